// C ABI of libffg: Pauli propagation (ffg_pauli_propagate) and the capture
// of dropped partners (ffg_pauli_propagate_capture, ffg_drops_*).
#include "ffg_engine_impl.cuh"


namespace {
// Body of ffg_pauli_propagate; with `capture` the orbit kernels also record
// the partners the degree filter drops (ctx->capture is set by the caller)
// and every commuting run goes through the orbit path.
int pauli_propagate_impl(ffg_ctx* ctx, const uint64_t* keys, const double* re, const double* im,
                         size_t n, const ffg_pauli_gate* gates, size_t ngates,
                         const ffg_pauli_params* params, int on_device, ffg_result** out, bool capture) {
    try {
        auto t0 = std::chrono::steady_clock::now();
        reset_profile(ctx);
        CK(cudaSetDevice(ctx->device));
        // validate gates; pick the key width
        bool wide = false;
        for (size_t i = 0; i < ngates; i++) {
            const ffg_pauli_gate& G = gates[i];
            if (G.kind < FFG_ROT || G.kind > FFG_CZ)
                return set_err(ctx, FFG_ERR_ARG, "gate " + std::to_string(i) + ": unknown kind");
            if (G.kind == FFG_ROT) {
                if (G.x[1] || G.z[1]) wide = true;
            } else {
                const bool two = G.kind >= FFG_CNOT;
                if (G.q0 < 0 || G.q0 >= 128 || (two && (G.q1 < 0 || G.q1 >= 128)))
                    return set_err(ctx, FFG_ERR_ARG, "gate " + std::to_string(i) + ": qubit index out of range");
                if (G.q0 >= 64 || (two && G.q1 >= 64)) wide = true;
            }
        }
        // complex mode when some coefficient has an imaginary part, or is not
        // finite (the real-mode reduction of the update holds for finite values)
        bool cplx = false;
        std::vector<uint64_t> hk;
        if (!on_device) {
            for (size_t i = 0; i < n && !wide; i++)
                if (keys[n + i] || keys[3 * n + i]) wide = true;
            for (size_t i = 0; i < n && !cplx; i++)
                if (!std::isfinite(re[i]) || (im && im[i] != 0.0)) cplx = true;
        } else {
            // device input: inspect on the host (one copy of the key planes)
            hk.resize(4 * n);
            std::vector<double> hre(n), him(n);
            if (n) {
                CK(cudaMemcpy(hk.data(), keys, 4 * n * 8, cudaMemcpyDeviceToHost));
                CK(cudaMemcpy(hre.data(), re, n * 8, cudaMemcpyDeviceToHost));
                if (im) CK(cudaMemcpy(him.data(), im, n * 8, cudaMemcpyDeviceToHost));
            }
            for (size_t i = 0; i < n && !wide; i++)
                if (hk[n + i] || hk[3 * n + i]) wide = true;
            for (size_t i = 0; i < n && !cplx; i++)
                if (!std::isfinite(hre[i]) || (im && him[i] != 0.0)) cplx = true;
        }
        const int nw = wide ? 2 : 1;
        std::vector<Op> ops;
        std::vector<RotArgs> rots;
        std::vector<TruncArgs> truncs;
        std::vector<GArgs> groups;
        std::vector<BatchInfo> binfo;
        std::vector<int> rot_gates;
        build_pauli_ops(gates, ngates, *params, nw, ops, rots, truncs, nullptr, &groups, ctx->group_d,
                        &binfo, capture ? &rot_gates : nullptr);
        int64_t nrot = 0;
        for (const auto& gr : groups) nrot += gr.ng;
        ctx->prof.n_gates = nrot;
        int rc = upload_cliffords(ctx, gates, ngates);
        if (rc) return rc;
        const bool det = params->deterministic != 0;
        const std::vector<int>* rg = capture ? &rot_gates : nullptr;
        const int min_gates = ctx->orbit_min_gates;
        if (capture) ctx->orbit_min_gates = 1;  // every run through the orbit kernels (they record)
        if (nw == 1 && !cplx)
            rc = run_engine<2, false, true>(ctx, keys, re, im, n, on_device, ops, rots, truncs, groups, det, out,
                                                &binfo, params->maxdegree, nullptr, rg);
        else if (nw == 1)
            rc = run_engine<2, true, true>(ctx, keys, re, im, n, on_device, ops, rots, truncs, groups, det, out,
                                                &binfo, params->maxdegree, nullptr, rg);
        else if (!cplx)
            rc = run_engine<4, false, true>(ctx, keys, re, im, n, on_device, ops, rots, truncs, groups, det, out,
                                                &binfo, params->maxdegree, nullptr, rg);
        else
            rc = run_engine<4, true, true>(ctx, keys, re, im, n, on_device, ops, rots, truncs, groups, det, out,
                                                &binfo, params->maxdegree, nullptr, rg);
        ctx->orbit_min_gates = min_gates;
        ctx->prof.seconds_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return rc;
    } catch (const std::exception& ex) {
        return set_err(ctx, FFG_ERR_STATE, ex.what());
    }
}

// keeps the capture records that are not repeats (gate >= 0), in any order
__global__ void capture_compact(CaptureArgs cp, u64 n, u64* key, double* re, double* im, int32_t* gate,
                                size_t stride, unsigned long long* cnt) {
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
        const int g = cp.gate[i];
        if (g < 0) continue;
        const u64 j = atomicAdd(cnt, 1ull);
        for (int w = 0; w < 4; w++) key[w * stride + j] = cp.key[(u64)w * cp.cap + i];
        re[j] = cp.re[i];
        im[j] = cp.im[i];
        gate[j] = g;
    }
}
}  // namespace

struct ffg_drops {
    int device = 0;
    size_t n = 0;
    u64* key = nullptr;     // [4][n] caller layout
    double* re = nullptr;
    double* im = nullptr;
    int32_t* gate = nullptr;
};

int ffg_pauli_propagate(ffg_ctx* ctx, const uint64_t* keys, const double* re, const double* im,
                        size_t n, const ffg_pauli_gate* gates, size_t ngates,
                        const ffg_pauli_params* params, int on_device, ffg_result** out) {
    if (!ctx || !out || !params || (n && (!keys || !re)) || (ngates && !gates)) return FFG_ERR_ARG;
    *out = nullptr;
    return pauli_propagate_impl(ctx, keys, re, im, n, gates, ngates, params, on_device, out, false);
}

void ffg_drops_free(ffg_drops* d) {
    if (!d) return;
    cudaSetDevice(d->device);
    if (d->key) cudaFree(d->key);
    if (d->re) cudaFree(d->re);
    if (d->im) cudaFree(d->im);
    if (d->gate) cudaFree(d->gate);
    delete d;
}

int ffg_pauli_propagate_capture(ffg_ctx* ctx, const uint64_t* keys, const double* re, const double* im,
                                size_t n, const ffg_pauli_gate* gates, size_t ngates,
                                const ffg_pauli_params* params, int on_device, int32_t capdeg, double min_abs,
                                ffg_result** out, ffg_drops** drops) {
    if (!ctx || !out || !drops || !params || (n && (!keys || !re)) || (ngates && !gates)) return FFG_ERR_ARG;
    *out = nullptr;
    *drops = nullptr;
    if (!params->batched || params->topk > 0)
        return set_err(ctx, FFG_ERR_ARG, "capture needs batched mode without top-k truncation");
    if (!(min_abs >= 0.0)) return set_err(ctx, FFG_ERR_ARG, "capture: min_abs must be >= 0");
    if (ctx->merge_sort || !ctx->orbit || !ctx->persistent || ctx->group_d != 1)
        return set_err(ctx, FFG_ERR_ARG, "capture needs the orbit path (merge_sort off, no FFG_* overrides)");
    if (capdeg <= params->maxdegree) return set_err(ctx, FFG_ERR_ARG, "capture: capdeg must exceed maxdegree");
    try {
        CK(cudaSetDevice(ctx->device));
        u64 cap = 1ull << 16;
        for (int attempt = 0; attempt < 8; attempt++) {
            const size_t need = align256(4 * cap * 8) + 2 * align256(cap * 8) + align256(cap * 4) +
                                align256(2 * cap * 4) + 256 + align256(sizeof(CaptureArgs));
            int rc = ensure_buf(ctx, ctx->capbuf, need);
            if (rc) return rc;
            char* p = ctx->capbuf.p;
            CaptureArgs cp{};
            cp.key = (u64*)p;
            p += align256(4 * cap * 8);
            cp.re = (double*)p;
            p += align256(cap * 8);
            cp.im = (double*)p;
            p += align256(cap * 8);
            cp.gate = (int*)p;
            p += align256(cap * 4);
            cp.slot = (u32*)p;
            p += align256(2 * cap * 4);
            cp.n = (u64*)p;
            cp.cap = cap;
            cp.maxdeg = capdeg;
            cp.min_abs = min_abs;
            CK(cudaMemsetAsync(cp.slot, 0, 2 * cap * 4 + 256, ctx->stream));  // index and counter
            CaptureArgs* cdev = (CaptureArgs*)(p + 256);
            CK(cudaMemcpyAsync(cdev, &cp, sizeof cp, cudaMemcpyHostToDevice, ctx->stream));
            ctx->capture = cp;
            ctx->capture_dev = cdev;
            ffg_result* r = nullptr;
            rc = pauli_propagate_impl(ctx, keys, re, im, n, gates, ngates, params, on_device, &r, true);
            ctx->capture = CaptureArgs{};
            ctx->capture_dev = nullptr;
            if (rc) return rc;
            u64 claimed = 0;
            CK(cudaMemcpyAsync(&claimed, cp.n, 8, cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaStreamSynchronize(ctx->stream));
            if (claimed > cap) {  // too small: run again with room for every record
                ffg_result_free(r);
                cap = pow2_at_least(2 * claimed);
                continue;
            }
            auto* d = new ffg_drops();
            std::unique_ptr<ffg_drops, void (*)(ffg_drops*)> guard(d, ffg_drops_free);
            d->device = ctx->device;
            const size_t m = std::max<u64>(claimed, 1);
            CK(cudaMalloc(&d->key, 4 * m * 8));
            CK(cudaMalloc(&d->re, m * 8));
            CK(cudaMalloc(&d->im, m * 8));
            CK(cudaMalloc(&d->gate, m * 4));
            unsigned long long* cnt = (unsigned long long*)cp.n;  // reused as the compaction counter
            CK(cudaMemsetAsync(cnt, 0, 8, ctx->stream));
            if (claimed) {
                capture_compact<<<grid_for(ctx, claimed), kBlock, 0, ctx->stream>>>(cp, claimed, d->key, d->re, d->im,
                                                                                   d->gate, m, cnt);
                CK(cudaGetLastError());
            }
            u64 kept = 0;
            CK(cudaMemcpyAsync(&kept, cnt, 8, cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaStreamSynchronize(ctx->stream));
            d->n = kept;
            // key planes were written with stride m; keep that stride as the
            // capacity and report kept entries
            if (kept != m && kept) {
                // repack the planes to stride kept
                u64* k2 = nullptr;
                CK(cudaMalloc(&k2, 4 * kept * 8));
                for (int w = 0; w < 4; w++)
                    CK(cudaMemcpyAsync(k2 + (size_t)w * kept, d->key + (size_t)w * m, kept * 8,
                                       cudaMemcpyDeviceToDevice, ctx->stream));
                CK(cudaStreamSynchronize(ctx->stream));
                cudaFree(d->key);
                d->key = k2;
            }
            *out = r;
            *drops = guard.release();
            return FFG_OK;
        }
        return set_err(ctx, FFG_ERR_STATE, "capture: record buffer kept overflowing");
    } catch (const std::exception& ex) {
        return set_err(ctx, FFG_ERR_STATE, ex.what());
    }
}

size_t ffg_drops_size(const ffg_drops* d) { return d ? d->n : 0; }

int ffg_drops_device(const ffg_drops* d, const uint64_t** keys, size_t* stride, const double** re,
                     const double** im, const int32_t** gate) {
    if (!d) return FFG_ERR_ARG;
    if (keys) *keys = (const uint64_t*)d->key;
    if (stride) *stride = d->n;
    if (re) *re = d->re;
    if (im) *im = d->im;
    if (gate) *gate = d->gate;
    return FFG_OK;
}

int ffg_drops_copy(const ffg_drops* d, uint64_t* keys, double* re, double* im, int32_t* gate) {
    if (!d || (d->n && (!keys || !re))) return FFG_ERR_ARG;
    const size_t n = d->n;
    if (!n) return FFG_OK;
    if (cudaSetDevice(d->device) != cudaSuccess) return FFG_ERR_CUDA;
    std::vector<u64> k(4 * n);
    std::vector<double> r(n), i(n);
    std::vector<int32_t> g(n);
    if (cudaMemcpy(k.data(), d->key, 4 * n * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(r.data(), d->re, n * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(i.data(), d->im, n * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(g.data(), d->gate, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
        return FFG_ERR_CUDA;
    // deterministic order: by gate, then key words 0..3
    std::vector<size_t> ord(n);
    for (size_t t = 0; t < n; t++) ord[t] = t;
    std::sort(ord.begin(), ord.end(), [&](size_t a, size_t b) {
        if (g[a] != g[b]) return g[a] < g[b];
        for (int w = 0; w < 4; w++)
            if (k[w * n + a] != k[w * n + b]) return k[w * n + a] < k[w * n + b];
        return false;
    });
    for (size_t t = 0; t < n; t++) {
        const size_t s = ord[t];
        for (int w = 0; w < 4; w++) keys[w * n + t] = k[w * n + s];
        re[t] = r[s];
        if (im) im[t] = i[s];
        if (gate) gate[t] = g[s];
    }
    return FFG_OK;
}
