// C ABI of libffg: batched instances (ffg_pauli_propagate_batched,
// ffg_pauli_propagate_instances) and the adjoint gradient (ffg_batch_*).
#include "ffg_engine_impl.cuh"


// ---------------------------------------------------------------------------
// batched instances and the adjoint
// ---------------------------------------------------------------------------
int ffg_pauli_propagate_batched(ffg_ctx* ctx, const uint64_t* keys, const double* re, size_t n,
                                const ffg_pauli_gate* gates, size_t ngates, const ffg_pauli_params* params,
                                const ffg_batch_params* bp, double* expect, ffg_batch** out) {
    return ffg_pauli_propagate_instances(ctx, keys, re, n, gates, ngates, params, bp, nullptr, expect, out);
}

int ffg_pauli_propagate_instances(ffg_ctx* ctx, const uint64_t* keys, const double* re, size_t n,
                                  const ffg_pauli_gate* gates, size_t ngates, const ffg_pauli_params* params,
                                  const ffg_batch_params* bp, const uint64_t* active, double* expect,
                                  ffg_batch** out) {
    if (!ctx || !params || !bp || !expect || (n && (!keys || !re)) || (ngates && !gates)) return FFG_ERR_ARG;
    if (out) *out = nullptr;
    const size_t ninst = bp->ninst;
    if (ninst == 0 || !bp->offsets) return set_err(ctx, FFG_ERR_ARG, "batched propagation: no instances");
    if (bp->offsets[0] != 0 || (size_t)bp->offsets[ninst] != n)
        return set_err(ctx, FFG_ERR_ARG, "batched propagation: offsets must start at 0 and end at n");
    for (size_t i = 0; i < ninst; i++)
        if (bp->offsets[i + 1] < bp->offsets[i])
            return set_err(ctx, FFG_ERR_ARG, "batched propagation: offsets must be non-decreasing");
    if (params->topk > 0) return set_err(ctx, FFG_ERR_ARG, "batched propagation does not support top-k truncation");
    if (params->max_xweight >= 0)
        return set_err(ctx, FFG_ERR_ARG, "batched propagation does not support X-weight truncation");
    if (bp->checkpoint_every < 0) return set_err(ctx, FFG_ERR_ARG, "checkpoint_every must be >= 0");
    if (active && bp->checkpoint_every > 0)
        return set_err(ctx, FFG_ERR_ARG, "per-instance active rotations do not support the adjoint");
    if (ctx->group_d != 1 || !ctx->orbit || !ctx->persistent)
        return set_err(ctx, FFG_ERR_ARG, "batched propagation needs the orbit and persistent paths (FFG_* overrides)");
    for (size_t i = 0; i < n; i++)
        if (!std::isfinite(re[i])) return set_err(ctx, FFG_ERR_ARG, "batched propagation needs finite coefficients");
    try {
        auto t0 = std::chrono::steady_clock::now();
        reset_profile(ctx);
        CK(cudaSetDevice(ctx->device));
        // qubits in use
        int nq = 0;
        size_t nrot = 0;
        auto use_bits = [&](uint64_t w, int word) {
            if (w) nq = std::max(nq, 64 * word + 64 - __builtin_clzll(w));
        };
        for (size_t i = 0; i < ngates; i++) {
            const ffg_pauli_gate& G = gates[i];
            if (G.kind < FFG_ROT || G.kind > FFG_CZ)
                return set_err(ctx, FFG_ERR_ARG, "gate " + std::to_string(i) + ": unknown kind");
            if (G.kind == FFG_ROT) {
                nrot++;
                for (int w = 0; w < 2; w++) {
                    use_bits(G.x[w], w);
                    use_bits(G.z[w], w);
                }
            } else {
                const bool two = G.kind >= FFG_CNOT;
                if (G.q0 < 0 || G.q0 >= 128 || (two && (G.q1 < 0 || G.q1 >= 128)))
                    return set_err(ctx, FFG_ERR_ARG, "gate " + std::to_string(i) + ": qubit index out of range");
                nq = std::max(nq, G.q0 + 1);
                if (two) nq = std::max(nq, G.q1 + 1);
            }
        }
        for (size_t i = 0; i < n; i++)
            for (int w = 0; w < 2; w++) {
                use_bits(keys[w * n + i], w);
                use_bits(keys[(2 + w) * n + i], w);
            }
        int b = 1;
        while (((size_t)1 << b) < ninst) b++;
        // instance code: x bits [shift, shift+b) of caller word `word`, complement in z
        int word, shift;
        if (nq + b <= 64) {
            word = 0;
            shift = nq;
        } else if (nq <= 64) {
            word = 1;
            shift = 0;
        } else if (nq + b <= 128) {
            word = 1;
            shift = nq - 64;
        } else {
            return set_err(ctx, FFG_ERR_ARG, "batched propagation: no free key bits for the instance code");
        }
        const bool wide = word == 1 || nq > 64;
        const int kw = wide ? 4 : 2;
        const u64 imask = (b == 64) ? ~0ull : ((1ull << b) - 1);
        auto* h = new ffg_batch();
        h->ctx = ctx;
        h->kw = kw;
        h->ninst = ninst;
        h->nrot = nrot;
        h->n_input = n;
        h->every = bp->checkpoint_every;
        h->gates.assign(gates, gates + ngates);
        h->inst_word = word;
        for (int w = 0; w < 2; w++) {
            const int lo = 64 * w, hi = 64 * w + 64;
            const int q1 = std::min(nq, hi);
            u64 m = 0;
            for (int q = lo; q < q1; q++) m |= 1ull << (q - lo);
            h->xmask[w] = m;
        }
        h->maxdeg = params->maxdegree + b;
        h->bc.ninst = (u32)ninst;
        h->bc.inst_plane = wide ? word : 0;  // x plane of that word in store order
        h->bc.inst_shift = shift;
        h->bc.inst_mask = imask;
        std::unique_ptr<ffg_batch, void (*)(ffg_batch*)> guard(h, ffg_batch_free);
        // encoded keys
        std::vector<uint64_t> ek(keys, keys + 4 * n);
        for (size_t i = 0; i < ninst; i++)
            for (int64_t t = bp->offsets[i]; t < bp->offsets[i + 1]; t++) {
                ek[(size_t)word * n + t] |= (u64)i << shift;
                ek[(size_t)(2 + word) * n + t] |= ((~(u64)i) & imask) << shift;
            }
        // schedule with the instance bits counted in the degree filter
        ffg_pauli_params p = *params;
        p.maxdegree = h->maxdeg;
        build_pauli_ops(gates, ngates, p, wide ? 2 : 1, h->ops, h->rots, h->truncs, nullptr, &h->groups, 1,
                        &h->binfo);
        size_t nbg = 0;
        for (const Op& o : h->ops) nbg += o.type == Op::GROUP;
        if (nbg != nrot) return set_err(ctx, FFG_ERR_STATE, "batched propagation: schedule does not cover every rotation");
        ctx->prof.n_gates = (int64_t)nrot;
        // per-instance (cos, sin); batch gate b is circuit rotation nrot-1-b
        std::vector<double> theta_of_rot;
        for (size_t i = 0; i < ngates; i++)
            if (gates[i].kind == FFG_ROT) theta_of_rot.push_back(gates[i].theta);
        std::vector<double2> cs(nbg * ninst);
        for (size_t bgi = 0; bgi < nbg; bgi++) {
            const size_t rot = nrot - 1 - bgi;
            for (size_t i = 0; i < ninst; i++) {
                const double th = bp->thetas ? bp->thetas[i * nrot + rot] : theta_of_rot[rot];
                cs[bgi * ninst + i] = make_double2(std::cos(th), std::sin(th));
            }
        }
        CK(cudaMalloc(&h->d_inst_cs, std::max<size_t>(cs.size(), 1) * sizeof(double2)));
        if (!cs.empty())
            CK(cudaMemcpy(h->d_inst_cs, cs.data(), cs.size() * sizeof(double2), cudaMemcpyHostToDevice));
        h->bc.d_inst_cs = h->d_inst_cs;
        h->bc.nrot = (u32)nrot;
        if (active) {
            const size_t words = std::max<size_t>((nrot + 63) / 64, 1);
            CK(cudaMalloc(&h->d_active, ninst * words * 8));
            CK(cudaMemcpy(h->d_active, active, ninst * words * 8, cudaMemcpyHostToDevice));
            h->bc.d_active = h->d_active;
            h->bc.active_words = (u32)words;
        }
        int rc = upload_cliffords(ctx, gates, ngates);
        if (rc) return rc;
        rc = kw == 2 ? batch_forward<2>(h, ek.data(), re, n, expect) : batch_forward<4>(h, ek.data(), re, n, expect);
        ctx->prof.seconds_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (rc) return rc;
        if (out) *out = guard.release();
        return FFG_OK;
    } catch (const std::exception& ex) {
        return set_err(ctx, FFG_ERR_STATE, ex.what());
    }
}

size_t ffg_batch_size(const ffg_batch* h) { return h ? (size_t)h->fn : 0; }

int ffg_batch_copy(const ffg_batch* h, uint64_t* keys, double* re, int64_t* inst) {
    if (!h || (h->fn && (!keys || !re))) return FFG_ERR_ARG;
    ffg_ctx* ctx = h->ctx;
    const size_t n = h->fn;
    if (!n) return FFG_OK;
    std::vector<u64> k((size_t)h->kw * n);
    CK(cudaSetDevice(ctx->device));
    CK(cudaMemcpy(k.data(), h->fkey, k.size() * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(re, h->fre, n * 8, cudaMemcpyDeviceToHost));
    const int nw = h->kw / 2;
    const u64 code = h->bc.inst_mask << h->bc.inst_shift;
    for (size_t i = 0; i < n; i++) {
        u64 x[2] = {k[i], nw > 1 ? k[n + i] : 0};
        u64 z[2] = {k[(size_t)nw * n + i], nw > 1 ? k[(size_t)(nw + 1) * n + i] : 0};
        const int wd = h->inst_word;
        if (inst) inst[i] = (int64_t)((x[wd] >> h->bc.inst_shift) & h->bc.inst_mask);
        x[wd] &= ~code;
        z[wd] &= ~code;
        keys[i] = x[0];
        keys[n + i] = x[1];
        keys[2 * n + i] = z[0];
        keys[3 * n + i] = z[1];
    }
    return FFG_OK;
}

int ffg_batch_adjoint(ffg_batch* h, const double* weights, double* grad_theta, double* grad_coef) {
    if (!h || !weights || !grad_theta) return FFG_ERR_ARG;
    try {
        return h->kw == 2 ? batch_adjoint<2>(h, weights, grad_theta, grad_coef)
                          : batch_adjoint<4>(h, weights, grad_theta, grad_coef);
    } catch (const std::exception& ex) {
        return set_err(h->ctx, FFG_ERR_STATE, ex.what());
    }
}

void ffg_batch_free(ffg_batch* h) {
    if (!h) return;
    if (h->ctx) cudaSetDevice(h->ctx->device);
    for (AdjRecord& r : h->recs) free_record(r);
    if (h->fkey) cudaFree(h->fkey);
    if (h->fre) cudaFree(h->fre);
    if (h->d_inst_cs) cudaFree(h->d_inst_cs);
    if (h->d_active) cudaFree(h->d_active);
    delete h;
}
