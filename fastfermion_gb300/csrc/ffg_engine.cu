// C ABI of libffg (include/ffg.h): contexts, profiling, results and their
// expectation values, the schedule query and the engine options.  The
// propagation entry points live in ffg_pauli.cu, ffg_majorana.cu,
// ffg_batch.cu and ffg_convert.cu; all share ffg_engine_impl.cuh.
#include "ffg_engine_impl.cuh"


// ===========================================================================
// C ABI (C linkage comes from the declarations in ffg.h)
// ===========================================================================

int ffg_create(ffg_ctx** out, int device) {
    if (!out) return FFG_ERR_ARG;
    *out = nullptr;
    ffg_ctx* ctx = new ffg_ctx();
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_ctr, sizeof(DevCounters));
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->h_ctr, sizeof(DevCounters));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_part, 2 * kMaxParts * sizeof(double) + 2 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_hist, 256 * 8);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_ps, sizeof(PersistState));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_oc, sizeof(OrbitCounters));
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->h_oc, sizeof(OrbitCounters));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_ocw, kOrbitWindowMax * sizeof(OrbitCounters));
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->h_ocw, kOrbitWindowMax * sizeof(OrbitCounters));
    if (e != cudaSuccess) {
        fprintf(stderr, "ffg_create: %s\n", cudaGetErrorString(e));
        ffg_destroy(ctx);
        return FFG_ERR_CUDA;
    }
    *out = ctx;
    return FFG_OK;
}

int ffg_destroy(ffg_ctx* ctx) {
    if (!ctx) return FFG_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (auto& b : ctx->buf)
        if (b.p) cudaFree(b.p);
    if (ctx->d_cliff) cudaFree(ctx->d_cliff);
    if (ctx->d_part) cudaFree(ctx->d_part);
    if (ctx->d_hist) cudaFree(ctx->d_hist);
    if (ctx->d_ties) cudaFree(ctx->d_ties);
    if (ctx->d_ps) cudaFree(ctx->d_ps);
    if (ctx->d_ops) cudaFree(ctx->d_ops);
    if (ctx->d_pairs) cudaFree(ctx->d_pairs);
    if (ctx->d_mrots) cudaFree(ctx->d_mrots);
    if (ctx->d_truncs) cudaFree(ctx->d_truncs);
    if (ctx->d_groups2) cudaFree(ctx->d_groups2);
    if (ctx->d_bgates) cudaFree(ctx->d_bgates);
    if (ctx->d_mgates) cudaFree(ctx->d_mgates);
    if (ctx->d_qidx) cudaFree(ctx->d_qidx);
    if (ctx->d_smscratch) cudaFree(ctx->d_smscratch);
    if (ctx->d_oscratch) cudaFree(ctx->d_oscratch);
    if (ctx->bigpool.p) cudaFree(ctx->bigpool.p);
    if (ctx->capbuf.p) cudaFree(ctx->capbuf.p);
    if (ctx->d_oc) cudaFree(ctx->d_oc);
    if (ctx->h_oc) cudaFreeHost(ctx->h_oc);
    if (ctx->d_ocw) cudaFree(ctx->d_ocw);
    if (ctx->h_ocw) cudaFreeHost(ctx->h_ocw);
    if (ctx->d_ctr) cudaFree(ctx->d_ctr);
    if (ctx->h_ctr) cudaFreeHost(ctx->h_ctr);
    for (auto e : ctx->free_events) cudaEventDestroy(e);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return FFG_OK;
}

const char* ffg_last_error(const ffg_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int ffg_set_profiling(ffg_ctx* ctx, int enabled) {
    if (!ctx) return FFG_ERR_ARG;
    ctx->profiling = enabled != 0;
    return FFG_OK;
}

int ffg_profile_get(const ffg_ctx* ctx, ffg_profile* out) {
    if (!ctx || !out) return FFG_ERR_ARG;
    *out = ctx->prof;
    return FFG_OK;
}

void* ffg_stream(const ffg_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

size_t ffg_result_size(const ffg_result* r) { return r ? r->n : 0; }
int ffg_result_kind(const ffg_result* r) { return r ? r->kind : 0; }

int ffg_result_copy(const ffg_result* r, uint64_t* keys, double* re, double* im) {
    if (!r) return FFG_ERR_ARG;
    ffg_ctx* ctx = r->ctx;
    auto t0 = std::chrono::steady_clock::now();
    cudaSetDevice(r->device);
    const size_t n = r->n;
    if (!r->deterministic) {
        // direct plane copies into the caller's layout
        if (n) {
            for (int w = 0; w < r->nplanes; w++) {
                int dst = w;
                if (r->kind == 1) {
                    const int nw = r->nplanes / 2;
                    dst = (w < nw) ? w : 2 + (w - nw);
                }
                CK(cudaMemcpyAsync(keys + (size_t)dst * n, r->key + (size_t)w * n, n * 8,
                                   cudaMemcpyDeviceToHost, ctx->stream));
            }
            for (int w = 0; w < 4; w++) {
                bool used = false;
                for (int v = 0; v < r->nplanes; v++) {
                    int dst = v;
                    if (r->kind == 1) {
                        const int nw = r->nplanes / 2;
                        dst = (v < nw) ? v : 2 + (v - nw);
                    }
                    used = used || dst == w;
                }
                if (!used) std::memset(keys + (size_t)w * n, 0, n * 8);
            }
            CK(cudaMemcpyAsync(re, r->re, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
            if (im) {
                if (r->cplx)
                    CK(cudaMemcpyAsync(im, r->im, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
                else
                    std::memset(im, 0, n * 8);
            }
            CK(cudaStreamSynchronize(ctx->stream));
        }
    } else {
        std::vector<uint64_t> k4;
        std::vector<double> hr, hi;
        int rc = result_to_host(r, k4, hr, hi);
        if (rc) return rc;
        if (n) {
            std::memcpy(keys, k4.data(), 4 * n * 8);
            std::memcpy(re, hr.data(), n * 8);
            if (im) std::memcpy(im, hi.data(), n * 8);
        }
    }
    ctx->prof.seconds_d2h += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return FFG_OK;
}

int ffg_result_device(const ffg_result* r, const uint64_t** keys, size_t* stride, int* nplanes,
                      const double** re, const double** im) {
    if (!r) return FFG_ERR_ARG;
    if (keys) *keys = (const uint64_t*)r->key;
    if (stride) *stride = r->n;
    if (nplanes) *nplanes = r->nplanes;
    if (re) *re = r->re;
    if (im) *im = r->cplx ? r->im : nullptr;
    return FFG_OK;
}

namespace {
template <int KW, bool CPLX>
void launch_expect(const ffg_result* r, StoreView v, int mode, int nw, u64 b0, u64 b1, int parts) {
    ffg_ctx* ctx = r->ctx;
    expect_kernel<KW, CPLX><<<parts, kBlock, 0, ctx->stream>>>(v, r->n, mode, nw, b0, b1, ctx->d_part,
                                                               ctx->d_part + kMaxParts);
}

int result_expect(const ffg_result* r, int mode, const uint64_t* b, double* ore, double* oim) {
    if (!r || !ore || !oim) return FFG_ERR_ARG;
    ffg_ctx* ctx = r->ctx;
    cudaSetDevice(r->device);
    const u64 b0 = b ? b[0] : 0, b1 = b ? b[1] : 0;
    if (r->deterministic) {
        std::vector<uint64_t> k4;
        std::vector<double> hr, hi;
        int rc = result_to_host(r, k4, hr, hi);
        if (rc) return rc;
        const size_t n = r->n;
        double sr = 0.0, si = 0.0;
        for (size_t i = 0; i < n; i++) {
            double vr = 0.0, vi = 0.0;
            bool use = false;
            if (mode == 0) {
                if (k4[i] == 0 && k4[n + i] == 0) {
                    const int par = popc64(k4[2 * n + i] & b0) + popc64(k4[3 * n + i] & b1);
                    const double sg = (par & 1) ? -1.0 : 1.0;
                    vr = hr[i] * sg - hi[i] * 0.0;
                    vi = hr[i] * 0.0 + hi[i] * sg;
                    use = true;
                }
            } else {
                bool paired = true;
                u64 J[2] = {0, 0};
                for (int w = 0; w < 4; w++) {
                    const u64 x = k4[(size_t)w * n + i];
                    const u64 ev = x & 0x5555555555555555ull, od = (x >> 1) & 0x5555555555555555ull;
                    paired = paired && ev == od;
                    u64 pj = 0;
                    for (int t = 0; t < 32; t++) pj |= ((ev >> (2 * t)) & 1ull) << t;
                    J[w >> 1] |= pj << (32 * (w & 1));
                }
                if (paired) {
                    const int ex = popc64(J[0]) + popc64(J[1]) + 2 * (popc64(J[0] & b0) + popc64(J[1] & b1));
                    double pr = 1.0, pi = 0.0;
                    switch (ex & 3) {
                        case 1: pr = 0.0; pi = 1.0; break;
                        case 2: pr = -1.0; pi = 0.0; break;
                        case 3: pr = 0.0; pi = -1.0; break;
                        default: break;
                    }
                    vr = hr[i] * pr - hi[i] * pi;
                    vi = hr[i] * pi + hi[i] * pr;
                    use = true;
                }
            }
            if (use) {
                sr = sr + vr;
                si = si + vi;
            }
        }
        *ore = sr;
        *oim = si;
        return FFG_OK;
    }
    StoreView v{};
    v.key = r->key;
    v.re = r->re;
    v.im = r->im;
    v.dead = r->dead;
    v.cap = r->n;
    const int parts = (int)std::max<u64>(1, std::min<u64>((r->n + kBlock - 1) / kBlock, kMaxParts));
    const int nw = r->kind == 1 ? r->nplanes / 2 : 0;
    if (r->kind == 1) {
        if (r->nplanes == 2 && !r->cplx) launch_expect<2, false>(r, v, mode, nw, b0, b1, parts);
        else if (r->nplanes == 2) launch_expect<2, true>(r, v, mode, nw, b0, b1, parts);
        else if (!r->cplx) launch_expect<4, false>(r, v, mode, nw, b0, b1, parts);
        else launch_expect<4, true>(r, v, mode, nw, b0, b1, parts);
    } else {
        switch (r->nplanes) {
            case 1: launch_expect<1, true>(r, v, mode, nw, b0, b1, parts); break;
            case 2: launch_expect<2, true>(r, v, mode, nw, b0, b1, parts); break;
            case 3: launch_expect<3, true>(r, v, mode, nw, b0, b1, parts); break;
            default: launch_expect<4, true>(r, v, mode, nw, b0, b1, parts); break;
        }
    }
    double* d_out = ctx->d_part + 2 * kMaxParts;
    expect_final_kernel<<<1, 32, 0, ctx->stream>>>(ctx->d_part, ctx->d_part + kMaxParts, parts, d_out);
    double h[2];
    CK(cudaMemcpyAsync(h, d_out, 16, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    *ore = h[0];
    *oim = h[1];
    return FFG_OK;
}
}  // namespace

int ffg_result_overlapwithzero(const ffg_result* r, double* re, double* im) {
    if (!r || r->kind != 1) return FFG_ERR_ARG;
    return result_expect(r, 0, nullptr, re, im);
}

int ffg_result_qubit_state(const ffg_result* r, const uint64_t* b, double* re, double* im) {
    if (!r || r->kind != 1) return FFG_ERR_ARG;
    return result_expect(r, 0, b, re, im);
}

int ffg_result_fock_state(const ffg_result* r, const uint64_t* b, double* re, double* im) {
    if (!r || r->kind != 2) return FFG_ERR_ARG;
    return result_expect(r, 1, b, re, im);
}

void ffg_result_free(ffg_result* r) {
    if (!r) return;
    cudaSetDevice(r->device);
    if (r->key) cudaFree(r->key);
    if (r->re) cudaFree(r->re);
    if (r->im) cudaFree(r->im);
    if (r->dead) cudaFree(r->dead);
    delete r;
}

int ffg_abs_le(double re, double im, double tau) { return abs_le(re, im, tau) ? 1 : 0; }

int64_t ffg_pauli_schedule(const ffg_pauli_gate* gates, size_t ngates, int batched, int64_t* sizes,
                           int64_t cap) {
    ffg_pauli_params p{};
    p.maxdegree = 128;
    p.batched = batched;
    p.mincoeff = 1.0;  // force a truncation op after every batch
    std::vector<Op> ops;
    std::vector<RotArgs> rots;
    std::vector<TruncArgs> truncs;
    std::vector<int64_t> b;
    build_pauli_ops(gates, ngates, p, 2, ops, rots, truncs, &b);
    for (int64_t i = 0; i < (int64_t)b.size() && i < cap; i++) sizes[i] = b[i];
    return (int64_t)b.size();
}


// ---------------------------------------------------------------------------
// engine options (the tuning knobs; defaults as measured on GB300)
// ---------------------------------------------------------------------------
namespace {
struct OptionRef {
    const char* name;
    int (*get)(const ffg_ctx*);
    bool (*set)(ffg_ctx*, int64_t);
};
const OptionRef kOptions[] = {
    {"orbit_route_big", [](const ffg_ctx* c) { return c->orbit_route_big; },
     [](ffg_ctx* c, int64_t v) { if (v < 1 || v > 1 << 20) return false; c->orbit_route_big = (int)v; return true; }},
    {"orbit_team", [](const ffg_ctx* c) { return (int)c->orbit_team; },
     [](ffg_ctx* c, int64_t v) { c->orbit_team = v != 0; return true; }},
    {"orbit_window", [](const ffg_ctx* c) { return c->orbit_window; },
     [](ffg_ctx* c, int64_t v) { if (v < 1 || v > kOrbitWindowMax) return false; c->orbit_window = (int)v; return true; }},
    {"orbit_min_gates", [](const ffg_ctx* c) { return c->orbit_min_gates; },
     [](ffg_ctx* c, int64_t v) { if (v < 1) return false; c->orbit_min_gates = (int)v; return true; }},
    {"orbit_qidx", [](const ffg_ctx* c) { return (int)c->orbit_qidx; },
     [](ffg_ctx* c, int64_t v) { c->orbit_qidx = v != 0; return true; }},
    {"pdl", [](const ffg_ctx* c) { return (int)c->pdl; }, [](ffg_ctx* c, int64_t v) { c->pdl = v != 0; return true; }},
    {"morbit", [](const ffg_ctx* c) { return (int)c->morbit; },
     [](ffg_ctx* c, int64_t v) { c->morbit = v != 0; return true; }},
    {"orbit_team_threads", [](const ffg_ctx* c) { return c->orbit_team_threads; },
     [](ffg_ctx* c, int64_t v) { if (v != 128 && v != 256) return false; c->orbit_team_threads = (int)v; return true; }},
    {"orbit_block_threads", [](const ffg_ctx* c) { return c->orbit_block_threads; },
     [](ffg_ctx* c, int64_t v) { if (v != 512 && v != 1024) return false; c->orbit_block_threads = (int)v; return true; }},
    {"merge_sort", [](const ffg_ctx* c) { return (int)c->merge_sort; },
     [](ffg_ctx* c, int64_t v) { c->merge_sort = v != 0; return true; }},
    {"morbit_min_gates", [](const ffg_ctx* c) { return c->morbit_min_gates; },
     [](ffg_ctx* c, int64_t v) { if (v < 1) return false; c->morbit_min_gates = (int)v; return true; }},
    {"morbit_route_big", [](const ffg_ctx* c) { return c->morbit_route_big; },
     [](ffg_ctx* c, int64_t v) { if (v < 1 || v > 1 << 20) return false; c->morbit_route_big = (int)v; return true; }},
    {"min_capacity", [](const ffg_ctx* c) { return (int)c->min_capacity; },
     [](ffg_ctx* c, int64_t v) {
         if (v < 64 || v > (1ll << 30) || (v & (v - 1))) return false;
         c->min_capacity = (u64)v;
         return true;
     }},
    {"barrier_limit_kcycles", [](const ffg_ctx* c) { return (int)(c->barrier_limit / 1000); },
     [](ffg_ctx* c, int64_t v) {
         if (v < 1 || v > kBarrierLimitCycles / 1000) return false;
         c->barrier_limit = v * 1000;
         return true;
     }},
    {"persistent", [](const ffg_ctx* c) { return (int)c->persistent; },
     [](ffg_ctx* c, int64_t v) { c->persistent = v != 0; return true; }},
    {"orbit", [](const ffg_ctx* c) { return (int)c->orbit; }, [](ffg_ctx* c, int64_t v) { c->orbit = v != 0; return true; }},
    {"group_d", [](const ffg_ctx* c) { return c->group_d; },
     [](ffg_ctx* c, int64_t v) { if (v < 1 || v > kGroupD) return false; c->group_d = (int)v; return true; }},
    {"persist_blocks_per_sm", [](const ffg_ctx* c) { return c->persist_blocks_per_sm; },
     [](ffg_ctx* c, int64_t v) { if (v < 1 || v > 8) return false; c->persist_blocks_per_sm = (int)v; return true; }},
    {"orbit_stats", [](const ffg_ctx* c) { return (int)c->orbit_stats; },
     [](ffg_ctx* c, int64_t v) { c->orbit_stats = v != 0; return true; }},
    {"store_headroom", [](const ffg_ctx* c) { return c->store_headroom; },
     [](ffg_ctx* c, int64_t v) {
         if (v < 1 || v > 64) return false;
         c->store_headroom = (int)v;
         return true;
     }},
    {"group_region_cap", [](const ffg_ctx* c) { return (int)c->group_region_cap; },
     [](ffg_ctx* c, int64_t v) {
         if (v < 64 || v > (1ll << 24) || (v & (v - 1))) return false;
         c->group_region_cap = (u64)v;
         return true;
     }},
};
}  // namespace

int ffg_set_option(ffg_ctx* ctx, const char* name, int64_t value) {
    if (!ctx || !name) return FFG_ERR_ARG;
    for (const OptionRef& o : kOptions)
        if (std::strcmp(o.name, name) == 0)
            return o.set(ctx, value) ? FFG_OK : set_err(ctx, FFG_ERR_ARG, std::string("bad value for ") + name);
    return set_err(ctx, FFG_ERR_ARG, std::string("unknown option ") + name);
}

int ffg_get_option(const ffg_ctx* ctx, const char* name, int64_t* value) {
    if (!ctx || !name || !value) return FFG_ERR_ARG;
    for (const OptionRef& o : kOptions)
        if (std::strcmp(o.name, name) == 0) {
            *value = o.get(ctx);
            return FFG_OK;
        }
    return FFG_ERR_ARG;
}
