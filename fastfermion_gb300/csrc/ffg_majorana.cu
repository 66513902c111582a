// C ABI of libffg: Majorana propagation (ffg_majorana_propagate).
#include "ffg_engine_impl.cuh"

int ffg_majorana_propagate(ffg_ctx* ctx, const uint64_t* keys, const double* re, const double* im,
                           size_t n, const ffg_majorana_gate* gates, size_t ngates,
                           const ffg_majorana_params* params, int on_device, ffg_result** out) {
    if (!ctx || !out || !params || (n && (!keys || !re)) || (ngates && !gates)) return FFG_ERR_ARG;
    *out = nullptr;
    try {
        auto t0 = std::chrono::steady_clock::now();
        reset_profile(ctx);
        CK(cudaSetDevice(ctx->device));
        int top = 0;  // highest plane used
        auto plane_of = [](const uint64_t* a4) {
            int t = 0;
            for (int w = 0; w < 4; w++)
                if (a4[w]) t = w;
            return t;
        };
        for (size_t i = 0; i < ngates; i++) top = std::max(top, plane_of(gates[i].alpha));
        std::vector<uint64_t> hk;
        const uint64_t* kp = keys;
        if (on_device && n) {
            hk.resize(4 * n);
            CK(cudaMemcpy(hk.data(), keys, 4 * n * 8, cudaMemcpyDeviceToHost));
            kp = hk.data();
        }
        for (size_t i = 0; i < n; i++)
            for (int w = 3; w > top; w--)
                if (kp[(size_t)w * n + i]) top = w;
        const int kw = top + 1;
        std::vector<Op> ops;
        std::vector<RotArgs> rots;
        std::vector<TruncArgs> truncs;
        TruncArgs t{};
        t.thr = params->mincoeff > 0;
        t.tau = params->mincoeff;
        t.max_xweight = -1;
        truncs.push_back(t);
        for (long long i = (long long)ngates - 1; i >= 0; i--) {
            const ffg_majorana_gate& G = gates[i];
            RotArgs a{};
            int deg = 0;
            for (int w = 0; w < 4; w++) {
                a.p[w] = G.alpha[w];
                deg += popc64(G.alpha[w]);
            }
            suffix_parity(G.alpha, a.mg);
            a.c = std::cos(G.theta);
            a.s = std::sin(G.theta);
            a.fr = G.r ? -a.s : 0.0;
            a.fi = G.r ? 0.0 : a.s;
            a.maxdeg = params->has_maxdegree ? params->maxdegree : 1 << 30;
            a.gate_odd = deg & 1;
            rots.push_back(a);
            ops.push_back({Op::ROT, (int)rots.size() - 1, 0, 0, 0});
            if (t.thr) ops.push_back({Op::TRUNC, 0, 0, 0, 0});
        }
        ctx->prof.n_gates = (int64_t)rots.size();
        // maximal runs of mutually commuting gates, application order
        // (commutation of Majorana strings: |a||b| - |a & b| even,
        // src/majorana_algebra.h:79-84)
        std::vector<std::pair<int, int>> runs;
        {
            auto commute = [&](const RotArgs& x, const RotArgs& y) {
                int dx = 0, dy = 0, dxy = 0;
                for (int w = 0; w < 4; w++) {
                    dx += popc64(x.p[w]);
                    dy += popc64(y.p[w]);
                    dxy += popc64(x.p[w] & y.p[w]);
                }
                return ((dx * dy - dxy) & 1) == 0;
            };
            int s0 = 0;
            for (int g = 1; g <= (int)rots.size(); g++) {
                bool ok = g < (int)rots.size();
                for (int u = s0; u < g && ok; u++) ok = commute(rots[u], rots[g]);
                if (!ok) {
                    runs.push_back({s0, g});
                    s0 = g;
                }
            }
        }
        const bool det = params->deterministic != 0;
        const int md = params->has_maxdegree ? params->maxdegree : 1 << 30;
        int rc;
        switch (kw) {
            case 1: rc = run_engine<1, true, false>(ctx, keys, re, im, n, on_device, ops, rots, truncs, {}, det, out, nullptr, md, &runs); break;
            case 2: rc = run_engine<2, true, false>(ctx, keys, re, im, n, on_device, ops, rots, truncs, {}, det, out, nullptr, md, &runs); break;
            case 3: rc = run_engine<3, true, false>(ctx, keys, re, im, n, on_device, ops, rots, truncs, {}, det, out, nullptr, md, &runs); break;
            default: rc = run_engine<4, true, false>(ctx, keys, re, im, n, on_device, ops, rots, truncs, {}, det, out, nullptr, md, &runs); break;
        }
        ctx->prof.seconds_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return rc;
    } catch (const std::exception& ex) {
        return set_err(ctx, FFG_ERR_STATE, ex.what());
    }
}
