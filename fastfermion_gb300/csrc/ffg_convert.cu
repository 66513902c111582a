// C ABI of libffg: conversions -- the Jordan-Wigner map
// (ffg_majorana_to_pauli) and sparse matrices (ffg_result_sparse).
#include "ffg_engine_impl.cuh"


// ---------------------------------------------------------------------------
// conversions: Jordan-Wigner map and sparse matrices
// ---------------------------------------------------------------------------
namespace {

// dst[t] = src[idx[t]] for 4 key planes and both coefficient arrays
__global__ void __launch_bounds__(kBlock) gather_terms(const u64* skey, u64 sn, const double* sre, const double* sim,
                                                       const u64* idx, u64 m, u64* dkey, double* dre, double* dim) {
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 t = (u64)blockIdx.x * blockDim.x + threadIdx.x; t < m; t += stride) {
        const u64 i = idx[t];
        for (int w = 0; w < 4; w++) dkey[(u64)w * m + t] = skey[(u64)w * sn + i];
        dre[t] = sre[i];
        dim[t] = sim[i];
    }
}

// device buffer freed at scope exit
struct DevBuf {
    void* p = nullptr;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

u64 flip_bits(u64 v, int n) {
    u64 r = 0;
    for (int q = 0; q < n; q++)
        if ((v >> q) & 1ull) r |= 1ull << (n - 1 - q);
    return r;
}

}  // namespace

int ffg_majorana_to_pauli(ffg_ctx* ctx, const uint64_t* keys, const double* re, const double* im, size_t n,
                          int on_device, ffg_result** out) {
    if (!ctx || !out || (n && (!keys || !re))) return FFG_ERR_ARG;
    *out = nullptr;
    try {
        CK(cudaSetDevice(ctx->device));
        const size_t m1 = std::max<size_t>(n, 1);
        DevBuf bk, bre, bim, pk, pre, pim, keep, idx;
        const u64* dk = (const u64*)keys;
        const double* dre = re;
        const double* dim = im;
        if (!on_device) {
            CK(cudaMalloc(&bk.p, 4 * m1 * 8));
            CK(cudaMalloc(&bre.p, m1 * 8));
            CK(cudaMalloc(&bim.p, m1 * 8));
            if (n) {
                CK(cudaMemcpyAsync(bk.p, keys, 4 * n * 8, cudaMemcpyHostToDevice, ctx->stream));
                CK(cudaMemcpyAsync(bre.p, re, n * 8, cudaMemcpyHostToDevice, ctx->stream));
                if (im)
                    CK(cudaMemcpyAsync(bim.p, im, n * 8, cudaMemcpyHostToDevice, ctx->stream));
                else
                    CK(cudaMemsetAsync(bim.p, 0, n * 8, ctx->stream));
            }
            dk = (const u64*)bk.p;
            dre = (const double*)bre.p;
            dim = (const double*)bim.p;
        }
        CK(cudaMalloc(&pk.p, 4 * m1 * 8));
        CK(cudaMalloc(&pre.p, m1 * 8));
        CK(cudaMalloc(&pim.p, m1 * 8));
        CK(cudaMalloc(&keep.p, m1));
        if (n)
            jw_kernel<<<grid_for(ctx, n), kBlock, 0, ctx->stream>>>(dk, 4, dre, dim, n, (u64*)pk.p, (double*)pre.p,
                                                                    (double*)pim.p, (unsigned char*)keep.p);
        CK(cudaGetLastError());
        std::vector<unsigned char> hk(n);
        if (n) CK(cudaMemcpyAsync(hk.data(), keep.p, n, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        std::vector<u64> kept;
        kept.reserve(n);
        for (size_t i = 0; i < n; i++)
            if (hk[i]) kept.push_back(i);
        const u64 m = kept.size();
        ffg_result* r = new ffg_result();
        r->kind = 1;
        r->nplanes = 4;
        r->cplx = true;
        r->n = m;
        r->ctx = ctx;
        r->device = ctx->device;
        const size_t mm = std::max<u64>(m, 1);
        cudaError_t e = cudaMalloc(&r->key, 4 * mm * 8);
        if (e == cudaSuccess) e = cudaMalloc(&r->re, mm * 8);
        if (e == cudaSuccess) e = cudaMalloc(&r->im, mm * 8);
        if (e == cudaSuccess) e = cudaMalloc(&r->dead, mm);
        if (e == cudaSuccess) e = cudaMalloc(&idx.p, mm * 8);
        if (e != cudaSuccess) {
            ffg_result_free(r);
            return set_err(ctx, FFG_ERR_CUDA, std::string("Jordan-Wigner result allocation: ") + cudaGetErrorString(e));
        }
        if (m) {
            CK(cudaMemcpyAsync(idx.p, kept.data(), m * 8, cudaMemcpyHostToDevice, ctx->stream));
            gather_terms<<<grid_for(ctx, m), kBlock, 0, ctx->stream>>>((const u64*)pk.p, n, (const double*)pre.p,
                                                                       (const double*)pim.p, (const u64*)idx.p, m,
                                                                       r->key, r->re, r->im);
        }
        CK(cudaMemsetAsync(r->dead, 0, mm, ctx->stream));
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(ctx->stream));
        *out = r;
        return FFG_OK;
    } catch (const std::exception& ex) {
        return set_err(ctx, FFG_ERR_STATE, ex.what());
    }
}

int ffg_result_sparse(const ffg_result* r, int n, int64_t* indptr, int64_t* indices, double* data_re,
                      double* data_im, size_t cap, size_t* nnz) {
    if (!r || !nnz || !indptr || n < 0 || n > 30) return FFG_ERR_ARG;
    ffg_ctx* ctx = r->ctx;
    if (r->kind != 1) return set_err(ctx, FFG_ERR_ARG, "sparse matrices are built for Pauli polynomials");
    try {
        CK(cudaSetDevice(r->device));
        std::vector<uint64_t> k4;
        std::vector<double> hr, hi;
        int rc = result_to_host(r, k4, hr, hi);
        if (rc) return rc;
        const size_t m = r->n;
        const u64 mask = n >= 64 ? ~0ull : ((1ull << n) - 1);
        // terms: flipped masks (qubit 0 = most significant bit; qubits >= n are
        // dropped as fliplr_bits does) and i^{#Y} c
        std::vector<u64> xf(m), zf(m);
        std::vector<double> cr(m), ci(m);
        for (size_t t = 0; t < m; t++) {
            const u64 x0 = k4[t], x1 = k4[m + t], z0 = k4[2 * m + t], z1 = k4[3 * m + t];
            xf[t] = flip_bits(x0 & mask, n);
            zf[t] = flip_bits(z0 & mask, n);
            const int ny = __builtin_popcountll(x0 & z0) + __builtin_popcountll(x1 & z1);
            // Ipow(ny) * c as a complex product (a.re*b.re - a.im*b.im, a.re*b.im + a.im*b.re)
            const double ar = (ny & 1) ? 0.0 : ((ny & 2) ? -1.0 : 1.0);
            const double ai = (ny & 1) ? ((ny & 2) ? -1.0 : 1.0) : 0.0;
            const double br = hr[t], bi = hi.empty() ? 0.0 : hi[t];
            volatile double p1 = ar * br, p2 = ai * bi, p3 = ar * bi, p4 = ai * br;
            cr[t] = p1 - p2;
            ci[t] = p3 + p4;
        }
        std::vector<size_t> ord(m);
        for (size_t t = 0; t < m; t++) ord[t] = t;
        // (xf, zf, position): equal masks (qubits >= n dropped) keep term order
        std::sort(ord.begin(), ord.end(), [&](size_t a, size_t b) {
            if (xf[a] != xf[b]) return xf[a] < xf[b];
            if (zf[a] != zf[b]) return zf[a] < zf[b];
            return a < b;
        });
        std::vector<u64> gxf, szf(m);
        std::vector<u32> gstart;
        std::vector<double> scr(m), sci(m);
        for (size_t t = 0; t < m; t++) {
            const size_t o = ord[t];
            if (t == 0 || xf[o] != xf[ord[t - 1]]) {
                gxf.push_back(xf[o]);
                gstart.push_back((u32)t);
            }
            szf[t] = zf[o];
            scr[t] = cr[o];
            sci[t] = ci[o];
        }
        gstart.push_back((u32)m);
        const u64 ncols = 1ull << n;
        const u32 ng = (u32)gxf.size();
        DevBuf d_gxf, d_gstart, d_zf, d_cr, d_ci, d_cnt, d_ptr, d_rows, d_vre, d_vim;
        const size_t m1 = std::max<size_t>(m, 1);
        CK(cudaMalloc(&d_gxf.p, std::max<size_t>(ng, 1) * 8));
        CK(cudaMalloc(&d_gstart.p, (ng + 1) * 4));
        CK(cudaMalloc(&d_zf.p, m1 * 8));
        CK(cudaMalloc(&d_cr.p, m1 * 8));
        CK(cudaMalloc(&d_ci.p, m1 * 8));
        CK(cudaMalloc(&d_cnt.p, ncols * 8));
        if (ng) CK(cudaMemcpyAsync(d_gxf.p, gxf.data(), ng * 8, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(d_gstart.p, gstart.data(), (ng + 1) * 4, cudaMemcpyHostToDevice, ctx->stream));
        if (m) {
            CK(cudaMemcpyAsync(d_zf.p, szf.data(), m * 8, cudaMemcpyHostToDevice, ctx->stream));
            CK(cudaMemcpyAsync(d_cr.p, scr.data(), m * 8, cudaMemcpyHostToDevice, ctx->stream));
            CK(cudaMemcpyAsync(d_ci.p, sci.data(), m * 8, cudaMemcpyHostToDevice, ctx->stream));
        }
        sparse_kernel<<<grid_for(ctx, ncols), kBlock, 0, ctx->stream>>>(
            ncols, (const u64*)d_gxf.p, (const u32*)d_gstart.p, ng, (const u64*)d_zf.p, (const double*)d_cr.p,
            (const double*)d_ci.p, (long long*)d_cnt.p, nullptr, nullptr, nullptr, nullptr, 0);
        CK(cudaGetLastError());
        std::vector<long long> cnt(ncols);
        CK(cudaMemcpyAsync(cnt.data(), d_cnt.p, ncols * 8, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        indptr[0] = 0;
        for (u64 b = 0; b < ncols; b++) indptr[b + 1] = indptr[b] + cnt[b];
        *nnz = (size_t)indptr[ncols];
        if (!indices || !data_re || !data_im || cap < *nnz || *nnz == 0) return FFG_OK;
        CK(cudaMalloc(&d_ptr.p, ncols * 8));
        CK(cudaMalloc(&d_rows.p, *nnz * 8));
        CK(cudaMalloc(&d_vre.p, *nnz * 8));
        CK(cudaMalloc(&d_vim.p, *nnz * 8));
        CK(cudaMemcpyAsync(d_ptr.p, indptr, ncols * 8, cudaMemcpyHostToDevice, ctx->stream));
        sparse_kernel<<<grid_for(ctx, ncols), kBlock, 0, ctx->stream>>>(
            ncols, (const u64*)d_gxf.p, (const u32*)d_gstart.p, ng, (const u64*)d_zf.p, (const double*)d_cr.p,
            (const double*)d_ci.p, nullptr, (const long long*)d_ptr.p, (long long*)d_rows.p, (double*)d_vre.p,
            (double*)d_vim.p, 1);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(indices, d_rows.p, *nnz * 8, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(data_re, d_vre.p, *nnz * 8, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(data_im, d_vim.p, *nnz * 8, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        return FFG_OK;
    } catch (const std::exception& ex) {
        return set_err(ctx, FFG_ERR_STATE, ex.what());
    }
}
