// Conversions of propagated polynomials, done on the GPU:
//
//  * Jordan-Wigner map of a Majorana polynomial to a Pauli polynomial
//    (src/transforms.h:124-151): Majorana index i = 2j + r maps to
//    Z_0 ... Z_{j-1} X_j (r = 0) or Z_0 ... Z_{j-1} Y_j (r = 1); a string is the
//    ordered product of its indices' images, the phase exponent accumulating
//    as in pauli_string_multiply (src/pauli/algebra.h:227-233).  The map is a
//    bijection on strings, so every term maps on its own; terms whose
//    coefficient is exactly zero are dropped (compress(0)).
//  * Sparse matrix (CSC, 2^n x 2^n) of a Pauli polynomial
//    (src/pauli/sparse.h:20-131): columns b are basis states with qubit 0 as
//    the most significant bit; the terms are grouped by their bit-reversed X
//    mask xf (ascending), and column b gets, for every group, the entry at
//    row b ^ xf with value sum over the group of (-1)^|b & zf| i^{#Y} c when
//    that sum is not zero.
#pragma once
#include "ffg_device.cuh"

namespace ffg {

// One Majorana string (KW planes) -> Pauli string (x0, x1, z0, z1) and i^jpow.
__device__ __forceinline__ void jw_string(const u64 (&a)[4], u64 (&x)[2], u64 (&z)[2], int& jpow) {
    x[0] = x[1] = z[0] = z[1] = 0;
    jpow = 0;
    for (int w = 0; w < 4; w++) {
        u64 bits = a[w];
        while (bits) {
            const int i = 64 * w + __ffsll((long long)bits) - 1;
            bits &= bits - 1;
            const int j = i >> 1, r = i & 1;
            // image of index i: x = bit j, z = bits [0, j) (+ bit j when r = 1)
            u64 bx[2] = {0, 0}, bz[2] = {0, 0};
            bx[j >> 6] = 1ull << (j & 63);
            for (int q = 0; q < 2; q++) {
                const int lo = 64 * q;
                const int end = j + r;  // bits [0, end)
                if (end >= lo + 64)
                    bz[q] = ~0ull;
                else if (end > lo)
                    bz[q] = (1ull << (end - lo)) - 1;
            }
            // pauli_string_multiply(res, jpow, b)
            jpow += __popcll(x[0] & z[0]) + __popcll(x[1] & z[1]) + __popcll(bx[0] & bz[0]) +
                    __popcll(bx[1] & bz[1]) + 2 * (__popcll(z[0] & bx[0]) + __popcll(z[1] & bx[1]));
            x[0] ^= bx[0];
            x[1] ^= bx[1];
            z[0] ^= bz[0];
            z[1] ^= bz[1];
            jpow -= __popcll(x[0] & z[0]) + __popcll(x[1] & z[1]);
        }
    }
}

// keys: kw planes (stride n) of Majorana strings; out: 4 Pauli planes (stride
// n).  keep[i] = 0 when the mapped coefficient is exactly zero.
static __global__ void __launch_bounds__(kBlock) jw_kernel(const u64* mkeys, int kw, const double* re, const double* im,
                                                    u64 n, u64* pkeys, double* ore, double* oim,
                                                    unsigned char* keep) {
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        u64 a[4] = {0, 0, 0, 0};
        for (int w = 0; w < kw; w++) a[w] = mkeys[(u64)w * n + i];
        u64 x[2], z[2];
        int jpow;
        jw_string(a, x, z, jpow);
        // res.terms[b] += v * i^jpow: complex product, then added to zero
        const cplx v = {re[i], im ? im[i] : 0.0};
        const cplx c = cadd({0.0, 0.0}, cmul(v, ipow(jpow)));
        pkeys[i] = x[0];
        pkeys[n + i] = x[1];
        pkeys[2 * n + i] = z[0];
        pkeys[3 * n + i] = z[1];
        ore[i] = c.re;
        oim[i] = c.im;
        keep[i] = (c.re != 0.0 || c.im != 0.0) ? 1 : 0;
    }
}

// Sparse matrix: groups g (ascending xf) with terms [gstart[g], gstart[g+1]);
// term t has the bit-reversed Z mask zf[t] and coefficient i^{#Y} c = (cr, ci).
// pass 0 counts the nonzero entries of every column, pass 1 writes them at
// colptr[b] (row indices and values).
static __global__ void __launch_bounds__(kBlock) sparse_kernel(u64 ncols, const u64* gxf, const u32* gstart, u32 ngroups,
                                                        const u64* zf, const double* cr, const double* ci,
                                                        long long* colcount, const long long* colptr,
                                                        long long* rows, double* vre, double* vim, int pass) {
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 b = (u64)blockIdx.x * blockDim.x + threadIdx.x; b < ncols; b += stride) {
        long long cnt = 0;
        long long at = pass ? colptr[b] : 0;
        for (u32 g = 0; g < ngroups; g++) {
            double sr = 0.0, si = 0.0;
            for (u32 t = gstart[g]; t < gstart[g + 1]; t++) {
                const double sg = (__popcll(b & zf[t]) & 1) ? -1.0 : 1.0;
                sr = __dadd_rn(sr, __dmul_rn(sg, cr[t]));
                si = __dadd_rn(si, __dmul_rn(sg, ci[t]));
            }
            if (sr != 0.0 || si != 0.0) {
                if (pass) {
                    rows[at] = (long long)(b ^ gxf[g]);
                    vre[at] = sr;
                    vim[at] = si;
                    at++;
                }
                cnt++;
            }
        }
        if (!pass) colcount[b] = cnt;
    }
}

}  // namespace ffg
