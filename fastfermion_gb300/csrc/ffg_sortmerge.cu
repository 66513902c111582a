// Sort-and-reduce merge for one Pauli rotation (the alternative to the hash
// index of the per-gate pass and to the batch-orbit engine; selected with the
// engine option merge_sort = 1, off by default: slower on GB300).
//
// One pass over the dense store emits, for every term Q, the kept entry
// (Q, c_Q cos) or (Q, c_Q) when Q commutes with the gate, and for every
// anticommuting Q whose partner K = P Q passes the degree filter the partner
// entry (K, c_Q (i sin) phase(P Q)) (src/pauli/propagate.h:71-89).  Entries are
// radix-sorted by (key, tag) with the kept entry (tag 0) before the partner
// entry (tag 1), so a key's run is at most [kept, partner] and the segmented
// reduce adds them in the reference's order: c_K cos first, then the partner
// (map[K] += p), or 0 + p when K was absent.  The sort is CUB's radix sort
// (a library primitive); the emit and reduce kernels are this file's.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cuda/std/tuple>

#include "ffg_sortmerge.h"
#include "ffg_device.cuh"

namespace ffg_sm {
using namespace ffg;

template <int KW>
struct SKey {
    u64 w[KW];  // key planes, most significant first in the decomposition
    u32 tag;    // 0 kept, 1 partner
};

template <int KW>
struct SKeyDecomposer;

template <>
struct SKeyDecomposer<2> {
    __host__ __device__ cuda::std::tuple<u64&, u64&, u32&> operator()(SKey<2>& k) const {
        return {k.w[0], k.w[1], k.tag};
    }
};

template <>
struct SKeyDecomposer<4> {
    __host__ __device__ cuda::std::tuple<u64&, u64&, u64&, u64&, u32&> operator()(SKey<4>& k) const {
        return {k.w[0], k.w[1], k.w[2], k.w[3], k.tag};
    }
};

template <int KW, bool CPLX>
__global__ void __launch_bounds__(kBlock) sm_emit(const u64* key, const double* re, const double* im, u64 n,
                                                  u64 stride, SmGate g, SKey<KW>* ek, u32* ev, double* cre,
                                                  double* cim, unsigned long long* counter) {
    constexpr int NW = KW / 2;
    const u64 step = (u64)gridDim.x * blockDim.x;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += step) {
        u64 q[KW];
#pragma unroll
        for (int w = 0; w < KW; w++) q[w] = key[(u64)w * stride + i];
        const cplx c = {re[i], CPLX ? im[i] : 0.0};
        u64 par = 0;
#pragma unroll
        for (int w = 0; w < NW; w++) par ^= (q[w] & g.p[NW + w]) ^ (q[NW + w] & g.p[w]);
        const bool anti = __popcll(par) & 1;
        // kept entry at slot 2i, partner at slot 2i + 1 (unused slots keep the
        // all-ones key and sort last)
        SKey<KW> kk;
#pragma unroll
        for (int w = 0; w < KW; w++) kk.w[w] = q[w];
        kk.tag = 0;
        ek[2 * i] = kk;
        ev[2 * i] = (u32)(2 * i);
        const cplx kept = anti ? rot_keep<CPLX>(c, g.c) : c;
        cre[2 * i] = kept.re;
        if (CPLX) cim[2 * i] = kept.im;
        SKey<KW> pk;
        pk.tag = 0xffffffffu;
#pragma unroll
        for (int w = 0; w < KW; w++) pk.w[w] = ~0ull;
        if (anti) {
            u64 k[KW];
            int yQ = 0, yK = 0, zxQ = 0, dK = 0;
#pragma unroll
            for (int w = 0; w < KW; w++) k[w] = q[w] ^ g.p[w];
#pragma unroll
            for (int w = 0; w < NW; w++) {
                yQ += __popcll(q[w] & q[NW + w]);
                yK += __popcll(k[w] & k[NW + w]);
                zxQ += __popcll(g.p[NW + w] & q[w]);
                dK += __popcll(k[w] | k[NW + w]);
            }
            if (dK <= g.maxdeg) {
                const cplx p = rot_partner<CPLX>(c, g.s, g.yP + yQ + 2 * zxQ - yK);
#pragma unroll
                for (int w = 0; w < KW; w++) pk.w[w] = k[w];
                pk.tag = 1;
                cre[2 * i + 1] = p.re;
                if (CPLX) cim[2 * i + 1] = p.im;
                atomicAdd(counter, 1ull);
            }
        }
        ek[2 * i + 1] = pk;
        ev[2 * i + 1] = (u32)(2 * i + 1);
    }
}

template <int KW>
__device__ __forceinline__ bool same_key(const SKey<KW>& a, const SKey<KW>& b) {
#pragma unroll
    for (int w = 0; w < KW; w++)
        if (a.w[w] != b.w[w]) return false;
    return true;
}

// head[p] = 1 when sorted entry p starts a key run of real entries
template <int KW>
__global__ void __launch_bounds__(kBlock) sm_heads(const SKey<KW>* sk, u64 m, u32* head) {
    const u64 step = (u64)gridDim.x * blockDim.x;
    for (u64 p = (u64)blockIdx.x * blockDim.x + threadIdx.x; p < m; p += step) {
        const bool real = sk[p].tag != 0xffffffffu;
        head[p] = (real && (p == 0 || !same_key<KW>(sk[p], sk[p - 1]))) ? 1u : 0u;
    }
}

template <int KW, bool CPLX>
__global__ void __launch_bounds__(kBlock) sm_reduce(const SKey<KW>* sk, const u32* sv, const double* cre,
                                                    const double* cim, u64 m, const u32* head, const u32* pos,
                                                    u64* okey, double* ore, double* oim, u64 ocap) {
    const u64 step = (u64)gridDim.x * blockDim.x;
    for (u64 p = (u64)blockIdx.x * blockDim.x + threadIdx.x; p < m; p += step) {
        if (!head[p]) continue;
        const u32 o = pos[p];
        if (o >= ocap) continue;
        const u32 a = sv[p];
        cplx v = {cre[a], CPLX ? cim[a] : 0.0};
        if (sk[p].tag == 1) {
            v = rot_add<CPLX>({0.0, 0.0}, v);  // partner of an absent key: 0 + p
        } else if (p + 1 < m && sk[p + 1].tag == 1 && same_key<KW>(sk[p], sk[p + 1])) {
            const u32 b = sv[p + 1];
            v = rot_add<CPLX>(v, cplx{cre[b], CPLX ? cim[b] : 0.0});  // c_K cos + partner
        }
#pragma unroll
        for (int w = 0; w < KW; w++) okey[(u64)w * ocap + o] = sk[p].w[w];
        ore[o] = v.re;
        if (CPLX) oim[o] = v.im;
    }
}

namespace {
size_t al(size_t b) { return (b + 255) & ~(size_t)255; }
}

template <int KW, bool CPLX>
static int rotation_t(cudaStream_t st, const u64* key, const double* re, const double* im, u64 n, u64 stride,
                      const SmGate& g, u64* okey, double* ore, double* oim, u64 ocap, u64* n_out, u64* emits,
                      void** scratch, size_t* scratch_bytes) {
    const u64 m = 2 * n;
    size_t sort_tmp = 0, scan_tmp = 0;
    cudaError_t e = cub::DeviceRadixSort::SortPairs(nullptr, sort_tmp, (SKey<KW>*)nullptr, (SKey<KW>*)nullptr,
                                                     (u32*)nullptr, (u32*)nullptr, (int64_t)m, SKeyDecomposer<KW>{},
                                                     0, (int)(KW * 64 + 32), st);
    if (e) return (int)e;
    e = cub::DeviceScan::ExclusiveSum(nullptr, scan_tmp, (u32*)nullptr, (u32*)nullptr, (int64_t)m, st);
    if (e) return (int)e;
    const size_t need = 2 * al(m * sizeof(SKey<KW>)) + 2 * al(m * 4) + 2 * al(m * 8) + 2 * al(m * 4) + al(sort_tmp) +
                        al(scan_tmp) + 256;
    if (*scratch_bytes < need) {
        if (*scratch) cudaFree(*scratch);
        *scratch = nullptr;
        *scratch_bytes = 0;
        e = cudaMalloc(scratch, need);
        if (e) return (int)e;
        *scratch_bytes = need;
    }
    char* p = (char*)*scratch;
    auto take = [&](size_t b) {
        char* r = p;
        p += al(b);
        return r;
    };
    SKey<KW>* k0 = (SKey<KW>*)take(m * sizeof(SKey<KW>));
    SKey<KW>* k1 = (SKey<KW>*)take(m * sizeof(SKey<KW>));
    u32* v0 = (u32*)take(m * 4);
    u32* v1 = (u32*)take(m * 4);
    double* cre = (double*)take(m * 8);
    double* cim = (double*)take(m * 8);
    u32* head = (u32*)take(m * 4);
    u32* pos = (u32*)take(m * 4);
    void* sortt = take(sort_tmp);
    void* scant = take(scan_tmp);
    unsigned long long* counter = (unsigned long long*)p;
    if ((e = cudaMemsetAsync(counter, 0, 8, st))) return (int)e;
    const int grid = (int)std::min<u64>((m + kBlock - 1) / kBlock + 1, 152 * 16);
    if (n) sm_emit<KW, CPLX><<<grid, kBlock, 0, st>>>(key, re, im, n, stride, g, k0, v0, cre, cim, counter);
    size_t tb = sort_tmp;
    e = cub::DeviceRadixSort::SortPairs(sortt, tb, k0, k1, v0, v1, (int64_t)m, SKeyDecomposer<KW>{}, 0,
                                        (int)(KW * 64 + 32), st);
    if (e) return (int)e;
    if (m) sm_heads<KW><<<grid, kBlock, 0, st>>>(k1, m, head);
    tb = scan_tmp;
    e = cub::DeviceScan::ExclusiveSum(scant, tb, head, pos, (int64_t)m, st);
    if (e) return (int)e;
    u32 last_pos = 0, last_head = 0;
    if (m) {
        if ((e = cudaMemcpyAsync(&last_pos, pos + m - 1, 4, cudaMemcpyDeviceToHost, st))) return (int)e;
        if ((e = cudaMemcpyAsync(&last_head, head + m - 1, 4, cudaMemcpyDeviceToHost, st))) return (int)e;
    }
    unsigned long long em = 0;
    if ((e = cudaMemcpyAsync(&em, counter, 8, cudaMemcpyDeviceToHost, st))) return (int)e;
    if ((e = cudaStreamSynchronize(st))) return (int)e;
    *n_out = (u64)last_pos + last_head;
    *emits = em;
    if (*n_out > ocap) return 0;  // the caller grows the output and calls again
    if (m) sm_reduce<KW, CPLX><<<grid, kBlock, 0, st>>>(k1, v1, cre, cim, m, head, pos, okey, ore, oim, ocap);
    return (int)cudaGetLastError();
}

int rotation(cudaStream_t st, int kw, bool cplx, const u64* key, const double* re, const double* im, u64 n, u64 stride,
             const SmGate& g, u64* okey, double* ore, double* oim, u64 ocap, u64* n_out, u64* emits, void** scratch,
             size_t* scratch_bytes) {
    if (kw == 2)
        return cplx ? rotation_t<2, true>(st, key, re, im, n, stride, g, okey, ore, oim, ocap, n_out, emits, scratch,
                                           scratch_bytes)
                    : rotation_t<2, false>(st, key, re, im, n, stride, g, okey, ore, oim, ocap, n_out, emits, scratch,
                                            scratch_bytes);
    return cplx ? rotation_t<4, true>(st, key, re, im, n, stride, g, okey, ore, oim, ocap, n_out, emits, scratch,
                                       scratch_bytes)
                : rotation_t<4, false>(st, key, re, im, n, stride, g, okey, ore, oim, ocap, n_out, emits, scratch,
                                        scratch_bytes);
}

}  // namespace ffg_sm
