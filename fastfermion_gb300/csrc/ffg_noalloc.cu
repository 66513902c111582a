// Allocation-free Pauli rotation entry point (ffg_pauli_rotations_noalloc).
//
// Some callers cannot allocate device memory at the moment they need this
// operation.  Two kinds are common: processes in which a framework's caching
// allocator has already reserved (nearly) all device memory for itself, so a
// cudaMalloc from a library fails or fragments that pool; and latency-critical
// loops that share the GPU with other streams, where cudaFree's implicit
// device-wide synchronisation is not acceptable.  For them this file keeps the
// term store in one statically sized device array, so the entry point creates
// no context and calls no cudaMalloc, cudaMallocHost, cudaFree or any
// allocating library routine.  The caller still provides the input and output
// arrays.
//
// Limits and sharing rules:
//  * the scratch array holds at most kNoAllocCap = 65536 terms; inputs may have
//    at most kNoAllocCap / 2 terms and a rotation that could push the store past
//    kNoAllocCap is reported as an error;
//  * every GPU that loads the library holds the array (about 4.3 MB) until the
//    process exits;
//  * every call on a device uses the same array and leaves the previous call's
//    contents in it; each call re-initialises what must start empty (counters,
//    index slots, dead flags) itself.  Two calls whose GPU work overlaps (for
//    example on two streams) race on the array and give wrong results;
//  * the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current and keeps it for the
//    process; make that first call before any stream capture begins.  A
//    cudaDeviceReset of that device invalidates the kept address: do not call
//    this entry point on that device after a reset;
//  * the call waits for its own work on `stream` to finish before it returns
//    (it reads the result size and the error flags back to the host).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/ffg.h"

// The propagation kernels, compiled into this translation unit under their own
// namespace so that their symbols stay separate from the context-based engine.
namespace ffg_noalloc_impl {
#include "ffg_kernels.cuh"
}

using namespace ffg_noalloc_impl::ffg;

namespace {

constexpr u64 kNoAllocCap = 1ull << 16;  // term capacity of the scratch store
constexpr int kKW = 4;                   // planes: x0, x1, z0, z1 (the caller's layout)

constexpr size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr size_t kOffKey = 0;
constexpr size_t kOffRe = kOffKey + al256(kKW * kNoAllocCap * 8);
constexpr size_t kOffIm = kOffRe + al256(kNoAllocCap * 8);
constexpr size_t kOffDead = kOffIm + al256(kNoAllocCap * 8);
constexpr size_t kOffSlots = kOffDead + al256(kNoAllocCap);
constexpr size_t kOffCtr = kOffSlots + al256(2 * kNoAllocCap * 8);
constexpr size_t kScratchBytes = kOffCtr + al256(sizeof(DevCounters));

// The scratch term store.  Host code must not use this name as an address: it
// only resolves to device memory through cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices] = {};
std::mutex g_setup_mutex;

int fail(char* errbuf, size_t errlen, int code, const char* msg) {
    if (errbuf && errlen) {
        std::strncpy(errbuf, msg, errlen - 1);
        errbuf[errlen - 1] = '\0';
    }
    return code;
}

__global__ void noalloc_reset_counters(DevCounters* c, u64 n) {
    DevCounters z{};
    z.n = n;
    z.alive = n;
    z.peak = n;
    *c = z;
}

}  // namespace

int ffg_pauli_rotations_noalloc(void* stream, const uint64_t* keys_in, const double* re_in,
                                const double* im_in, size_t n, const ffg_pauli_gate* gates,
                                size_t ngates, int32_t maxdegree, uint64_t* keys_out,
                                double* re_out, double* im_out, size_t out_cap, size_t* n_out,
                                char* errbuf, size_t errlen) {
    char msg[256];
    if (n_out) *n_out = 0;
    if ((n && (!keys_in || !re_in)) || (ngates && !gates) || !keys_out || !re_out || !im_out || !n_out)
        return fail(errbuf, errlen, FFG_ERR_ARG, "ffg_pauli_rotations_noalloc: null argument");
    if (n > kNoAllocCap / 2) {
        std::snprintf(msg, sizeof msg,
                      "ffg_pauli_rotations_noalloc: %zu input terms exceed the fixed scratch "
                      "limit of %llu terms",
                      n, (unsigned long long)(kNoAllocCap / 2));
        return fail(errbuf, errlen, FFG_ERR_ARG, msg);
    }
    for (size_t i = 0; i < ngates; i++)
        if (gates[i].kind != FFG_ROT)
            return fail(errbuf, errlen, FFG_ERR_ARG,
                        "ffg_pauli_rotations_noalloc: only FFG_ROT gates are accepted");
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return fail(errbuf, errlen, FFG_ERR_CUDA, "ffg_pauli_rotations_noalloc: no current CUDA device");
    if (dev < 0 || dev >= kMaxDevices) {
        std::snprintf(msg, sizeof msg,
                      "ffg_pauli_rotations_noalloc: device ordinal %d is beyond the %d devices this entry "
                      "point supports",
                      dev, kMaxDevices);
        return fail(errbuf, errlen, FFG_ERR_ARG, msg);
    }
    // once per device, with that device current: device address of the array
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_addr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                std::snprintf(msg, sizeof msg, "ffg_pauli_rotations_noalloc: cudaGetSymbolAddress: %s",
                              cudaGetErrorString(e));
                return fail(errbuf, errlen, FFG_ERR_CUDA, msg);
            }
            g_scratch_addr[dev] = p;
        }
    }
    unsigned char* base = (unsigned char*)g_scratch_addr[dev];
    StoreView v{};
    v.cap = kNoAllocCap;
    v.key = (u64*)(base + kOffKey);
    v.re = (double*)(base + kOffRe);
    v.im = (double*)(base + kOffIm);
    v.dead = base + kOffDead;
    v.slots = (u64*)(base + kOffSlots);
    v.hmask = 2 * kNoAllocCap - 1;
    DevCounters* ctr = (DevCounters*)(base + kOffCtr);

#define NA_CK(call)                                                                            \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess) {                                                               \
            std::snprintf(msg, sizeof msg, "ffg_pauli_rotations_noalloc: %s", cudaGetErrorString(e_)); \
            return fail(errbuf, errlen, FFG_ERR_CUDA, msg);                                    \
        }                                                                                      \
    } while (0)

    // reset what must start empty, then load the input
    noalloc_reset_counters<<<1, 1, 0, st>>>(ctr, n);
    NA_CK(cudaMemsetAsync(v.dead, 0, kNoAllocCap, st));
    if (n) {
        for (int w = 0; w < kKW; w++)
            NA_CK(cudaMemcpyAsync(v.key + (size_t)w * kNoAllocCap, keys_in + (size_t)w * n, n * 8,
                                  cudaMemcpyDeviceToDevice, st));
        NA_CK(cudaMemcpyAsync(v.re, re_in, n * 8, cudaMemcpyDeviceToDevice, st));
        if (im_in)
            NA_CK(cudaMemcpyAsync(v.im, im_in, n * 8, cudaMemcpyDeviceToDevice, st));
        else
            NA_CK(cudaMemsetAsync(v.im, 0, n * 8, st));
    }
    const int grid = 256;
    clear_slots_kernel<<<grid, kBlock, 0, st>>>(v.slots, v.hmask + 1);
    index_kernel<kKW><<<grid, kBlock, 0, st>>>(v, ctr, 1);
    // rotations, last gate first, each exactly as one reference conjugation
    for (size_t t = 0; t < ngates; t++) {
        const ffg_pauli_gate& G = gates[ngates - 1 - t];
        RotArgs a{};
        a.p[0] = G.x[0];
        a.p[1] = G.x[1];
        a.p[2] = G.z[0];
        a.p[3] = G.z[1];
        a.c = std::cos(G.theta);
        a.s = std::sin(G.theta);
        a.maxdeg = maxdegree;
        a.yP = __builtin_popcountll(G.x[0] & G.z[0]) + __builtin_popcountll(G.x[1] & G.z[1]);
        a.op = (u32)t;
        pauli_rot_kernel<2, true><<<grid, kBlock, 0, st>>>(v, ctr, a);
    }
    NA_CK(cudaGetLastError());
    DevCounters h;
    NA_CK(cudaMemcpyAsync(&h, ctr, sizeof h, cudaMemcpyDeviceToHost, st));
    NA_CK(cudaStreamSynchronize(st));
    if (h.error & 1u) return fail(errbuf, errlen, FFG_ERR_ARG, "ffg_pauli_rotations_noalloc: input contains duplicate keys");
    if (h.error) return fail(errbuf, errlen, FFG_ERR_STATE, "ffg_pauli_rotations_noalloc: index probe overrun");
    if (h.overflow) {
        // h.overflow - 1 counts rotations in application order (last gate first)
        const size_t applied = (size_t)(h.overflow - 1);
        std::snprintf(msg, sizeof msg,
                      "ffg_pauli_rotations_noalloc: the polynomial outgrew the fixed scratch limit "
                      "of %llu terms at gates[%zu]",
                      (unsigned long long)kNoAllocCap, ngates - 1 - applied);
        return fail(errbuf, errlen, FFG_ERR_ARG, msg);
    }
    *n_out = (size_t)h.n;
    if (h.n > out_cap) {
        std::snprintf(msg, sizeof msg, "ffg_pauli_rotations_noalloc: result has %llu terms, out_cap is %zu",
                      (unsigned long long)h.n, out_cap);
        return fail(errbuf, errlen, FFG_ERR_ARG, msg);
    }
    if (h.n) {
        for (int w = 0; w < kKW; w++)
            NA_CK(cudaMemcpyAsync(keys_out + (size_t)w * out_cap, v.key + (size_t)w * kNoAllocCap,
                                  h.n * 8, cudaMemcpyDeviceToDevice, st));
        NA_CK(cudaMemcpyAsync(re_out, v.re, h.n * 8, cudaMemcpyDeviceToDevice, st));
        NA_CK(cudaMemcpyAsync(im_out, v.im, h.n * 8, cudaMemcpyDeviceToDevice, st));
    }
    NA_CK(cudaStreamSynchronize(st));
#undef NA_CK
    return FFG_OK;
}
