// The learned truncation correction's network on sm_103a tensor cores, and the
// features of the partners that the degree filter drops.  No counterpart in
// the reference (its propagate discards those partners,
// src/pauli/propagate.h:71-89).
//
// Network: 32 -> 128 -> 128 -> 128 -> 1 with GELU after each hidden layer.
// The three hidden GEMMs run on the tensor cores (tcgen05.mma kind::f16, BF16
// operands staged in shared memory, FP32 accumulators in TMEM); the 128 -> 1
// output layer, the biases, the activations and the optimizer are FP32 on the
// CUDA cores.  Master parameters are FP32; every update rewrites their BF16
// images.  One CTA of 128 threads handles a tile of 128 rows: thread r owns
// row r of the tile, which is TMEM lane r of the accumulators.
//
// Kernels:
//   mlp_forward_kernel     inference: y = f(x) for every row (persistent over tiles)
//   mlp_rows_kernel        training, per row: forward, loss, backward through
//                          the layers (the dH GEMMs also on the tensor cores);
//                          writes the activations and the pre-activation
//                          gradients that the weight gradients need, and
//                          accumulates the bias and output-layer gradients
//   mlp_wgrad_kernel       weight gradients dW = dZ^T H, a GEMM whose K runs over
//                          rows (split across CTAs, FP32 atomics at the end)
//   mlp_adam_kernel        Adam step on the FP32 parameters + BF16 images
//   drop_features_kernel   32 features of each dropped partner
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/ffg.h"
#include "ffg_tc.cuh"

using namespace ffg_tc;

namespace {

constexpr int kIn = 32;
constexpr int kHid = 128;
constexpr int kTile = 128;     // rows per CTA tile (= TMEM lanes = threads)
constexpr int kThreads = 128;

// flat FP32 parameter vector
constexpr int oW1 = 0;                      // [128][32]  (out, in)
constexpr int oB1 = oW1 + kHid * kIn;       // [128]
constexpr int oW2 = oB1 + kHid;             // [128][128]
constexpr int oB2 = oW2 + kHid * kHid;
constexpr int oW3 = oB2 + kHid;
constexpr int oB3 = oW3 + kHid * kHid;
constexpr int oW4 = oB3 + kHid;             // [128]
constexpr int oB4 = oW4 + kHid;             // scalar
constexpr int kNumParams = oB4 + 1;
static_assert(kNumParams == FFG_MLP_NPARAMS, "parameter count");

// weight images (bytes): the forward prefix [W1 | W2 | W3 | bias block] and,
// for training, [W2^T | W3^T]; the same layout in global and shared memory
constexpr uint32_t kImgW1 = 0;                         // 128 x 32
constexpr uint32_t kImgW2 = kImgW1 + kHid * kIn * 2;   // 128 x 128
constexpr uint32_t kImgW3 = kImgW2 + kHid * kHid * 2;
constexpr uint32_t kImgBias = kImgW3 + kHid * kHid * 2;  // floats: b1, b2, b3, w4, b4, pad
constexpr uint32_t kBiasFloats = 544;
constexpr uint32_t kImgW2T = kImgBias + kBiasFloats * 4;
constexpr uint32_t kImgW3T = kImgW2T + kHid * kHid * 2;
constexpr uint32_t kImgBytes = kImgW3T + kHid * kHid * 2;
constexpr uint32_t kFwdImgBytes = kImgW2T;
static_assert(kImgW2T % 128 == 0 && kFwdImgBytes % 16 == 0 && kImgBytes % 16 == 0, "image alignment");

constexpr uint32_t kIdescN128 = idesc_bf16(128, 128);
constexpr uint32_t kIdescN32 = idesc_bf16(128, 32);

// status bits of a launch
constexpr int kStatusTimeout = 1;

// GELU in its tanh form (Hendrycks and Gimpel, "Gaussian Error Linear Units",
// 2016):  gelu(z) = z/2 (1 + tanh(u)),  u = sqrt(2/pi) (z + 0.044715 z^3),
// with tanh from the hardware approximation (tanh.approx.f32, one MUFU
// instruction, relative error about 2^-11, below the BF16 rounding that
// follows it).  gelu_grad is its exact derivative with the same tanh.
constexpr float kGeluK = 0.7978845608028654f;     // sqrt(2/pi)
constexpr float kGeluK3 = 0.035677408136300125f;  // 0.044715 sqrt(2/pi)
constexpr float kGeluK3d = 0.10703222440890037f;  // 3 x 0.044715 sqrt(2/pi)

__device__ __forceinline__ float tanh_approx(float u) {
    float t;
    asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(u));
    return t;
}
__device__ __forceinline__ float gelu(float z) {
    const float u = z * fmaf(kGeluK3, z * z, kGeluK);
    const float hz = 0.5f * z;
    return fmaf(hz, tanh_approx(u), hz);
}
__device__ __forceinline__ float gelu_grad(float z) {
    const float z2 = z * z;
    const float t = tanh_approx(z * fmaf(kGeluK3, z2, kGeluK));
    // d/dz: (1 + t)/2 + z/2 (1 - t^2) sqrt(2/pi) (1 + 3 x 0.044715 z^2)
    return fmaf(0.5f * z * fmaf(kGeluK3d, z2, kGeluK), fmaf(-t, t, 1.0f), 0.5f + 0.5f * t);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);  // .x = a (low half), .y = b
    return *reinterpret_cast<const uint32_t*>(&h);
}

// 16 values of row r, columns c0..c0+15, into an operand image of width K
__device__ __forceinline__ void store_row16(uint8_t* img, int r, int c0, int K, const float (&v)[16]) {
    uint4 a, b;
    a.x = pack_bf16(v[0], v[1]);
    a.y = pack_bf16(v[2], v[3]);
    a.z = pack_bf16(v[4], v[5]);
    a.w = pack_bf16(v[6], v[7]);
    b.x = pack_bf16(v[8], v[9]);
    b.y = pack_bf16(v[10], v[11]);
    b.z = pack_bf16(v[12], v[13]);
    b.w = pack_bf16(v[14], v[15]);
    *reinterpret_cast<uint4*>(img + img_off(r, c0, K)) = a;
    *reinterpret_cast<uint4*>(img + img_off(r, c0 + 8, K)) = b;
}

// the same 16 values as a row-major bf16 row segment in global memory
__device__ __forceinline__ void store_global16(__nv_bfloat16* row, int c0, const float (&v)[16]) {
    uint4 a, b;
    a.x = pack_bf16(v[0], v[1]);
    a.y = pack_bf16(v[2], v[3]);
    a.z = pack_bf16(v[4], v[5]);
    a.w = pack_bf16(v[6], v[7]);
    b.x = pack_bf16(v[8], v[9]);
    b.y = pack_bf16(v[10], v[11]);
    b.z = pack_bf16(v[12], v[13]);
    b.w = pack_bf16(v[14], v[15]);
    reinterpret_cast<uint4*>(row + c0)[0] = a;
    reinterpret_cast<uint4*>(row + c0)[1] = b;
}

// Issues D = A * B^T over K (multiple of 16) from one thread: A image of
// width K at a_s (M = 128 rows), B image of width K at b_s (N rows).
__device__ __forceinline__ void issue_gemm(uint32_t tmem_d, uint32_t a_s, uint32_t b_s, int K, uint32_t idesc) {
    const uint32_t sbo = (uint32_t)K * 16;
    for (int s = 0; s < K / 16; s++)
        mma_bf16(tmem_d, sdesc(a_s + 256 * s, 128, sbo), sdesc(b_s + 256 * s, 128, sbo), idesc, s > 0 ? 1u : 0u);
}

// Loads row `row` (row < n, else zeros) of a row-major bf16 [n][32] matrix
// into the K = 32 operand image at row r.
__device__ __forceinline__ void stage_x(uint8_t* img, int r, const __nv_bfloat16* x, size_t n, size_t row) {
    uint4 v[4] = {};
    if (row < n) {
        const uint4* src = reinterpret_cast<const uint4*>(x + row * kIn);
#pragma unroll
        for (int c = 0; c < 4; c++) v[c] = __ldg(src + c);
    }
#pragma unroll
    for (int c = 0; c < 4; c++) *reinterpret_cast<uint4*>(img + img_off(r, 8 * c, kIn)) = v[c];
}

// ---------------------------------------------------------------------------
// tensor-core GEMM self-test: D[128][N] = A[128][K] B[N][K]^T (one CTA)
// ---------------------------------------------------------------------------
struct __align__(128) GemmTestSmem {
    uint8_t a[128 * 128 * 2];
    uint8_t b[256 * 128 * 2];
    uint64_t bar;
    uint32_t tmem;
};

__global__ void __launch_bounds__(kThreads, 1)
    gemm_test_kernel(const __nv_bfloat16* a, const __nv_bfloat16* b, float* d, int N, int K, int* status) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    GemmTestSmem& S = *reinterpret_cast<GemmTestSmem*>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int i = tid; i < 128 * K; i += kThreads) {
        const int r = i / K, k = i % K;
        *reinterpret_cast<__nv_bfloat16*>(S.a + img_off(r, k, K)) = a[i];
    }
    for (int i = tid; i < N * K; i += kThreads) {
        const int r = i / K, k = i % K;
        *reinterpret_cast<__nv_bfloat16*>(S.b + img_off(r, k, K)) = b[i];
    }
    if (tid == 0) {
        mbar_init(&S.bar, 1);
        mbar_fence_init();
    }
    if (warp == 0) tmem_alloc(&S.tmem, 256);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem;
    if (tid == 0) {
        issue_gemm(tmem, smem_u32(S.a), smem_u32(S.b), K, idesc_bf16(128, N));
        mma_commit(&S.bar);
    }
    const bool ok = __syncthreads_and(mbar_wait(&S.bar, 0));
    tc_fence_after();
    if (ok) {
        for (int c = 0; c < N; c += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c, v);
            for (int j = 0; j < 16; j++) d[(size_t)tid * N + c + j] = v[j];
        }
    } else if (tid == 0) {
        atomicOr(status, kStatusTimeout);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, 256);
    }
}

// ---------------------------------------------------------------------------
// inference
// ---------------------------------------------------------------------------
// Inference keeps kFwdGroups tiles in flight per CTA, one per warpgroup of 128
// threads.  Each warpgroup owns an activation image and 128 TMEM columns,
// issues its own GEMMs and runs its own epilogues, meeting only its own warps
// at named barriers; so while one warpgroup waits for its tile's MMAs, the
// others run FP32 epilogues (bias, GELU, BF16 packing), which bound this
// kernel.  A tile's input image sits at the start of its activation image: the
// layer-1 epilogue overwrites it only after the layer-1 MMAs have read it.  The
// weight images are loaded once per CTA and shared.  The epilogue runs on
// pairs of columns with the packed FP32 instructions (add/mul/fma .f32x2,
// round to nearest, as the scalar ones).
constexpr int kFwdGroups = 4;
constexpr int kFwdThreads = 128 * kFwdGroups;
constexpr uint32_t kFwdTmemCols = kFwdGroups <= 2 ? 256 : 512;  // a power of two >= 128 x groups
static_assert(kTile * kIn * 2 <= kTile * kHid * 2, "input image inside the activation image");

struct __align__(1024) FwdSmem {
    uint8_t w[kFwdImgBytes];                  // W1 | W2 | W3 images, bias block
    uint8_t h[kFwdGroups][kTile * kHid * 2];  // input (K = 32), then hidden activation (K = 128) images
    uint64_t bar_w;
    uint64_t bar_mma[kFwdGroups];
    uint32_t tmem;
};

// Barrier over the 128 threads of warpgroup g (ids 1..kFwdGroups; 0 is
// __syncthreads), returning the AND of v over them.
__device__ __forceinline__ bool group_sync_and(int g, bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.and.pred q, %2, 128, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}\n"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(g + 1)
        : "memory");
    return r != 0;
}

// 32 consecutive 32-bit TMEM columns of this thread's lane (one wait)
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// --- two FP32 values in one 64-bit register (low half first) -----------------
__device__ __forceinline__ uint64_t f2(float a, float b) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void f2_split(uint64_t r, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ uint64_t add2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t mul2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t fma2(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// gelu of two values, the same operations (and results) as the scalar gelu
__device__ __forceinline__ uint64_t gelu2(uint64_t z) {
    const uint64_t u = mul2(z, fma2(f2(kGeluK3, kGeluK3), mul2(z, z), f2(kGeluK, kGeluK)));
    float u0, u1;
    f2_split(u, u0, u1);
    const uint64_t hz = mul2(f2(0.5f, 0.5f), z);
    return fma2(hz, f2(tanh_approx(u0), tanh_approx(u1)), hz);
}

// bias + GELU of 32 accumulator columns (v) with bias b[0..31], in pairs
__device__ __forceinline__ void bias_gelu32(float (&v)[32], const float* b) {
    const float4* b4 = reinterpret_cast<const float4*>(b);
#pragma unroll
    for (int j = 0; j < 8; j++) {
        const float4 bb = b4[j];
        const uint64_t h0 = gelu2(add2(f2(v[4 * j], v[4 * j + 1]), f2(bb.x, bb.y)));
        const uint64_t h1 = gelu2(add2(f2(v[4 * j + 2], v[4 * j + 3]), f2(bb.z, bb.w)));
        f2_split(h0, v[4 * j], v[4 * j + 1]);
        f2_split(h1, v[4 * j + 2], v[4 * j + 3]);
    }
}

// hidden-layer epilogue of one thread: bias + GELU of the 128 columns of its
// accumulator row into the next layer's operand image
__device__ __forceinline__ void hidden_epilogue(uint32_t trow, const float* bias, uint8_t* img, int r) {
#pragma unroll 1
    for (int c = 0; c < kHid; c += 32) {
        float v[32];
        tmem_ld32(trow + (uint32_t)c, v);
        bias_gelu32(v, bias + c);
        store_row16(img, r, c, kHid, *reinterpret_cast<const float(*)[16]>(&v[0]));
        store_row16(img, r, c + 16, kHid, *reinterpret_cast<const float(*)[16]>(&v[16]));
    }
}

__global__ void __launch_bounds__(kFwdThreads, 1)
    mlp_forward_kernel(const uint8_t* __restrict__ wimg, const __nv_bfloat16* __restrict__ x, size_t n,
                       float* __restrict__ y, int* status) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    FwdSmem& S = *reinterpret_cast<FwdSmem*>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int g = warp >> 2;                     // warpgroup = tile slot
    const int r = tid & 127;                     // row of the tile = TMEM lane
    const size_t ntiles = (n + kTile - 1) / kTile;
    if (tid == 0) {
        mbar_init(&S.bar_w, 1);
        for (int i = 0; i < kFwdGroups; i++) mbar_init(&S.bar_mma[i], 1);
        mbar_fence_init();
    }
    if (warp == 0) tmem_alloc(&S.tmem, kFwdTmemCols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem + (uint32_t)(128 * g);
    const uint32_t trow = tmem + ((uint32_t)(32 * (warp & 3)) << 16);
    if (tid == 0) {
        mbar_expect_tx(&S.bar_w, kFwdImgBytes);
        bulk_g2s(S.w, wimg, kFwdImgBytes, &S.bar_w);
    }
    bool ok = __syncthreads_and(mbar_wait(&S.bar_w, 0));
    const float* bias = reinterpret_cast<const float*>(S.w + kImgBias);
    uint8_t* himg = S.h[g];
    const uint32_t sh = smem_u32(himg);
    uint64_t* bar = &S.bar_mma[g];
    const bool issuer = r == 0;
    uint32_t phase = 0;
    // one GEMM of this warpgroup's tile: issue, then wait for it (bounded)
    auto gemm = [&](uint32_t a_s, uint32_t b_off, int K) {
        if (issuer) {
            tc_fence_after();
            issue_gemm(tmem, a_s, smem_u32(S.w + b_off), K, kIdescN128);
            mma_commit(bar);
        }
        const bool done = group_sync_and(g, mbar_wait(bar, phase));
        phase ^= 1;
        tc_fence_after();
        return done;
    };
    auto operands_ready = [&]() {
        fence_async_smem();
        tc_fence_before();
        group_sync_and(g, true);
    };
    for (size_t tile = (size_t)blockIdx.x * kFwdGroups + g; ok && tile < ntiles;
         tile += (size_t)gridDim.x * kFwdGroups) {
        const size_t row = tile * kTile + r;
        stage_x(himg, r, x, n, row);
        operands_ready();
        if (!(ok = gemm(sh, kImgW1, kIn))) break;
        hidden_epilogue(trow, bias, himg, r);
        operands_ready();
        if (!(ok = gemm(sh, kImgW2, kHid))) break;
        hidden_epilogue(trow, bias + kHid, himg, r);
        operands_ready();
        if (!(ok = gemm(sh, kImgW3, kHid))) break;
        // layer 3 and the output layer
        uint64_t acc = f2(0.0f, 0.0f);  // even and odd columns
#pragma unroll 1
        for (int c = 0; c < kHid; c += 32) {
            float v[32];
            tmem_ld32(trow + (uint32_t)c, v);
            bias_gelu32(v, bias + 2 * kHid + c);
            const float4* w4 = reinterpret_cast<const float4*>(bias + 3 * kHid + c);
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const float4 w = w4[j];
                acc = fma2(f2(v[4 * j], v[4 * j + 1]), f2(w.x, w.y), acc);
                acc = fma2(f2(v[4 * j + 2], v[4 * j + 3]), f2(w.z, w.w), acc);
            }
        }
        float acc0, acc1;
        f2_split(acc, acc0, acc1);
        if (row < n) y[row] = (acc0 + acc1) + bias[4 * kHid];
        // this tile's TMEM reads are done before the next tile's first MMA
        tc_fence_before();
        group_sync_and(g, true);
    }
    if (!ok && r == 0) atomicOr(status, kStatusTimeout);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(S.tmem, kFwdTmemCols);
    }
}

// ---------------------------------------------------------------------------
// training: per-row forward and backward
// ---------------------------------------------------------------------------
struct __align__(1024) RowsSmem {
    uint8_t w[kImgBytes];           // all weight images and the bias block
    uint8_t x[kTile * kIn * 2];
    uint8_t a[kTile * kHid * 2];    // operand image: H1, H2, dZ3, dZ2 in turn
    float red[5][kHid];             // this CTA's b1, b2, b3, w4 gradients and b4 (red[4][0])
    uint64_t bar_w, bar_mma;
    uint32_t tmem;
    float loss;
};

// TMEM columns of the training kernel
constexpr uint32_t kColZ1 = 0, kColZ2 = 128, kColZ3 = 256, kColWork = 384;

// Adds the 128 values v (this thread's row, columns c..c+15 of a 128-wide
// quantity) to red[...], rotating the column order by the row so that the 128
// threads of a tile hit 128 different words at every step.
__device__ __forceinline__ void red_add16(float* red, int c, const float (&v)[16], int r) {
#pragma unroll
    for (int j0 = 0; j0 < 16; j0++) {
        const int j = (j0 + r) & 15;
        atomicAdd(&red[c + j], v[j]);
    }
}

struct RowsArgs {
    const uint8_t* wimg;
    const __nv_bfloat16* x;  // [n][32]
    const float* target;     // [n]
    const float* weight;     // [n] loss weights
    size_t n;
    __nv_bfloat16* h1;       // [n][128] activations and pre-activation gradients (bf16, row-major)
    __nv_bfloat16* h2;
    __nv_bfloat16* dz1;
    __nv_bfloat16* dz2;
    __nv_bfloat16* dz3;
    float* grad;             // FP32 gradient accumulators (parameter layout)
    double* loss;            // sum of weight (y - target)^2
    float* y;                // [n] predictions (may be null)
    int* status;
};

__global__ void __launch_bounds__(kThreads, 1) mlp_rows_kernel(RowsArgs A) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    RowsSmem& S = *reinterpret_cast<RowsSmem*>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5;
    const size_t ntiles = (A.n + kTile - 1) / kTile;
    for (int i = tid; i < 5 * kHid; i += kThreads) (&S.red[0][0])[i] = 0.0f;
    if (tid == 0) {
        S.loss = 0.0f;
        mbar_init(&S.bar_w, 1);
        mbar_init(&S.bar_mma, 1);
        mbar_fence_init();
    }
    if (warp == 0) tmem_alloc(&S.tmem, 512);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem;
    const uint32_t trow = tmem + ((uint32_t)(32 * warp) << 16);
    if (tid == 0) {
        mbar_expect_tx(&S.bar_w, kImgBytes);
        bulk_g2s(S.w, A.wimg, kImgBytes, &S.bar_w);
    }
    bool ok = __syncthreads_and(mbar_wait(&S.bar_w, 0));
    const float* bias = reinterpret_cast<const float*>(S.w + kImgBias);
    const float* b1 = bias;
    const float* b2 = bias + kHid;
    const float* b3 = bias + 2 * kHid;
    const float* w4 = bias + 3 * kHid;
    const float b4 = bias[4 * kHid];
    const uint32_t sx = smem_u32(S.x), sa = smem_u32(S.a);
    uint32_t phase = 0;
    auto gemm = [&](uint32_t col, uint32_t a_s, uint32_t b_off, int K) {
        if (tid == 0) {
            tc_fence_after();
            issue_gemm(tmem + col, a_s, smem_u32(S.w + b_off), K, kIdescN128);
            mma_commit(&S.bar_mma);
        }
        const bool r = __syncthreads_and(mbar_wait(&S.bar_mma, phase));
        phase ^= 1;
        tc_fence_after();
        return r;
    };
    auto sync_operands = [&]() {
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
    };
    for (size_t tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x) {
        const size_t row = tile * kTile + tid;
        const bool live = row < A.n;
        stage_x(S.x, tid, A.x, A.n, row);
        sync_operands();
        // forward: Z1, Z2, Z3 stay in TMEM for the backward pass
        if (!(ok = gemm(kColZ1, sx, kImgW1, kIn))) break;
#pragma unroll 1
        for (int c = 0; c < kHid; c += 16) {
            float v[16];
            tmem_ld16(trow + kColZ1 + c, v);
#pragma unroll
            for (int j = 0; j < 16; j++) v[j] = gelu(v[j] + b1[c + j]);
            store_row16(S.a, tid, c, kHid, v);
            if (live) store_global16(A.h1 + row * kHid, c, v);
        }
        sync_operands();
        if (!(ok = gemm(kColZ2, sa, kImgW2, kHid))) break;
#pragma unroll 1
        for (int c = 0; c < kHid; c += 16) {
            float v[16];
            tmem_ld16(trow + kColZ2 + c, v);
#pragma unroll
            for (int j = 0; j < 16; j++) v[j] = gelu(v[j] + b2[c + j]);
            store_row16(S.a, tid, c, kHid, v);
            if (live) store_global16(A.h2 + row * kHid, c, v);
        }
        sync_operands();
        if (!(ok = gemm(kColZ3, sa, kImgW3, kHid))) break;
        // output, loss, dy
        float y = 0.0f;
#pragma unroll 1
        for (int c = 0; c < kHid; c += 16) {
            float v[16];
            tmem_ld16(trow + kColZ3 + c, v);
#pragma unroll
            for (int j = 0; j < 16; j++) y = fmaf(gelu(v[j] + b3[c + j]), w4[c + j], y);
        }
        y += b4;
        float dy = 0.0f;
        if (live) {
            const float e = y - A.target[row];
            const float w = A.weight[row];
            dy = 2.0f * w * e;
            atomicAdd(&S.loss, w * e * e);
            if (A.y) A.y[row] = y;
        }
        // dw4, db4, dZ3 (and db3)
#pragma unroll 1
        for (int c = 0; c < kHid; c += 16) {
            float v[16], h[16], dz[16];
            tmem_ld16(trow + kColZ3 + c, v);
#pragma unroll
            for (int j = 0; j < 16; j++) {
                const float z = v[j] + b3[c + j];
                h[j] = dy * gelu(z);
                dz[j] = dy * w4[c + j] * gelu_grad(z);
            }
            red_add16(S.red[3], c, h, tid);
            red_add16(S.red[2], c, dz, tid);
            store_row16(S.a, tid, c, kHid, dz);
            if (live) store_global16(A.dz3 + row * kHid, c, dz);
        }
        if (dy != 0.0f) atomicAdd(&S.red[4][0], dy);
        sync_operands();
        // dH2 = dZ3 W3
        if (!(ok = gemm(kColWork, sa, kImgW3T, kHid))) break;
#pragma unroll 1
        for (int c = 0; c < kHid; c += 16) {
            float v[16], z[16];
            tmem_ld16(trow + kColWork + c, v);
            tmem_ld16(trow + kColZ2 + c, z);
#pragma unroll
            for (int j = 0; j < 16; j++) v[j] *= gelu_grad(z[j] + b2[c + j]);
            red_add16(S.red[1], c, v, tid);
            store_row16(S.a, tid, c, kHid, v);
            if (live) store_global16(A.dz2 + row * kHid, c, v);
        }
        sync_operands();
        // dH1 = dZ2 W2
        if (!(ok = gemm(kColWork, sa, kImgW2T, kHid))) break;
#pragma unroll 1
        for (int c = 0; c < kHid; c += 16) {
            float v[16], z[16];
            tmem_ld16(trow + kColWork + c, v);
            tmem_ld16(trow + kColZ1 + c, z);
#pragma unroll
            for (int j = 0; j < 16; j++) v[j] *= gelu_grad(z[j] + b1[c + j]);
            red_add16(S.red[0], c, v, tid);
            if (live) store_global16(A.dz1 + row * kHid, c, v);
        }
        tc_fence_before();
        __syncthreads();
    }
    if (!ok && tid == 0) atomicOr(A.status, kStatusTimeout);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, 512);
    }
    // this CTA's bias / output-layer gradients and loss
    for (int i = tid; i < kHid; i += kThreads) {
        atomicAdd(&A.grad[oB1 + i], S.red[0][i]);
        atomicAdd(&A.grad[oB2 + i], S.red[1][i]);
        atomicAdd(&A.grad[oB3 + i], S.red[2][i]);
        atomicAdd(&A.grad[oW4 + i], S.red[3][i]);
    }
    if (tid == 0) {
        atomicAdd(&A.grad[oB4], S.red[4][0]);
        atomicAdd(A.loss, (double)S.loss);
    }
}

// ---------------------------------------------------------------------------
// training: weight gradients dW[o][i] = sum_r dZ[r][o] H[r][i]
// ---------------------------------------------------------------------------
struct __align__(1024) WgradSmem {
    uint8_t a[kHid * kTile * 2];   // dZ^T image: [o][r], K = rows of the chunk
    uint8_t b[kHid * kTile * 2];   // H^T image: [i][r]
    uint64_t bar;
    uint32_t tmem;
};

// Writes the transpose of a row-major bf16 [rows][width] chunk (rows < nrows
// valid, the rest zero) into an image of shape [width][128] (K = rows).
__device__ __forceinline__ void stage_transposed(uint8_t* img, const __nv_bfloat16* src, size_t row0, size_t n,
                                                 int width, int tid) {
    const size_t row = row0 + tid;
    for (int c = 0; c < width; c += 8) {
        uint4 v = {0u, 0u, 0u, 0u};
        if (row < n) v = __ldg(reinterpret_cast<const uint4*>(src + row * width + c));
        const uint16_t* e = reinterpret_cast<const uint16_t*>(&v);
#pragma unroll
        for (int j = 0; j < 8; j++) *reinterpret_cast<uint16_t*>(img + img_off(c + j, tid, kTile)) = e[j];
    }
}

struct WgradArgs {
    const __nv_bfloat16* x;   // [n][32]
    const __nv_bfloat16* h1;  // [n][128]
    const __nv_bfloat16* h2;
    const __nv_bfloat16* dz1;
    const __nv_bfloat16* dz2;
    const __nv_bfloat16* dz3;
    size_t n;
    float* grad;
    int* status;
};

constexpr uint32_t kColD1 = 0, kColD2 = 128, kColD3 = 256;  // dW1 (32 columns), dW2, dW3

__global__ void __launch_bounds__(kThreads, 1) mlp_wgrad_kernel(WgradArgs A) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    WgradSmem& S = *reinterpret_cast<WgradSmem*>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5;
    const size_t nchunks = (A.n + kTile - 1) / kTile;
    if (tid == 0) {
        mbar_init(&S.bar, 1);
        mbar_fence_init();
    }
    if (warp == 0) tmem_alloc(&S.tmem, 512);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem;
    const uint32_t sa = smem_u32(S.a), sb = smem_u32(S.b);
    uint32_t phase = 0;
    bool ok = true;
    bool any = false;
    // three GEMMs per chunk of 128 rows, each accumulating into its TMEM columns
    for (size_t ch = blockIdx.x; ok && ch < nchunks; ch += gridDim.x) {
        const size_t r0 = ch * kTile;
        for (int g = 0; g < 3 && ok; g++) {
            const __nv_bfloat16* dz = g == 0 ? A.dz1 : (g == 1 ? A.dz2 : A.dz3);
            const __nv_bfloat16* h = g == 0 ? A.x : (g == 1 ? A.h1 : A.h2);
            const int width = g == 0 ? kIn : kHid;
            stage_transposed(S.a, dz, r0, A.n, kHid, tid);
            stage_transposed(S.b, h, r0, A.n, width, tid);
            fence_async_smem();
            tc_fence_before();
            __syncthreads();
            if (tid == 0) {
                tc_fence_after();
                const uint32_t col = g == 0 ? kColD1 : (g == 1 ? kColD2 : kColD3);
                const uint32_t sbo = kTile * 16;
                for (int s = 0; s < kTile / 16; s++)
                    mma_bf16(tmem + col, sdesc(sa + 256 * s, 128, sbo), sdesc(sb + 256 * s, 128, sbo),
                             g == 0 ? kIdescN32 : kIdescN128, (any || s > 0) ? 1u : 0u);
                mma_commit(&S.bar);
            }
            ok = __syncthreads_and(mbar_wait(&S.bar, phase));
            phase ^= 1;
            tc_fence_after();
        }
        any = true;
    }
    if (ok && any) {
        const uint32_t trow = tmem + ((uint32_t)(32 * warp) << 16);
        const int o = tid;  // TMEM lane = output unit
        for (int c = 0; c < kIn; c += 16) {
            float v[16];
            tmem_ld16(trow + kColD1 + c, v);
            for (int j = 0; j < 16; j++) atomicAdd(&A.grad[oW1 + o * kIn + c + j], v[j]);
        }
        for (int c = 0; c < kHid; c += 16) {
            float v[16];
            tmem_ld16(trow + kColD2 + c, v);
            for (int j = 0; j < 16; j++) atomicAdd(&A.grad[oW2 + o * kHid + c + j], v[j]);
            tmem_ld16(trow + kColD3 + c, v);
            for (int j = 0; j < 16; j++) atomicAdd(&A.grad[oW3 + o * kHid + c + j], v[j]);
        }
    }
    if (!ok && tid == 0) atomicOr(A.status, kStatusTimeout);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, 512);
    }
}

// ---------------------------------------------------------------------------
// parameters: Adam step and BF16 images
// ---------------------------------------------------------------------------
// Writes parameter i (value p) into the weight images.
__device__ __forceinline__ void image_param(uint8_t* img, int i, float p) {
    const __nv_bfloat16 b = __float2bfloat16_rn(p);
    if (i < oB1) {
        const int o = i / kIn, k = i % kIn;
        *reinterpret_cast<__nv_bfloat16*>(img + kImgW1 + img_off(o, k, kIn)) = b;
    } else if (i < oW2) {
        reinterpret_cast<float*>(img + kImgBias)[i - oB1] = p;
    } else if (i < oB2) {
        const int o = (i - oW2) / kHid, k = (i - oW2) % kHid;
        *reinterpret_cast<__nv_bfloat16*>(img + kImgW2 + img_off(o, k, kHid)) = b;
        *reinterpret_cast<__nv_bfloat16*>(img + kImgW2T + img_off(k, o, kHid)) = b;
    } else if (i < oW3) {
        reinterpret_cast<float*>(img + kImgBias)[kHid + i - oB2] = p;
    } else if (i < oB3) {
        const int o = (i - oW3) / kHid, k = (i - oW3) % kHid;
        *reinterpret_cast<__nv_bfloat16*>(img + kImgW3 + img_off(o, k, kHid)) = b;
        *reinterpret_cast<__nv_bfloat16*>(img + kImgW3T + img_off(k, o, kHid)) = b;
    } else {
        reinterpret_cast<float*>(img + kImgBias)[2 * kHid + i - oB3] = p;  // b3, w4, b4
    }
}

__global__ void mlp_pack_kernel(const float* __restrict__ params, uint8_t* img) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kNumParams; i += gridDim.x * blockDim.x)
        image_param(img, i, params[i]);
}

struct AdamArgs {
    float* params;
    float* m;
    float* v;
    float* grad;   // cleared after use
    uint8_t* img;
    float lr, beta1, beta2, eps;
    float c1, c2;  // bias corrections 1 - beta^t
};

__global__ void mlp_adam_kernel(AdamArgs A) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kNumParams; i += gridDim.x * blockDim.x) {
        const float g = A.grad[i];
        const float m = A.beta1 * A.m[i] + (1.0f - A.beta1) * g;
        const float v = A.beta2 * A.v[i] + (1.0f - A.beta2) * g * g;
        A.m[i] = m;
        A.v[i] = v;
        const float p = A.params[i] - A.lr * (m / A.c1) / (sqrtf(v / A.c2) + A.eps);
        A.params[i] = p;
        A.grad[i] = 0.0f;
        image_param(A.img, i, p);
    }
}

// ---------------------------------------------------------------------------
// features of the dropped partners
// ---------------------------------------------------------------------------
struct FeatGate {
    uint64_t sup[2];  // qubits the gate acts on
    float abs_sin;    // |sin theta| (rotations), 0 for Clifford gates
    int rot;          // 1 for a rotation
};

struct FeatArgs {
    const uint64_t* key;   // [4][stride] caller layout
    size_t stride;
    const double* coef;    // [n] real parts
    const int32_t* gate;   // [n]
    size_t n;
    const FeatGate* gates; // [ngates] circuit order
    const int32_t* batch_of_gate;  // [ngates] commuting-run index in application order
    int ngates, nbatches, maxdeg, obs;
    const float* coords;   // [2][128] lattice coordinates of the qubits
    float lx, ly;          // lattice extents
    float* feat;           // [n][32] FP32 (may be null)
    __nv_bfloat16* x;      // [n][32] BF16 network input (may be null): (f - shift) * scale
    const float* shift;    // [32] (null: 0)
    const float* scale;    // [32] (null: 1)
};

__global__ void drop_features_kernel(FeatArgs A) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    if (A.gate[i] < 0 || A.gate[i] >= A.ngates) {  // not a gate of this circuit: zero features
        if (A.feat)
            for (int k = 0; k < 32; k++) A.feat[i * 32 + k] = 0.0f;
        if (A.x)
            for (int k = 0; k < 32; k++) A.x[i * 32 + k] = __float2bfloat16_rn(0.0f);
        return;
    }
    const uint64_t x0 = A.key[i], x1 = A.key[A.stride + i];
    const uint64_t z0 = A.key[2 * A.stride + i], z1 = A.key[3 * A.stride + i];
    const uint64_t s0 = x0 | z0, s1 = x1 | z1;
    const int nx = __popcll(x0 & ~z0) + __popcll(x1 & ~z1);
    const int ny = __popcll(x0 & z0) + __popcll(x1 & z1);
    const int nz = __popcll(z0 & ~x0) + __popcll(z1 & ~x1);
    const int w = nx + ny + nz;
    const float ox = A.coords[A.obs], oy = A.coords[128 + A.obs];
    float xmin = 1e9f, xmax = -1e9f, ymin = 1e9f, ymax = -1e9f, cx = 0.0f, cy = 0.0f, dmin = 1e9f;
    float near[3] = {0.0f, 0.0f, 0.0f}, mid[3] = {0.0f, 0.0f, 0.0f};
    for (int wd = 0; wd < 2; wd++) {
        uint64_t s = wd ? s1 : s0;
        const uint64_t xw = wd ? x1 : x0, zw = wd ? z1 : z0;
        while (s) {
            const int b = __ffsll((long long)s) - 1;
            s &= s - 1;
            const int q = 64 * wd + b;
            const float qx = A.coords[q], qy = A.coords[128 + q];
            xmin = fminf(xmin, qx);
            xmax = fmaxf(xmax, qx);
            ymin = fminf(ymin, qy);
            ymax = fmaxf(ymax, qy);
            cx += qx;
            cy += qy;
            const float d = fabsf(qx - ox) + fabsf(qy - oy);
            dmin = fminf(dmin, d);
            const int xb = (int)((xw >> b) & 1ull), zb = (int)((zw >> b) & 1ull);
            const int type = xb && zb ? 1 : (xb ? 0 : 2);  // X, Y, Z
            if (d <= 1.0f) near[type] += 1.0f;
            else if (d <= 3.0f) mid[type] += 1.0f;
        }
    }
    const float inv_w = w ? 1.0f / (float)w : 0.0f;
    cx *= inv_w;
    cy *= inv_w;
    // backward light cone through the gates still to come: gates [0, g)
    const int g = A.gate[i];
    uint64_t c0 = s0, c1 = s1;
    int cone = 0;
    float sin_sum = 0.0f;
    for (int j = g - 1; j >= 0; j--) {
        const FeatGate G = A.gates[j];
        if ((G.sup[0] & c0) | (G.sup[1] & c1)) {
            cone++;
            sin_sum += G.abs_sin;
            c0 |= G.sup[0];
            c1 |= G.sup[1];
        }
    }
    const FeatGate Gg = A.gates[g];
    const double c = A.coef[i];
    const float span = A.lx + A.ly;
    float f[32];
    f[0] = w / 8.0f;
    f[1] = nx / 8.0f;
    f[2] = ny / 8.0f;
    f[3] = nz / 8.0f;
    f[4] = xmin / A.lx;
    f[5] = xmax / A.lx;
    f[6] = ymin / A.ly;
    f[7] = ymax / A.ly;
    f[8] = (xmax - xmin + 1.0f) * (ymax - ymin + 1.0f) / (A.lx * A.ly);
    f[9] = (float)(log10(fabs(c) + 1e-300) / 8.0 + 1.0);
    f[10] = c < 0.0 ? -1.0f : 1.0f;
    f[11] = (float)A.batch_of_gate[g] / (float)A.nbatches;
    f[12] = (float)g / (float)A.ngates;
    f[13] = (float)cone / (float)A.ngates;
    f[14] = cone ? sin_sum / (float)cone : 0.0f;
    f[15] = Gg.abs_sin;
    f[16] = Gg.rot ? sqrtf(fmaxf(0.0f, 1.0f - Gg.abs_sin * Gg.abs_sin)) : 1.0f;
    f[17] = dmin / span;
    f[18] = (fabsf(cx - ox) + fabsf(cy - oy)) / span;
    f[19] = (((A.obs < 64 ? s0 >> A.obs : s1 >> (A.obs - 64)) & 1ull) != 0) ? 1.0f : 0.0f;
    f[20] = (nx + ny) / 8.0f;
    f[21] = near[0] / 5.0f;
    f[22] = near[1] / 5.0f;
    f[23] = near[2] / 5.0f;
    f[24] = mid[0] / 8.0f;
    f[25] = mid[1] / 8.0f;
    f[26] = mid[2] / 8.0f;
    f[27] = (w - A.maxdeg) / 4.0f;
    f[28] = (float)(__popcll(c0) + __popcll(c1)) / (A.lx * A.ly);
    f[29] = (float)(A.nbatches - A.batch_of_gate[g]) / (float)A.nbatches;
    f[30] = (cx - ox) / A.lx;
    f[31] = (cy - oy) / A.ly;
    if (A.feat)
        for (int k = 0; k < 32; k++) A.feat[i * 32 + k] = f[k];
    if (A.x) {
        if (A.shift)
            for (int k = 0; k < 32; k++) f[k] = (f[k] - A.shift[k]) * A.scale[k];
        for (int k = 0; k < 32; k += 2)
            *reinterpret_cast<uint32_t*>(A.x + i * 32 + k) = pack_bf16(f[k], f[k + 1]);
    }
}

// sum over rows of coef[r] * t[r] (the predicted correction), one block
__global__ void correction_sum_kernel(const double* coef, const float* t, size_t n, double* out) {
    __shared__ double part[256];
    double s = 0.0;
    for (size_t i = threadIdx.x; i < n; i += blockDim.x) s += coef[i] * (double)t[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = part[0];
}

// Set-level training targets.  For segments s (rows seg[s] .. seg[s+1]) with
// targets delta[s] the loss is
//     L = sum_s R_s^2 + sum_r lw_r (y_r - label_r)^2,  R_s = sum_{r in s} c_r y_r - delta_s,
// so dL/dy_r = 2 R_s c_r + 2 lw_r (y_r - label_r).  The per-row training
// kernel minimises sum_r w_r (y_r - t_r)^2, whose gradient is 2 w_r (y_r - t_r):
// with w_r = omega + lw_r and t_r = y_r - (R_s c_r + lw_r (y_r - label_r)) / w_r
// its step is a step on L.
__global__ void segment_residual_kernel(const float* y, const double* coef, const int64_t* seg,
                                        const double* delta, double* R, double* loss) {
    __shared__ double part[256];
    const int s = blockIdx.x;
    double acc = 0.0;
    for (int64_t r = seg[s] + threadIdx.x; r < seg[s + 1]; r += blockDim.x) acc += coef[r] * (double)y[r];
    part[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double r = part[0] - delta[s];
        R[s] = r;
        atomicAdd(&loss[0], r * r);
    }
}

__global__ void set_targets_kernel(const float* y, const double* coef, const int64_t* seg, int nseg,
                                   const double* R, const float* label, const float* lw, float omega, size_t n,
                                   float* target, float* weight, double* loss) {
    const size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    int lo = 0, hi = nseg - 1;  // segment of row r: seg[lo] <= r < seg[lo + 1]
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (seg[mid] <= (int64_t)r) lo = mid;
        else hi = mid - 1;
    }
    double g = R[lo] * coef[r];
    float w = omega;
    if (label) {
        const float e = y[r] - label[r];
        g += (double)lw[r] * e;
        w += lw[r];
        atomicAdd(&loss[1], (double)lw[r] * e * e);
    }
    weight[r] = w;
    target[r] = (float)((double)y[r] - g / w);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
template <typename K>
cudaError_t set_smem(K kern, size_t bytes) {
    return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

}  // namespace

struct ffg_mlp {
    ffg_ctx* ctx = nullptr;
    int device = 0;
    cudaStream_t stream = nullptr;
    int num_sms = 148;
    float* params = nullptr;  // FP32 master parameters
    float* m = nullptr;
    float* v = nullptr;
    float* grad = nullptr;
    uint8_t* img = nullptr;
    double* loss = nullptr;
    int* status = nullptr;
    long long step = 0;
    // training scratch: h1, h2, dz1, dz2, dz3 ([rows][128] bf16 each)
    __nv_bfloat16* act = nullptr;
    size_t act_rows = 0;
    // set-level targets: predictions, segment residuals, two loss terms
    float* ys = nullptr;
    size_t ys_rows = 0;
    double* R = nullptr;
    size_t R_segs = 0;
    double* loss2 = nullptr;
    std::string err;
};

namespace {
int mlp_err(ffg_mlp* m, int code, const std::string& msg) {
    if (m) m->err = msg;
    return code;
}

#define MCK(call)                                                                         \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) return mlp_err(m, FFG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

int mlp_check_status(ffg_mlp* m) {
    int st = 0;
    MCK(cudaMemcpyAsync(&st, m->status, 4, cudaMemcpyDeviceToHost, m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    if (st) return mlp_err(m, FFG_ERR_STATE, "MLP kernel: a tensor-core wait timed out");
    return FFG_OK;
}

int ensure_act(ffg_mlp* m, size_t rows) {
    if (m->act_rows >= rows) return FFG_OK;
    if (m->act) MCK(cudaFree(m->act));
    m->act = nullptr;
    m->act_rows = 0;
    const size_t r = ((rows + kTile - 1) / kTile) * kTile;
    MCK(cudaMalloc(&m->act, 5 * r * kHid * sizeof(__nv_bfloat16)));
    m->act_rows = r;
    return FFG_OK;
}

int grid_rows(const ffg_mlp* m, size_t n) {
    const size_t tiles = (n + kTile - 1) / kTile;
    return (int)std::max<size_t>(1, std::min<size_t>(tiles, (size_t)m->num_sms));
}

// inference CTAs: kFwdGroups tiles at a time, at most one CTA per SM
int grid_fwd(const ffg_mlp* m, size_t n) {
    const size_t slots = (n + (size_t)kTile * kFwdGroups - 1) / ((size_t)kTile * kFwdGroups);
    return (int)std::max<size_t>(1, std::min<size_t>(slots, (size_t)m->num_sms));
}

// forward and backward over n rows into m->grad (cleared first when clear)
int run_gradient(ffg_mlp* m, const uint16_t* x, const float* target, const float* weight, size_t n,
                 float* y) {
    int rc = ensure_act(m, n);
    if (rc) return rc;
    const size_t r = m->act_rows;
    RowsArgs A{};
    A.wimg = m->img;
    A.x = reinterpret_cast<const __nv_bfloat16*>(x);
    A.target = target;
    A.weight = weight;
    A.n = n;
    A.h1 = m->act;
    A.h2 = m->act + r * kHid;
    A.dz1 = m->act + 2 * r * kHid;
    A.dz2 = m->act + 3 * r * kHid;
    A.dz3 = m->act + 4 * r * kHid;
    A.grad = m->grad;
    A.loss = m->loss;
    A.y = y;
    A.status = m->status;
    MCK(cudaMemsetAsync(m->loss, 0, 8, m->stream));
    mlp_rows_kernel<<<grid_rows(m, n), kThreads, sizeof(RowsSmem), m->stream>>>(A);
    MCK(cudaGetLastError());
    WgradArgs W{};
    W.x = A.x;
    W.h1 = A.h1;
    W.h2 = A.h2;
    W.dz1 = A.dz1;
    W.dz2 = A.dz2;
    W.dz3 = A.dz3;
    W.n = n;
    W.grad = m->grad;
    W.status = m->status;
    mlp_wgrad_kernel<<<grid_rows(m, n), kThreads, sizeof(WgradSmem), m->stream>>>(W);
    MCK(cudaGetLastError());
    return FFG_OK;
}
}  // namespace

extern "C" {

const char* ffg_mlp_last_error(const ffg_mlp* m) { return m ? m->err.c_str() : "null network"; }

int ffg_mlp_create(ffg_ctx* ctx, ffg_mlp** out) {
    if (!ctx || !out) return FFG_ERR_ARG;
    *out = nullptr;
    auto* m = new ffg_mlp();
    std::unique_ptr<ffg_mlp, void (*)(ffg_mlp*)> guard(m, ffg_mlp_free);
    m->ctx = ctx;
    m->stream = (cudaStream_t)ffg_stream(ctx);
    MCK(cudaGetDevice(&m->device));
    MCK(cudaDeviceGetAttribute(&m->num_sms, cudaDevAttrMultiProcessorCount, m->device));
    MCK(cudaMalloc(&m->params, kNumParams * 4));
    MCK(cudaMalloc(&m->m, kNumParams * 4));
    MCK(cudaMalloc(&m->v, kNumParams * 4));
    MCK(cudaMalloc(&m->grad, kNumParams * 4));
    MCK(cudaMalloc(&m->img, kImgBytes));
    MCK(cudaMalloc(&m->loss, 8));
    MCK(cudaMalloc(&m->status, 4));
    MCK(cudaMemsetAsync(m->params, 0, kNumParams * 4, m->stream));
    MCK(cudaMemsetAsync(m->m, 0, kNumParams * 4, m->stream));
    MCK(cudaMemsetAsync(m->v, 0, kNumParams * 4, m->stream));
    MCK(cudaMemsetAsync(m->grad, 0, kNumParams * 4, m->stream));
    MCK(cudaMemsetAsync(m->img, 0, kImgBytes, m->stream));
    MCK(cudaMemsetAsync(m->status, 0, 4, m->stream));
    static int attr_dev = -1;
    if (attr_dev != m->device) {
        MCK(set_smem(mlp_forward_kernel, sizeof(FwdSmem)));
        MCK(set_smem(mlp_rows_kernel, sizeof(RowsSmem)));
        MCK(set_smem(mlp_wgrad_kernel, sizeof(WgradSmem)));
        MCK(set_smem(gemm_test_kernel, sizeof(GemmTestSmem)));
        attr_dev = m->device;
    }
    MCK(cudaStreamSynchronize(m->stream));
    *out = guard.release();
    return FFG_OK;
}

void ffg_mlp_free(ffg_mlp* m) {
    if (!m) return;
    cudaSetDevice(m->device);
    if (m->stream) cudaStreamSynchronize(m->stream);
    for (void* p : {(void*)m->params, (void*)m->m, (void*)m->v, (void*)m->grad, (void*)m->img, (void*)m->loss,
                    (void*)m->status, (void*)m->act, (void*)m->ys, (void*)m->R, (void*)m->loss2})
        if (p) cudaFree(p);
    delete m;
}

int ffg_mlp_set_params(ffg_mlp* m, const float* params) {
    if (!m || !params) return FFG_ERR_ARG;
    MCK(cudaMemcpyAsync(m->params, params, kNumParams * 4, cudaMemcpyHostToDevice, m->stream));
    MCK(cudaMemsetAsync(m->m, 0, kNumParams * 4, m->stream));
    MCK(cudaMemsetAsync(m->v, 0, kNumParams * 4, m->stream));
    MCK(cudaMemsetAsync(m->grad, 0, kNumParams * 4, m->stream));
    mlp_pack_kernel<<<(kNumParams + 255) / 256, 256, 0, m->stream>>>(m->params, m->img);
    MCK(cudaGetLastError());
    MCK(cudaStreamSynchronize(m->stream));
    m->step = 0;
    return FFG_OK;
}

int ffg_mlp_get_params(const ffg_mlp* mc, float* params) {
    ffg_mlp* m = const_cast<ffg_mlp*>(mc);
    if (!m || !params) return FFG_ERR_ARG;
    MCK(cudaMemcpyAsync(params, m->params, kNumParams * 4, cudaMemcpyDeviceToHost, m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    return FFG_OK;
}

int ffg_mlp_forward(ffg_mlp* m, const uint16_t* x, size_t n, float* y) {
    if (!m || (n && (!x || !y))) return FFG_ERR_ARG;
    if (!n) return FFG_OK;
    if (((uintptr_t)x & 15) != 0) return mlp_err(m, FFG_ERR_ARG, "x must be 16-byte aligned");
    mlp_forward_kernel<<<grid_fwd(m, n), kFwdThreads, sizeof(FwdSmem), m->stream>>>(
        m->img, reinterpret_cast<const __nv_bfloat16*>(x), n, y, m->status);
    MCK(cudaGetLastError());
    return mlp_check_status(m);
}

int ffg_mlp_gradient(ffg_mlp* m, const uint16_t* x, const float* target, const float* weight, size_t n,
                     float* grad, double* loss) {
    if (!m || !grad || (n && (!x || !target || !weight))) return FFG_ERR_ARG;
    if (((uintptr_t)x & 15) != 0) return mlp_err(m, FFG_ERR_ARG, "x must be 16-byte aligned");
    MCK(cudaMemsetAsync(m->grad, 0, kNumParams * 4, m->stream));
    if (n) {
        int rc = run_gradient(m, x, target, weight, n, nullptr);
        if (rc) return rc;
    } else {
        MCK(cudaMemsetAsync(m->loss, 0, 8, m->stream));
    }
    int rc = mlp_check_status(m);
    if (rc) return rc;
    MCK(cudaMemcpyAsync(grad, m->grad, kNumParams * 4, cudaMemcpyDeviceToHost, m->stream));
    if (loss) MCK(cudaMemcpyAsync(loss, m->loss, 8, cudaMemcpyDeviceToHost, m->stream));
    MCK(cudaMemsetAsync(m->grad, 0, kNumParams * 4, m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    return FFG_OK;
}

int ffg_mlp_adam_step(ffg_mlp* m, const uint16_t* x, const float* target, const float* weight, size_t n,
                      float lr, float beta1, float beta2, float eps, double* loss) {
    if (!m || (n && (!x || !target || !weight))) return FFG_ERR_ARG;
    if (((uintptr_t)x & 15) != 0) return mlp_err(m, FFG_ERR_ARG, "x must be 16-byte aligned");
    if (n) {
        int rc = run_gradient(m, x, target, weight, n, nullptr);
        if (rc) return rc;
    }
    m->step++;
    AdamArgs A{};
    A.params = m->params;
    A.m = m->m;
    A.v = m->v;
    A.grad = m->grad;
    A.img = m->img;
    A.lr = lr;
    A.beta1 = beta1;
    A.beta2 = beta2;
    A.eps = eps;
    A.c1 = 1.0f - std::pow(beta1, (float)m->step);
    A.c2 = 1.0f - std::pow(beta2, (float)m->step);
    mlp_adam_kernel<<<(kNumParams + 255) / 256, 256, 0, m->stream>>>(A);
    MCK(cudaGetLastError());
    if (loss) {
        int rc = mlp_check_status(m);
        if (rc) return rc;
        MCK(cudaMemcpyAsync(loss, m->loss, 8, cudaMemcpyDeviceToHost, m->stream));
        MCK(cudaStreamSynchronize(m->stream));
    }
    return FFG_OK;
}

int ffg_mlp_correction(ffg_mlp* m, const uint16_t* x, const double* coef, size_t n, float* t, double* out) {
    if (!m || !out || (n && (!x || !coef || !t))) return FFG_ERR_ARG;
    *out = 0.0;
    if (!n) return FFG_OK;
    int rc = ffg_mlp_forward(m, x, n, t);
    if (rc) return rc;
    double* d = reinterpret_cast<double*>(m->loss);  // reused as the one-value output
    correction_sum_kernel<<<1, 256, 0, m->stream>>>(coef, t, n, d);
    MCK(cudaGetLastError());
    MCK(cudaMemcpyAsync(out, d, 8, cudaMemcpyDeviceToHost, m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    return FFG_OK;
}

int ffg_mlp_set_targets(ffg_mlp* m, const uint16_t* x, size_t n, const double* coef, const int64_t* seg,
                        const double* delta, size_t nseg, const float* label, const float* label_weight,
                        float* target, float* weight, double* loss) {
    if (!m || !n || !nseg || !x || !coef || !seg || !delta || !target || !weight || (label && !label_weight))
        return FFG_ERR_ARG;
    if (((uintptr_t)x & 15) != 0) return mlp_err(m, FFG_ERR_ARG, "x must be 16-byte aligned");
    if (m->ys_rows < n) {
        if (m->ys) MCK(cudaFree(m->ys));
        m->ys = nullptr;
        MCK(cudaMalloc(&m->ys, n * 4));
        m->ys_rows = n;
    }
    if (m->R_segs < nseg) {
        if (m->R) MCK(cudaFree(m->R));
        m->R = nullptr;
        MCK(cudaMalloc(&m->R, nseg * 8));
        m->R_segs = nseg;
    }
    if (!m->loss2) MCK(cudaMalloc(&m->loss2, 16));
    MCK(cudaMemsetAsync(m->loss2, 0, 16, m->stream));
    mlp_forward_kernel<<<grid_fwd(m, n), kFwdThreads, sizeof(FwdSmem), m->stream>>>(
        m->img, reinterpret_cast<const __nv_bfloat16*>(x), n, m->ys, m->status);
    MCK(cudaGetLastError());
    segment_residual_kernel<<<(unsigned)nseg, 256, 0, m->stream>>>(m->ys, coef, seg, delta, m->R, m->loss2);
    MCK(cudaGetLastError());
    set_targets_kernel<<<(unsigned)((n + 255) / 256), 256, 0, m->stream>>>(
        m->ys, coef, seg, (int)nseg, m->R, label, label_weight, 1.0f / (float)n, n, target, weight, m->loss2);
    MCK(cudaGetLastError());
    if (loss) {
        int rc = mlp_check_status(m);
        if (rc) return rc;
        MCK(cudaMemcpyAsync(loss, m->loss2, 16, cudaMemcpyDeviceToHost, m->stream));
        MCK(cudaStreamSynchronize(m->stream));
    }
    return FFG_OK;
}

int ffg_mlp_selftest_gemm(ffg_mlp* m, int N, int K, const uint16_t* a, const uint16_t* b, float* d) {
    if (!m || !a || !b || !d) return FFG_ERR_ARG;
    if (K <= 0 || K > 128 || K % 16 || N < 16 || N > 256 || N % 16)
        return mlp_err(m, FFG_ERR_ARG, "self-test GEMM: K in 16..128 and N in 16..256, multiples of 16");
    void *da = nullptr, *db = nullptr, *dd = nullptr;
    MCK(cudaMalloc(&da, 128 * K * 2));
    MCK(cudaMalloc(&db, (size_t)N * K * 2));
    MCK(cudaMalloc(&dd, (size_t)128 * N * 4));
    cudaError_t e = cudaMemcpyAsync(da, a, 128 * K * 2, cudaMemcpyHostToDevice, m->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(db, b, (size_t)N * K * 2, cudaMemcpyHostToDevice, m->stream);
    if (e == cudaSuccess) {
        gemm_test_kernel<<<1, kThreads, sizeof(GemmTestSmem), m->stream>>>(
            (const __nv_bfloat16*)da, (const __nv_bfloat16*)db, (float*)dd, N, K, m->status);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(d, dd, (size_t)128 * N * 4, cudaMemcpyDeviceToHost, m->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    cudaFree(da);
    cudaFree(db);
    cudaFree(dd);
    if (e != cudaSuccess) return mlp_err(m, FFG_ERR_CUDA, cudaGetErrorString(e));
    return mlp_check_status(m);
}

int ffg_drop_features(ffg_ctx* ctx, const uint64_t* keys, size_t stride, const double* coef, const int32_t* gate,
                      size_t n, const ffg_pauli_gate* gates, size_t ngates, const int32_t* batch_of_gate,
                      int32_t nbatches, const float* coords, int32_t obs_qubit, int32_t maxdegree,
                      const float* shift, const float* scale, float* feat, uint16_t* x) {
    if (!ctx || (n && (!keys || !coef || !gate)) || !gates || !ngates || !batch_of_gate || nbatches < 1 || !coords ||
        obs_qubit < 0 || obs_qubit >= 128 || (!shift != !scale))
        return FFG_ERR_ARG;
    if (!n) return FFG_OK;
    cudaStream_t st = (cudaStream_t)ffg_stream(ctx);
    std::vector<FeatGate> fg(ngates);
    float lx = 1.0f, ly = 1.0f;
    for (int q = 0; q < 128; q++) {
        lx = std::max(lx, coords[q] + 1.0f);
        ly = std::max(ly, coords[128 + q] + 1.0f);
    }
    for (size_t j = 0; j < ngates; j++) {
        const ffg_pauli_gate& G = gates[j];
        FeatGate f{};
        if (G.kind == FFG_ROT) {
            f.sup[0] = G.x[0] | G.z[0];
            f.sup[1] = G.x[1] | G.z[1];
            f.abs_sin = (float)std::fabs(std::sin(G.theta));
            f.rot = 1;
        } else {
            for (int q : {G.q0, G.q1}) {
                if (q < 0 || q >= 128 || (q == G.q1 && (G.kind == FFG_H || G.kind == FFG_S))) continue;
                f.sup[q >> 6] |= 1ull << (q & 63);
            }
        }
        fg[j] = f;
    }
    FeatGate* dg = nullptr;
    int32_t* db = nullptr;
    float* dc = nullptr;
    auto cleanup = [&]() {
        if (dg) cudaFree(dg);
        if (db) cudaFree(db);
        if (dc) cudaFree(dc);
    };
    cudaError_t e = cudaMalloc(&dg, ngates * sizeof(FeatGate));
    if (e == cudaSuccess) e = cudaMalloc(&db, ngates * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dc, 320 * 4);  // coords, then shift and scale
    if (e == cudaSuccess) e = cudaMemcpyAsync(dg, fg.data(), ngates * sizeof(FeatGate), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(db, batch_of_gate, ngates * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dc, coords, 256 * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && shift) e = cudaMemcpyAsync(dc + 256, shift, 32 * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && scale) e = cudaMemcpyAsync(dc + 288, scale, 32 * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        FeatArgs A{};
        A.key = keys;
        A.stride = stride;
        A.coef = coef;
        A.gate = gate;
        A.n = n;
        A.gates = dg;
        A.batch_of_gate = db;
        A.ngates = (int)ngates;
        A.nbatches = nbatches;
        A.maxdeg = maxdegree;
        A.obs = obs_qubit;
        A.coords = dc;
        A.lx = lx;
        A.ly = ly;
        A.feat = feat;
        A.x = reinterpret_cast<__nv_bfloat16*>(x);
        A.shift = shift ? dc + 256 : nullptr;
        A.scale = scale ? dc + 288 : nullptr;
        drop_features_kernel<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(A);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cleanup();
    return e == cudaSuccess ? FFG_OK : FFG_ERR_CUDA;
}

}  // extern "C"
