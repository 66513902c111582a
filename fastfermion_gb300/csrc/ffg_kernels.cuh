// Propagation kernels (sm_103a).  One rotation gate = one launch of
// pauli_rot_kernel / majorana_rot_kernel over the term store; truncation,
// Clifford segments, compaction and index rebuilds are separate passes.
//
// Per-gate update (src/pauli/propagate.h:71-89, src/majorana_gates.h:67-103).
// For a gate axis P every anticommuting term Q has exactly one partner key
// K = P*Q, and K anticommutes with P too, so the update is a 2x2 butterfly on
// the pair (Q, K):
//     c_Q' = c_Q cos + [deg Q <= W] * c_K * (i sin) * phase(P*K)
//     c_K' = c_K cos + [deg K <= W] * c_Q * (i sin) * phase(P*Q)
// where an absent partner contributes nothing (and an absent K that passes the
// degree filter is created with value 0 + c_Q (i sin) phase(P*Q)).  Each pair
// is owned by the thread of its lower store position, so the update is done in
// place without atomics on coefficients, and each coefficient sees exactly the
// one rounding per operation that the reference applies.
// The kernel headers are included by several translation units of libffg:
// templates and inline functions may repeat across them, and the few
// non-template kernels are declared static (internal linkage).
#pragma once
#include "ffg_device.cuh"

namespace ffg {

struct RotArgs {
    u64 p[8];      // Pauli: x words [0, NW), z words [NW, 2NW); Majorana: alpha words
    u64 mg[4];     // Majorana: bit t = parity of #{g in gate : g > t}
    double c, s;   // cos(theta), sin(theta) from the host C library
    double fr, fi; // Majorana: i * i^r * sin(theta)
    int maxdeg;    // partner filter
    int gate_odd;  // Majorana: odd gate degree
    int yP;        // Pauli: popc(x_P & z_P)
    u32 op;        // position in the op list (overflow reporting)
};

struct TruncArgs {
    double tau;      // erase |c| <= tau when thr != 0
    int thr;
    int max_xweight; // erase popc(x) > max_xweight when >= 0 (Pauli)
    u32 op;
};

struct CliffordOp {
    int kind, q0, q1, pad;
};

enum { kH = 1, kS = 2, kCNOT = 3, kSWAP = 4, kCZ = 5 };

// ---------------------------------------------------------------------------
// kernel entry / exit bookkeeping
// ---------------------------------------------------------------------------
struct Entry {
    u64 n, alive;
    int skip;
};

// need: store positions the kernel may fill (checked against cap)
__device__ __forceinline__ void kernel_enter(DevCounters* C, u64 cap, bool doubles, u32 op,
                                             Entry* e) {
    if (threadIdx.x == 0) {
        volatile DevCounters* V = C;
        const u64 n = V->n;
        int skip = V->overflow != 0 || V->error != 0;
        if (!skip && doubles && 2 * n > cap) {
            atomicCAS(&C->overflow, 0u, op + 1u);
            skip = 1;
        }
        e->n = n;
        e->alive = V->alive;
        e->skip = skip;
    }
    __syncthreads();
}

// Folds the block's live-count change into the counters; the last block to
// finish commits n, alive, apps and peak for the next kernel.
__device__ __forceinline__ void kernel_exit(DevCounters* C, const Entry& e, long long d_alive,
                                            long long* sh, bool is_rot, long long emits = 0) {
    const long long tot = block_sum_ll(d_alive, sh);
    const long long em = is_rot ? block_sum_ll(emits, sh) : 0;
    if (threadIdx.x == 0) {
        if (tot) atomicAdd((u64*)&C->d_alive, (u64)tot);
        if (em) atomicAdd(&C->emits, (u64)em);
        __threadfence();
        const u32 prev = atomicAdd(&C->done, 1u);
        if (prev == gridDim.x - 1) {
            __threadfence();
            volatile DevCounters* V = C;
            const u64 app = V->d_app;
            const long long da = V->d_alive;
            V->n = e.n + app;
            const u64 a = (u64)((long long)e.alive + da);
            V->alive = a;
            if (is_rot && !e.skip) {
                V->apps = V->apps + e.alive;
                if (a > V->peak) V->peak = a;
            }
            V->d_app = 0;
            V->d_alive = 0;
            V->done = 0;
            __threadfence();
        }
    }
}

template <bool CPLX>
__device__ __forceinline__ cplx load_coef(const StoreView& s, u64 i) {
    return {s.re[i], CPLX ? s.im[i] : 0.0};
}

template <bool CPLX>
__device__ __forceinline__ void store_coef(const StoreView& s, u64 i, cplx v) {
    s.re[i] = v.re;
    if (CPLX) s.im[i] = v.im;
}

// Creates the entry for key k with value v at a fresh position after n_in and
// returns the live-count change.  When k is held by a dead entry (truncated
// earlier, not yet compacted away; dead_slot names its index slot) the index
// slot is re-pointed to the new position and the dead entry stays dead.  A
// dead entry is never revived in place: its own thread in this kernel could
// then see it live and process the pair a second time.
template <int KW, bool CPLX>
__device__ __forceinline__ int emit_partner(const StoreView& s, DevCounters* C, u64 n_in,
                                            long long dead_slot, const u64 (&k)[KW], cplx v) {
    const cplx nv = rot_add<CPLX>({0.0, 0.0}, v);  // operator[] starts from complex zero
    const u64 pos = n_in + atomicAdd(&C->d_app, 1ull);
#pragma unroll
    for (int w = 0; w < KW; w++) s.key[(u64)w * s.cap + pos] = k[w];
    store_coef<CPLX>(s, pos, nv);
    s.dead[pos] = 0;
    __threadfence();
    if (dead_slot >= 0) {
        const u64 e = __ldcg(&s.slots[dead_slot]);
        atomicExch(&s.slots[dead_slot], (e & 0xffffffff00000000ull) | pos);
    } else {
        insert<KW>(s, k, (u32)pos, &C->error, false);
    }
    return 1;
}

// ---------------------------------------------------------------------------
// Pauli rotation  exp(-i theta/2 P)
// ---------------------------------------------------------------------------
template <int NW, bool CPLX>
__global__ void __launch_bounds__(kBlock) pauli_rot_kernel(StoreView s, DevCounters* C, RotArgs a) {
    constexpr int KW = 2 * NW;
    __shared__ Entry e;
    __shared__ long long sh[kBlock / 32];
    kernel_enter(C, s.cap, true, a.op, &e);
    long long d_alive = 0, emits = 0;
    if (!e.skip) {
        const u64 n_in = e.n;
        const u64 stride = (u64)gridDim.x * blockDim.x;
        const cplx isin = {0.0, a.s};
        for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n_in; i += stride) {
            // anticommutation parity from the planes the axis touches only
            u64 par = 0;
#pragma unroll
            for (int w = 0; w < NW; w++) {
                if (a.p[NW + w]) par ^= s.key[(u64)w * s.cap + i] & a.p[NW + w];
                if (a.p[w]) par ^= s.key[(u64)(NW + w) * s.cap + i] & a.p[w];
            }
            if (!(__popcll(par) & 1)) continue;
            if (s.dead[i]) continue;
            u64 q[KW], k[KW];
            load_key<KW>(s, i, q);
#pragma unroll
            for (int w = 0; w < KW; w++) k[w] = q[w] ^ a.p[w];
            int yQ = 0, yK = 0, zxQ = 0, zxK = 0, dQ = 0, dK = 0;
#pragma unroll
            for (int w = 0; w < NW; w++) {
                yQ += __popcll(q[w] & q[NW + w]);
                yK += __popcll(k[w] & k[NW + w]);
                zxQ += __popcll(a.p[NW + w] & q[w]);
                zxK += __popcll(a.p[NW + w] & k[w]);
                dQ += __popcll(q[w] | q[NW + w]);
                dK += __popcll(k[w] | k[NW + w]);
            }
            // pauli_string_multiply(P, Q): src/pauli/algebra.h:227-233
            const int jQ = a.yP + yQ + 2 * zxQ - yK;
            const int jK = a.yP + yK + 2 * zxK - yQ;
            u64 js = 0;
            const long long j = lookup<KW>(s, k, &C->error, &js);
            const cplx ci = load_coef<CPLX>(s, i);
            if (j >= 0 && !s.dead[j]) {
                if ((u64)j < i) continue;  // the pair belongs to position j
                const cplx cj = load_coef<CPLX>(s, (u64)j);
                cplx ni = rot_keep<CPLX>(ci, a.c), nj = rot_keep<CPLX>(cj, a.c);
                if (dQ <= a.maxdeg) ni = rot_add<CPLX>(ni, rot_partner<CPLX>(cj, isin.im, jK));
                if (dK <= a.maxdeg) nj = rot_add<CPLX>(nj, rot_partner<CPLX>(ci, isin.im, jQ));
                emits += (dQ <= a.maxdeg) + (dK <= a.maxdeg);
                store_coef<CPLX>(s, i, ni);
                store_coef<CPLX>(s, (u64)j, nj);
            } else {
                store_coef<CPLX>(s, i, rot_keep<CPLX>(ci, a.c));
                if (dK <= a.maxdeg) {
                    d_alive += emit_partner<KW, CPLX>(s, C, n_in, j >= 0 ? (long long)js : -1, k,
                                                      rot_partner<CPLX>(ci, isin.im, jQ));
                    emits++;
                }
            }
        }
    }
    kernel_exit(C, e, d_alive, sh, true, emits);
}

// ---------------------------------------------------------------------------
// Majorana rotation  exp(-i theta/2 i^r gamma_S)
// ---------------------------------------------------------------------------
template <int KW>
__global__ void __launch_bounds__(kBlock) majorana_rot_kernel(StoreView s, DevCounters* C, RotArgs a) {
    __shared__ Entry e;
    __shared__ long long sh[kBlock / 32];
    kernel_enter(C, s.cap, true, a.op, &e);
    long long d_alive = 0, emits = 0;
    if (!e.skip) {
        const u64 n_in = e.n;
        const u64 stride = (u64)gridDim.x * blockDim.x;
        const cplx F = {a.fr, a.fi};
        for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n_in; i += stride) {
            // (|a||b| - |a & b|) odd  <=>  popc(a & g) odd (even |g|) or popc(a & ~g) odd (odd |g|)
            u64 par = 0;
#pragma unroll
            for (int w = 0; w < KW; w++) {
                if (a.gate_odd)
                    par ^= s.key[(u64)w * s.cap + i] & ~a.p[w];
                else if (a.p[w])
                    par ^= s.key[(u64)w * s.cap + i] & a.p[w];
            }
            if (!(__popcll(par) & 1)) continue;
            if (s.dead[i]) continue;
            u64 q[KW], k[KW];
            load_key<KW>(s, i, q);
            int dQ = 0, dK = 0, mQ = 0, mK = 0;
#pragma unroll
            for (int w = 0; w < KW; w++) {
                k[w] = q[w] ^ a.p[w];
                dQ += __popcll(q[w]);
                dK += __popcll(k[w]);
                mQ += __popcll(q[w] & a.mg[w]);
                mK += __popcll(k[w] & a.mg[w]);
            }
            // sign of gamma_S * gamma_Q: (-1)^merge_parity(Q, S) (src/bits_utils.h:14-38)
            const cplx sQ = {(mQ & 1) ? -1.0 : 1.0, 0.0};
            const cplx sK = {(mK & 1) ? -1.0 : 1.0, 0.0};
            u64 js = 0;
            const long long j = lookup<KW>(s, k, &C->error, &js);
            const cplx ci = load_coef<true>(s, i);
            if (j >= 0 && !s.dead[j]) {
                if ((u64)j < i) continue;
                const cplx cj = load_coef<true>(s, (u64)j);
                cplx ni = cscale(ci, a.c), nj = cscale(cj, a.c);
                if (dQ <= a.maxdeg) ni = cadd(ni, cmul(cmul(cj, F), sK));
                if (dK <= a.maxdeg) nj = cadd(nj, cmul(cmul(ci, F), sQ));
                emits += (dQ <= a.maxdeg) + (dK <= a.maxdeg);
                store_coef<true>(s, i, ni);
                store_coef<true>(s, (u64)j, nj);
            } else {
                store_coef<true>(s, i, cscale(ci, a.c));
                if (dK <= a.maxdeg) {
                    d_alive += emit_partner<KW, true>(s, C, n_in, j >= 0 ? (long long)js : -1, k,
                                                      cmul(cmul(ci, F), sQ));
                    emits++;
                }
            }
        }
    }
    kernel_exit(C, e, d_alive, sh, true, emits);
}

// ---------------------------------------------------------------------------
// truncation: |c| <= tau and X/Y weight (src/pauli/truncate.h:16-57)
// ---------------------------------------------------------------------------
template <int KW, bool CPLX, int NWX>
__global__ void __launch_bounds__(kBlock) truncate_kernel(StoreView s, DevCounters* C, TruncArgs t) {
    __shared__ Entry e;
    __shared__ long long sh[kBlock / 32];
    kernel_enter(C, s.cap, false, t.op, &e);
    long long d_alive = 0;
    if (!e.skip) {
        const u64 stride = (u64)gridDim.x * blockDim.x;
        for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < e.n; i += stride) {
            if (s.dead[i]) continue;
            bool kill = false;
            if (t.thr) {
                const double re = s.re[i];
                kill = CPLX ? abs_le(re, s.im[i], t.tau) : (fabs(re) <= t.tau);
            }
            if (!kill && NWX > 0 && t.max_xweight >= 0) {
                int xw = 0;
#pragma unroll
                for (int w = 0; w < NWX; w++) xw += __popcll(s.key[(u64)w * s.cap + i]);
                kill = xw > t.max_xweight;
            }
            if (kill) {
                s.dead[i] = 1;
                d_alive -= 1;
            }
        }
    }
    kernel_exit(C, e, d_alive, sh, false);
}

// ---------------------------------------------------------------------------
// Clifford segment (src/pauli/gates.h:15-69, 273-301): every term maps 1:1,
// gates applied last to first; keys change, so the index is rebuilt after.
// ---------------------------------------------------------------------------
template <int NW>
__device__ __forceinline__ u64 bit_at(const u64 (&w)[NW], int i) {
    return (w[i >> 6] >> (i & 63)) & 1ull;
}
template <int NW>
__device__ __forceinline__ void set_bit(u64 (&w)[NW], int i, u64 b) {
    w[i >> 6] = (w[i >> 6] & ~(1ull << (i & 63))) | (b << (i & 63));
}

// Maps the key (x, z) through the Clifford gates ops[nops-1] .. ops[0] (the
// Heisenberg order) and returns the number of sign flips.
template <int NW>
__device__ __forceinline__ int clifford_map(u64 (&x)[NW], u64 (&z)[NW], const CliffordOp* ops, int nops) {
    int flips = 0;
    for (int g = nops - 1; g >= 0; g--) {
        const CliffordOp o = ops[g];
        const int a = o.q0, b = o.q1;
        switch (o.kind) {
            case kH: {
                const u64 xa = bit_at<NW>(x, a), za = bit_at<NW>(z, a);
                set_bit<NW>(x, a, za);
                set_bit<NW>(z, a, xa);
                flips += (int)(xa & za);
                break;
            }
            case kS: {
                const u64 xa = bit_at<NW>(x, a), za = bit_at<NW>(z, a);
                set_bit<NW>(z, a, xa ^ za);
                flips += (int)(xa & (za ^ 1ull));
                break;
            }
            case kCNOT: {
                const u64 xa = bit_at<NW>(x, a), xb = bit_at<NW>(x, b);
                const u64 za = bit_at<NW>(z, a), zb = bit_at<NW>(z, b);
                set_bit<NW>(x, b, xa ^ xb);
                set_bit<NW>(z, a, za ^ zb);
                flips += (int)(xa & zb & ((za ^ xb) ^ 1ull));
                break;
            }
            case kSWAP: {
                const u64 xa = bit_at<NW>(x, a), xb = bit_at<NW>(x, b);
                const u64 za = bit_at<NW>(z, a), zb = bit_at<NW>(z, b);
                set_bit<NW>(x, a, xb);
                set_bit<NW>(x, b, xa);
                set_bit<NW>(z, a, zb);
                set_bit<NW>(z, b, za);
                break;
            }
            case kCZ: {
                const u64 xa = bit_at<NW>(x, a), xb = bit_at<NW>(x, b);
                const u64 za = bit_at<NW>(z, a), zb = bit_at<NW>(z, b);
                flips += (int)(xa & xb & (za ^ zb));
                u64 m[NW];
#pragma unroll
                for (int w = 0; w < NW; w++) m[w] = 0;
                m[a >> 6] |= xb << (a & 63);
                m[b >> 6] |= xa << (b & 63);
#pragma unroll
                for (int w = 0; w < NW; w++) z[w] ^= m[w];
                break;
            }
            default:
                break;
        }
    }
    return flips;
}

template <int NW, bool CPLX>
__global__ void __launch_bounds__(kBlock) clifford_kernel(StoreView s, DevCounters* C,
                                                          const CliffordOp* ops, int nops, u32 op) {
    __shared__ Entry e;
    __shared__ long long sh[kBlock / 32];
    kernel_enter(C, s.cap, false, op, &e);
    if (!e.skip) {
        const u64 stride = (u64)gridDim.x * blockDim.x;
        for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < e.n; i += stride) {
            u64 x[NW], z[NW];
#pragma unroll
            for (int w = 0; w < NW; w++) {
                x[w] = s.key[(u64)w * s.cap + i];
                z[w] = s.key[(u64)(NW + w) * s.cap + i];
            }
            const int flips = clifford_map<NW>(x, z, ops, nops);
#pragma unroll
            for (int w = 0; w < NW; w++) {
                s.key[(u64)w * s.cap + i] = x[w];
                s.key[(u64)(NW + w) * s.cap + i] = z[w];
            }
            if (flips & 1) {
                // mult * coeff with mult = (-1, -0): exact negation
                s.re[i] = __dmul_rn(s.re[i], -1.0);
                if (CPLX) s.im[i] = __dmul_rn(s.im[i], -1.0);
            }
        }
    }
    kernel_exit(C, e, 0, sh, false);
}

// ---------------------------------------------------------------------------
// index maintenance
// ---------------------------------------------------------------------------
static __global__ void clear_slots_kernel(u64* slots, u64 nslots) {
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < nslots; i += stride) slots[i] = kEmptySlot;
}

// Rebuilds the index from the live entries only.  A dead entry may share its
// key with a live one (a key truncated away and re-created later), so dead
// entries must not be indexed.
template <int KW>
__global__ void __launch_bounds__(kBlock) index_kernel(StoreView s, DevCounters* C, int check_dup) {
    const u64 n = *(volatile u64*)&C->n;
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (s.dead[i]) continue;
        u64 k[KW];
        load_key<KW>(s, i, k);
        insert<KW>(s, k, (u32)i, &C->error, check_dup != 0);
    }
}

// ---------------------------------------------------------------------------
// order-preserving compaction of live entries: src -> dst
// ---------------------------------------------------------------------------
constexpr int kTileItems = kBlock * 8;

static __global__ void __launch_bounds__(kBlock) tile_count_kernel(StoreView s, DevCounters* C, u64* counts) {
    const u64 n = *(volatile u64*)&C->n;
    const u64 ntiles = (n + kTileItems - 1) / kTileItems;
    __shared__ int red[kBlock / 32];
    for (u64 t = blockIdx.x; t < ntiles; t += gridDim.x) {
        int c = 0;
        for (int r = 0; r < 8; r++) {
            const u64 i = t * kTileItems + (u64)r * kBlock + threadIdx.x;
            if (i < n && !s.dead[i]) c++;
        }
        for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
        __syncthreads();
        if (threadIdx.x == 0) {
            int tot = 0;
            for (int w = 0; w < kBlock / 32; w++) tot += red[w];
            counts[t] = (u64)tot;
        }
        __syncthreads();
    }
}

// exclusive scan of the tile counts (one block); writes the live total
static __global__ void __launch_bounds__(1024) tile_scan_kernel(DevCounters* C, u64* counts) {
    const u64 n = *(volatile u64*)&C->n;
    const u64 ntiles = (n + kTileItems - 1) / kTileItems;
    __shared__ u64 carry;
    __shared__ u64 warp_tot[32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (u64 base = 0; base < ntiles; base += blockDim.x) {
        const u64 t = base + threadIdx.x;
        const u64 v = t < ntiles ? counts[t] : 0;
        u64 x = v;
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        for (int o = 1; o < 32; o <<= 1) {
            const u64 y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[wid] = x;
        __syncthreads();
        if (wid == 0) {
            u64 w = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const u64 y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            warp_tot[lane] = w;
        }
        __syncthreads();
        const u64 incl = x + (wid > 0 ? warp_tot[wid - 1] : 0);
        if (t < ntiles) counts[t] = carry + incl - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) counts[ntiles] = carry;
}

template <int KW, bool CPLX>
__global__ void __launch_bounds__(kBlock) scatter_kernel(StoreView src, StoreView dst, DevCounters* C,
                                                         const u64* offsets) {
    const u64 n = *(volatile u64*)&C->n;
    const u64 ntiles = (n + kTileItems - 1) / kTileItems;
    __shared__ int wsum[kBlock / 32];
    __shared__ int run;
    for (u64 t = blockIdx.x; t < ntiles; t += gridDim.x) {
        if (threadIdx.x == 0) run = 0;
        __syncthreads();
        const u64 base = offsets[t];
        for (int r = 0; r < 8; r++) {
            const u64 i = t * kTileItems + (u64)r * kBlock + threadIdx.x;
            const bool live = i < n && !src.dead[i];
            const u32 vote = __ballot_sync(0xffffffffu, live);
            const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
            if (lane == 0) wsum[wid] = __popc(vote);
            __syncthreads();
            int before = run;
            for (int w = 0; w < wid; w++) before += wsum[w];
            before += __popc(vote & ((1u << lane) - 1u));
            if (live) {
                const u64 o = base + (u64)before;
#pragma unroll
                for (int w = 0; w < KW; w++) dst.key[(u64)w * dst.cap + o] = src.key[(u64)w * src.cap + i];
                dst.re[o] = src.re[i];
                if (CPLX) dst.im[o] = src.im[i];
                dst.dead[o] = 0;
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                int tot = 0;
                for (int w = 0; w < kBlock / 32; w++) tot += wsum[w];
                run += tot;
            }
            __syncthreads();
        }
    }
}

static __global__ void compact_commit_kernel(DevCounters* C, const u64* counts) {
    volatile DevCounters* V = C;
    const u64 n = V->n;
    const u64 ntiles = (n + kTileItems - 1) / kTileItems;
    const u64 live = counts[ntiles];
    V->n = live;
    V->alive = live;
}

// ---------------------------------------------------------------------------
// expectation values (masked reductions)
// ---------------------------------------------------------------------------
// mode 0: Pauli product state b: x == 0 terms, sign (-1)^{|z & b|}
//         (src/qubitproductstate.h:73-88; b = 0 is overlapwithzero)
// mode 1: Majorana Fock state b: fully paired strings, i^{|J| + 2|b & J|}
//         (src/fockstate.h:95-114)
template <int KW, bool CPLX>
__global__ void __launch_bounds__(kBlock) expect_kernel(StoreView s, u64 n, int mode, int nw, u64 b0,
                                                        u64 b1, double* part_re, double* part_im) {
    double r = 0.0, im = 0.0;
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (s.dead[i]) continue;
        u64 k[KW];
        load_key<KW>(s, i, k);
        const cplx c = load_coef<CPLX>(s, i);
        if (mode == 0) {
            bool zero_x = true;
            int par = 0;
            for (int w = 0; w < nw; w++) {
                zero_x = zero_x && k[w] == 0;
                par += __popcll(k[nw + w] & (w == 0 ? b0 : b1));
            }
            if (!zero_x) continue;
            const cplx v = cmul(c, {(par & 1) ? -1.0 : 1.0, 0.0});
            r = __dadd_rn(r, v.re);
            im = __dadd_rn(im, v.im);
        } else {
            bool paired = true;
            u64 J[2] = {0, 0};
#pragma unroll
            for (int w = 0; w < KW; w++) {
                const u64 ev = k[w] & 0x5555555555555555ull, od = (k[w] >> 1) & 0x5555555555555555ull;
                paired = paired && ev == od;
                u64 p = 0;
                for (int t = 0; t < 32; t++) p |= ((ev >> (2 * t)) & 1ull) << t;
                J[w >> 1] |= p << (32 * (w & 1));
            }
            if (!paired) continue;
            const int ex = __popcll(J[0]) + __popcll(J[1]) + 2 * (__popcll(J[0] & b0) + __popcll(J[1] & b1));
            const cplx v = cmul(c, ipow(ex));
            r = __dadd_rn(r, v.re);
            im = __dadd_rn(im, v.im);
        }
    }
    __shared__ double sr[kBlock / 32], si[kBlock / 32];
    for (int o = 16; o > 0; o >>= 1) {
        r = __dadd_rn(r, __shfl_down_sync(0xffffffffu, r, o));
        im = __dadd_rn(im, __shfl_down_sync(0xffffffffu, im, o));
    }
    if ((threadIdx.x & 31) == 0) {
        sr[threadIdx.x >> 5] = r;
        si[threadIdx.x >> 5] = im;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < kBlock / 32; w++) {
            a = __dadd_rn(a, sr[w]);
            b = __dadd_rn(b, si[w]);
        }
        part_re[blockIdx.x] = a;
        part_im[blockIdx.x] = b;
    }
}

static __global__ void expect_final_kernel(const double* part_re, const double* part_im, int nparts, double* out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int i = 0; i < nparts; i++) {
            a = __dadd_rn(a, part_re[i]);
            b = __dadd_rn(b, part_im[i]);
        }
        out[0] = a;
        out[1] = b;
    }
}

// ---------------------------------------------------------------------------
// top-k support: histogram of |c| bit patterns (8-bit digit, MSB first)
// ---------------------------------------------------------------------------
template <bool CPLX>
__device__ __forceinline__ u64 mag_bits(const StoreView& s, u64 i) {
    const double m = CPLX ? hypot(s.re[i], s.im[i]) : fabs(s.re[i]);
    return (u64)__double_as_longlong(m);
}

template <bool CPLX>
__global__ void __launch_bounds__(kBlock) mag_hist_kernel(StoreView s, DevCounters* C, int shift,
                                                          u64 prefix, u64 prefix_mask, u64* hist) {
    __shared__ unsigned int h[256];
    for (int b = threadIdx.x; b < 256; b += blockDim.x) h[b] = 0;
    __syncthreads();
    const u64 n = *(volatile u64*)&C->n;
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (s.dead[i]) continue;
        const u64 m = mag_bits<CPLX>(s, i);
        if ((m & prefix_mask) != prefix) continue;
        atomicAdd(&h[(m >> shift) & 255], 1u);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < 256; b += blockDim.x)
        if (h[b]) atomicAdd(&hist[b], (u64)h[b]);
}

// kills live entries with |c| < cut; gathers positions with |c| == cut
template <bool CPLX>
__global__ void __launch_bounds__(kBlock) topk_cut_kernel(StoreView s, DevCounters* C, u64 cut,
                                                          u64* ties, u64* nties, u64 max_ties) {
    __shared__ Entry e;
    __shared__ long long sh[kBlock / 32];
    kernel_enter(C, s.cap, false, 0u, &e);
    long long d_alive = 0;
    if (!e.skip) {
        const u64 stride = (u64)gridDim.x * blockDim.x;
        for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < e.n; i += stride) {
            if (s.dead[i]) continue;
            const u64 m = mag_bits<CPLX>(s, i);
            if (m < cut) {
                s.dead[i] = 1;
                d_alive -= 1;
            } else if (m == cut) {
                const u64 p = atomicAdd(nties, 1ull);
                if (p < max_ties) ties[p] = i;
            }
        }
    }
    kernel_exit(C, e, d_alive, sh, false);
}

static __global__ void kill_list_kernel(StoreView s, DevCounters* C, const u64* list, u64 m) {
    for (u64 t = (u64)blockIdx.x * blockDim.x + threadIdx.x; t < m; t += (u64)gridDim.x * blockDim.x)
        s.dead[list[t]] = 1;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        volatile DevCounters* V = C;
        V->alive = V->alive - m;
    }
}

}  // namespace ffg

namespace ffg {

// ---------------------------------------------------------------------------
// Fused pass over a group of up to D consecutive rotations of one commuting
// batch whose axes are linearly independent (as GF(2) vectors).
//
// For a term Q let A = {t : Q anticommutes with P_t}.  Because the axes commute,
// every member of the orbit M_S = Q * prod_{t in S} P_t (S subset of A) has the
// same A, the members are distinct (independent axes), and the gates of the
// group only ever pair members of the same orbit.  Applying the group gate by
// gate is therefore, orbit by orbit, a sequence of butterflies over the
// hypercube of subsets of A, taken in gate order: stage t pairs M_S with
// M_{S+t}.  The present member with the lowest store position owns the orbit,
// gathers the present members, runs the stages in registers with the
// reference's exact per-gate arithmetic, degree filter and creation rule, and
// writes the members back (new ones are appended and indexed).
// ---------------------------------------------------------------------------
template <int D>
struct GroupArgs {
    u64 psub[1 << D][4];  // XOR of the axes of each gate subset (planes in store order)
    double c[D], s[D];
    int yP[D];
    int ng;               // gates in the group (1..D)
    int maxdeg;
    u32 need;             // bit w: key plane w takes part in the anticommutation test
    u32 op;
};

template <int NW>
__device__ __forceinline__ int popc_planes(const u64 (&k)[2 * NW], int lo) {
    int r = 0;
#pragma unroll
    for (int w = 0; w < NW; w++) r += __popcll(k[lo + w]);
    return r;
}

// Processes the orbit of the live term at position i (anticommutation pattern
// A) when i owns it.  Adds to the thread's live-count, emitted-partner and
// in-pass application counters.
template <int NW, bool CPLX, int D>
__device__ __forceinline__ void group_orbit(const StoreView& s, DevCounters* C, const GroupArgs<D>& a,
                                            u64 n_in, u64 i, u32 A, long long& d_alive,
                                            long long& emits, long long& extra_apps,
                                            u64* app_ctr = nullptr) {
    constexpr int KW = 2 * NW;
    constexpr int M = 1 << D;
    u64 q[KW];
    load_key<KW>(s, i, q);
    // look up every member of the orbit; loc[m] = store position of a present
    // member, or the index slot of a dead one
    u32 loc[M];
    u32 present = 1u, wasdead = 0u;
    loc[0] = (u32)i;
    bool owner = true;
#pragma unroll
    for (int m = 1; m < M; m++) {
        loc[m] = 0u;
        if ((m & ~A) != 0) continue;
        u64 k[KW];
#pragma unroll
        for (int w = 0; w < KW; w++) k[w] = q[w] ^ a.psub[m][w];
        u64 sl = 0;
        const long long j = lookup<KW>(s, k, &C->error, &sl);
        if (j >= 0) {
            if (!s.dead[j]) {
                present |= 1u << m;
                loc[m] = (u32)j;
                if ((u64)j < i) owner = false;
            } else {
                wasdead |= 1u << m;
                loc[m] = (u32)sl;
            }
        }
    }
    if (!owner) return;
    cplx c[M];
#pragma unroll
    for (int m = 0; m < M; m++) {
        c[m] = {0.0, 0.0};
        if ((present >> m) & 1u) c[m] = load_coef<CPLX>(s, loc[m]);
    }
    const u32 present0 = present;
    // stages in gate order
#pragma unroll
    for (int t = 0; t < D; t++) {
        if (t >= a.ng || !((A >> t) & 1u)) continue;
        const u64* P = a.psub[1 << t];
        const cplx isin = {0.0, a.s[t]};
        int created = 0;
#pragma unroll
        for (int u = 0; u < M; u++) {
            if ((u & ~A) != 0 || ((u >> t) & 1)) continue;
            const int v = u | (1 << t);
            const bool pu = (present >> u) & 1u, pv = (present >> v) & 1u;
            if (!pu && !pv) continue;
            // degrees, Y counts and phases of P_t * member
            // (pauli_string_multiply, src/pauli/algebra.h:227-233)
            int du = 0, dv = 0, yu = 0, yv = 0, zxu = 0, zxv = 0;
#pragma unroll
            for (int w = 0; w < NW; w++) {
                const u64 xu = q[w] ^ a.psub[u][w], zu = q[NW + w] ^ a.psub[u][NW + w];
                const u64 xv = q[w] ^ a.psub[v][w], zv = q[NW + w] ^ a.psub[v][NW + w];
                du += __popcll(xu | zu);
                dv += __popcll(xv | zv);
                yu += __popcll(xu & zu);
                yv += __popcll(xv & zv);
                zxu += __popcll(P[NW + w] & xu);
                zxv += __popcll(P[NW + w] & xv);
            }
            const int ju = a.yP[t] + yu + 2 * zxu - yv;  // P_t * M_u -> M_v
            const int jv = a.yP[t] + yv + 2 * zxv - yu;  // P_t * M_v -> M_u
            const bool to_u = pv && du <= a.maxdeg;
            const bool to_v = pu && dv <= a.maxdeg;
            cplx nu = c[u], nv = c[v];
            if (pu) nu = rot_keep<CPLX>(c[u], a.c[t]);
            if (pv) nv = rot_keep<CPLX>(c[v], a.c[t]);
            if (to_u) nu = rot_add<CPLX>(pu ? nu : cplx{0.0, 0.0}, rot_partner<CPLX>(c[v], isin.im, jv));
            if (to_v) nv = rot_add<CPLX>(pv ? nv : cplx{0.0, 0.0}, rot_partner<CPLX>(c[u], isin.im, ju));
            emits += (int)to_u + (int)to_v;
            if (!pu && to_u) {
                present |= 1u << u;
                created++;
            }
            if (!pv && to_v) {
                present |= 1u << v;
                created++;
            }
            c[u] = nu;
            c[v] = nv;
        }
        extra_apps += (long long)created * (a.ng - 1 - t);
    }
    // write back
#pragma unroll
    for (int m = 0; m < M; m++) {
        if (!((present >> m) & 1u)) continue;
        if ((present0 >> m) & 1u) {
            store_coef<CPLX>(s, loc[m], c[m]);
            continue;
        }
        u64 k[KW];
#pragma unroll
        for (int w = 0; w < KW; w++) k[w] = q[w] ^ a.psub[m][w];
        const u64 pos = n_in + atomicAdd(app_ctr ? app_ctr : &C->d_app, 1ull);
#pragma unroll
        for (int w = 0; w < KW; w++) s.key[(u64)w * s.cap + pos] = k[w];
        store_coef<CPLX>(s, pos, c[m]);
        s.dead[pos] = 0;
        __threadfence();
        if ((wasdead >> m) & 1u) {
            const u64 ent = __ldcg(&s.slots[loc[m]]);
            atomicExch(&s.slots[loc[m]], (ent & 0xffffffff00000000ull) | pos);
        } else {
            insert<KW>(s, k, (u32)pos, &C->error, false);
        }
        d_alive += 1;
    }
}

constexpr int kScanR = 8;                     // terms tested per thread per tile
constexpr int kTile = kBlock * kScanR;

// One pass of a rotation group over the store.  Each block walks tiles of
// kTile positions: every thread first issues the loads of its kScanR terms
// together (the planes the axes touch plus the dead flags) and queues the
// anticommuting live ones in shared memory; then the block works through the
// queue, one orbit per thread.
template <int NW, bool CPLX, int D>
__global__ void __launch_bounds__(kBlock) pauli_group_kernel(StoreView s, DevCounters* C,
                                                             GroupArgs<D> a) {
    constexpr int KW = 2 * NW;
    __shared__ Entry e;
    __shared__ long long sh[kBlock / 32];
    __shared__ u32 queue[kTile];
    __shared__ u32 qn;
    if (threadIdx.x == 0) {
        volatile DevCounters* V = C;
        const u64 n = V->n;
        int skip = V->overflow != 0 || V->error != 0;
        // an orbit of 2^ng members may be created from each present term
        if (!skip && (n << a.ng) > s.cap) {
            atomicCAS(&C->overflow, 0u, a.op + 1u);
            skip = 1;
        }
        e.n = n;
        e.alive = V->alive;
        e.skip = skip;
    }
    __syncthreads();
    long long d_alive = 0, emits = 0, extra_apps = 0;
    if (!e.skip) {
        const u64 n_in = e.n;
        const u64 ntiles = (n_in + kTile - 1) / kTile;
        for (u64 tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
            if (threadIdx.x == 0) qn = 0;
            __syncthreads();
            const u64 base = tile * kTile;
            u64 pl[kScanR][KW];
            unsigned char dd[kScanR];
#pragma unroll
            for (int r = 0; r < kScanR; r++) {
                const u64 i = base + (u64)r * kBlock + threadIdx.x;
                const bool in = i < n_in;
#pragma unroll
                for (int w = 0; w < KW; w++)
                    pl[r][w] = (in && ((a.need >> w) & 1u)) ? s.key[(u64)w * s.cap + i] : 0ull;
                dd[r] = in ? s.dead[i] : 1;
            }
#pragma unroll
            for (int r = 0; r < kScanR; r++) {
                u32 A = 0;
#pragma unroll
                for (int t = 0; t < D; t++) {
                    if (t >= a.ng) break;
                    const u64* P = a.psub[1 << t];
                    u64 par = 0;
#pragma unroll
                    for (int w = 0; w < NW; w++) par ^= (pl[r][w] & P[NW + w]) ^ (pl[r][NW + w] & P[w]);
                    A |= (u32)(__popcll(par) & 1) << t;
                }
                const bool act = A != 0 && !dd[r];
                const u32 vote = __ballot_sync(0xffffffffu, act);
                if (vote) {
                    const int lane = threadIdx.x & 31;
                    u32 slot0 = 0;
                    if (lane == 0) slot0 = atomicAdd(&qn, (u32)__popc(vote));
                    slot0 = __shfl_sync(0xffffffffu, slot0, 0);
                    if (act) queue[slot0 + __popc(vote & ((1u << lane) - 1u))] =
                        ((u32)(r * kBlock + threadIdx.x) << 4) | A;
                }
            }
            __syncthreads();
            const u32 nq = qn;
            for (u32 k = threadIdx.x; k < nq; k += blockDim.x) {
                const u32 ent = queue[k];
                group_orbit<NW, CPLX, D>(s, C, a, n_in, base + (ent >> 4), ent & 15u, d_alive, emits,
                                         extra_apps);
            }
            __syncthreads();
        }
    }
    // fold counters; apps = sum over the group's gates of the live terms entering it
    const long long tot = block_sum_ll(d_alive, sh);
    const long long em = block_sum_ll(emits, sh);
    const long long xa = block_sum_ll(extra_apps, sh);
    if (threadIdx.x == 0) {
        if (tot) atomicAdd((u64*)&C->d_alive, (u64)tot);
        if (em) atomicAdd(&C->emits, (u64)em);
        if (xa) atomicAdd(&C->d_apps, (u64)xa);
        __threadfence();
        const u32 prev = atomicAdd(&C->done, 1u);
        if (prev == gridDim.x - 1) {
            __threadfence();
            volatile DevCounters* V = C;
            const u64 app = V->d_app;
            const long long da = V->d_alive;
            V->n = e.n + app;
            const u64 al = (u64)((long long)e.alive + da);
            V->alive = al;
            if (!e.skip) {
                V->apps = V->apps + (u64)a.ng * e.alive + V->d_apps;
                if (al > V->peak) V->peak = al;
            }
            V->d_app = 0;
            V->d_alive = 0;
            V->d_apps = 0;
            V->done = 0;
            __threadfence();
        }
    }
}

}  // namespace ffg

namespace ffg {

// ---------------------------------------------------------------------------
// Lean single-rotation pass (the pair butterfly of pauli_rot_kernel) tuned for
// memory-level parallelism: few registers so that many terms are in flight,
// and the dependent loads of a pair grouped into as few round trips as
// possible:
//   1. the planes the axis touches + the dead flag of position i
//   2. (anticommuting, live) the remaining planes + the coefficient of i
//   3. the index probe for the partner key
//   4. the partner's key words, dead flag and coefficient, issued together
// ---------------------------------------------------------------------------
struct PairArgs {
    u64 p[4];        // axis planes in store order (x words, then z words)
    double c, s;
    int yP;
    int maxdeg;
    u32 need;        // planes that take part in the anticommutation test
    u32 op;
};

template <int NW, bool CPLX>
__global__ void __launch_bounds__(kBlock, 5) pauli_pair_kernel(StoreView s, DevCounters* C, PairArgs a) {
    constexpr int KW = 2 * NW;
    __shared__ Entry e;
    __shared__ long long sh[kBlock / 32];
    kernel_enter(C, s.cap, true, a.op, &e);
    long long d_alive = 0, emits = 0;
    if (!e.skip) {
        const u64 n_in = e.n;
        const u64 stride = (u64)gridDim.x * blockDim.x;
        for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n_in; i += stride) {
            u64 q[KW];
#pragma unroll
            for (int w = 0; w < KW; w++) q[w] = ((a.need >> w) & 1u) ? s.key[(u64)w * s.cap + i] : 0ull;
            const unsigned char di = s.dead[i];
            u64 par = 0;
#pragma unroll
            for (int w = 0; w < NW; w++) par ^= (q[w] & a.p[NW + w]) ^ (q[NW + w] & a.p[w]);
            if (!(__popcll(par) & 1) || di) continue;
#pragma unroll
            for (int w = 0; w < KW; w++)
                if (!((a.need >> w) & 1u)) q[w] = s.key[(u64)w * s.cap + i];
            const cplx ci = load_coef<CPLX>(s, i);
            // partner key K = P*Q, its degree and the two phases
            int yQ = 0, yK = 0, zxQ = 0, zxK = 0, dQ = 0, dK = 0;
#pragma unroll
            for (int w = 0; w < NW; w++) {
                const u64 xk = q[w] ^ a.p[w], zk = q[NW + w] ^ a.p[NW + w];
                yQ += __popcll(q[w] & q[NW + w]);
                yK += __popcll(xk & zk);
                zxQ += __popcll(a.p[NW + w] & q[w]);
                zxK += __popcll(a.p[NW + w] & xk);
                dQ += __popcll(q[w] | q[NW + w]);
                dK += __popcll(xk | zk);
            }
            const int jQ = a.yP + yQ + 2 * zxQ - yK;  // P*Q -> K
            const int jK = a.yP + yK + 2 * zxK - yQ;  // P*K -> Q
            // probe for K; at a fingerprint match fetch key, dead flag and
            // coefficient of the candidate in one round trip
            u64 k[KW];
#pragma unroll
            for (int w = 0; w < KW; w++) k[w] = q[w] ^ a.p[w];
            const u64 h = hash_key<KW>(k);
            const u32 fp = (u32)(h >> 32);
            u64 pos = h & s.hmask;
            long long j = -1;
            u64 jslot = 0;
            bool jdead = false;
            cplx cj = {0.0, 0.0};
            for (u64 probe = 0; probe <= s.hmask; probe++) {
                const u64 ent = __ldcg(&s.slots[pos]);
                if (ent == kEmptySlot) break;
                if ((u32)(ent >> 32) == fp) {
                    const u32 idx = (u32)ent;
                    bool eq = true;
                    u64 kk[KW];
#pragma unroll
                    for (int w = 0; w < KW; w++) kk[w] = __ldcg(&s.key[(u64)w * s.cap + idx]);
                    const unsigned char dj = s.dead[idx];
                    const cplx cc = {s.re[idx], CPLX ? s.im[idx] : 0.0};
#pragma unroll
                    for (int w = 0; w < KW; w++) eq = eq && kk[w] == k[w];
                    if (eq) {
                        j = idx;
                        jslot = pos;
                        jdead = dj != 0;
                        cj = cc;
                        break;
                    }
                }
                pos = (pos + 1) & s.hmask;
                if (probe == s.hmask) atomicOr(&C->error, 2u);
            }
            const cplx isin = {0.0, a.s};
            if (j >= 0 && !jdead) {
                if ((u64)j < i) continue;  // the pair belongs to position j
                cplx ni = rot_keep<CPLX>(ci, a.c), nj = rot_keep<CPLX>(cj, a.c);
                if (dQ <= a.maxdeg) ni = rot_add<CPLX>(ni, rot_partner<CPLX>(cj, isin.im, jK));
                if (dK <= a.maxdeg) nj = rot_add<CPLX>(nj, rot_partner<CPLX>(ci, isin.im, jQ));
                emits += (dQ <= a.maxdeg) + (dK <= a.maxdeg);
                store_coef<CPLX>(s, i, ni);
                store_coef<CPLX>(s, (u64)j, nj);
            } else {
                store_coef<CPLX>(s, i, rot_keep<CPLX>(ci, a.c));
                if (dK <= a.maxdeg) {
                    d_alive += emit_partner<KW, CPLX>(s, C, n_in, j >= 0 ? (long long)jslot : -1, k,
                                                      rot_partner<CPLX>(ci, isin.im, jQ));
                    emits++;
                }
            }
        }
    }
    kernel_exit(C, e, d_alive, sh, true, emits);
}

}  // namespace ffg
