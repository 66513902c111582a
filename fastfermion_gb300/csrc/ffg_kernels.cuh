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
    const cplx nv = cadd({0.0, 0.0}, v);  // operator[] starts from complex zero
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
                cplx ni = cscale(ci, a.c), nj = cscale(cj, a.c);
                if (dQ <= a.maxdeg) ni = cadd(ni, cmul(cmul(cj, isin), ipow(jK)));
                if (dK <= a.maxdeg) nj = cadd(nj, cmul(cmul(ci, isin), ipow(jQ)));
                emits += (dQ <= a.maxdeg) + (dK <= a.maxdeg);
                store_coef<CPLX>(s, i, ni);
                store_coef<CPLX>(s, (u64)j, nj);
            } else {
                store_coef<CPLX>(s, i, cscale(ci, a.c));
                if (dK <= a.maxdeg) {
                    d_alive += emit_partner<KW, CPLX>(s, C, n_in, j >= 0 ? (long long)js : -1, k,
                                                      cmul(cmul(ci, isin), ipow(jQ)));
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
__global__ void clear_slots_kernel(u64* slots, u64 nslots) {
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

__global__ void __launch_bounds__(kBlock) tile_count_kernel(StoreView s, DevCounters* C, u64* counts) {
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
__global__ void __launch_bounds__(1024) tile_scan_kernel(DevCounters* C, u64* counts) {
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

__global__ void compact_commit_kernel(DevCounters* C, const u64* counts) {
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

__global__ void expect_final_kernel(const double* part_re, const double* part_im, int nparts, double* out) {
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

__global__ void kill_list_kernel(StoreView s, DevCounters* C, const u64* list, u64 m) {
    for (u64 t = (u64)blockIdx.x * blockDim.x + threadIdx.x; t < m; t += (u64)gridDim.x * blockDim.x)
        s.dead[list[t]] = 1;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        volatile DevCounters* V = C;
        V->alive = V->alive - m;
    }
}

}  // namespace ffg
