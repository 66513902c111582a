// Persistent propagation kernel: one cooperative launch runs a whole run of
// ops (rotations, truncations, Clifford segments) with a grid barrier after
// each op instead of one kernel launch per op.  Every block keeps its own copy
// of the store size and live count; per-op changes are accumulated in three
// rotating delta slots so that one barrier per op suffices:
//   op o adds to slot o%3; after the barrier every block folds slot o%3 into
//   its copy; during op o block 0 zeroes slot (o+1)%3, whose last readers
//   passed the barrier of op o-1 and whose next writers start after the
//   barrier of op o.
// The kernel stops early (returning to the host) when a rotation could
// overflow the store, or when a truncation leaves more dead than live
// entries (the host then compacts).  Grid barriers spin with a time limit and
// report a timeout instead of waiting forever.
#pragma once
#include "ffg_kernels.cuh"

namespace ffg {

struct DevOp {
    int type;   // 0 pair rotation (Pauli), 1 truncation, 2 Clifford segment, 3 Majorana rotation
    int idx;    // args index (rotation / truncation)
    int begin;  // Clifford range [begin, end) in the circuit table
    int end;
};

enum { OP_PAIR = 0, OP_TRUNC = 1, OP_CLIFF = 2, OP_MROT = 3, OP_GROUP2 = 4 };
constexpr int kScanUnroll = 4;  // scan loads in flight per thread

struct PersistState {
    u64 d_app[3];
    long long d_alive[3];
    u64 d_emit[3];
    u64 d_xapps[3];   // fused groups: live terms created inside the op that enter its later gates
    u32 bar_count;
    u32 bar_gen;
    u32 bar_timeout;
    u32 stop_reason;  // 0 finished, 1 overflow, 2 compaction wanted, 3 barrier timeout
    u32 next_op;      // first op not executed
    u32 pad;
    u64 bcast[4];     // Bcast record released by grid barriers (own 32-byte line)
};

constexpr long long kBarrierLimitCycles = 4000000000ll;  // default wait limit: about 2 s at 2 GHz
constexpr int kPBlock = 512;                             // threads per block of the persistent kernel

// Grid-wide barrier for a cooperative launch that also folds the op's delta
// slot: the last block to arrive copies slot values into ps->bcast before
// releasing the others, so every block reads them from the line it polls.
// Returns false after a timeout.
struct Bcast {
    u64 app;
    long long alive;
    u64 emit;
    u32 gen;
    u32 xapps;
};

__device__ __forceinline__ bool grid_sync_fold(PersistState* ps, Bcast* bc, int slot, Bcast* out,
                                               long long limit) {
    __shared__ int ok;
    __shared__ Bcast sb;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile Bcast* vb = bc;
        const u32 g = vb->gen;
        __threadfence();
        const u32 arrived = atomicAdd(&ps->bar_count, 1u);
        ok = 1;
        if (arrived == gridDim.x - 1) {
            atomicExch(&ps->bar_count, 0u);
            __threadfence();
            Bcast b;
            b.app = *(volatile u64*)&ps->d_app[slot];
            b.alive = *(volatile long long*)&ps->d_alive[slot];
            b.emit = *(volatile u64*)&ps->d_emit[slot];
            b.xapps = (u32)*(volatile u64*)&ps->d_xapps[slot];
            vb->app = b.app;
            vb->alive = b.alive;
            vb->emit = b.emit;
            vb->xapps = b.xapps;
            __threadfence();
            vb->gen = g + 1;
            b.gen = g + 1;
            sb = b;
        } else {
            const long long t0 = clock64();
            for (;;) {
                if (vb->gen != g) break;
                if (*(volatile u32*)&ps->bar_timeout) {
                    ok = 0;
                    break;
                }
                if (clock64() - t0 > limit) {
                    atomicExch(&ps->bar_timeout, 1u);
                    ok = 0;
                    break;
                }
            }
            __threadfence();
            sb.app = vb->app;
            sb.alive = vb->alive;
            sb.emit = vb->emit;
            sb.xapps = vb->xapps;
        }
    }
    __syncthreads();
    *out = sb;
    return ok != 0;
}

// Plain grid barrier (used between the phases of a Clifford segment).
__device__ __forceinline__ bool grid_sync(PersistState* ps, Bcast* bc, long long limit) {
    Bcast dummy;
    return grid_sync_fold(ps, bc, 0, &dummy, limit);
}

// --- one Pauli rotation over positions [0, n_in) (pair butterfly) ----------
template <int NW, bool CPLX>
__device__ __forceinline__ void pair_one(const StoreView& s, DevCounters* C, u64* app_ctr,
                                         const PairArgs& a, u64 n_in, u64 i, long long& d_alive,
                                         long long& emits) {
    constexpr int KW = 2 * NW;
    u64 q[KW];
    load_key<KW>(s, i, q);
    const cplx ci = load_coef<CPLX>(s, i);
    int yQ = 0, yK = 0, zxQ = 0, zxK = 0, dQ = 0, dK = 0;
    u64 k[KW];
#pragma unroll
    for (int w = 0; w < NW; w++) {
        const u64 xk = q[w] ^ a.p[w], zk = q[NW + w] ^ a.p[NW + w];
        k[w] = xk;
        k[NW + w] = zk;
        yQ += __popcll(q[w] & q[NW + w]);
        yK += __popcll(xk & zk);
        zxQ += __popcll(a.p[NW + w] & q[w]);
        zxK += __popcll(a.p[NW + w] & xk);
        dQ += __popcll(q[w] | q[NW + w]);
        dK += __popcll(xk | zk);
    }
    const int jQ = a.yP + yQ + 2 * zxQ - yK;  // P*Q -> K
    const int jK = a.yP + yK + 2 * zxK - yQ;  // P*K -> Q
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
            u64 kk[KW];
#pragma unroll
            for (int w = 0; w < KW; w++) kk[w] = __ldcg(&s.key[(u64)w * s.cap + idx]);
            const unsigned char dj = __ldcg(&s.dead[idx]);
            const cplx cc = {__ldcg(&s.re[idx]), CPLX ? __ldcg(&s.im[idx]) : 0.0};
            bool eq = true;
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
        if ((u64)j < i) return;  // the pair belongs to position j
        cplx ni = rot_keep<CPLX>(ci, a.c), nj = rot_keep<CPLX>(cj, a.c);
        if (dQ <= a.maxdeg) ni = rot_add<CPLX>(ni, rot_partner<CPLX>(cj, isin.im, jK));
        if (dK <= a.maxdeg) nj = rot_add<CPLX>(nj, rot_partner<CPLX>(ci, isin.im, jQ));
        emits += (dQ <= a.maxdeg) + (dK <= a.maxdeg);
        store_coef<CPLX>(s, i, ni);
        store_coef<CPLX>(s, (u64)j, nj);
    } else {
        store_coef<CPLX>(s, i, rot_keep<CPLX>(ci, a.c));
        if (dK <= a.maxdeg) {
            const cplx nv = rot_add<CPLX>({0.0, 0.0}, rot_partner<CPLX>(ci, isin.im, jQ));
            const u64 p = n_in + atomicAdd(app_ctr, 1ull);
#pragma unroll
            for (int w = 0; w < KW; w++) s.key[(u64)w * s.cap + p] = k[w];
            store_coef<CPLX>(s, p, nv);
            s.dead[p] = 0;
            __threadfence();
            if (j >= 0) {
                const u64 ent = __ldcg(&s.slots[jslot]);
                atomicExch(&s.slots[jslot], (ent & 0xffffffff00000000ull) | p);
            } else {
                insert<KW>(s, k, (u32)p, &C->error, false);
            }
            d_alive += 1;
            emits++;
        }
    }
}

template <int NW, bool CPLX>
__device__ __forceinline__ void pass_pair(const StoreView& s, DevCounters* C, u64* app_ctr,
                                          const PairArgs& a, u64 n_in, long long& d_alive,
                                          long long& emits) {
    constexpr int KW = 2 * NW;
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n_in; i += stride) {
        u64 par = 0;
#pragma unroll
        for (int w = 0; w < NW; w++) {
            if ((a.need >> w) & 1u) par ^= s.key[(u64)w * s.cap + i] & a.p[NW + w];
            if ((a.need >> (NW + w)) & 1u) par ^= s.key[(u64)(NW + w) * s.cap + i] & a.p[w];
        }
        const unsigned char di = s.dead[i];
        if (!(__popcll(par) & 1) || di) continue;
        pair_one<NW, CPLX>(s, C, app_ctr, a, n_in, i, d_alive, emits);
    }
    (void)KW;
}

// Scan of [0, n_in): each thread tests kScanUnroll positions per round with
// all their loads issued together, then processes the anticommuting live ones.
// test(planes) returns the anticommutation pattern (0 = commutes with all).
template <int NW, class Test, class Proc>
__device__ __forceinline__ void scan_pass(const StoreView& s, u32 need, u64 n_in, Test test, Proc proc) {
    constexpr int KW = 2 * NW;
    constexpr int R = kScanUnroll;
    const u64 nth = (u64)gridDim.x * blockDim.x;
    const u64 t0 = (u64)blockIdx.x * blockDim.x + threadIdx.x;
    for (u64 base = 0; base < n_in; base += nth * R) {
        u64 pl[R][KW];
        unsigned char dd[R];
#pragma unroll
        for (int r = 0; r < R; r++) {
            const u64 i = base + t0 + (u64)r * nth;
            const bool in = i < n_in;
#pragma unroll
            for (int w = 0; w < KW; w++)
                pl[r][w] = (in && ((need >> w) & 1u)) ? s.key[(u64)w * s.cap + i] : 0ull;
            dd[r] = in ? s.dead[i] : (unsigned char)1;
        }
#pragma unroll
        for (int r = 0; r < R; r++) {
            const u32 A = test(pl[r]);
            if (A && !dd[r]) proc(base + t0 + (u64)r * nth, A);
        }
    }
}

// --- one Majorana rotation (src/majorana_gates.h:67-103) -------------------
template <int KW>
__device__ __forceinline__ void pass_mrot(const StoreView& s, DevCounters* C, u64* app_ctr,
                                          const RotArgs& a, u64 n_in, long long& d_alive,
                                          long long& emits) {
    const u64 stride = (u64)gridDim.x * blockDim.x;
    const cplx F = {a.fr, a.fi};
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n_in; i += stride) {
        u64 q[KW];
        load_key<KW>(s, i, q);
        const unsigned char di = s.dead[i];
        u64 par = 0;
#pragma unroll
        for (int w = 0; w < KW; w++) par ^= q[w] & (a.gate_odd ? ~a.p[w] : a.p[w]);
        if (!(__popcll(par) & 1) || di) continue;
        const cplx ci = load_coef<true>(s, i);
        u64 k[KW];
        int dQ = 0, dK = 0, mQ = 0, mK = 0;
#pragma unroll
        for (int w = 0; w < KW; w++) {
            k[w] = q[w] ^ a.p[w];
            dQ += __popcll(q[w]);
            dK += __popcll(k[w]);
            mQ += __popcll(q[w] & a.mg[w]);
            mK += __popcll(k[w] & a.mg[w]);
        }
        const cplx sQ = {(mQ & 1) ? -1.0 : 1.0, 0.0};
        const cplx sK = {(mK & 1) ? -1.0 : 1.0, 0.0};
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
                u64 kk[KW];
#pragma unroll
                for (int w = 0; w < KW; w++) kk[w] = __ldcg(&s.key[(u64)w * s.cap + idx]);
                const unsigned char dj = __ldcg(&s.dead[idx]);
                const cplx cc = {__ldcg(&s.re[idx]), __ldcg(&s.im[idx])};
                bool eq = true;
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
        if (j >= 0 && !jdead) {
            if ((u64)j < i) continue;
            cplx ni = cscale(ci, a.c), nj = cscale(cj, a.c);
            if (dQ <= a.maxdeg) ni = cadd(ni, cmul(cmul(cj, F), sK));
            if (dK <= a.maxdeg) nj = cadd(nj, cmul(cmul(ci, F), sQ));
            emits += (dQ <= a.maxdeg) + (dK <= a.maxdeg);
            store_coef<true>(s, i, ni);
            store_coef<true>(s, (u64)j, nj);
        } else {
            store_coef<true>(s, i, cscale(ci, a.c));
            if (dK <= a.maxdeg) {
                const cplx nv = cadd({0.0, 0.0}, cmul(cmul(ci, F), sQ));
                const u64 p = n_in + atomicAdd(app_ctr, 1ull);
#pragma unroll
                for (int w = 0; w < KW; w++) s.key[(u64)w * s.cap + p] = k[w];
                store_coef<true>(s, p, nv);
                s.dead[p] = 0;
                __threadfence();
                if (j >= 0) {
                    const u64 ent = __ldcg(&s.slots[jslot]);
                    atomicExch(&s.slots[jslot], (ent & 0xffffffff00000000ull) | p);
                } else {
                    insert<KW>(s, k, (u32)p, &C->error, false);
                }
                d_alive += 1;
                emits++;
            }
        }
    }
}

// --- truncation pass --------------------------------------------------------
template <int KW, bool CPLX, int NWX>
__device__ __forceinline__ void pass_trunc(const StoreView& s, const TruncArgs& t, u64 n,
                                           long long& d_alive) {
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (s.dead[i]) continue;
        bool kill = false;
        if (t.thr) {
            const double re = s.re[i];
            kill = CPLX ? abs_le(re, s.im[i], t.tau) : (fabs(re) <= t.tau);
        }
        if (!kill && NWX > 0 && t.max_xweight >= 0) {
            int xw = 0;
#pragma unroll
            for (int w = 0; w < (NWX > 0 ? NWX : 1); w++) xw += __popcll(s.key[(u64)w * s.cap + i]);
            kill = xw > t.max_xweight;
        }
        if (kill) {
            s.dead[i] = 1;
            d_alive -= 1;
        }
    }
}

// --- Clifford segment: map every key, then rebuild the index ----------------
template <int NW, bool CPLX>
__device__ __forceinline__ void pass_cliff_map(const StoreView& s, const CliffordOp* ops, int nops, u64 n) {
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
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
            s.re[i] = __dmul_rn(s.re[i], -1.0);
            if (CPLX) s.im[i] = __dmul_rn(s.im[i], -1.0);
        }
    }
}

__device__ __forceinline__ void pass_clear_slots(const StoreView& s) {
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i <= s.hmask; i += stride)
        s.slots[i] = kEmptySlot;
}

template <int KW>
__device__ __forceinline__ void pass_index(const StoreView& s, DevCounters* C, u64 n) {
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (s.dead[i]) continue;
        u64 k[KW];
        load_key<KW>(s, i, k);
        insert<KW>(s, k, (u32)i, &C->error, false);
    }
}

struct PersistArgs {
    const DevOp* ops;
    const PairArgs* pairs;
    const RotArgs* mrots;
    const TruncArgs* truncs;
    const CliffordOp* cliff;
    const GroupArgs<2>* groups2;
    int op_begin, op_end;
    int compact_min;  // stop for compaction when dead > alive and dead > compact_min
    long long barrier_limit;  // clock cycles a block waits at a grid barrier before giving up
};

template <int KW, bool CPLX, bool PAULI, bool FUSE2>
__global__ void __launch_bounds__(kPBlock, 2) persistent_kernel(StoreView s, DevCounters* C, PersistState* ps,
                                                                PersistArgs pa) {
    constexpr int NW = PAULI ? KW / 2 : 1;
    __shared__ long long sh[kPBlock / 32];
    __shared__ DevOp sop;
    __shared__ PairArgs spair;
    __shared__ RotArgs smrot;
    __shared__ TruncArgs strunc;
    __shared__ GroupArgs<2> sgroup;
    Bcast* bc = (Bcast*)ps->bcast;
    // every block keeps the committed counters
    u64 n = *(volatile u64*)&C->n;
    u64 alive = *(volatile u64*)&C->alive;
    u64 apps = *(volatile u64*)&C->apps;
    u64 peak = *(volatile u64*)&C->peak;
    u64 emits_tot = *(volatile u64*)&C->emits;
    u32 stop = 0;  // the host launches only with the error and overflow flags clear
    int o = pa.op_begin;
    // stage the first op's arguments in shared memory
    auto stage = [&](int which) {
        if (threadIdx.x == 0 && which < pa.op_end) {
            const DevOp op = pa.ops[which];
            sop = op;
            if (op.type == OP_PAIR) spair = pa.pairs[op.idx];
            else if (op.type == OP_GROUP2) sgroup = pa.groups2[op.idx];
            else if (op.type == OP_MROT) smrot = pa.mrots[op.idx];
            else if (op.type == OP_TRUNC) strunc = pa.truncs[op.idx];
        }
    };
    stage(o);
    __syncthreads();
    for (; o < pa.op_end && !stop; o++) {
        const int slot = o % 3;
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            const int nx = (o + 1) % 3;
            ps->d_app[nx] = 0;
            ps->d_alive[nx] = 0;
            ps->d_emit[nx] = 0;
            ps->d_xapps[nx] = 0;
        }
        const DevOp op = sop;
        long long d_alive = 0, emits = 0, xapps = 0;
        int ng_op = 1;
        bool is_rot = false;
        if (FUSE2 && op.type == OP_GROUP2 && PAULI) {
            const GroupArgs<2> a = sgroup;
            is_rot = true;
            if ((n << a.ng) > s.cap) {
                stop = 1;
                break;
            }
            u64* ac = &ps->d_app[slot];
            const u64 n_in = n;
            scan_pass<NW>(s, a.need, n_in,
                [&](const u64 (&q)[2 * NW]) -> u32 {
                    u32 A = 0;
#pragma unroll
                    for (int t = 0; t < 2; t++) {
                        if (t >= a.ng) break;
                        const u64* P = a.psub[1 << t];
                        u64 par = 0;
#pragma unroll
                        for (int w = 0; w < NW; w++) par ^= (q[w] & P[NW + w]) ^ (q[NW + w] & P[w]);
                        A |= (u32)(__popcll(par) & 1) << t;
                    }
                    return A;
                },
                [&](u64 i, u32 A) {
                    group_orbit<NW, CPLX, 2>(s, C, a, n_in, i, A, d_alive, emits, xapps, ac);
                });
            ng_op = a.ng;
        } else if (op.type == OP_PAIR || op.type == OP_MROT) {
            is_rot = true;
            if (2 * n > s.cap) {
                stop = 1;  // identical decision in every block
                break;
            }
            if (PAULI && op.type == OP_PAIR) {
                const PairArgs a = spair;
                pass_pair<NW, CPLX>(s, C, &ps->d_app[slot], a, n, d_alive, emits);
            }
            if (!PAULI && op.type == OP_MROT) {
                const RotArgs a = smrot;
                pass_mrot<KW>(s, C, &ps->d_app[slot], a, n, d_alive, emits);
            }
        } else if (op.type == OP_TRUNC) {
            const TruncArgs t = strunc;
            pass_trunc<KW, CPLX, (PAULI ? NW : 0)>(s, t, n, d_alive);
        } else if (op.type == OP_CLIFF && PAULI) {
            pass_cliff_map<NW, CPLX>(s, pa.cliff + op.begin, op.end - op.begin, n);
            if (!grid_sync(ps, bc, pa.barrier_limit)) { stop = 3; break; }
            pass_clear_slots(s);
            if (!grid_sync(ps, bc, pa.barrier_limit)) { stop = 3; break; }
            pass_index<KW>(s, C, n);
        }
        const long long bd = block_sum_ll(d_alive, sh);
        const long long be = block_sum_ll(emits, sh);
        const long long bx = block_sum_ll(xapps, sh);
        if (threadIdx.x == 0) {
            if (bd) atomicAdd((u64*)&ps->d_alive[slot], (u64)bd);
            if (be) atomicAdd(&ps->d_emit[slot], (u64)be);
            if (bx) atomicAdd(&ps->d_xapps[slot], (u64)bx);
        }
        stage(o + 1);  // prefetch the next op while waiting at the barrier
        Bcast f;
        if (!grid_sync_fold(ps, bc, slot, &f, pa.barrier_limit)) {
            stop = 3;
            break;
        }
        if (is_rot) apps += (u64)ng_op * alive + f.xapps;
        n += f.app;
        alive = (u64)((long long)alive + f.alive);
        emits_tot += f.emit;
        if (is_rot && alive > peak) peak = alive;
        if (op.type == OP_TRUNC && n - alive > alive && n - alive > (u64)pa.compact_min) {
            stop = 2;
            o++;
            break;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        volatile DevCounters* V = C;
        V->n = n;
        V->alive = alive;
        V->apps = apps;
        V->peak = peak;
        V->emits = emits_tot;
        if (stop == 1) V->overflow = (u32)o + 1u;
        ps->stop_reason = stop;
        ps->next_op = (u32)o;
        __threadfence();
    }
}

}  // namespace ffg
