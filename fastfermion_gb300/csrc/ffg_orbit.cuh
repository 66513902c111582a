// Batch-orbit processing of a run of mutually commuting Pauli rotations.
//
// Within a commuting batch (src/pauli/propagate.h:272-291) a term Q is acted on
// only by the gates A(Q) = {t : Q anticommutes with P_t}, and every product
// Q * P_t (t in A) has the same set A (the axes commute).  The gates therefore
// never pair terms whose sets A differ, nor terms that differ outside the
// bits U_A touched by the axes of A.  Terms are grouped by the key
// (A, Q & ~U_A); each group is a union of orbits Q * <P_t : t in A> and is
// processed on its own, gate by gate in batch order, with exactly the
// per-gate arithmetic, degree filter and creation rule of the reference
// (src/pauli/propagate.h:71-89).  The per-gate update of a group only involves
// its own members, so the result is bit-identical to applying the whole
// store gate by gate, while the work scales with the number of member updates
// rather than with (gates x store size).
//
// Kernels of one batch:
//   orbit_gate       opens the batch: input size from the previous batch's
//                    counters, or skip when that batch did not complete
//   orbit_classify   A(Q) and the group key of every input term; terms with
//                    A = {} are final and go straight to the output store
//   orbit_group      representative of every term's group (hash of the key)
//   orbit_offsets / orbit_scatter
//                    group ranges, members (keys, coefficients) copied into
//                    group order
//   orbit_process    one warp per group: members in a shared-memory table,
//                    gates applied in order, survivors of the batch-end
//                    truncation appended to the output store
//   orbit_process_big
//                    groups that outgrow a warp table, or whose |A| reaches
//                    the routing threshold: a thread team with a larger
//                    shared-memory table, then a block with a global-memory
//                    region
// An output store that would overflow stops the batch (the host grows it and
// runs the batch again from its intact input).
#pragma once
#include "ffg_kernels.cuh"

namespace ffg {

constexpr int kMaxBatchGates = 256;        // gates per orbit batch (longer runs are split)
constexpr int kAW = kMaxBatchGates / 64;   // words of a gate-subset mask
constexpr int kOrbitCap = 512;             // members of one group held in shared memory
constexpr int kOrbitWarps = 4;             // groups in flight per block

struct BatchGate {
    u64 p[4];     // axis planes in store order (the NW x words, then the NW z words)
    double c, s;
    int yP;
    int gidx;     // index of the gate in the caller's circuit (capture records)
};

struct OrbitScratch {
    u64* amask;    // [kAW][cap_in] gate-subset mask of each input term
    u64* gkey;     // [4][cap_in] key outside U_A
    u32* rep;      // [cap_in] representative of the term's group (0xffffffff = final)
    u32* cnt;      // [cap_in] members of the group represented by a term
    u32* off;      // [cap_in] first position of that group in `order`
    u32* fill;     // [cap_in]
    u32* order;    // [cap_in] input positions grouped
    u32* groups;   // [cap_in] list of representatives
    u32* big;      // [cap_in] representatives of groups too large for a warp table
    u32* list2;    // [cap_in] groups passed on by the Majorana sub-warp tier
    double* gcoef; // [2][cap_in] coefficients in group order (re, then im); after the
                   // scatter gkey holds the keys in group order too
    u64* gslots;   // [2*cap_in] group index: (fingerprint << 32) | representative
    u64 gmask;
    u64 cap_in;
};

struct OrbitCounters {
    u64 n_out;         // entries written to the output store
    u64 created;       // members created inside the batch
    u64 xapps;         // sum over created members of the batch gates after their creation
    u64 emits;
    u32 ngroups;
    u32 overflow;      // 1: output store too small, 2: a group outgrew kOrbitCap
    u32 error;
    u32 max_members;   // largest group seen (members at the end, or on input when too large)
    u32 nbig;          // groups left for the block-level pass (list in OrbitScratch::big)
    u32 big_overflow;  // a block-level group outgrew its region
    u32 chk_code;      // self-check builds: first failed check (0 = none)
    u32 chk_a, chk_b, chk_c;
    u32 hist[16];      // completed groups by floor(log2(final members))
    u32 hist_a[16];    // completed groups by |A| (capped at 15)
    u32 wasted;        // groups abandoned by the warp pass after growing past its table
    u32 skip;          // 1: an earlier batch of the window did not complete; this one does nothing
    u32 member_total;  // members placed by orbit_offsets
    u32 nrest;         // groups left by a thread-level pass for the warp tier (list in OrbitScratch::fill)
    u32 nrest2;        // groups left by a sub-warp pass (list in OrbitScratch::list2)
    u64 n_in;          // terms entering the batch (set by orbit_gate)
    u64 gmask;         // group-index slots - 1 for this batch (set by orbit_gate)
    u32 fetch[2];      // groups handed out by the team and block passes beyond their first round
    u32 pad;
};

#ifdef FFG_ORBIT_CHECK
#define OCHK(cond, code, a_, b_, c_)                                              \
    if (!(cond)) {                                                               \
        if (atomicCAS(&oc->chk_code, 0u, (u32)(code)) == 0u) {                   \
            oc->chk_a = (u32)(a_);                                               \
            oc->chk_b = (u32)(b_);                                               \
            oc->chk_c = (u32)(c_);                                               \
        }                                                                        \
        continue;                                                                \
    }
#else
#define OCHK(cond, code, a_, b_, c_)
#endif

// Partners that the degree filter drops, recorded for the learned correction
// (no counterpart in the reference): every partner of degree in
// (maxdeg of the batch, cap.maxdeg] whose |value| exceeds cap.min_abs (every
// one when min_abs is 0), with the
// index of the circuit gate that created it.  A group or batch that is run
// again (a table or the output store overflowed) records its drops again; the
// index over (key, gate) keeps the first record and marks later ones with
// gate = -1.  Off when n is null.
struct CaptureArgs {
    u64* key;        // [4][cap] caller layout: xory words 0, 1, yorz words 0, 1
    double* re;      // [cap]
    double* im;      // [cap]
    int* gate;       // [cap] circuit gate index, -1 = repeat of an earlier record
    u32* slot;       // [2 * cap] index over (key, gate): record + 1, 0 = empty
    u64* n;          // records claimed (> cap: the buffer was too small)
    u64 cap;         // power of two
    int maxdeg;
    int pad;
    double min_abs;
};

struct OrbitBatchArgs {
    const BatchGate* gates;  // k gates of the batch, application order
    int k;
    int maxdeg;
    // fused batch-end truncation
    int thr;
    double tau;
    int max_xweight;
    int route_big;  // groups with at least this many gates in A go straight to the block-level pass
    // batched instances (null inst_cs: one instance, angles from `gates`).  The
    // instance of a term is (key plane inst_plane >> inst_shift) & inst_mask;
    // gate t of instance i uses inst_cs[t * ninst + i] = (cos, sin).
    const double2* inst_cs;
    u32 ninst;
    int inst_plane;
    int inst_shift;
    u64 inst_mask;
    // qubit -> gates index of the batch (null: test every gate): gates touching
    // qubit q are qidx[129 + qidx[q] .. 129 + qidx[q + 1]).  A Pauli gate
    // anticommutes only with terms whose support it touches.
    const u32* qidx;
    // per-instance active rotations (null: every rotation acts on every
    // instance).  Rotation r (circuit order among the rotations) acts on
    // instance i iff bit r of active[i * active_words + r / 64]; batch gate t
    // is rotation act_r0 - t.  An inactive gate leaves the instance's terms
    // untouched; the batch-end truncation still runs.
    const u64* active;
    u32 active_words;
    int act_r0;
    const CaptureArgs* cap;  // record of dropped partners (device copy; null: off)
};

// whether batch gate t acts on instance inst
__device__ __forceinline__ bool gate_active(const OrbitBatchArgs& a, u32 inst, int t) {
    const int r = a.act_r0 - t;
    return (__ldg(&a.active[(u64)inst * a.active_words + (u32)(r >> 6)]) >> (r & 63)) & 1ull;
}

template <int NW>
__device__ __forceinline__ u64 capture_hash(const u64 (&c)[4], int gidx) {
    u64 h = mix64(c[0] ^ 0x9e3779b97f4a7c15ull ^ ((u64)(u32)gidx << 32));
#pragma unroll
    for (int w = 1; w < 4; w++) h = mix64(h ^ c[w]);
    return h;
}

// Records one dropped partner (key k in store order, value v) created by the
// circuit gate gidx.
template <int NW, bool CPLX>
__device__ void capture_drop(const CaptureArgs& cp, const u64* k, cplx v, int gidx) {
    if (cp.min_abs > 0.0) {  // min_abs = 0 records every dropped partner, exact zeros included
        const bool small = CPLX ? abs_le(v.re, v.im, cp.min_abs) : (fabs(v.re) <= cp.min_abs);
        if (small) return;
    }
    const u64 idx = atomicAdd(cp.n, 1ull);
    if (idx >= cp.cap) return;  // the host sees n > cap and runs again with more room
    const u64 c[4] = {k[0], NW == 2 ? k[1] : 0ull, k[NW], NW == 2 ? k[NW + 1] : 0ull};
#pragma unroll
    for (int w = 0; w < 4; w++) cp.key[(u64)w * cp.cap + idx] = c[w];
    cp.re[idx] = v.re;
    cp.im[idx] = CPLX ? v.im : 0.0;
    cp.gate[idx] = gidx;
    __threadfence();
    const u64 mask = 2 * cp.cap - 1;
    u64 pos = capture_hash<NW>(c, gidx) & mask;
    for (u64 probe = 0; probe <= mask; probe++) {
        const u32 e = atomicCAS(&cp.slot[pos], 0u, (u32)idx + 1u);
        if (e == 0u) return;
        const u64 j = e - 1u;
        bool same = __ldcg(&cp.gate[j]) == gidx;
#pragma unroll
        for (int w = 0; w < 4; w++) same = same && __ldcg(&cp.key[(u64)w * cp.cap + j]) == c[w];
        if (same) {
            cp.gate[idx] = -1;
            return;
        }
        pos = (pos + 1) & mask;
    }
}

// Waits until the grid this one depends on (programmatic dependent launch)
// has completed and its memory is visible; returns at once for a normal launch.
__device__ __forceinline__ void wait_prior_grid() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// barrier of a team of TEAM threads (a warp, or the whole block)
template <int TEAM>
__device__ __forceinline__ void team_sync() {
    if constexpr (TEAM < 32) {
        // the TEAM-lane slice of the warp that this thread belongs to
        const unsigned lane = threadIdx.x & 31;
        __syncwarp(((1u << TEAM) - 1) << (lane & ~(unsigned)(TEAM - 1)));
    } else if constexpr (TEAM == 32) {
        __syncwarp();
    } else {
        __syncthreads();
    }
}

// instance of the group represented by input position rep
__device__ __forceinline__ u32 group_instance(const StoreView& in, const OrbitBatchArgs& a, u32 rep) {
    if (!a.inst_cs) return 0;
    return (u32)((in.key[(u64)a.inst_plane * in.cap + rep] >> a.inst_shift) & a.inst_mask);
}

// (cos, sin) of batch gate t for instance inst
__device__ __forceinline__ void gate_cs(const OrbitBatchArgs& a, const BatchGate& G, int t, u32 inst,
                                        double& c, double& s) {
    if (a.inst_cs) {
        const double2 v = a.inst_cs[(u64)t * a.ninst + inst];
        c = v.x;
        s = v.y;
    } else {
        c = G.c;
        s = G.s;
    }
}

template <int NW, bool CPLX>
__device__ __forceinline__ bool survives(const u64* key, cplx c, const OrbitBatchArgs& a) {
    if (a.thr) {
        const bool small = CPLX ? abs_le(c.re, c.im, a.tau) : abs_le_bits(c.re, a.tau);
        if (small) return false;
    }
    if (a.max_xweight >= 0) {
        int xw = 0;
#pragma unroll
        for (int w = 0; w < NW; w++) xw += __popcll(key[w]);
        if (xw > a.max_xweight) return false;
    }
    return true;
}

// Appends the entries of the calling lanes that keep theirs with one atomic
// per set of converged lanes (warp ballot, then each lane's rank in it).
// Every converged lane calls it, keep or not.
template <int KW, bool CPLX>
__device__ __forceinline__ void out_append_warp(const StoreView& o, OrbitCounters* oc, const u64* key, cplx c,
                                                bool keep) {
    const unsigned mask = __activemask();
    const unsigned ball = __ballot_sync(mask, keep);
    if (!ball) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(ball) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(&oc->n_out, (u64)__popc(ball));
    base = __shfl_sync(mask, base, leader);
    if (!keep) return;
    const u64 pos = base + (u64)__popc(ball & ((1u << lane) - 1u));
    if (pos >= o.cap) {
        atomicOr(&oc->overflow, 1u);
        return;
    }
#pragma unroll
    for (int w = 0; w < KW; w++) o.key[(u64)w * o.cap + pos] = key[w];
    o.re[pos] = c.re;
    if (CPLX) o.im[pos] = c.im;
    o.dead[pos] = 0;
}

// Reserves one slot of the counter *ctr for each calling lane, with one atomic
// per set of converged lanes that name the same counter (a group's new members
// are numbered this way: a same-address atomic per lane serialises every
// creating thread of a gate; lanes of one warp may serve different groups);
// returns this lane's slot.
__device__ __forceinline__ u32 warp_reserve(u32* ctr) {
    const unsigned mask = __match_any_sync(__activemask(), (unsigned long long)ctr);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    u32 base = 0;
    if (lane == leader) base = atomicAdd(ctr, (u32)__popc(mask));
    base = __shfl_sync(mask, base, leader);
    return base + (u32)__popc(mask & ((1u << lane) - 1u));
}

template <int KW, bool CPLX>
__device__ __forceinline__ void out_append(const StoreView& o, OrbitCounters* oc, const u64* key, cplx c) {
    const u64 pos = atomicAdd(&oc->n_out, 1ull);
    if (pos >= o.cap) {
        atomicOr(&oc->overflow, 1u);
        return;
    }
#pragma unroll
    for (int w = 0; w < KW; w++) o.key[(u64)w * o.cap + pos] = key[w];
    o.re[pos] = c.re;
    if (CPLX) o.im[pos] = c.im;
    o.dead[pos] = 0;
}

// Opens a batch (one warp): clears its counters and, unless an earlier batch
// of the window did not complete (overflowed its output store, failed a
// check, or left groups for the host in nretry[1]), sets the number of input
// terms (the previous batch's output, or n_first) and the group-index size,
// and clears the two retry counts.  Otherwise the batch is marked skipped and
// every kernel of it returns at once, leaving the scratch as the incomplete
// batch left it.
static __global__ void orbit_gate(OrbitCounters* cur, const OrbitCounters* prev, u64 n_first, u64 gslots_cap,
                           u32* nretry) {
    wait_prior_grid();
    constexpr u32 nw = sizeof(OrbitCounters) / 4;
    for (u32 i = threadIdx.x; i < nw; i += blockDim.x) ((u32*)cur)[i] = 0;
    __syncwarp();
    if (threadIdx.x != 0) return;
    const bool bad = prev && (prev->skip || (prev->overflow & 1u) || prev->error || prev->chk_code ||
                              nretry[1] != 0);
    if (bad) {
        cur->skip = 1;
        return;
    }
    const u64 n = prev ? prev->n_out : n_first;
    u64 slots = 1024;
    while (slots < 2 * n) slots <<= 1;
    if (slots > gslots_cap) {  // more input terms than the window was sized for
        cur->skip = 1;
        cur->overflow = 1;
        cur->n_out = n;
        return;
    }
    cur->n_in = n;
    cur->gmask = slots - 1;
    nretry[0] = 0;
    nretry[1] = 0;
}

// A(Q) for every input term; group key; final terms go to the output.
// ACT: per-instance active rotations (a.active) are honoured; the plain
// instantiation carries no trace of them.
template <int NW, bool CPLX, bool ACT = false>
__global__ void __launch_bounds__(kBlock) orbit_classify(StoreView in, StoreView out, OrbitScratch sc,
                                                         OrbitCounters* oc, OrbitBatchArgs a) {
    wait_prior_grid();
    constexpr int KW = 2 * NW;
    if (*(volatile u32*)&oc->skip) return;
    const u64 n_in = *(volatile u64*)&oc->n_in;
    const u64 nslots = *(volatile u64*)&oc->gmask + 1;
    __shared__ u64 gp[kMaxBatchGates][KW];
    for (int t = threadIdx.x; t < a.k; t += blockDim.x)
        for (int w = 0; w < KW; w++) gp[t][w] = a.gates[t].p[w];
    __syncthreads();
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < nslots; i += stride) sc.gslots[i] = kEmptySlot;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n_in; i += stride) {
        u64 q[KW];
        load_key<KW>(in, i, q);
        u64 A[kAW] = {};
        u64 U[KW] = {};
        const u32 inst = ACT ? (u32)((q[a.inst_plane] >> a.inst_shift) & a.inst_mask) : 0u;
        if (a.qidx) {
            // candidates: the gates on the term's support
#pragma unroll
            for (int ws = 0; ws < NW; ws++) {
                u64 sup = q[ws] | q[NW + ws];
                while (sup) {
                    const int qb = 64 * ws + __ffsll((long long)sup) - 1;
                    sup &= sup - 1;
                    const u32 e1 = __ldg(&a.qidx[qb + 1]);
                    for (u32 e = __ldg(&a.qidx[qb]); e < e1; e++) {
                        const int t = (int)__ldg(&a.qidx[129 + e]);
                        if ((A[t >> 6] >> (t & 63)) & 1ull) continue;
                        if (ACT && !gate_active(a, inst, t)) continue;
                        u64 par = 0;
#pragma unroll
                        for (int w = 0; w < NW; w++) par ^= (q[w] & gp[t][NW + w]) ^ (q[NW + w] & gp[t][w]);
                        if (__popcll(par) & 1) {
                            A[t >> 6] |= 1ull << (t & 63);
#pragma unroll
                            for (int w = 0; w < KW; w++) U[w] |= gp[t][w];
                        }
                    }
                }
            }
        } else {
            for (int t = 0; t < a.k; t++) {
                if (ACT && !gate_active(a, inst, t)) continue;
                u64 par = 0;
#pragma unroll
                for (int w = 0; w < NW; w++) par ^= (q[w] & gp[t][NW + w]) ^ (q[NW + w] & gp[t][w]);
                if (__popcll(par) & 1) {
                    A[t >> 6] |= 1ull << (t & 63);
#pragma unroll
                    for (int w = 0; w < KW; w++) U[w] |= gp[t][w];
                }
            }
        }
        bool any = false;
#pragma unroll
        for (int w = 0; w < kAW; w++) any = any || A[w];
        if (!any) {
            sc.rep[i] = 0xffffffffu;
            const cplx c = load_coef<CPLX>(in, i);
            out_append_warp<KW, CPLX>(out, oc, q, c, survives<NW, CPLX>(q, c, a));
            continue;
        }
#pragma unroll
        for (int w = 0; w < kAW; w++) sc.amask[(u64)w * sc.cap_in + i] = A[w];
#pragma unroll
        for (int w = 0; w < KW; w++) sc.gkey[(u64)w * sc.cap_in + i] = q[w] & ~U[w];
        sc.cnt[i] = 0;
        sc.fill[i] = 0;
        sc.rep[i] = 0xfffffffeu;  // grouped in the next pass
    }
}

template <int KW>
__device__ __forceinline__ u64 group_hash(const OrbitScratch& sc, u64 i) {
    u64 h = 0x51ed270b27e41b3bull;
#pragma unroll
    for (int w = 0; w < kAW; w++) h = mix64(h ^ sc.amask[(u64)w * sc.cap_in + i]);
#pragma unroll
    for (int w = 0; w < KW; w++) h = mix64(h ^ sc.gkey[(u64)w * sc.cap_in + i]);
    return h;
}

template <int KW>
__device__ __forceinline__ bool same_group(const OrbitScratch& sc, u64 i, u64 j) {
#pragma unroll
    for (int w = 0; w < kAW; w++)
        if (sc.amask[(u64)w * sc.cap_in + i] != sc.amask[(u64)w * sc.cap_in + j]) return false;
#pragma unroll
    for (int w = 0; w < KW; w++)
        if (sc.gkey[(u64)w * sc.cap_in + i] != sc.gkey[(u64)w * sc.cap_in + j]) return false;
    return true;
}

// representative of each term's group: the term that claims the index slot
template <int KW>
__global__ void __launch_bounds__(kBlock) orbit_group(OrbitScratch sc, OrbitCounters* oc) {
    wait_prior_grid();
    if (*(volatile u32*)&oc->skip) return;
    const u64 n_in = *(volatile u64*)&oc->n_in;
    const u64 gmask = *(volatile u64*)&oc->gmask;
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n_in; i += stride) {
        if (sc.rep[i] == 0xffffffffu) continue;
        const u64 h = group_hash<KW>(sc, i);
        const u32 fp = (u32)(h >> 32);
        u64 pos = h & gmask;
        u32 rep = 0xffffffffu;
        for (u64 probe = 0; probe <= gmask; probe++) {
            u64 e = __ldcg(&sc.gslots[pos]);
            if (e == kEmptySlot) {
                e = atomicCAS(&sc.gslots[pos], kEmptySlot, ((u64)fp << 32) | i);
                if (e == kEmptySlot) {
                    rep = (u32)i;
                    break;
                }
            }
            if ((u32)(e >> 32) == fp && same_group<KW>(sc, i, (u32)e)) {
                rep = (u32)e;
                break;
            }
            pos = (pos + 1) & gmask;
        }
        if (rep == 0xffffffffu) {
            atomicOr(&oc->error, 1u);
            rep = (u32)i;
        }
        sc.rep[i] = rep;
        atomicAdd(&sc.cnt[rep], 1u);
        if (rep == (u32)i) {
            const u32 g = atomicAdd(&oc->ngroups, 1u);
            sc.groups[g] = (u32)i;
        }
    }
}

// first member position of every group (groups listed in sc.groups).  Any
// placement of the groups works (each group is processed on its own), so the
// ranges come from warp-aggregated atomic additions, in parallel.
static __global__ void __launch_bounds__(kBlock) orbit_offsets(OrbitScratch sc, OrbitCounters* oc) {
    wait_prior_grid();
    if (*(volatile u32*)&oc->skip) return;
    const u32 ng = *(volatile u32*)&oc->ngroups;
    const int lane = threadIdx.x & 31;
    const u32 stride = gridDim.x * blockDim.x;
    // every warp runs the same number of iterations so that the shuffles see full warps
    const u32 tid = blockIdx.x * blockDim.x + threadIdx.x;
    const u32 rounds = (ng + stride - 1) / stride;
    for (u32 r = 0; r < rounds; r++) {
        const u32 g = tid + r * stride;
        const u32 rep = g < ng ? sc.groups[g] : 0u;
        const u32 v = g < ng ? sc.cnt[rep] : 0u;
        u32 x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const u32 y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        u32 base = 0;
        if (lane == 31 && x) base = atomicAdd(&oc->member_total, x);
        base = __shfl_sync(0xffffffffu, base, 31);
        if (g < ng) sc.off[rep] = base + x - v;
    }
}

// Members made contiguous: position p of a group's range gets the input
// position (order) and a copy of the key planes (into gkey, no longer needed
// for grouping) and of the coefficient, so that group processing reads one
// contiguous range instead of gathering from the store.
template <int KW, bool CPLX>
__global__ void __launch_bounds__(kBlock) orbit_scatter(StoreView in, OrbitScratch sc, const OrbitCounters* oc) {
    wait_prior_grid();
    if (*(volatile const u32*)&oc->skip) return;
    const u64 n_in = *(volatile const u64*)&oc->n_in;
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n_in; i += stride) {
        const u32 r = sc.rep[i];
        if (r == 0xffffffffu) continue;
        const u32 p = sc.off[r] + atomicAdd(&sc.fill[r], 1u);
        sc.order[p] = (u32)i;
#pragma unroll
        for (int w = 0; w < KW; w++) sc.gkey[(u64)w * sc.cap_in + p] = in.key[(u64)w * in.cap + i];
        sc.gcoef[p] = in.re[i];
        if (CPLX) sc.gcoef[sc.cap_in + p] = in.im[i];
    }
}

// --- group processing: one warp per group ----------------------------------
template <int KW, bool CPLX>
struct OrbitTable {
    u64 key[kOrbitCap][KW];
    double re[kOrbitCap];
    double im[CPLX ? kOrbitCap : 1];
    unsigned short slot[2 * kOrbitCap];  // index of members, 0xffff = empty
    unsigned int cnt;                     // members in the table
    unsigned int flag;                    // the group outgrew the table
};

// Hash of a key for the per-group tables, on the critical path of every
// member update: each key word is multiplied by its own odd constant (the
// four products are independent), the products are rotated apart and XORed
// (a multiplication carries into higher bits only, so the rotations keep the
// top-bit flips of different words from cancelling), and one 64-bit mixing
// round spreads the result.  Bits 32.. are the table position, bits 13..31 a
// fingerprint; the hash is computed once per member and gate and reused by
// the insert.  (Hashes that first fold the key words by XOR map keys that
// differ on particular qubit pairs to the same value; on the large W = 10
// groups that lengthened the probe chains and slowed the workload by a
// third.)  A full key match is still required to find a member, so the hash
// only decides where members sit in a table, never the results.
__device__ __forceinline__ u64 rotl64(u64 x, int r) { return r ? (x << r) | (x >> (64 - r)) : x; }

template <int KW>
__device__ __forceinline__ u64 tab_hash(const u64* k) {
    constexpr u64 mul[4] = {0x9e3779b97f4a7c15ull, 0xc2b2ae3d27d4eb4full, 0x165667b19e3779f9ull,
                            0xd6e8feb86659fd93ull};
    constexpr int rot[4] = {0, 17, 31, 47};
    u64 x = k[0] * mul[0];
#pragma unroll
    for (int w = 1; w < KW; w++) x ^= rotl64(k[w] * mul[w & 3], rot[w & 3]);
    return mix64(x);
}
__device__ __forceinline__ u32 tab_pos(u64 h) { return (u32)(h >> 32); }
__device__ __forceinline__ u32 tab_fp(u64 h) { return (u32)h >> 13; }  // 19 bits

template <int KW>
__device__ __forceinline__ u32 small_hash(const u64* k) {
    return tab_pos(tab_hash<KW>(k));
}

// member index of key k or -1 (lanes of one warp share the table)
// hp: small_hash of the key
template <int KW, bool CPLX>
__device__ __forceinline__ int table_find(const OrbitTable<KW, CPLX>& T, const u64* k, u32 hp) {
    u32 pos = hp & (2 * kOrbitCap - 1);
    for (int probe = 0; probe < 2 * kOrbitCap; probe++) {
        const unsigned short m = ((volatile unsigned short*)T.slot)[pos];
        if (m == 0xffff) return -1;
        bool eq = true;
#pragma unroll
        for (int w = 0; w < KW; w++) eq = eq && T.key[m][w] == k[w];
        if (eq) return m;
        pos = (pos + 1) & (2 * kOrbitCap - 1);
    }
    return -1;
}

template <int KW, bool CPLX>
__device__ __forceinline__ void table_insert(OrbitTable<KW, CPLX>& T, u32 hp, unsigned short m) {
    u32 pos = hp & (2 * kOrbitCap - 1);
    for (int probe = 0; probe < 2 * kOrbitCap; probe++) {
        unsigned int* word = (unsigned int*)&T.slot[pos & ~1u];
        const int hi = pos & 1;
        unsigned int old = *(volatile unsigned int*)word;
        for (;;) {
            const unsigned short cur = hi ? (unsigned short)(old >> 16) : (unsigned short)(old & 0xffff);
            if (cur != 0xffff) break;
            const unsigned int nw = hi ? ((old & 0x0000ffffu) | ((u32)m << 16)) : ((old & 0xffff0000u) | m);
            const unsigned int seen = atomicCAS(word, old, nw);
            if (seen == old) return;
            old = seen;
        }
        pos = (pos + 1) & (2 * kOrbitCap - 1);
    }
}

// REC: dropped partners are recorded into *a.cap (capture runs); the plain
// instantiation carries no trace of the record.
template <int NW, bool CPLX, bool REC = false>
__global__ void __launch_bounds__(32 * kOrbitWarps, 4) orbit_process(StoreView in, StoreView out, OrbitScratch sc,
                                                                  OrbitCounters* oc, OrbitBatchArgs a) {
    wait_prior_grid();
    constexpr int KW = 2 * NW;
    extern __shared__ unsigned char smem[];
    OrbitTable<KW, CPLX>* tables = (OrbitTable<KW, CPLX>*)smem;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    OrbitTable<KW, CPLX>& T = tables[warp];
    const u32 ng = *(volatile u32*)&oc->ngroups;
    long long emits = 0, created = 0, xapps = 0;
    for (u32 g = blockIdx.x * kOrbitWarps + warp; g < ng; g += gridDim.x * kOrbitWarps) {
        long long g_emits = 0, g_created = 0, g_xapps = 0;
        OCHK(g < sc.cap_in, 13, g, ng, 0)
        const u32 rep = sc.groups[g];
        OCHK(rep < sc.cap_in, 14, rep, g, ng)
        const u32 m0 = sc.cnt[rep];
        const u32 base = sc.off[rep];
        int na = 0;
#pragma unroll
        for (int w = 0; w < kAW; w++) na += __popcll(sc.amask[(u64)w * sc.cap_in + rep]);
        if (m0 > kOrbitCap || na >= a.route_big) {
            if (lane == 0) {
                sc.big[atomicAdd(&oc->nbig, 1u)] = rep;
                atomicMax(&oc->max_members, m0);
            }
            continue;
        }
        // load members
        for (int s = lane; s < 2 * kOrbitCap; s += 32) T.slot[s] = 0xffff;
        __syncwarp();
        for (u32 m = lane; m < m0; m += 32) {
            OCHK((u64)base + m < sc.cap_in, 11, base, m, rep)
            const u64 pm = (u64)base + m;
#pragma unroll
            for (int w = 0; w < KW; w++) T.key[m][w] = sc.gkey[(u64)w * sc.cap_in + pm];
            T.re[m] = sc.gcoef[pm];
            if (CPLX) T.im[m] = sc.gcoef[sc.cap_in + pm];
            table_insert<KW, CPLX>(T, small_hash<KW>(T.key[m]), (unsigned short)m);
        }
        if (lane == 0) {
            T.cnt = m0;
            T.flag = 0;
        }
        __syncwarp();
        const u32 inst = group_instance(in, a, rep);
        // gates of A in batch order
        u64 A[kAW];
#pragma unroll
        for (int w = 0; w < kAW; w++) A[w] = sc.amask[(u64)w * sc.cap_in + rep];
        for (int wd = 0; wd < kAW; wd++) {
            u64 bits = A[wd];
            while (bits) {
                const int t = 64 * wd + __ffsll((long long)bits) - 1;
                bits &= bits - 1;
                const BatchGate G = a.gates[t];
                double gc, gs;
                gate_cs(a, G, t, inst, gc, gs);
                const bool unit = !CPLX && unit_sine(gs);
                auto partner = [&](cplx b, int jj) {
                    return unit ? rot_partner_unit<CPLX>(b, gs, jj) : rot_partner<CPLX>(b, gs, jj);
                };
                u64 P[KW];
#pragma unroll
                for (int w = 0; w < KW; w++) P[w] = G.p[w];
                const int cnt0 = (int)*(volatile unsigned int*)&T.cnt;
                __syncwarp();
                for (int m = lane; m < cnt0; m += 32) {
                    u64 q[KW], k[KW];
#pragma unroll
                    for (int w = 0; w < KW; w++) {
                        q[w] = T.key[m][w];
                        k[w] = q[w] ^ P[w];
                    }
                    int yQ = 0, yK = 0, zxQ = 0, zxK = 0, dQ = 0, dK = 0;
#pragma unroll
                    for (int w = 0; w < NW; w++) {
                        yQ += __popcll(q[w] & q[NW + w]);
                        yK += __popcll(k[w] & k[NW + w]);
                        zxQ += __popcll(P[NW + w] & q[w]);
                        zxK += __popcll(P[NW + w] & k[w]);
                        dQ += __popcll(q[w] | q[NW + w]);
                        dK += __popcll(k[w] | k[NW + w]);
                    }
                    const int jQ = G.yP + yQ + 2 * zxQ - yK;  // P*Q -> K
                    const int jK = G.yP + yK + 2 * zxK - yQ;  // P*K -> Q
                    const cplx ci = {T.re[m], CPLX ? T.im[m] : 0.0};
                    const u32 hk = small_hash<KW>(k);
                    const int j = table_find<KW, CPLX>(T, k, hk);
                    if (j >= 0 && j < cnt0) {
                        if (j < m) continue;  // the pair belongs to member j
                        const cplx cj = {T.re[j], CPLX ? T.im[j] : 0.0};
                        cplx ni = rot_keep<CPLX>(ci, gc), nj = rot_keep<CPLX>(cj, gc);
                        if (dQ <= a.maxdeg) ni = rot_add<CPLX>(ni, partner(cj, jK));
                        else if (REC && a.cap && dQ <= a.cap->maxdeg)
                            capture_drop<NW, CPLX>(*a.cap, q, partner(cj, jK), G.gidx);
                        if (dK <= a.maxdeg) nj = rot_add<CPLX>(nj, partner(ci, jQ));
                        else if (REC && a.cap && dK <= a.cap->maxdeg)
                            capture_drop<NW, CPLX>(*a.cap, k, partner(ci, jQ), G.gidx);
                        g_emits += (dQ <= a.maxdeg) + (dK <= a.maxdeg);
                        T.re[m] = ni.re;
                        T.re[j] = nj.re;
                        if (CPLX) {
                            T.im[m] = ni.im;
                            T.im[j] = nj.im;
                        }
                    } else {
                        const cplx ni = rot_keep<CPLX>(ci, gc);
                        T.re[m] = ni.re;
                        if (CPLX) T.im[m] = ni.im;
                        if (dK <= a.maxdeg) {
                            g_emits++;
                            const cplx nv = rot_new<CPLX>(partner(ci, jQ));
                            const unsigned int idx = warp_reserve(&T.cnt);
                            if (idx >= (unsigned int)kOrbitCap) {
                                atomicExch(&T.flag, 1u);
                            } else {
#pragma unroll
                                for (int w = 0; w < KW; w++) T.key[idx][w] = k[w];
                                T.re[idx] = nv.re;
                                if (CPLX) T.im[idx] = nv.im;
                                __threadfence_block();
                                table_insert<KW, CPLX>(T, hk, (unsigned short)idx);
                                g_created++;
                                g_xapps += a.k - 1 - t;
                            }
                        } else if (REC && a.cap && dK <= a.cap->maxdeg) {
                            capture_drop<NW, CPLX>(*a.cap, k, partner(ci, jQ), G.gidx);
                        }
                    }
                }
                __syncwarp();
                if (*(volatile unsigned int*)&T.flag) break;
            }
            if (*(volatile unsigned int*)&T.flag) break;
        }
        __syncwarp();
        if (*(volatile unsigned int*)&T.flag) {
            if (lane == 0) {
                sc.big[atomicAdd(&oc->nbig, 1u)] = rep;
                atomicAdd(&oc->wasted, 1u);
            }
            continue;
        }
        emits += g_emits;
        created += g_created;
        xapps += g_xapps;
        // survivors of the batch-end truncation go to the output store
        const int cnt = (int)*(volatile unsigned int*)&T.cnt;
        if (lane == 0) {
            atomicMax(&oc->max_members, (u32)cnt);
            atomicAdd(&oc->hist[31 - __clz(cnt | 1)], 1u);
            int na = 0;
            for (int w = 0; w < kAW; w++) na += __popcll(A[w]);
            atomicAdd(&oc->hist_a[na < 15 ? na : 15], 1u);
        }
        for (int m = lane; m < cnt; m += 32) {
            const cplx c = {T.re[m], CPLX ? T.im[m] : 0.0};
            out_append_warp<KW, CPLX>(out, oc, T.key[m], c, survives<NW, CPLX>(T.key[m], c, a));
        }
        __syncwarp();
    }
    // block totals
    for (int o = 16; o > 0; o >>= 1) {
        emits += __shfl_down_sync(0xffffffffu, emits, o);
        created += __shfl_down_sync(0xffffffffu, created, o);
        xapps += __shfl_down_sync(0xffffffffu, xapps, o);
    }
    if (lane == 0) {
        if (emits) atomicAdd(&oc->emits, (u64)emits);
        if (created) atomicAdd(&oc->created, (u64)created);
        if (xapps) atomicAdd(&oc->xapps, (u64)xapps);
    }
}

// --- groups too large for a warp: one block per group, table in global memory
struct BigPool {
    char* base;      // regions of region_bytes each
    u64 region_bytes;
    u32 rcap;        // members per region (power of two)
    u32* retry;      // representatives of groups that outgrew their region
    u32* nretry;
    u32* fetch;      // counter of groups handed out after each block's first (null: blocks stride the list)
};

template <int KW, bool CPLX>
struct BigRegion {
    u64* key;      // [KW][rcap]
    double* re;
    double* im;
    u32* slot;     // [2*rcap], 0xffffffff = empty; (fingerprint << 12) | member in shared memory
    u32* cnt;      // members when the group was loaded (the kernel keeps the running count in registers)
    u32* flag;     // the group outgrew the table
};

template <int KW, bool CPLX>
__device__ __forceinline__ BigRegion<KW, CPLX> big_region(const BigPool& bp, u32 r) {
    BigRegion<KW, CPLX> g;
    char* p = bp.base + (u64)r * bp.region_bytes;
    g.key = (u64*)p;
    p += (u64)KW * bp.rcap * 8;
    g.re = (double*)p;
    p += (u64)bp.rcap * 8;
    g.im = (double*)p;
    if (CPLX) p += (u64)bp.rcap * 8;
    g.slot = (u32*)p;
    p += (u64)2 * bp.rcap * 4;
    g.cnt = (u32*)p;
    g.flag = g.cnt + 1;
    return g;
}

// loads from a block-level table: L2 for global-memory regions, volatile for
// shared memory
template <bool SM, typename T>
__device__ __forceinline__ T tld(const T* p) {
    if (SM) return *(const volatile T*)p;
    return __ldcg(p);
}

// Block-level tables in shared memory (FP) keep a fingerprint with each
// member index, (tab_fp << 12) | index (tables of at most 4096 members, the
// top bit never set), so that a probe reads the member's key only when the
// fingerprints agree; global-memory regions (any size) keep the index alone.
// Both take the key's tab_hash h.
constexpr u32 kFpShift = 12;

template <int KW, bool CPLX, bool SM = false, bool FP = false>
__device__ __forceinline__ int big_find(const BigRegion<KW, CPLX>& G, u32 rcap, const u64* k, u64 h) {
    const u32 mask = 2 * rcap - 1;
    u32 pos = tab_pos(h) & mask;
    const u32 fp = tab_fp(h);
    for (u32 probe = 0; probe <= mask; probe++) {
        const u32 e = tld<SM>(&G.slot[pos]);
        if (e == 0xffffffffu) return -1;
        if (!FP || (e >> kFpShift) == fp) {
            const u32 m = FP ? (e & ((1u << kFpShift) - 1)) : e;
#ifdef FFG_ORBIT_CHECK
            if (m >= rcap) return (int)0x7fffffff;
#endif
            bool eq = true;
#pragma unroll
            for (int w = 0; w < KW; w++) eq = eq && tld<SM>(&G.key[(u64)w * rcap + m]) == k[w];
            if (eq) return (int)m;
        }
        pos = (pos + 1) & mask;
    }
    return -1;
}

template <int KW, bool CPLX, bool FP = false>
__device__ __forceinline__ void big_insert(const BigRegion<KW, CPLX>& G, u32 rcap, u32 m, u64 h) {
    const u32 mask = 2 * rcap - 1;
    u32 pos = tab_pos(h) & mask;
    const u32 e = FP ? ((tab_fp(h) << kFpShift) | m) : m;
    for (u32 probe = 0; probe <= mask; probe++) {
        if (atomicCAS(&G.slot[pos], 0xffffffffu, e) == 0xffffffffu) return;
        pos = (pos + 1) & mask;
    }
}

constexpr u32 kBlockCap = 4096;  // members of a block-level table held in shared memory
constexpr u32 kTeamCap = 1024;   // members of a team-level table (256-thread blocks, several per SM)

template <int KW, bool CPLX, u32 CAP = kBlockCap>
constexpr size_t block_table_bytes() {
    return (size_t)KW * CAP * 8 + CAP * 8 * (CPLX ? 2 : 1) + 2 * CAP * 4 + 16;
}

// One member of a block-level group at gate t of the batch: pairs it with its
// partner K = Q * P_t when K is a member that existed before the gate (the
// lower index of the two does the update), or creates K (index cnt0 + the
// gate's creation count *ctr) when the degree filter admits it; the
// reference's arithmetic, filter and creation rule (src/pauli/propagate.h:71-89).
// UNIT: the gate's |sin theta| is 1 (partners by sign flip, rot_partner_unit).
template <int NW, bool CPLX, bool SM, bool REC, bool UNIT>
__device__ __forceinline__ void big_member(const BigRegion<2 * NW, CPLX>& G, u32 rcap, u32 m, u32 cnt0, int t,
                                           const BatchGate& Gt, double gc, double gs, const OrbitBatchArgs& a,
                                           u32* ctr, u32& g_emits, u32& g_created, u32& g_xapps) {
    constexpr int KW = 2 * NW;
    auto partner = [&](cplx b, int j) {
        return UNIT ? rot_partner_unit<CPLX>(b, gs, j) : rot_partner<CPLX>(b, gs, j);
    };
    u64 q[KW], k[KW];
#pragma unroll
    for (int w = 0; w < KW; w++) {
        q[w] = tld<SM>(&G.key[(u64)w * rcap + m]);
        k[w] = q[w] ^ Gt.p[w];
    }
    int yQ = 0, yK = 0, zxQ = 0, zxK = 0, dQ = 0, dK = 0;
#pragma unroll
    for (int w = 0; w < NW; w++) {
        yQ += __popcll(q[w] & q[NW + w]);
        yK += __popcll(k[w] & k[NW + w]);
        zxQ += __popcll(Gt.p[NW + w] & q[w]);
        zxK += __popcll(Gt.p[NW + w] & k[w]);
        dQ += __popcll(q[w] | q[NW + w]);
        dK += __popcll(k[w] | k[NW + w]);
    }
    const int jQ = Gt.yP + yQ + 2 * zxQ - yK;
    const int jK = Gt.yP + yK + 2 * zxK - yQ;
    const cplx ci = {tld<SM>(&G.re[m]), CPLX ? tld<SM>(&G.im[m]) : 0.0};
    const u64 hk = tab_hash<KW>(k);
    const int j = big_find<KW, CPLX, SM, SM>(G, rcap, k, hk);
    if (j >= 0 && (u32)j < cnt0) {
        if ((u32)j < m) return;
        const cplx cj = {tld<SM>(&G.re[j]), CPLX ? tld<SM>(&G.im[j]) : 0.0};
        cplx ni = rot_keep<CPLX>(ci, gc), nj = rot_keep<CPLX>(cj, gc);
        if (dQ <= a.maxdeg) ni = rot_add<CPLX>(ni, partner(cj, jK));
        else if (REC && a.cap && dQ <= a.cap->maxdeg)
            capture_drop<NW, CPLX>(*a.cap, q, partner(cj, jK), Gt.gidx);
        if (dK <= a.maxdeg) nj = rot_add<CPLX>(nj, partner(ci, jQ));
        else if (REC && a.cap && dK <= a.cap->maxdeg)
            capture_drop<NW, CPLX>(*a.cap, k, partner(ci, jQ), Gt.gidx);
        g_emits += (dQ <= a.maxdeg) + (dK <= a.maxdeg);
        G.re[m] = ni.re;
        G.re[j] = nj.re;
        if (CPLX) {
            G.im[m] = ni.im;
            G.im[j] = nj.im;
        }
    } else {
        const cplx ni = rot_keep<CPLX>(ci, gc);
        G.re[m] = ni.re;
        if (CPLX) G.im[m] = ni.im;
        if (dK <= a.maxdeg) {
            g_emits++;
            const cplx nv = rot_new<CPLX>(partner(ci, jQ));
            const u32 idx = cnt0 + warp_reserve(ctr);
            if (idx >= rcap) {
                atomicExch(G.flag, 1u);
            } else {
#pragma unroll
                for (int w = 0; w < KW; w++) G.key[(u64)w * rcap + idx] = k[w];
                G.re[idx] = nv.re;
                if (CPLX) G.im[idx] = nv.im;
                __threadfence_block();
                big_insert<KW, CPLX, SM>(G, rcap, idx, hk);
                g_created++;
                g_xapps += a.k - 1 - t;
            }
        } else if (REC && a.cap && dK <= a.cap->maxdeg) {
            capture_drop<NW, CPLX>(*a.cap, k, partner(ci, jQ), Gt.gidx);
        }
    }
}


// Block-level group processing with TB threads per block.  SM: the table lives
// in dynamic shared memory (CAP members); otherwise in the block's
// global-memory region of bp.
template <int NW, bool CPLX, bool SM, int TB = 1024, u32 CAP = kBlockCap, bool REC = false>
__global__ void __launch_bounds__(TB, TB <= 256 ? 4 : 1) orbit_process_big(StoreView in, StoreView out, OrbitScratch sc,
                                                          OrbitCounters* oc, OrbitBatchArgs a, BigPool bp,
                                                          const u32* list, u32 nlist, const u32* nlist_dev) {
    wait_prior_grid();
    constexpr int KW = 2 * NW;
    static_assert(!SM || CAP <= (1u << kFpShift), "member indexes of a shared-memory table fit beside the fingerprint");
    __shared__ long long red[3][32];
    __shared__ u32 big_cr[3];  // members created by a gate (ring of three)
    extern __shared__ __align__(16) unsigned char btab[];
    if (*(volatile u32*)&oc->skip) return;
    if (nlist_dev) nlist = *(volatile const u32*)nlist_dev;  // list length written by an earlier kernel
    long long emits = 0, created = 0, xapps = 0;
    // Groups differ in cost by orders of magnitude: after its first group a
    // block takes the next unclaimed one (bp.fetch) rather than striding.
    __shared__ u32 big_next;
    auto next_group = [&](u32 g) -> u32 {
        if (!bp.fetch) return g + gridDim.x;
        __syncthreads();
        if (threadIdx.x == 0) big_next = gridDim.x + atomicAdd(bp.fetch, 1u);
        __syncthreads();
        return big_next;
    };
    for (u32 gi = blockIdx.x; gi < nlist; gi = next_group(gi)) {
        OCHK(gi < sc.cap_in, 8, gi, nlist, 0)
        const u32 rep = list[gi];
        OCHK(rep < sc.cap_in, 9, rep, gi, nlist)
        BigRegion<KW, CPLX> G;
        u32 rcap;
        if (SM) {
            rcap = CAP;
            char* p = (char*)btab;
            G.key = (u64*)p;
            p += (size_t)KW * CAP * 8;
            G.re = (double*)p;
            p += CAP * 8;
            G.im = (double*)p;
            if (CPLX) p += CAP * 8;
            G.slot = (u32*)p;
            p += 2 * CAP * 4;
            G.cnt = (u32*)p;
            G.flag = G.cnt + 1;
        } else {
            G = big_region<KW, CPLX>(bp, blockIdx.x);
            rcap = bp.rcap;
        }
        const u32 m0 = sc.cnt[rep];
        const u32 base = sc.off[rep];
        for (u32 s2 = threadIdx.x; s2 < 2 * rcap; s2 += blockDim.x) G.slot[s2] = 0xffffffffu;
        if (threadIdx.x == 0) {
            *G.cnt = m0;
            *G.flag = m0 > rcap ? 1u : 0u;
            big_cr[0] = 0;
        }
        __syncthreads();
        if (*(volatile u32*)G.flag) {
            if (threadIdx.x == 0) bp.retry[atomicAdd(bp.nretry, 1u)] = rep;
            __syncthreads();
            continue;
        }
        for (u32 m = threadIdx.x; m < m0; m += blockDim.x) {
            OCHK((u64)base + m < sc.cap_in, 1, base, m, rep)
            OCHK(m < rcap, 3, m, rcap, rep)
            const u64 pm = (u64)base + m;
            u64 k[KW];
#pragma unroll
            for (int w = 0; w < KW; w++) {
                k[w] = sc.gkey[(u64)w * sc.cap_in + pm];
                G.key[(u64)w * rcap + m] = k[w];
            }
            G.re[m] = sc.gcoef[pm];
            if (CPLX) G.im[m] = sc.gcoef[sc.cap_in + pm];
            __threadfence_block();
            big_insert<KW, CPLX, SM>(G, rcap, m, tab_hash<KW>(k));
        }
        __syncthreads();
        u32 g_emits = 0, g_created = 0, g_xapps = 0;  // this thread, this group
        const u32 inst = group_instance(in, a, rep);
        const u64* A = sc.amask + rep;  // word w of the group's gate set at A[w * cap_in]
        u32 cnt0 = m0;   // members before the current gate (the same in every thread)
        // Gates in order, every thread, one block barrier per gate.  Creations
        // of gate i count in big_cr[i % 3]; the slot of gate i + 1 is cleared
        // during gate i (its last readers passed the barrier of gate i - 1).
        {
            int gi = 0;
            bool stop = *(volatile u32*)G.flag != 0;
            for (int wd = 0; wd < kAW && !stop; wd++) {
                u64 bits = A[(u64)wd * sc.cap_in];
                while (bits && !stop) {
                    const int t = 64 * wd + __ffsll((long long)bits) - 1;
                    bits &= bits - 1;
                    u32* ctr = &big_cr[gi++ % 3];
                    if (threadIdx.x == 0) big_cr[gi % 3] = 0;
                    const BatchGate Gt = a.gates[t];
                    double gc, gs;
                    gate_cs(a, Gt, t, inst, gc, gs);
                    if (!CPLX && unit_sine(gs)) {
                        for (u32 m = threadIdx.x; m < cnt0; m += blockDim.x)
                            big_member<NW, CPLX, SM, REC, true>(G, rcap, m, cnt0, t, Gt, gc, gs, a, ctr, g_emits,
                                                                 g_created, g_xapps);
                    } else {
                        for (u32 m = threadIdx.x; m < cnt0; m += blockDim.x)
                            big_member<NW, CPLX, SM, REC, false>(G, rcap, m, cnt0, t, Gt, gc, gs, a, ctr, g_emits,
                                                                  g_created, g_xapps);
                    }
                    __syncthreads();
                    cnt0 += *(volatile u32*)ctr;
                    stop = *(volatile u32*)G.flag != 0;
                }
            }
        }
        __syncthreads();
        if (*(volatile u32*)G.flag) {
            if (threadIdx.x == 0) bp.retry[atomicAdd(bp.nretry, 1u)] = rep;
            __syncthreads();
            continue;
        }
        emits += g_emits;
        created += g_created;
        xapps += g_xapps;
        const u32 cnt = cnt0;
        if (threadIdx.x == 0) {
            atomicMax(&oc->max_members, cnt);
            atomicAdd(&oc->hist[31 - __clz(cnt | 1)], 1u);
            int na = 0;
            for (int w = 0; w < kAW; w++) na += __popcll(sc.amask[(u64)w * sc.cap_in + rep]);
            atomicAdd(&oc->hist_a[na < 15 ? na : 15], 1u);
        }
        for (u32 m = threadIdx.x; m < cnt; m += blockDim.x) {
            OCHK(m < rcap, 7, m, cnt, rcap)
            u64 k[KW];
#pragma unroll
            for (int w = 0; w < KW; w++) k[w] = tld<SM>(&G.key[(u64)w * rcap + m]);
            const cplx c = {tld<SM>(&G.re[m]), CPLX ? tld<SM>(&G.im[m]) : 0.0};
            out_append_warp<KW, CPLX>(out, oc, k, c, survives<NW, CPLX>(k, c, a));
        }
        __syncthreads();
    }
    // block totals
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        emits += __shfl_down_sync(0xffffffffu, emits, o);
        created += __shfl_down_sync(0xffffffffu, created, o);
        xapps += __shfl_down_sync(0xffffffffu, xapps, o);
    }
    if (lane == 0) {
        red[0][wid] = emits;
        red[1][wid] = created;
        red[2][wid] = xapps;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long e = 0, c = 0, x = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            e += red[0][w];
            c += red[1][w];
            x += red[2][w];
        }
        if (e) atomicAdd(&oc->emits, (u64)e);
        if (c) atomicAdd(&oc->created, (u64)c);
        if (x) atomicAdd(&oc->xapps, (u64)x);
    }
}

}  // namespace ffg
