// Batch-orbit processing of a run of mutually commuting Majorana rotations
// with the reference's threshold after every gate
// (src/majorana_propagation.h:18-33, src/majorana_gates.h:67-103).
//
// The commutation form of Majorana strings, |a||b| - |a & b| mod 2, is
// bilinear over GF(2) (|a ^ c| = |a| + |c| and |(a ^ c) & b| = |a & b| + |c & b|
// mod 2), so within a commuting run a string Q and every Q * G_t (t in A(Q))
// anticommute with the same gates, exactly as for Pauli strings.  Terms are
// grouped by (A, Q & ~U_A) and every group is processed on its own, gate by
// gate in run order, with the reference's per-gate arithmetic:
//     c_Q' = c_Q cos + [deg Q <= W] (c_K F) s_K     (F = i i^r sin, s = merge sign)
// and after each gate every member with |c| <= tau is removed; a removed
// member that a later gate re-creates starts again from 0 + p.  A gate leaves
// the terms it commutes with unchanged, and a threshold leaves an unchanged
// coefficient that already passed it in place, so processing groups one at
// a time reproduces the gate-by-gate result bit for bit, provided every term
// entering the run has already passed the threshold (the driver applies the
// circuit's first gate with the per-gate kernel, so this holds).
//
// Apps (live terms entering each gate of the run) are counted per term from
// its alive intervals: an untouched term is alive for all k gates; a group
// member alive from gate entry `since` until the gate t after which it is
// removed counts t + 1 - since, or k - since if it survives the run.
#pragma once
#include "ffg_orbit.cuh"

namespace ffg {

struct MBatchGate {
    u64 p[4];      // Majorana string of the gate
    u64 mg[4];     // bit t = parity of #{s in gate : s > t} (merge sign)
    double c;      // cos theta
    double fr, fi; // i * i^r * sin theta
    int odd;       // odd gate degree
    int pad;
};

struct MOrbitArgs {
    const MBatchGate* gates;  // k gates of the run, application order
    int k;
    int maxdeg;               // partner filter (1 << 30: none)
    int thr;                  // threshold after every gate
    double tau;
    int route_big;            // groups with at least this many gates skip the warp tier
    // mode -> gates index of the run when every gate has even degree (null
    // otherwise): an even string anticommutes only with strings that overlap
    // it.  Gates touching mode i are midx[257 + midx[i] .. 257 + midx[i + 1]).
    const u32* midx;
};

template <int KW>
__device__ __forceinline__ bool manti(const u64* q, const u64* p, int odd) {
    u64 par = 0;
#pragma unroll
    for (int w = 0; w < KW; w++) par ^= q[w] & (odd ? ~p[w] : p[w]);
    return __popcll(par) & 1;
}

// A(Q) for every input term and its group key; untouched terms go straight to
// the output (they count k apps each).
template <int KW>
__global__ void __launch_bounds__(kBlock) morbit_classify(StoreView in, StoreView out, OrbitScratch sc,
                                                          OrbitCounters* oc, MOrbitArgs a) {
    wait_prior_grid();
    if (*(volatile u32*)&oc->skip) return;
    const u64 n_in = *(volatile u64*)&oc->n_in;
    const u64 nslots = *(volatile u64*)&oc->gmask + 1;
    __shared__ u64 gp[kMaxBatchGates][KW];
    __shared__ int godd[kMaxBatchGates];
    __shared__ long long sh[kBlock / 32];
    for (int t = threadIdx.x; t < a.k; t += blockDim.x) {
        for (int w = 0; w < KW; w++) gp[t][w] = a.gates[t].p[w];
        godd[t] = a.gates[t].odd;
    }
    __syncthreads();
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < nslots; i += stride) sc.gslots[i] = kEmptySlot;
    long long apps = 0;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n_in; i += stride) {
        u64 q[KW];
        load_key<KW>(in, i, q);
        u64 A[kAW] = {};
        u64 U[KW] = {};
        if (a.midx) {
            // candidates: the gates on the string's modes
#pragma unroll
            for (int ws = 0; ws < KW; ws++) {
                u64 sup = q[ws];
                while (sup) {
                    const int md = 64 * ws + __ffsll((long long)sup) - 1;
                    sup &= sup - 1;
                    const u32 e1 = __ldg(&a.midx[md + 1]);
                    for (u32 e = __ldg(&a.midx[md]); e < e1; e++) {
                        const int t = (int)__ldg(&a.midx[257 + e]);
                        if ((A[t >> 6] >> (t & 63)) & 1ull) continue;
                        if (manti<KW>(q, gp[t], 0)) {
                            A[t >> 6] |= 1ull << (t & 63);
#pragma unroll
                            for (int w = 0; w < KW; w++) U[w] |= gp[t][w];
                        }
                    }
                }
            }
        } else {
            for (int t = 0; t < a.k; t++) {
                if (manti<KW>(q, gp[t], godd[t])) {
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
            const cplx c = load_coef<true>(in, i);
            apps += a.k;
            out_append_warp<KW, true>(out, oc, q, c, !a.thr || !abs_le(c.re, c.im, a.tau));
            continue;
        }
#pragma unroll
        for (int w = 0; w < kAW; w++) sc.amask[(u64)w * sc.cap_in + i] = A[w];
#pragma unroll
        for (int w = 0; w < KW; w++) sc.gkey[(u64)w * sc.cap_in + i] = q[w] & ~U[w];
        sc.cnt[i] = 0;
        sc.fill[i] = 0;
        sc.rep[i] = 0xfffffffeu;
    }
    const long long tot = block_sum_ll(apps, sh);
    if (threadIdx.x == 0 && tot) atomicAdd(&oc->xapps, (u64)tot);
}

// Member table of one group (shared or global memory).
template <int KW>
struct MTable {
    u64* key;             // [KW][cap]
    double* re;           // [cap]
    double* im;           // [cap]
    u32* slot;            // [2 cap], 0xffffffff = empty
    u32* cnt;
    u32* flag;
    unsigned short* since;  // gate entry from which the member is alive
    unsigned char* st;    // bit 0: alive at gate start; bit 1: created by this gate
    u32 cap;
    u32 mask;             // index slots in use - 1 (a power of two minus one, < 2 cap)
};

template <int KW>
__host__ __device__ constexpr size_t mtable_bytes(u32 cap) {
    return ((size_t)KW * cap * 8 + (size_t)2 * cap * 8 + (size_t)2 * cap * 4 + 8 + (size_t)cap * 2 + cap + 255) &
           ~(size_t)255;
}

template <int KW>
__device__ __forceinline__ MTable<KW> mcarve(char* p, u32 cap) {
    MTable<KW> T;
    T.cap = cap;
    T.key = (u64*)p;
    p += (size_t)KW * cap * 8;
    T.re = (double*)p;
    p += (size_t)cap * 8;
    T.im = (double*)p;
    p += (size_t)cap * 8;
    T.slot = (u32*)p;
    p += (size_t)2 * cap * 4;
    T.cnt = (u32*)p;
    T.flag = T.cnt + 1;
    p += 8;
    T.since = (unsigned short*)p;
    p += (size_t)cap * 2;
    T.st = (unsigned char*)p;
    T.mask = 2 * cap - 1;
    return T;
}

template <int KW>
__device__ __forceinline__ int mfind(const MTable<KW>& T, const u64* k) {
    const u32 mask = T.mask;
    u32 pos = small_hash<KW>(k) & mask;
    for (u32 probe = 0; probe <= mask; probe++) {
        const u32 m = *(volatile u32*)&T.slot[pos];
        if (m == 0xffffffffu) return -1;
        bool eq = true;
#pragma unroll
        for (int w = 0; w < KW; w++) eq = eq && *(volatile u64*)&T.key[(u64)w * T.cap + m] == k[w];
        if (eq) return (int)m;
        pos = (pos + 1) & mask;
    }
    return -1;
}

template <int KW>
__device__ __forceinline__ void minsert(const MTable<KW>& T, const u64* k, u32 m) {
    const u32 mask = T.mask;
    u32 pos = small_hash<KW>(k) & mask;
    for (u32 probe = 0; probe <= mask; probe++) {
        if (atomicCAS(&T.slot[pos], 0xffffffffu, m) == 0xffffffffu) return;
        pos = (pos + 1) & mask;
    }
    atomicExch(T.flag, 1u);  // index full: the group goes to the next tier
}

// Processes the group represented by input position rep with TEAM threads.
// Returns false, with nothing written, when the group outgrew the table.
template <int KW, int TEAM>
__device__ bool mgroup(const StoreView& in, const StoreView& out, const OrbitScratch& sc, OrbitCounters* oc,
                       const MOrbitArgs& a, const MTable<KW>& T0, u32 rep, int rank, long long& apps,
                       long long& emits) {
    const u32 m0 = sc.cnt[rep];
    const u32 base = sc.off[rep];
    if (m0 > T0.cap) return false;
    u64 Am[kAW];
    int na = 0;
#pragma unroll
    for (int w = 0; w < kAW; w++) {
        Am[w] = sc.amask[(u64)w * sc.cap_in + rep];
        na += __popcll(Am[w]);
    }
    // index sized for the orbit bound m0 * 2^|A| at half load (at most 2 cap slots)
    MTable<KW> T = T0;
    {
        u32 slots = 8;
        const u64 bound = na < 24 ? ((u64)m0 << na) : ~0ull;
        while ((u64)slots < 2 * bound && slots < 2 * T.cap) slots <<= 1;
        T.mask = slots - 1;
    }
    for (u32 s2 = rank; s2 <= T.mask; s2 += TEAM) T.slot[s2] = 0xffffffffu;
    if (rank == 0) {
        *T.cnt = m0;
        *T.flag = 0;
    }
    team_sync<TEAM>();
    for (u32 m = rank; m < m0; m += TEAM) {
        const u64 pm = (u64)base + m;
        u64 k[KW];
#pragma unroll
        for (int w = 0; w < KW; w++) {
            k[w] = sc.gkey[(u64)w * sc.cap_in + pm];
            T.key[(u64)w * T.cap + m] = k[w];
        }
        T.re[m] = sc.gcoef[pm];
        T.im[m] = sc.gcoef[sc.cap_in + pm];
        T.st[m] = 1;
        T.since[m] = 0;
        __threadfence_block();
        minsert<KW>(T, k, m);
    }
    team_sync<TEAM>();
    if (*(volatile u32*)T.flag) return false;
    long long g_apps = 0, g_emits = 0;
    for (int wd = 0; wd < kAW; wd++) {
        u64 bits = Am[wd];
        while (bits) {
            const int t = 64 * wd + __ffsll((long long)bits) - 1;
            bits &= bits - 1;
            const MBatchGate& G = a.gates[t];
            u64 P[KW], MG[KW];
#pragma unroll
            for (int w = 0; w < KW; w++) {
                P[w] = G.p[w];
                MG[w] = G.mg[w];
            }
            const double gc = G.c;
            const cplx F = {G.fr, G.fi};
            const u32 cnt0 = *(volatile u32*)T.cnt;
            for (u32 m = rank; m < cnt0; m += TEAM) {
                if (!(*(volatile unsigned char*)&T.st[m] & 1)) continue;  // not alive at gate start
                u64 q[KW], k[KW];
                int dQ = 0, dK = 0, mQ = 0, mK = 0;
#pragma unroll
                for (int w = 0; w < KW; w++) {
                    q[w] = T.key[(u64)w * T.cap + m];
                    k[w] = q[w] ^ P[w];
                    dQ += __popcll(q[w]);
                    dK += __popcll(k[w]);
                    mQ += __popcll(q[w] & MG[w]);
                    mK += __popcll(k[w] & MG[w]);
                }
                const cplx sQ = {(mQ & 1) ? -1.0 : 1.0, 0.0};
                const cplx sK = {(mK & 1) ? -1.0 : 1.0, 0.0};
                const cplx ci = {T.re[m], T.im[m]};
                const int j = mfind<KW>(T, k);
                const bool jal = j >= 0 && (u32)j < cnt0 && (*(volatile unsigned char*)&T.st[j] & 1);
                if (jal) {
                    if ((u32)j < m) continue;  // the pair belongs to member j
                    const cplx cj = {T.re[j], T.im[j]};
                    cplx ni = cscale(ci, gc), nj = cscale(cj, gc);
                    if (dQ <= a.maxdeg) ni = cadd(ni, cmul(cmul(cj, F), sK));
                    if (dK <= a.maxdeg) nj = cadd(nj, cmul(cmul(ci, F), sQ));
                    g_emits += (dQ <= a.maxdeg) + (dK <= a.maxdeg);
                    T.re[m] = ni.re;
                    T.im[m] = ni.im;
                    T.re[j] = nj.re;
                    T.im[j] = nj.im;
                } else {
                    const cplx ni = cscale(ci, gc);
                    T.re[m] = ni.re;
                    T.im[m] = ni.im;
                    if (dK <= a.maxdeg) {
                        g_emits++;
                        const cplx nv = cadd({0.0, 0.0}, cmul(cmul(ci, F), sQ));
                        if (j >= 0) {
                            // removed by an earlier threshold: re-created from zero
                            T.re[j] = nv.re;
                            T.im[j] = nv.im;
                            T.st[j] = 2;
                        } else {
                            const u32 idx = warp_reserve(T.cnt);
                            if (idx >= T.cap) {
                                atomicExch(T.flag, 1u);
                            } else {
#pragma unroll
                                for (int w = 0; w < KW; w++) T.key[(u64)w * T.cap + idx] = k[w];
                                T.re[idx] = nv.re;
                                T.im[idx] = nv.im;
                                T.st[idx] = 2;
                                __threadfence_block();
                                minsert<KW>(T, k, idx);
                            }
                        }
                    }
                }
            }
            team_sync<TEAM>();
            if (*(volatile u32*)T.flag) return false;
            // threshold after the gate; alive intervals for the apps count
            const u32 cnt1 = *(volatile u32*)T.cnt;
            for (u32 m = rank; m < cnt1; m += TEAM) {
                const unsigned char s = T.st[m];
                if (!s) continue;
                const bool keep = !a.thr || !abs_le(T.re[m], T.im[m], a.tau);
                if (s & 1) {
                    if (!keep) {
                        g_apps += (long long)(t + 1) - T.since[m];
                        T.st[m] = 0;
                    }
                } else {
                    if (keep) {
                        T.since[m] = (unsigned short)(t + 1);
                        T.st[m] = 1;
                    } else {
                        T.st[m] = 0;
                    }
                }
            }
            team_sync<TEAM>();
        }
    }
    const u32 cnt = *(volatile u32*)T.cnt;
    for (u32 m = rank; m < cnt; m += TEAM) {
        const bool live = (T.st[m] & 1) != 0;
        if (live) g_apps += (long long)a.k - T.since[m];
        u64 k[KW];
#pragma unroll
        for (int w = 0; w < KW; w++) k[w] = T.key[(u64)w * T.cap + m];
        out_append_warp<KW, true>(out, oc, k, cplx{T.re[m], T.im[m]}, live);
    }
    team_sync<TEAM>();
    apps += g_apps;
    emits += g_emits;
    return true;
}

// Thread tier: groups acted on by a single gate of the run (|A| = 1) whose
// input members are one term Q, or the pair Q, Q*G: one butterfly (or one
// partner creation), the threshold and the apps bookkeeping in registers.
// Every other group is listed in sc.fill (count oc->nrest) for the warp tier.
template <int KW>
__global__ void __launch_bounds__(kBlock) morbit_single(StoreView in, StoreView out, OrbitScratch sc,
                                                        OrbitCounters* oc, MOrbitArgs a) {
    wait_prior_grid();
    if (*(volatile u32*)&oc->skip) return;
    const u32 ng = *(volatile u32*)&oc->ngroups;
    __shared__ long long sh[kBlock / 32];
    long long apps = 0, emits = 0;
    const u32 stride = gridDim.x * blockDim.x;
    for (u32 g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += stride) {
        const u32 rep = sc.groups[g];
        const u32 m0 = sc.cnt[rep];
        int na = 0, t = -1;
#pragma unroll
        for (int w = 0; w < kAW; w++) {
            const u64 am = sc.amask[(u64)w * sc.cap_in + rep];
            na += __popcll(am);
            if (am && t < 0) t = 64 * w + __ffsll((long long)am) - 1;
        }
        bool simple = na == 1 && m0 <= 2;
        u64 q0[KW], q1[KW];
        u64 i0 = 0, i1 = 0;  // positions in group order (sc.gkey / sc.gcoef)
        const MBatchGate& G = a.gates[t < 0 ? 0 : t];
        if (simple) {
            const u32 base = sc.off[rep];
            i0 = base;
#pragma unroll
            for (int w = 0; w < KW; w++) q0[w] = sc.gkey[(u64)w * sc.cap_in + i0];
            if (m0 == 2) {
                i1 = (u64)base + 1;
#pragma unroll
                for (int w = 0; w < KW; w++) q1[w] = sc.gkey[(u64)w * sc.cap_in + i1];
#pragma unroll
                for (int w = 0; w < KW; w++) simple = simple && (q1[w] == (q0[w] ^ G.p[w]));
            }
        }
        if (!simple) {
            sc.fill[atomicAdd(&oc->nrest, 1u)] = rep;
            continue;
        }
        // members: Q = q0, K = q0 ^ p (present when m0 == 2)
        u64 k[KW];
        int dQ = 0, dK = 0, mQ = 0, mK = 0;
#pragma unroll
        for (int w = 0; w < KW; w++) {
            k[w] = q0[w] ^ G.p[w];
            dQ += __popcll(q0[w]);
            dK += __popcll(k[w]);
            mQ += __popcll(q0[w] & G.mg[w]);
            mK += __popcll(k[w] & G.mg[w]);
        }
        const cplx sQ = {(mQ & 1) ? -1.0 : 1.0, 0.0};
        const cplx sK = {(mK & 1) ? -1.0 : 1.0, 0.0};
        const cplx F = {G.fr, G.fi};
        const cplx cq = {sc.gcoef[i0], sc.gcoef[sc.cap_in + i0]};
        cplx nq, nk;
        bool has_k;
        if (m0 == 2) {
            const cplx ck = {sc.gcoef[i1], sc.gcoef[sc.cap_in + i1]};
            nq = cscale(cq, G.c);
            nk = cscale(ck, G.c);
            if (dQ <= a.maxdeg) nq = cadd(nq, cmul(cmul(ck, F), sK));
            if (dK <= a.maxdeg) nk = cadd(nk, cmul(cmul(cq, F), sQ));
            emits += (dQ <= a.maxdeg) + (dK <= a.maxdeg);
            has_k = true;
        } else {
            nq = cscale(cq, G.c);
            has_k = dK <= a.maxdeg;
            if (has_k) {
                nk = cadd({0.0, 0.0}, cmul(cmul(cq, F), sQ));
                emits++;
            }
        }
        // threshold after the gate; apps: inputs alive for entries [0, t], a
        // created member from t + 1, survivors until the end of the run
        const bool kq = !a.thr || !abs_le(nq.re, nq.im, a.tau);
        apps += kq ? a.k : t + 1;
        out_append_warp<KW, true>(out, oc, q0, nq, kq);
        if (has_k) {
            const bool kk = !a.thr || !abs_le(nk.re, nk.im, a.tau);
            if (m0 == 2)
                apps += kk ? a.k : t + 1;
            else if (kk)
                apps += a.k - (t + 1);
            out_append_warp<KW, true>(out, oc, k, nk, kk);
        }
    }
    long long tot = block_sum_ll(apps, sh);
    if (threadIdx.x == 0 && tot) atomicAdd(&oc->xapps, (u64)tot);
    tot = block_sum_ll(emits, sh);
    if (threadIdx.x == 0 && tot) atomicAdd(&oc->emits, (u64)tot);
}

constexpr u32 kMSubCap = 64;      // sub-warp tier: members per group table
constexpr int kMSubLanes = 8;     // sub-warp tier: lanes per group (4 groups per warp)
constexpr int kMSubWarps = 8;     // sub-warp tier: warps per block

// Sub-warp tier: 8 lanes per group, 64-member tables in shared memory, for the
// groups whose orbit bound m0 * 2^|A| is at most 64 (they cannot outgrow the
// table); the others go to sc.list2 for the warp tier.
template <int KW>
__global__ void __launch_bounds__(32 * kMSubWarps, 2) morbit_sub(StoreView in, StoreView out, OrbitScratch sc,
                                                            OrbitCounters* oc, MOrbitArgs a) {
    wait_prior_grid();
    extern __shared__ __align__(16) unsigned char msm[];
    if (*(volatile u32*)&oc->skip) return;
    constexpr int kTeams = 32 * kMSubWarps / kMSubLanes;
    const int team = threadIdx.x / kMSubLanes, rank = threadIdx.x % kMSubLanes;
    const MTable<KW> T = mcarve<KW>((char*)msm + team * mtable_bytes<KW>(kMSubCap), kMSubCap);
    const u32 ng = *(volatile u32*)&oc->nrest;  // groups left by morbit_single, listed in sc.fill
    long long apps = 0, emits = 0;
    for (u32 g = blockIdx.x * kTeams + team; g < ng; g += gridDim.x * kTeams) {
        const u32 rep = sc.fill[g];
        int na = 0;
#pragma unroll
        for (int w = 0; w < kAW; w++) na += __popcll(sc.amask[(u64)w * sc.cap_in + rep]);
        const u32 m0 = sc.cnt[rep];
        bool done = false;
        if (na < 7 && ((u64)m0 << na) <= kMSubCap)
            done = mgroup<KW, kMSubLanes>(in, out, sc, oc, a, T, rep, rank, apps, emits);
        if (!done && rank == 0) sc.list2[atomicAdd(&oc->nrest2, 1u)] = rep;
        team_sync<kMSubLanes>();
    }
    for (int o = 16; o > 0; o >>= 1) {
        apps += __shfl_down_sync(0xffffffffu, apps, o);
        emits += __shfl_down_sync(0xffffffffu, emits, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (apps) atomicAdd(&oc->xapps, (u64)apps);
        if (emits) atomicAdd(&oc->emits, (u64)emits);
    }
}

constexpr u32 kMWarpCap = 256;    // warp tier: members per group table
constexpr int kMWarps = 8;        // warp tier: groups per block
constexpr u32 kMTeamCap = 1024;   // team tier (256 threads)

// Warp tier: one warp per group, tables in shared memory; groups that do not
// fit (or have route_big or more gates) are listed in sc.big.
template <int KW>
__global__ void __launch_bounds__(32 * kMWarps, 2) morbit_warp(StoreView in, StoreView out, OrbitScratch sc,
                                                          OrbitCounters* oc, MOrbitArgs a) {
    wait_prior_grid();
    extern __shared__ __align__(16) unsigned char msm[];
    if (*(volatile u32*)&oc->skip) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const MTable<KW> T = mcarve<KW>((char*)msm + warp * mtable_bytes<KW>(kMWarpCap), kMWarpCap);
    const u32 ng = *(volatile u32*)&oc->nrest2;  // groups left by morbit_sub, listed in sc.list2
    long long apps = 0, emits = 0;
    for (u32 g = blockIdx.x * kMWarps + warp; g < ng; g += gridDim.x * kMWarps) {
        const u32 rep = sc.list2[g];
        int na = 0;
#pragma unroll
        for (int w = 0; w < kAW; w++) na += __popcll(sc.amask[(u64)w * sc.cap_in + rep]);
        bool done = false;
        if (na < a.route_big && sc.cnt[rep] <= kMWarpCap)
            done = mgroup<KW, 32>(in, out, sc, oc, a, T, rep, lane, apps, emits);
        if (!done && lane == 0) sc.big[atomicAdd(&oc->nbig, 1u)] = rep;
        __syncwarp();
    }
    for (int o = 16; o > 0; o >>= 1) {
        apps += __shfl_down_sync(0xffffffffu, apps, o);
        emits += __shfl_down_sync(0xffffffffu, emits, o);
    }
    if (lane == 0) {
        if (apps) atomicAdd(&oc->xapps, (u64)apps);
        if (emits) atomicAdd(&oc->emits, (u64)emits);
    }
}

// Team / block tiers: one block of TB threads per group, table of `cap`
// members in dynamic shared memory (SM) or in the block's region of `pool`;
// groups that outgrow it go to `retry`.  The list length is read from
// nlist_dev when given.
template <int KW, int TB, bool SM>
__global__ void __launch_bounds__(TB) morbit_block(StoreView in, StoreView out, OrbitScratch sc, OrbitCounters* oc,
                                                   MOrbitArgs a, u32 cap, char* pool, u64 region_bytes,
                                                   const u32* list, u32 nlist, const u32* nlist_dev, u32* retry,
                                                   u32* nretry) {
    wait_prior_grid();
    extern __shared__ __align__(16) unsigned char msm[];
    if (*(volatile u32*)&oc->skip) return;
    if (nlist_dev) nlist = *(volatile const u32*)nlist_dev;
    const MTable<KW> T = mcarve<KW>(SM ? (char*)msm : pool + (u64)blockIdx.x * region_bytes, cap);
    long long apps = 0, emits = 0;
    for (u32 gi = blockIdx.x; gi < nlist; gi += gridDim.x) {
        const u32 rep = list[gi];
        const bool done = mgroup<KW, TB>(in, out, sc, oc, a, T, rep, threadIdx.x, apps, emits);
        if (!done && threadIdx.x == 0) retry[atomicAdd(nretry, 1u)] = rep;
        __syncthreads();
    }
    for (int o = 16; o > 0; o >>= 1) {
        apps += __shfl_down_sync(0xffffffffu, apps, o);
        emits += __shfl_down_sync(0xffffffffu, emits, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (apps) atomicAdd(&oc->xapps, (u64)apps);
        if (emits) atomicAdd(&oc->emits, (u64)emits);
    }
}

}  // namespace ffg
