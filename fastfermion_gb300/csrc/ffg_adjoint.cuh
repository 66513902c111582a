// Batched instances and reverse-mode differentiation of truncated Pauli
// propagation (real coefficients).
//
// Batched instances.  Many observables that go through the same circuit
// structure (same gate axes and Clifford gates, per-instance angles) share one
// term store.  Instance i is written into key bits that no gate touches: the
// binary code of i in x-plane bits [shift, shift+b) and its complement in the
// z-plane bits at the same positions.  Those bits never change anticommutation
// (no gate has them set), never form a Y (x & z is 0 there), and add exactly b
// to every term's weight popc(x | z), so the degree filter runs with
// maxdegree + b and every instance's term set is bit-identical to a
// propagation of that instance alone.  Grouping by (A, Q & ~U_A) keeps the
// instance bits in the group key, so no orbit group mixes instances; the orbit
// kernels read each gate's (cos, sin) per instance.
//
// Adjoint.  With the truncation pattern held fixed, every coefficient after a
// rotation is linear in the coefficients before it:
//     c'_Q = cos c_Q + [deg Q <= W] sin e_KQ c_K          (K = P Q, e = +-1)
// and f = sum over terms with x = 0 of the final coefficients.  The backward
// pass runs the ops in reverse.  For an orbit batch it re-forms the groups of
// the batch's input term set (a checkpoint), replays each group's forward gate
// by gate in the same arithmetic while keeping each member's coefficient
// before every gate (history), then sweeps the gates backward:
//     abar_Q(before) = cos abar_Q(after) + [K exists after, deg K <= W] sin e_QK abar_K(after)
//     dF/dtheta     += abar_Q(after) (-sin c_Q + [K existed, deg Q <= W] cos e_KQ c_K)
//                      (+ abar_K(after) cos e_QK c_Q when K was created by Q)
// A truncated term has abar 0 (it is absent from the next term set).  A
// Clifford segment maps terms 1:1 with a sign, so abar_in = sign abar_out(map(Q)).
#pragma once
#include "ffg_orbit.cuh"

namespace ffg {

constexpr u32 kAdjWarpCap = 256;     // members of a group held in shared memory (warp tier)
constexpr u32 kAdjWarpGates = 9;     // gates of a warp-tier group (history rows in shared memory)
constexpr int kAdjWarps = 3;          // groups in flight per block (warp tier; 3 keeps two blocks per SM)
constexpr unsigned short kInputMember = 0xffff;

// Tables of one group.  Warp tier: in shared memory; block tier: in the block's
// global-memory region.  history[m * na + ti] = coefficient of member m before
// the group's ti-th gate.
template <int KW>
struct AdjTable {
    u64* key;               // [KW][cap]
    u32* slot;              // [2 cap], 0xffffffff = empty
    unsigned short* ct;     // [cap] gate ordinal that created the member (kInputMember)
    double* c;              // [cap] coefficient during the replay
    double* an;             // [cap] abar after the current gate
    double* ao;             // [cap] abar before the current gate
    double* hist;           // [cap * na]
    u32* cnt;
    u32* flag;
    u32 cap;
};

template <int KW>
__host__ __device__ constexpr size_t adj_table_bytes(u32 cap, u32 na) {
    return ((size_t)KW * cap * 8 + (size_t)2 * cap * 4 + (size_t)cap * 2 + 8 + (size_t)3 * cap * 8 +
            (size_t)cap * na * 8 + 255) & ~(size_t)255;
}

template <int KW>
__device__ __forceinline__ AdjTable<KW> adj_carve(char* p, u32 cap, u32 na) {
    AdjTable<KW> T;
    T.cap = cap;
    T.key = (u64*)p;
    p += (size_t)KW * cap * 8;
    T.c = (double*)p;
    p += (size_t)cap * 8;
    T.an = (double*)p;
    p += (size_t)cap * 8;
    T.ao = (double*)p;
    p += (size_t)cap * 8;
    T.hist = (double*)p;
    p += (size_t)cap * na * 8;
    T.slot = (u32*)p;
    p += (size_t)2 * cap * 4;
    T.cnt = (u32*)p;
    T.flag = T.cnt + 1;
    p += 8;
    T.ct = (unsigned short*)p;
    return T;
}

template <int KW>
__device__ __forceinline__ int adj_find(const AdjTable<KW>& T, const u64* k) {
    const u32 mask = 2 * T.cap - 1;
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
__device__ __forceinline__ void adj_insert(const AdjTable<KW>& T, const u64* k, u32 m) {
    const u32 mask = 2 * T.cap - 1;
    u32 pos = small_hash<KW>(k) & mask;
    for (u32 probe = 0; probe <= mask; probe++) {
        if (atomicCAS(&T.slot[pos], 0xffffffffu, m) == 0xffffffffu) return;
        pos = (pos + 1) & mask;
    }
}

struct AdjArgs {
    OrbitBatchArgs a;     // the batch (gates, k, maxdeg, truncation, instances)
    StoreView out;        // term set after the batch (index over its live keys)
    const double* abar_out;
    double* abar_in;      // [n_in]
    double* grad;         // [k][ninst] gradient of the batch's gates
    u32* err;
};

__device__ __forceinline__ double real_factor(int j) {
    // re(i * i^j) for odd j: the real factor of (i sin) * phase in real mode
    return ((j & 3) == 1) ? -1.0 : 1.0;
}

// Processes the group represented by input position rep with TEAM threads
// (rank = this thread's index in the team).  Returns false, with no output
// written, when the group outgrew the table.
template <int NW, int TEAM>
__device__ bool adj_group(const StoreView& in, const OrbitScratch& sc, const AdjArgs& A,
                          const AdjTable<2 * NW>& T, u32 rep, int rank) {
    constexpr int KW = 2 * NW;
    const OrbitBatchArgs& a = A.a;
    const u32 m0 = sc.cnt[rep];
    const u32 base = sc.off[rep];
    u64 Am[kAW];
    int na = 0;
#pragma unroll
    for (int w = 0; w < kAW; w++) {
        Am[w] = sc.amask[(u64)w * sc.cap_in + rep];
        na += __popcll(Am[w]);
    }
    const u32 inst = group_instance(in, a, rep);
    if (m0 > T.cap) return false;
    for (u32 s2 = rank; s2 < 2 * T.cap; s2 += TEAM) T.slot[s2] = 0xffffffffu;
    if (rank == 0) {
        *T.cnt = m0;
        *T.flag = 0;
    }
    team_sync<TEAM>();
    for (u32 m = rank; m < m0; m += TEAM) {
        const u32 i = sc.order[base + m];
        u64 k[KW];
#pragma unroll
        for (int w = 0; w < KW; w++) {
            k[w] = in.key[(u64)w * in.cap + i];
            T.key[(u64)w * T.cap + m] = k[w];
        }
        T.c[m] = in.re[i];
        T.ct[m] = kInputMember;
        __threadfence_block();
        adj_insert<KW>(T, k, m);
    }
    team_sync<TEAM>();
    // ---- forward replay, coefficient history before every gate ----
    int ti = 0;
    for (int wd = 0; wd < kAW; wd++) {
        u64 bits = Am[wd];
        while (bits) {
            const int t = 64 * wd + __ffsll((long long)bits) - 1;
            bits &= bits - 1;
            const BatchGate G = a.gates[t];
            double gc, gs;
            gate_cs(a, G, t, inst, gc, gs);
            const u32 cnt0 = *(volatile u32*)T.cnt;
            for (u32 m = rank; m < cnt0; m += TEAM) T.hist[(u64)m * na + ti] = T.c[m];
            team_sync<TEAM>();
            for (u32 m = rank; m < cnt0; m += TEAM) {
                u64 q[KW], k[KW];
#pragma unroll
                for (int w = 0; w < KW; w++) {
                    q[w] = T.key[(u64)w * T.cap + m];
                    k[w] = q[w] ^ G.p[w];
                }
                int yQ = 0, yK = 0, zxQ = 0, zxK = 0, dQ = 0, dK = 0;
#pragma unroll
                for (int w = 0; w < NW; w++) {
                    yQ += __popcll(q[w] & q[NW + w]);
                    yK += __popcll(k[w] & k[NW + w]);
                    zxQ += __popcll(G.p[NW + w] & q[w]);
                    zxK += __popcll(G.p[NW + w] & k[w]);
                    dQ += __popcll(q[w] | q[NW + w]);
                    dK += __popcll(k[w] | k[NW + w]);
                }
                const int jQ = G.yP + yQ + 2 * zxQ - yK;
                const int jK = G.yP + yK + 2 * zxK - yQ;
                const cplx ci = {T.c[m], 0.0};
                const int j = adj_find<KW>(T, k);
                if (j >= 0 && (u32)j < cnt0) {
                    if ((u32)j < m) continue;  // the pair belongs to member j
                    const cplx cj = {T.c[j], 0.0};
                    cplx ni = rot_keep<false>(ci, gc), nj = rot_keep<false>(cj, gc);
                    if (dQ <= a.maxdeg) ni = rot_add<false>(ni, rot_partner<false>(cj, gs, jK));
                    if (dK <= a.maxdeg) nj = rot_add<false>(nj, rot_partner<false>(ci, gs, jQ));
                    T.c[m] = ni.re;
                    T.c[j] = nj.re;
                } else {
                    T.c[m] = rot_keep<false>(ci, gc).re;
                    if (dK <= a.maxdeg) {
                        const cplx nv = rot_add<false>({0.0, 0.0}, rot_partner<false>(ci, gs, jQ));
                        const u32 idx = warp_reserve(T.cnt);
                        if (idx >= T.cap) {
                            atomicExch(T.flag, 1u);
                        } else {
#pragma unroll
                            for (int w = 0; w < KW; w++) T.key[(u64)w * T.cap + idx] = k[w];
                            T.c[idx] = nv.re;
                            T.ct[idx] = (unsigned short)ti;
                            __threadfence_block();
                            adj_insert<KW>(T, k, idx);
                        }
                    }
                }
            }
            team_sync<TEAM>();
            if (*(volatile u32*)T.flag) return false;
            ti++;
        }
    }
    const u32 cnt = *(volatile u32*)T.cnt;
    // ---- abar after the batch: the member's value in the next term set ----
    for (u32 m = rank; m < cnt; m += TEAM) {
        u64 k[KW];
#pragma unroll
        for (int w = 0; w < KW; w++) k[w] = T.key[(u64)w * T.cap + m];
        const long long pos = lookup<KW>(A.out, k, A.err);
        T.an[m] = pos >= 0 ? A.abar_out[pos] : 0.0;
    }
    team_sync<TEAM>();
    // ---- backward sweep ----
    double* an = T.an;
    double* ao = T.ao;
    for (int tb = na - 1; tb >= 0; tb--) {
        // gate of ordinal tb: the tb-th set bit of Am
        int t = -1;
        {
            int left = tb;
            for (int wd = 0; wd < kAW && t < 0; wd++) {
                u64 bits = Am[wd];
                const int pc = __popcll(bits);
                if (left >= pc) {
                    left -= pc;
                    continue;
                }
                for (int r = 0; r < left; r++) bits &= bits - 1;
                t = 64 * wd + __ffsll((long long)bits) - 1;
            }
        }
        const BatchGate G = a.gates[t];
        double gc, gs;
        gate_cs(a, G, t, inst, gc, gs);
        double gsum = 0.0;
        for (u32 m = rank; m < cnt; m += TEAM) {
            const unsigned short ctm = T.ct[m];
            if (ctm != kInputMember && (int)ctm >= tb) {
                ao[m] = 0.0;  // not present before this gate
                continue;
            }
            u64 q[KW], k[KW];
#pragma unroll
            for (int w = 0; w < KW; w++) {
                q[w] = T.key[(u64)w * T.cap + m];
                k[w] = q[w] ^ G.p[w];
            }
            int yQ = 0, yK = 0, zxQ = 0, zxK = 0, dQ = 0, dK = 0;
#pragma unroll
            for (int w = 0; w < NW; w++) {
                yQ += __popcll(q[w] & q[NW + w]);
                yK += __popcll(k[w] & k[NW + w]);
                zxQ += __popcll(G.p[NW + w] & q[w]);
                zxK += __popcll(G.p[NW + w] & k[w]);
                dQ += __popcll(q[w] | q[NW + w]);
                dK += __popcll(k[w] | k[NW + w]);
            }
            const double eQK = real_factor(G.yP + yQ + 2 * zxQ - yK);  // Q -> K
            const double eKQ = real_factor(G.yP + yK + 2 * zxK - yQ);  // K -> Q
            const int j = adj_find<KW>(T, k);
            const unsigned short ctj = j >= 0 ? T.ct[j] : 0;
            const bool jex = j >= 0 && (ctj == kInputMember || (int)ctj < tb);
            const bool jnew = j >= 0 && (int)ctj == tb;
            const double cm = T.hist[(u64)m * na + tb];
            const double cj = jex ? T.hist[(u64)j * na + tb] : 0.0;
            const double am = an[m];
            const double aj = (jex || jnew) ? an[j] : 0.0;
            double v = gc * am;
            if ((jex || jnew) && dK <= a.maxdeg) v += gs * eQK * aj;
            ao[m] = v;
            double d = -gs * cm;
            if (jex && dQ <= a.maxdeg) d += gc * eKQ * cj;
            gsum += am * d;
            if (jnew) gsum += aj * gc * eQK * cm;
        }
        // team total -> one atomic per warp
        for (int o = 16; o > 0; o >>= 1) gsum += __shfl_down_sync(0xffffffffu, gsum, o);
        if ((rank & 31) == 0 && gsum != 0.0) atomicAdd(&A.grad[(u64)t * a.ninst + inst], gsum);
        team_sync<TEAM>();
        double* tmp = an;
        an = ao;
        ao = tmp;
    }
    // abar before the batch for the input members
    for (u32 m = rank; m < m0; m += TEAM) A.abar_in[sc.order[base + m]] = an[m];
    team_sync<TEAM>();
    return true;
}

// Warp tier: one warp per group, tables in shared memory (groups with at most
// kAdjWarpCap members and fewer than a.route_big gates); other groups are
// listed in sc.big for the block tier.
template <int NW>
__global__ void __launch_bounds__(32 * kAdjWarps) adj_orbit_warp(StoreView in, OrbitScratch sc, OrbitCounters* oc,
                                                                AdjArgs A) {
    constexpr int KW = 2 * NW;
    constexpr u32 na_max = kAdjWarpGates;
    extern __shared__ __align__(16) unsigned char adj_smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t tb = adj_table_bytes<KW>(kAdjWarpCap, na_max);
    const AdjTable<KW> T = adj_carve<KW>((char*)adj_smem + warp * tb, kAdjWarpCap, na_max);
    const u32 ng = *(volatile u32*)&oc->ngroups;
    for (u32 g = blockIdx.x * kAdjWarps + warp; g < ng; g += gridDim.x * kAdjWarps) {
        const u32 rep = sc.groups[g];
        int na = 0;
#pragma unroll
        for (int w = 0; w < kAW; w++) na += __popcll(sc.amask[(u64)w * sc.cap_in + rep]);
        bool done = false;
        if ((u32)na <= na_max && sc.cnt[rep] <= kAdjWarpCap && na < A.a.route_big)
            done = adj_group<NW, 32>(in, sc, A, T, rep, lane);
        if (!done && lane == 0) sc.big[atomicAdd(&oc->nbig, 1u)] = rep;
        __syncwarp();
    }
}

// Block tier: one block per group, tables in the block's region of `pool`
// (region_bytes each, capacity cap); groups that outgrow it go to `retry`.
template <int NW>
__global__ void __launch_bounds__(1024) adj_orbit_block(StoreView in, OrbitScratch sc, AdjArgs A, char* pool,
                                                        u64 region_bytes, u32 cap, u32 na_max, const u32* list,
                                                        u32 nlist, u32* retry, u32* nretry) {
    constexpr int KW = 2 * NW;
    const AdjTable<KW> T = adj_carve<KW>(pool + (u64)blockIdx.x * region_bytes, cap, na_max);
    for (u32 gi = blockIdx.x; gi < nlist; gi += gridDim.x) {
        const u32 rep = list[gi];
        const bool done = adj_group<NW, 1024>(in, sc, A, T, rep, threadIdx.x);
        if (!done && threadIdx.x == 0) retry[atomicAdd(nretry, 1u)] = rep;
        __syncthreads();
    }
}

// Terms that no gate of the batch acts on: abar passes through unchanged
// (0 when the batch-end truncation removed the term).
template <int KW>
__global__ void __launch_bounds__(kBlock) adj_passthrough(StoreView in, u64 n_in, OrbitScratch sc, AdjArgs A) {
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n_in; i += stride) {
        if (sc.rep[i] != 0xffffffffu) continue;
        u64 k[KW];
        load_key<KW>(in, i, k);
        const long long pos = lookup<KW>(A.out, k, A.err);
        A.abar_in[i] = pos >= 0 ? A.abar_out[pos] : 0.0;
    }
}

// Clifford segments: abar_in(Q) = sign(Q) abar_out(map(Q)); the segments in
// `segs` ([begin, end) gate ranges of `ops`) are applied in list order, each
// from its last gate to its first.
template <int NW>
__global__ void __launch_bounds__(kBlock) adj_clifford(StoreView in, u64 n_in, const CliffordOp* ops,
                                                       const int2* segs, int nsegs, StoreView out,
                                                       const double* abar_out, double* abar_in, u32* err) {
    constexpr int KW = 2 * NW;
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n_in; i += stride) {
        u64 x[NW], z[NW];
#pragma unroll
        for (int w = 0; w < NW; w++) {
            x[w] = in.key[(u64)w * in.cap + i];
            z[w] = in.key[(u64)(NW + w) * in.cap + i];
        }
        int flips = 0;
        for (int sgi = 0; sgi < nsegs; sgi++) flips += clifford_map<NW>(x, z, ops + segs[sgi].x, segs[sgi].y - segs[sgi].x);
        u64 k[KW];
#pragma unroll
        for (int w = 0; w < NW; w++) {
            k[w] = x[w];
            k[NW + w] = z[w];
        }
        const long long pos = lookup<KW>(out, k, err);
        const double v = pos >= 0 ? abar_out[pos] : 0.0;
        abar_in[i] = (flips & 1) ? -v : v;
    }
}

// Index over the first n entries of a dense term set (no dead entries).
template <int KW>
__global__ void __launch_bounds__(kBlock) adj_index(StoreView s, u64 n, u32* err) {
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        u64 k[KW];
        load_key<KW>(s, i, k);
        insert<KW>(s, k, (u32)i, err, true);
    }
}

// Per-instance <0|O|0> of the final term set and the initial abar of a
// weighted sum of them: terms whose x planes (without the instance bits) are
// zero.  xmask[w] selects the qubit bits of x plane w.
template <int NW>
__global__ void __launch_bounds__(kBlock) batch_expect(StoreView s, u64 n, u64 xm0, u64 xm1, int inst_plane,
                                                       int inst_shift, u64 inst_mask, double* expect,
                                                       const double* weights, double* abar) {
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const u64 x0 = s.key[i] & xm0;
        const u64 x1 = NW > 1 ? (s.key[s.cap + i] & xm1) : 0;
        const u32 inst = (u32)((s.key[(u64)inst_plane * s.cap + i] >> inst_shift) & inst_mask);
        const bool zero = (x0 | x1) == 0;
        if (expect && zero) atomicAdd(&expect[inst], s.re[i]);
        if (abar) abar[i] = zero ? weights[inst] : 0.0;
    }
}

}  // namespace ffg
