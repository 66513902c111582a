// Internal header of libffg's host engine: the context, result and batch
// objects behind the C ABI, term-store memory, the propagation schedule and
// the runners that launch the kernels.  Each translation unit of the C ABI
// (ffg_engine.cu: context, results, options; ffg_pauli.cu; ffg_majorana.cu;
// ffg_batch.cu; ffg_convert.cu) includes it and instantiates the runners it
// uses.
//
// Host engine of libffg: term-store memory, the propagation schedule and the
// C ABI declared in include/ffg.h.
//
// Schedule (src/pauli/propagate.h:297-493): the circuit is walked last gate
// first; consecutive Clifford gates form a segment applied term by term;
// rotations are buffered and split greedily into maximal runs of mutually
// commuting axes (batch_commuting_gates, :272-291); truncation runs after each
// run (batched) or after each rotation (unbatched) with the reference's
// rot_count bookkeeping for the X-weight period.  Majorana circuits apply
// every gate last to first with a threshold after each gate
// (src/majorana_propagation.h:18-33).
//
// The schedule is turned into a flat op list once; ops are enqueued on the
// context stream in chunks without host round trips (kernels agree on the
// store size through device counters).  After each chunk the host reads the
// counters once: a rotation that found the store too small set the overflow
// flag and every later op of the chunk skipped itself, so the host grows the
// store and replays from that op.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/ffg.h"
#include "ffg_kernels.cuh"
#include "ffg_persist.cuh"
#include "ffg_orbit.cuh"
#include "ffg_adjoint.cuh"
#include "ffg_morbit.cuh"
#include "ffg_transforms.cuh"
#include "ffg_sortmerge.h"

using namespace ffg;

namespace {

struct RawBuf {
    char* p = nullptr;
    size_t bytes = 0;
};

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

size_t store_bytes(int kw, bool cplx, u64 cap) {
    size_t b = align256((size_t)kw * cap * 8);
    b += align256(cap * 8);
    if (cplx) b += align256(cap * 8);
    b += align256(cap);
    b += align256(2 * cap * 8);                      // index slots (load <= 1/2)
    b += align256((cap / kTileItems + 2) * 8);       // compaction tile offsets
    return b;
}

struct Store {
    StoreView v{};
    u64* tiles = nullptr;
    RawBuf* buf = nullptr;
};

Store carve(RawBuf& rb, int kw, bool cplx, u64 cap) {
    Store s;
    char* p = rb.p;
    s.v.cap = cap;
    s.v.key = (u64*)p;
    p += align256((size_t)kw * cap * 8);
    s.v.re = (double*)p;
    p += align256(cap * 8);
    s.v.im = nullptr;
    if (cplx) {
        s.v.im = (double*)p;
        p += align256(cap * 8);
    }
    s.v.dead = (unsigned char*)p;
    p += align256(cap);
    s.v.slots = (u64*)p;
    s.v.hmask = 2 * cap - 1;
    p += align256(2 * cap * 8);
    s.tiles = (u64*)p;
    s.buf = &rb;
    return s;
}

u64 pow2_at_least(u64 x) {
    u64 c = 1;
    while (c < x) c <<= 1;
    return c;
}

int popc64(u64 x) { return __builtin_popcountll(x); }

constexpr int kGroupD = 4;  // largest number of rotations fused in one pass (Pauli)
typedef GroupArgs<kGroupD> GArgs;

struct Op {
    enum Type { ROT, TRUNC, CLIFF, GROUP } type;
    int idx;     // ROT: rot args; TRUNC: trunc args; GROUP: group args
    int begin;   // CLIFF: circuit range [begin, end)
    int end;
    int topk;    // TRUNC: top-k after threshold/x-weight
};

// One commuting run of rotations and the truncation that follows it.
struct BatchInfo {
    int first;   // op index of the first rotation
    int nrot;    // rotation ops (consecutive)
    int trunc;   // op index of the trailing truncation, or -1
};

struct PendingEvent {
    cudaEvent_t a, b;
    int phase;
};

constexpr int kOrbitWindowMax = 16;  // orbit batches enqueued per host round trip (at most)

// One step of a batched propagation, kept for the adjoint: a range of Clifford
// ops run by the persistent kernel, or one orbit batch.
struct AdjRecord {
    enum Type { CLIFF, ORBIT } type;
    size_t op_begin = 0, op_end = 0;  // CLIFF: ops [op_begin, op_end)
    int g0 = 0, k = 0;                // ORBIT: batch gates [g0, g0 + k)
    bool has_trunc = false;
    TruncArgs trunc{};
    u64 n_in = 0;                     // terms entering the step
    u64* key = nullptr;               // checkpoint of the terms entering the step:
    double* re = nullptr;             //   KW planes of n_in keys (stride n_in) + coefficients
    bool temp = false;                // recomputed during the backward pass
};

// Instance layout of a batched propagation (see ffg_adjoint.cuh).
struct BatchCtx {
    const double2* d_inst_cs = nullptr;  // [batch gates][ninst] (cos, sin)
    u32 ninst = 0;
    int inst_plane = 0;                  // store plane of the instance code
    int inst_shift = 0;
    u64 inst_mask = 0;
    const u64* d_active = nullptr;       // [ninst][active_words] active rotations (null: all)
    u32 active_words = 0;
    u32 nrot = 0;                        // rotations of the circuit (batch gate b = rotation nrot-1-b)
};

}  // namespace

struct ffg_ctx {
    int device = 0;
    int num_sms = 152;
    cudaStream_t stream = nullptr;
    DevCounters* d_ctr = nullptr;
    DevCounters* h_ctr = nullptr;  // pinned
    RawBuf buf[2];
    CliffordOp* d_cliff = nullptr;
    size_t cliff_cap = 0;
    double* d_part = nullptr;  // expectation partial sums (2 * kMaxParts)
    u64* d_hist = nullptr;     // 256 bins
    u64* d_ties = nullptr;
    size_t ties_cap = 0;
    std::string err;
    bool profiling = false;
    int group_d = 1;  // rotations fused per pass (1..4; option group_d)
    bool persistent = true;  // one cooperative launch per run of ops (option persistent)
    int persist_blocks_per_sm = 2;  // blocks per SM of the persistent kernel (option persist_blocks_per_sm)
    PersistState* d_ps = nullptr;
    DevOp* d_ops = nullptr;
    size_t ops_cap = 0;
    PairArgs* d_pairs = nullptr;
    size_t pairs_cap = 0;
    RotArgs* d_mrots = nullptr;
    size_t mrots_cap = 0;
    TruncArgs* d_truncs = nullptr;
    size_t truncs_cap = 0;
    GroupArgs<2>* d_groups2 = nullptr;
    size_t groups2_cap = 0;
    bool orbit = true;          // batch-orbit path for long commuting runs (option orbit)
    int orbit_min_gates = 4;    // shortest run sent to the batch-orbit path
    int orbit_route_big = 8;    // |A| from which a group skips the warp-level pass (option orbit_route_big)
    bool orbit_team = true;     // 256-thread team pass before the 1024-thread pass (option orbit_team)
    bool morbit = true;         // batch-orbit path for commuting Majorana runs (option morbit)
    bool pdl = true;            // programmatic dependent launch of the orbit kernels (option pdl)
    bool orbit_qidx = true;     // classify against the gates on each term's support (option orbit_qidx)
    int orbit_window = kOrbitWindowMax;  // orbit batches per host round trip (1..kOrbitWindowMax)
    bool merge_sort = false;    // per-gate sort-and-reduce merge instead of the hash / orbit paths
    int orbit_team_threads = 256;   // threads of a team-tier group (128 or 256)
    int orbit_block_threads = 1024; // threads of a block-tier group (512 or 1024)
    void* d_smscratch = nullptr;
    size_t smscratch_bytes = 0;
    int morbit_min_gates = 2;   // shortest Majorana run sent to the batch-orbit path
    u64 min_capacity = 1ull << 16;      // smallest term-store capacity (option min_capacity)
    long long barrier_limit = kBarrierLimitCycles;  // grid-barrier wait limit, cycles (option barrier_limit_kcycles)
    bool orbit_stats = false;           // print per-batch group statistics to stderr (option orbit_stats)
    int store_headroom = 4;             // orbit windows size their stores for this many times
                                        // the entering terms (option store_headroom)
    u64 group_region_cap = 1ull << 14;  // members of a first global-memory group region (Pauli;
                                        // Majorana starts at a quarter of it)
    int morbit_route_big = 12;  // |A| from which a Majorana group skips the warp tier (option morbit_route_big);
                                // 6x6 Hubbard: 323 ms at 12 or 16, 329 ms at 10, 356 ms at 8
    MBatchGate* d_mgates = nullptr;
    size_t mgates_cap = 0;
    u32* d_qidx = nullptr;      // qubit -> gate indexes of the orbit batches of a window call
    size_t qidx_cap = 0;
    BatchGate* d_bgates = nullptr;
    size_t bgates_cap = 0;
    char* d_oscratch = nullptr;
    size_t oscratch_bytes = 0;
    OrbitCounters* d_oc = nullptr;
    OrbitCounters* h_oc = nullptr;  // pinned
    OrbitCounters* d_ocw = nullptr;  // counters of a window of orbit batches (kOrbitWindowMax)
    OrbitCounters* h_ocw = nullptr;  // pinned
    RawBuf bigpool;                 // global-memory tables of large orbit groups
    const BatchCtx* batch = nullptr;  // set while a batched propagation runs
    CaptureArgs capture{};            // set while a capture propagation runs (n null: off)
    const CaptureArgs* capture_dev = nullptr;  // its device copy (the kernels' argument)
    RawBuf capbuf;                    // capture records and their index
    ffg_profile prof{};
    std::vector<PendingEvent> events;
    std::vector<cudaEvent_t> free_events;
};

struct ffg_result {
    int kind = 1;   // 1 Pauli, 2 Majorana
    int nplanes = 4;
    bool cplx = false;
    bool deterministic = false;
    size_t n = 0;
    int device = 0;
    u64* key = nullptr;   // nplanes * n
    double* re = nullptr;
    double* im = nullptr;
    unsigned char* dead = nullptr;  // zeros (lets the reduction kernels share the store view)
    ffg_ctx* ctx = nullptr;
};

// A batched propagation: the final term set, the schedule and the checkpoints
// the adjoint needs.  Device memory here belongs to the handle.
struct ffg_batch {
    ffg_ctx* ctx = nullptr;
    int kw = 2;                      // key planes (2: qubits and instance bits below 64; 4 otherwise)
    size_t ninst = 0, nrot = 0, n_input = 0;
    BatchCtx bc{};
    double2* d_inst_cs = nullptr;
    u64* d_active = nullptr;         // per-instance active rotations (null: all)
    u64 xmask[2] = {0, 0};           // qubit bits of the x planes (caller words 0, 1)
    int inst_word = 0;               // caller word that holds the instance code
    int maxdeg = 128;                // degree filter including the instance bits
    std::vector<ffg_pauli_gate> gates;
    std::vector<Op> ops;
    std::vector<RotArgs> rots;
    std::vector<TruncArgs> truncs;
    std::vector<GArgs> groups;
    std::vector<BatchInfo> binfo;
    std::vector<AdjRecord> recs;
    int every = 0;                   // checkpoint every `every` steps (0: none)
    u64* fkey = nullptr;             // final term set: kw planes, stride fn
    double* fre = nullptr;
    u64 fn = 0;
};

namespace {

constexpr int kMaxParts = 1024;
constexpr int kChunkOps = 128;

#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);                \
            return FFG_ERR_CUDA;                                                          \
        }                                                                                 \
    } while (0)

#ifdef FFG_ORBIT_CHECK
#define OSTEP(name)                                              \
    do {                                                         \
        cudaError_t e_ = cudaGetLastError();                     \
        if (e_ == cudaSuccess) e_ = cudaStreamSynchronize(ctx->stream); \
        if (e_ != cudaSuccess) {                                 \
            ctx->err = std::string(name) + ": " + cudaGetErrorString(e_); \
            return FFG_ERR_CUDA;                                 \
        }                                                        \
    } while (0)
#else
#define OSTEP(name) CK(cudaGetLastError())
#endif

int set_err(ffg_ctx* ctx, int code, const std::string& m) {
    ctx->err = m;
    return code;
}

int ensure_buf(ffg_ctx* ctx, RawBuf& rb, size_t bytes) {
    if (rb.bytes >= bytes) return FFG_OK;
    if (rb.p) {
        const cudaError_t e = cudaFree(rb.p);
        if (e != cudaSuccess) {
            char m[256];
            snprintf(m, sizeof m, "cudaFree of a %zu-byte buffer at %p (growing to %zu bytes): %s", rb.bytes,
                     (void*)rb.p, bytes, cudaGetErrorString(e));
            ctx->err = m;
            return FFG_ERR_CUDA;
        }
    }
    rb.p = nullptr;
    rb.bytes = 0;
    const cudaError_t e = cudaMalloc(&rb.p, bytes);
    if (e != cudaSuccess) {
        char m[256];
        snprintf(m, sizeof m, "cudaMalloc of %zu bytes: %s", bytes, cudaGetErrorString(e));
        ctx->err = m;
        rb.p = nullptr;
        return FFG_ERR_CUDA;
    }
    rb.bytes = bytes;
    return FFG_OK;
}

int grid_for(const ffg_ctx* ctx, u64 items) {
    u64 b = (items + kBlock - 1) / kBlock;
    u64 lim = (u64)ctx->num_sms * 8;
    if (b < 1) b = 1;
    return (int)std::min(b, lim);
}

// Kernel launch that may start while the previous kernel on the stream is
// finishing (programmatic dependent launch): the kernel's blocks are scheduled
// early and wait in griddepcontrol.wait (wait_prior_grid) until the previous
// grid has completed.  Every kernel launched this way calls wait_prior_grid
// before touching memory.
template <typename... KArgs, typename... Args>
cudaError_t launch_k(bool pdl, void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                     Args... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

// ---------------------------------------------------------------------------
// profiling events
// ---------------------------------------------------------------------------
enum { PH_ROT = 0, PH_TRUNC, PH_CLIFF, PH_COMPACT };

cudaEvent_t get_event(ffg_ctx* ctx) {
    if (!ctx->free_events.empty()) {
        cudaEvent_t e = ctx->free_events.back();
        ctx->free_events.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

struct PhaseScope {
    ffg_ctx* ctx;
    int phase;
    cudaEvent_t a{}, b{};
    PhaseScope(ffg_ctx* c, int ph) : ctx(c), phase(ph) {
        if (ctx->profiling) {
            a = get_event(ctx);
            cudaEventRecord(a, ctx->stream);
        }
    }
    ~PhaseScope() {
        if (ctx->profiling) {
            b = get_event(ctx);
            cudaEventRecord(b, ctx->stream);
            ctx->events.push_back({a, b, phase});
        }
    }
};

void drain_events(ffg_ctx* ctx) {
    for (auto& e : ctx->events) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e.a, e.b);
        double s = ms * 1e-3;
        switch (e.phase) {
            case PH_ROT: ctx->prof.seconds_rotations += s; break;
            case PH_TRUNC: ctx->prof.seconds_truncate += s; break;
            case PH_CLIFF: ctx->prof.seconds_clifford += s; break;
            default: ctx->prof.seconds_compact += s; break;
        }
        ctx->free_events.push_back(e.a);
        ctx->free_events.push_back(e.b);
    }
    ctx->events.clear();
}

// ---------------------------------------------------------------------------
// Engine: one term store layout (KW key planes, real or complex coefficients)
// ---------------------------------------------------------------------------
template <int KW, bool CPLX, bool PAULI>
struct Engine {
    static constexpr int NW = PAULI ? KW / 2 : 0;
    ffg_ctx* ctx;
    int active = 0;  // which RawBuf holds the live store
    Store cur;
    u64 cap = 0;
    // circuit gate index of every group (one rotation per group), for the
    // capture records; null when not needed
    const std::vector<int>* group_gate = nullptr;

    explicit Engine(ffg_ctx* c) : ctx(c) {}

    int sync_counters() {
        CK(cudaMemcpyAsync(ctx->h_ctr, ctx->d_ctr, sizeof(DevCounters), cudaMemcpyDeviceToHost,
                           ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        ctx->prof.syncs++;
        if (ctx->profiling) drain_events(ctx);
        if (ctx->h_ctr->error & 1u) return set_err(ctx, FFG_ERR_ARG, "input contains duplicate keys");
        if (ctx->h_ctr->error) return set_err(ctx, FFG_ERR_STATE, "term-store index probe overrun");
        return FFG_OK;
    }

    void reindex(Store& s, int check_dup) {
        const u64 nslots = s.v.hmask + 1;
        clear_slots_kernel<<<grid_for(ctx, nslots), kBlock, 0, ctx->stream>>>(s.v.slots, nslots);
        index_kernel<KW><<<grid_for(ctx, s.v.cap), kBlock, 0, ctx->stream>>>(s.v, ctx->d_ctr, check_dup);
        ctx->prof.kernel_launches += 2;
    }

    // order-preserving compaction of live entries into buffer `to` (capacity newcap)
    int compact_into(int to, u64 newcap) {
        PhaseScope ps(ctx, PH_COMPACT);
        int rc = ensure_buf(ctx, ctx->buf[to], store_bytes(KW, CPLX, newcap));
        if (rc) return rc;
        Store dst = carve(ctx->buf[to], KW, CPLX, newcap);
        const u64 ntiles = (cap + kTileItems - 1) / kTileItems;
        const int g = (int)std::min<u64>(std::max<u64>(ntiles, 1), (u64)ctx->num_sms * 8);
        tile_count_kernel<<<g, kBlock, 0, ctx->stream>>>(cur.v, ctx->d_ctr, cur.tiles);
        tile_scan_kernel<<<1, 1024, 0, ctx->stream>>>(ctx->d_ctr, cur.tiles);
        scatter_kernel<KW, CPLX><<<g, kBlock, 0, ctx->stream>>>(cur.v, dst.v, ctx->d_ctr, cur.tiles);
        compact_commit_kernel<<<1, 1, 0, ctx->stream>>>(ctx->d_ctr, cur.tiles);
        ctx->prof.kernel_launches += 4;
        cur = dst;
        cap = newcap;
        active = to;
        reindex(cur, 0);
        index_valid = true;
        ctx->prof.compactions++;
        CK(cudaGetLastError());
        return FFG_OK;
    }

    int load(const uint64_t* keys, const double* re, const double* im, size_t n, int on_device,
             int pauli_nw_in /* planes layout of the caller: 4 planes */) {
        (void)pauli_nw_in;
        cap = pow2_at_least(std::max<u64>((u64)n * 4, ctx->min_capacity));
        int rc = ensure_buf(ctx, ctx->buf[0], store_bytes(KW, CPLX, cap));
        if (rc) return rc;
        active = 0;
        cur = carve(ctx->buf[0], KW, CPLX, cap);
        auto t0 = std::chrono::steady_clock::now();
        const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
        if (n) {
            for (int w = 0; w < KW; w++) {
                // caller plane for store plane w
                int src = w;
                if (PAULI) src = (w < NW) ? w : 2 + (w - NW);
                CK(cudaMemcpyAsync(cur.v.key + (size_t)w * cap, keys + (size_t)src * n, n * 8, kind,
                                   ctx->stream));
            }
            CK(cudaMemcpyAsync(cur.v.re, re, n * 8, kind, ctx->stream));
            if (CPLX) {
                if (im)
                    CK(cudaMemcpyAsync(cur.v.im, im, n * 8, kind, ctx->stream));
                else
                    CK(cudaMemsetAsync(cur.v.im, 0, n * 8, ctx->stream));
            }
        }
        CK(cudaMemsetAsync(cur.v.dead, 0, cap, ctx->stream));
        DevCounters h{};
        h.n = n;
        h.alive = n;
        h.peak = n;
        *ctx->h_ctr = h;
        CK(cudaMemcpyAsync(ctx->d_ctr, ctx->h_ctr, sizeof(DevCounters), cudaMemcpyHostToDevice,
                           ctx->stream));
        reindex(cur, 1);
        rc = sync_counters();
        ctx->prof.seconds_h2d += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return rc;
    }

    void launch_rot(const RotArgs& a) {
        PhaseScope ps(ctx, PH_ROT);
        const int g = grid_for(ctx, cap / 2);
        if (PAULI)
            pauli_rot_kernel<(NW > 0 ? NW : 1), CPLX><<<g, kBlock, 0, ctx->stream>>>(cur.v, ctx->d_ctr, a);
        else
            majorana_rot_kernel<KW><<<g, kBlock, 0, ctx->stream>>>(cur.v, ctx->d_ctr, a);
        ctx->prof.kernel_launches++;
    }

    void launch_trunc(const TruncArgs& t) {
        PhaseScope ps(ctx, PH_TRUNC);
        truncate_kernel<KW, CPLX, (PAULI ? NW : 0)><<<grid_for(ctx, cap / 2), kBlock, 0, ctx->stream>>>(
            cur.v, ctx->d_ctr, t);
        ctx->prof.kernel_launches++;
    }

    void launch_cliff(int begin, int end, u32 op) {
        PhaseScope ps(ctx, PH_CLIFF);
        clifford_kernel<(NW > 0 ? NW : 1), CPLX><<<grid_for(ctx, cap / 2), kBlock, 0, ctx->stream>>>(
            cur.v, ctx->d_ctr, ctx->d_cliff + begin, end - begin, op);
        ctx->prof.kernel_launches++;
        reindex(cur, 0);
    }

    // top-k (src/pauli/truncate.h:21-38): keep the k largest |c|.  Ties at the
    // cut are resolved by keeping the smallest keys (the reference keeps the
    // ones that come first in its hash-map iteration order).
    int topk(int k) {
        int rc = sync_counters();
        if (rc) return rc;
        const u64 alive = ctx->h_ctr->alive;
        if (k <= 0 || alive <= (u64)k) return FFG_OK;
        // radix select of the (k+1)-th largest magnitude, 8 bits at a time
        u64 prefix = 0, pmask = 0, rank = (u64)k;  // 0-based rank from the top
        std::vector<u64> hist(256);
        for (int shift = 56; shift >= 0; shift -= 8) {
            CK(cudaMemsetAsync(ctx->d_hist, 0, 256 * 8, ctx->stream));
            mag_hist_kernel<CPLX><<<grid_for(ctx, cap / 2), kBlock, 0, ctx->stream>>>(
                cur.v, ctx->d_ctr, shift, prefix, pmask, ctx->d_hist);
            CK(cudaMemcpyAsync(hist.data(), ctx->d_hist, 256 * 8, cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaStreamSynchronize(ctx->stream));
            ctx->prof.kernel_launches++;
            int b = 255;
            for (; b >= 0; b--) {
                if (rank < hist[b]) break;
                rank -= hist[b];
            }
            if (b < 0) b = 0;
            prefix |= (u64)b << shift;
            pmask |= 255ull << shift;
        }
        const u64 cut = prefix;
        // kill |c| < cut, gather ties
        if (ctx->ties_cap < alive) {
            if (ctx->d_ties) CK(cudaFree(ctx->d_ties));
            ctx->ties_cap = std::max<size_t>(alive, 1024);
            CK(cudaMalloc(&ctx->d_ties, (ctx->ties_cap + 1) * 8));
        }
        u64* d_nties = ctx->d_ties + ctx->ties_cap;
        CK(cudaMemsetAsync(d_nties, 0, 8, ctx->stream));
        topk_cut_kernel<CPLX><<<grid_for(ctx, cap / 2), kBlock, 0, ctx->stream>>>(
            cur.v, ctx->d_ctr, cut, ctx->d_ties, d_nties, ctx->ties_cap);
        ctx->prof.kernel_launches++;
        u64 nties = 0;
        CK(cudaMemcpyAsync(&nties, d_nties, 8, cudaMemcpyDeviceToHost, ctx->stream));
        rc = sync_counters();
        if (rc) return rc;
        const u64 now = ctx->h_ctr->alive;
        if (now <= (u64)k) return FFG_OK;
        u64 drop = now - (u64)k;
        if (drop > nties) drop = nties;
        // order ties by key, drop the largest keys
        std::vector<u64> pos(nties);
        CK(cudaMemcpy(pos.data(), ctx->d_ties, nties * 8, cudaMemcpyDeviceToHost));
        std::vector<u64> keys((size_t)nties * KW);
        for (u64 t = 0; t < nties; t++)
            for (int w = 0; w < KW; w++)
                CK(cudaMemcpy(&keys[t * KW + w], cur.v.key + (size_t)w * cap + pos[t], 8,
                              cudaMemcpyDeviceToHost));
        std::vector<u64> ord(nties);
        for (u64 t = 0; t < nties; t++) ord[t] = t;
        std::sort(ord.begin(), ord.end(), [&](u64 a, u64 b) {
            // store planes are in the caller's lexicographic order
            for (int w = 0; w < KW; w++)
                if (keys[a * KW + w] != keys[b * KW + w]) return keys[a * KW + w] < keys[b * KW + w];
            return false;
        });
        std::vector<u64> kill(drop);
        for (u64 t = 0; t < drop; t++) kill[t] = pos[ord[nties - 1 - t]];
        CK(cudaMemcpy(ctx->d_ties, kill.data(), drop * 8, cudaMemcpyHostToDevice));
        kill_list_kernel<<<grid_for(ctx, drop), kBlock, 0, ctx->stream>>>(cur.v, ctx->d_ctr, ctx->d_ties, drop);
        ctx->prof.kernel_launches++;
        return sync_counters();
    }

    template <int D>
    void launch_group_d(const GArgs& a) {
        GroupArgs<D> b{};
        for (int m = 0; m < (1 << D); m++)
            for (int w = 0; w < 4; w++) b.psub[m][w] = a.psub[m][w];
        for (int t = 0; t < D; t++) {
            b.c[t] = a.c[t];
            b.s[t] = a.s[t];
            b.yP[t] = a.yP[t];
        }
        b.ng = a.ng;
        b.maxdeg = a.maxdeg;
        b.need = a.need;
        b.op = a.op;
        const int g = grid_for(ctx, cap / 2);
        pauli_group_kernel<(NW > 0 ? NW : 1), CPLX, D><<<g, kBlock, 0, ctx->stream>>>(cur.v, ctx->d_ctr, b);
    }

    void launch_pair(const GArgs& a) {
        PairArgs b{};
        for (int w = 0; w < 4; w++) b.p[w] = a.psub[1][w];
        b.c = a.c[0];
        b.s = a.s[0];
        b.yP = a.yP[0];
        b.maxdeg = a.maxdeg;
        b.need = a.need;
        b.op = a.op;
        const int g = grid_for(ctx, cap / 2);
        pauli_pair_kernel<(NW > 0 ? NW : 1), CPLX><<<g, kBlock, 0, ctx->stream>>>(cur.v, ctx->d_ctr, b);
    }

    void launch_group(const GArgs& a) {
        PhaseScope ps(ctx, PH_ROT);
        if (!PAULI) return;
        if (a.ng == 1) {
            launch_pair(a);
            ctx->prof.kernel_launches++;
            return;
        }
        switch (ctx->group_d) {
            case 1: launch_group_d<1>(a); break;
            case 2: launch_group_d<2>(a); break;
            case 3: launch_group_d<3>(a); break;
            default: launch_group_d<4>(a); break;
        }
        ctx->prof.kernel_launches++;
    }

    int run(const std::vector<Op>& ops, const std::vector<RotArgs>& rots,
            const std::vector<TruncArgs>& truncs, const std::vector<GArgs>& groups) {
        size_t i = 0;
        while (i < ops.size()) {
            size_t j = i;
            int pending_topk = -1;
            for (; j < ops.size() && j - i < (size_t)kChunkOps; j++) {
                const Op& o = ops[j];
                if (o.type == Op::ROT) {
                    RotArgs a = rots[o.idx];
                    a.op = (u32)j;
                    launch_rot(a);
                } else if (o.type == Op::TRUNC) {
                    TruncArgs t = truncs[o.idx];
                    t.op = (u32)j;
                    if (t.thr || t.max_xweight >= 0) launch_trunc(t);
                    if (o.topk > 0) {
                        pending_topk = o.topk;
                        j++;
                        break;
                    }
                } else if (o.type == Op::GROUP) {
                    GArgs a = groups[o.idx];
                    a.op = (u32)j;
                    launch_group(a);
                } else {
                    launch_cliff(o.begin, o.end, (u32)j);
                }
            }
            CK(cudaGetLastError());
            int rc = sync_counters();
            if (rc) return rc;
            const DevCounters h = *ctx->h_ctr;
            if (h.overflow) {
                const size_t k = h.overflow - 1;
                // grow: at least twice the entries the failed op could create
                const u64 need = pow2_at_least(std::max<u64>((u64)(2 << ctx->group_d) * h.n, 2 * cap));
                DevCounters c = h;
                c.overflow = 0;
                *ctx->h_ctr = c;
                CK(cudaMemcpyAsync(ctx->d_ctr, ctx->h_ctr, sizeof(DevCounters), cudaMemcpyHostToDevice,
                                   ctx->stream));
                rc = compact_into(1 - active, need);
                if (rc) return rc;
                ctx->prof.regrows++;
                // the other buffer is re-carved at the next compaction
                i = k;
                continue;
            }
            if (pending_topk > 0) {
                rc = topk(pending_topk);
                if (rc) return rc;
            }
            // compact when more than half of the positions are dead
            const u64 dead = ctx->h_ctr->n - ctx->h_ctr->alive;
            if (dead > 4096 && dead > ctx->h_ctr->alive) {
                rc = compact_into(1 - active, cap);
                if (rc) return rc;
            }
            i = j;
        }
        int rc = sync_counters();
        if (rc) return rc;
        if (ctx->h_ctr->n != ctx->h_ctr->alive) {
            rc = compact_into(1 - active, cap);
            if (rc) return rc;
            rc = sync_counters();
            if (rc) return rc;
        }
        return FFG_OK;
    }

    template <typename T>
    int upload(T*& dptr, size_t& dcap, const std::vector<T>& h) {
        if (dcap < h.size()) {
            if (dptr) CK(cudaFree(dptr));
            dcap = std::max<size_t>(h.size(), 64);
            CK(cudaMalloc(&dptr, dcap * sizeof(T)));
        }
        if (!h.empty())
            CK(cudaMemcpyAsync(dptr, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
        return FFG_OK;
    }

    // ---------------------------------------------------------------------
    // persistent runs
    // ---------------------------------------------------------------------
    std::vector<DevOp> dops;
    void (*pkern)(StoreView, DevCounters*, PersistState*, PersistArgs) = nullptr;
    int pgrid = 0;
    bool index_valid = true;  // the index describes the live entries of cur

    int prepare_persistent(const std::vector<Op>& ops, const std::vector<RotArgs>& rots,
                           const std::vector<TruncArgs>& truncs, const std::vector<GArgs>& groups) {
        std::vector<PairArgs> pairs;
        std::vector<GroupArgs<2>> g2;
        dops.clear();
        dops.reserve(ops.size());
        for (const Op& o : ops) {
            if (o.type == Op::GROUP && groups[o.idx].ng == 2) {
                const GArgs& a = groups[o.idx];
                GroupArgs<2> b{};
                for (int m = 0; m < 4; m++)
                    for (int w = 0; w < 4; w++) b.psub[m][w] = a.psub[m][w];
                for (int t = 0; t < 2; t++) {
                    b.c[t] = a.c[t];
                    b.s[t] = a.s[t];
                    b.yP[t] = a.yP[t];
                }
                b.ng = 2;
                b.maxdeg = a.maxdeg;
                b.need = a.need;
                g2.push_back(b);
                dops.push_back({OP_GROUP2, (int)g2.size() - 1, 0, 0});
            } else if (o.type == Op::GROUP) {
                const GArgs& a = groups[o.idx];
                PairArgs b{};
                for (int w = 0; w < 4; w++) b.p[w] = a.psub[1][w];
                b.c = a.c[0];
                b.s = a.s[0];
                b.yP = a.yP[0];
                b.maxdeg = a.maxdeg;
                b.need = a.need;
                pairs.push_back(b);
                dops.push_back({OP_PAIR, (int)pairs.size() - 1, 0, 0});
            } else if (o.type == Op::ROT) {
                dops.push_back({OP_MROT, o.idx, 0, 0});
            } else if (o.type == Op::TRUNC) {
                dops.push_back({OP_TRUNC, o.idx, 0, 0});
            } else {
                dops.push_back({OP_CLIFF, 0, o.begin, o.end});
            }
        }
        int rc = upload(ctx->d_ops, ctx->ops_cap, dops);
        if (!rc) rc = upload(ctx->d_pairs, ctx->pairs_cap, pairs);
        if (!rc && !PAULI) rc = upload(ctx->d_mrots, ctx->mrots_cap, rots);
        if (!rc) rc = upload(ctx->d_truncs, ctx->truncs_cap, truncs);
        if (!rc) rc = upload(ctx->d_groups2, ctx->groups2_cap, g2);
        if (rc) return rc;
        pkern = g2.empty() ? persistent_kernel<KW, CPLX, PAULI, false> : persistent_kernel<KW, CPLX, PAULI, PAULI>;
        int per_sm = 0;
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pkern, kPBlock, 0));
        if (per_sm < 1) return set_err(ctx, FFG_ERR_STATE, "persistent kernel does not fit on an SM");
        pgrid = ctx->num_sms * std::min(per_sm, ctx->persist_blocks_per_sm);
        return FFG_OK;
    }

    void launch_reindex() {
        reindex(cur, 0);
        index_valid = true;
    }

    // Runs ops [begin, end) with the persistent kernel; the host only steps in
    // to grow or compact the store.
    int exec_persistent(size_t begin, size_t end) {
        if (!index_valid) launch_reindex();
        size_t i = begin;
        int rc = FFG_OK;
        while (i < end) {
            CK(cudaMemsetAsync(ctx->d_ps, 0, sizeof(PersistState), ctx->stream));
            PersistArgs pa{};
            pa.ops = ctx->d_ops;
            pa.pairs = ctx->d_pairs;
            pa.mrots = ctx->d_mrots;
            pa.truncs = ctx->d_truncs;
            pa.cliff = ctx->d_cliff;
            pa.groups2 = ctx->d_groups2;
            pa.op_begin = (int)i;
            pa.op_end = (int)end;
            pa.compact_min = 4096;
            pa.barrier_limit = ctx->barrier_limit;
            StoreView v = cur.v;
            DevCounters* C = ctx->d_ctr;
            PersistState* ps = ctx->d_ps;
            void* args[] = {(void*)&v, (void*)&C, (void*)&ps, (void*)&pa};
            {
                PhaseScope sc(ctx, PH_ROT);
                CK(cudaLaunchCooperativeKernel((void*)pkern, dim3(pgrid), dim3(kPBlock), args, 0, ctx->stream));
            }
            ctx->prof.kernel_launches++;
            PersistState h{};
            CK(cudaMemcpyAsync(&h, ctx->d_ps, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
            rc = sync_counters();
            if (rc) return rc;
            if (h.stop_reason == 3) return set_err(ctx, FFG_ERR_STATE, "grid barrier timed out");
            const DevCounters c = *ctx->h_ctr;
            if (h.stop_reason == 1) {
                const u64 need = pow2_at_least(std::max<u64>(8 * c.n, 2 * cap));
                DevCounters z = c;
                z.overflow = 0;
                *ctx->h_ctr = z;
                CK(cudaMemcpyAsync(ctx->d_ctr, ctx->h_ctr, sizeof(DevCounters), cudaMemcpyHostToDevice,
                                   ctx->stream));
                rc = compact_into(1 - active, need);
                if (rc) return rc;
                ctx->prof.regrows++;
            } else if (h.stop_reason == 2) {
                rc = compact_into(1 - active, cap);
                if (rc) return rc;
            }
            i = h.next_op;
        }
        return rc;
    }

    int finish() {
        int rc = sync_counters();
        if (rc) return rc;
        if (ctx->h_ctr->n != ctx->h_ctr->alive) {
            rc = compact_into(1 - active, cap);
            if (rc) return rc;
            rc = sync_counters();
        }
        return rc;
    }

    int run_persistent(const std::vector<Op>& ops, const std::vector<RotArgs>& rots,
                       const std::vector<TruncArgs>& truncs, const std::vector<GArgs>& groups) {
        int rc = prepare_persistent(ops, rots, truncs, groups);
        if (!rc) rc = exec_persistent(0, dops.size());
        if (!rc) rc = finish();
        return rc;
    }

    // ---------------------------------------------------------------------
    // batch-orbit runs (Pauli, batched mode)
    // ---------------------------------------------------------------------
    u32* retry_list = nullptr;
    u32* nretry = nullptr;

    // Big-group tiers.  launch_big_tiers enqueues the shared-memory passes right
    // after the warp pass, reading the list lengths on the device (no host
    // round trip): 256-thread teams with kTeamCap-member tables (several blocks
    // per SM), then 1024-thread blocks with kBlockCap-member tables over the
    // team pass's overflow.  Groups left after both (more than kBlockCap
    // members) are listed in sc.big with their count in nretry[1];
    // finish_big_groups runs them with global-memory regions (x4 per pass).
    int launch_big_tiers(const StoreView& in, const StoreView& out, OrbitScratch& sc, const OrbitBatchArgs& a,
                         OrbitCounters* oc) {
        constexpr int NWo = PAULI ? NW : 1;
        const size_t tb = block_table_bytes<KW, CPLX>();
        const size_t tt = block_table_bytes<KW, CPLX, kTeamCap>();
        // the tier kernels at each thread count (options orbit_team_threads, orbit_block_threads)
        const bool rec = ctx->capture_dev != nullptr;  // capture runs record the dropped partners
        auto team_k = ctx->orbit_team_threads == 128
                          ? (rec ? orbit_process_big<NWo, CPLX, true, 128, kTeamCap, true>
                                 : orbit_process_big<NWo, CPLX, true, 128, kTeamCap>)
                          : (rec ? orbit_process_big<NWo, CPLX, true, 256, kTeamCap, true>
                                 : orbit_process_big<NWo, CPLX, true, 256, kTeamCap>);
        auto block_k = ctx->orbit_block_threads == 512
                           ? (rec ? orbit_process_big<NWo, CPLX, true, 512, kBlockCap, true>
                                  : orbit_process_big<NWo, CPLX, true, 512, kBlockCap>)
                           : (rec ? orbit_process_big<NWo, CPLX, true, 1024, kBlockCap, true>
                                  : orbit_process_big<NWo, CPLX, true, 1024, kBlockCap>);
        // function attributes are set once per device (bit `device` of attr_devs)
        static u64 attr_devs = 0;
        static int team_per_sm = 1;
        if (!((attr_devs >> (ctx->device & 63)) & 1ull)) {
            for (auto k : {orbit_process_big<NWo, CPLX, true, 512, kBlockCap>,
                           orbit_process_big<NWo, CPLX, true, 1024, kBlockCap>,
                           orbit_process_big<NWo, CPLX, true, 512, kBlockCap, true>,
                           orbit_process_big<NWo, CPLX, true, 1024, kBlockCap, true>})
                CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tb));
            for (auto k : {orbit_process_big<NWo, CPLX, true, 128, kTeamCap>,
                           orbit_process_big<NWo, CPLX, true, 256, kTeamCap>,
                           orbit_process_big<NWo, CPLX, true, 128, kTeamCap, true>,
                           orbit_process_big<NWo, CPLX, true, 256, kTeamCap, true>})
                CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tt));
            CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &team_per_sm, orbit_process_big<NWo, CPLX, true, 256, kTeamCap>, 256, tt));
            team_per_sm = std::max(team_per_sm, 1);
            attr_devs |= 1ull << (ctx->device & 63);
        }
        const int tthreads = ctx->orbit_team_threads == 128 ? 128 : 256;
        const int bthreads = ctx->orbit_block_threads == 512 ? 512 : 1024;
        BigPool bp{};
        const u32* nbig_dev = &oc->nbig;
        PhaseScope ps(ctx, PH_ROT);
        if (ctx->orbit_team) {
            // sc.big -> retry_list (count nretry[0]) -> sc.big (count nretry[1])
            bp.retry = retry_list;
            bp.nretry = nretry;
            bp.fetch = &oc->fetch[0];
            CK(launch_k(ctx->pdl, team_k, ctx->num_sms * team_per_sm, tthreads, tt, ctx->stream, in, out, sc, oc, a,
                        bp, (const u32*)sc.big, 0u, nbig_dev));
            bp.retry = sc.big;
            bp.nretry = nretry + 1;
            bp.fetch = &oc->fetch[1];
            CK(launch_k(ctx->pdl, block_k, ctx->num_sms, bthreads, tb, ctx->stream, in, out, sc, oc, a, bp,
                        (const u32*)retry_list, 0u, (const u32*)nretry));
            ctx->prof.kernel_launches += 2;
        } else {
            // sc.big -> retry_list (count nretry[1])
            bp.retry = retry_list;
            bp.nretry = nretry + 1;
            bp.fetch = &oc->fetch[1];
            CK(launch_k(ctx->pdl, block_k, ctx->num_sms, bthreads, tb, ctx->stream, in, out, sc, oc, a, bp,
                        (const u32*)sc.big, 0u, nbig_dev));
            ctx->prof.kernel_launches++;
        }
        OSTEP("orbit_process_big");
        return FFG_OK;
    }

    // Global-memory passes over the nleft groups left by launch_big_tiers;
    // returns 0 when every group fit, 2 when the output store overflowed, else
    // a negative status.
    int finish_big_groups(const StoreView& in, const StoreView& out, OrbitScratch& sc, const OrbitBatchArgs& a,
                          u32 nleft, OrbitCounters* oc, OrbitCounters* hoc) {
        constexpr int NWo = PAULI ? NW : 1;
        u32* list = ctx->orbit_team ? sc.big : retry_list;
        u32* other = ctx->orbit_team ? retry_list : sc.big;
        u64 rcap = ctx->group_region_cap;
        while (nleft > 0) {
            const u32 grid = std::min<u32>(nleft, (u32)ctx->num_sms);
            BigPool bp{};
            bp.retry = other;
            bp.nretry = nretry;
            const u64 region = align256((size_t)KW * rcap * 8 + rcap * 8 * (CPLX ? 2 : 1) + 2 * rcap * 4 + 8);
            int rc = ensure_buf(ctx, ctx->bigpool, region * grid);
            if (rc) return rc;
            bp.base = ctx->bigpool.p;
            bp.region_bytes = region;
            bp.rcap = (u32)rcap;
            CK(cudaMemsetAsync(nretry, 0, 4, ctx->stream));
            {
                PhaseScope ps(ctx, PH_ROT);
                if (ctx->capture_dev)
                    orbit_process_big<NWo, CPLX, false, 1024, kBlockCap, true><<<grid, 1024, 0, ctx->stream>>>(
                        in, out, sc, oc, a, bp, list, nleft, nullptr);
                else
                    orbit_process_big<NWo, CPLX, false><<<grid, 1024, 0, ctx->stream>>>(in, out, sc, oc, a, bp, list,
                                                                                       nleft, nullptr);
                OSTEP("orbit_process_big");
                ctx->prof.kernel_launches++;
            }
            u32 hr = 0;
            CK(cudaMemcpyAsync(hoc, oc, sizeof(OrbitCounters), cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaMemcpyAsync(&hr, nretry, 4, cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaStreamSynchronize(ctx->stream));
            ctx->prof.syncs++;
            if (hoc->chk_code)
                return set_err(ctx, FFG_ERR_STATE, "orbit self-check " + std::to_string(hoc->chk_code) + " a=" +
                                                       std::to_string(hoc->chk_a) + " b=" + std::to_string(hoc->chk_b) +
                                                       " c=" + std::to_string(hoc->chk_c));
            if (hoc->overflow & 1u) return 2;
            if (hr == 0) return 0;
            std::swap(list, other);
            nleft = hr;
            rcap *= 4;
            if (rcap > (1ull << 26)) return set_err(ctx, FFG_ERR_STATE, "orbit group larger than 2^26 terms");
        }
        return 0;
    }

    OrbitScratch carve_scratch(u64 cap_in) {
        OrbitScratch sc{};
        u64 hc = pow2_at_least(std::max<u64>(2 * cap_in, 1024));
        size_t need = align256((size_t)kAW * cap_in * 8) + align256((size_t)KW * cap_in * 8) +
                      9 * align256(cap_in * 4) + align256(2 * cap_in * 8) + align256(hc * 8) + 256;
        if (ctx->oscratch_bytes < need) {
            if (ctx->d_oscratch && cudaFree(ctx->d_oscratch) != cudaSuccess) return sc;
            ctx->d_oscratch = nullptr;
            ctx->oscratch_bytes = 0;
            if (cudaMalloc(&ctx->d_oscratch, need) != cudaSuccess) return sc;
            ctx->oscratch_bytes = need;
        }
        char* p = ctx->d_oscratch;
        sc.amask = (u64*)p;
        p += align256((size_t)kAW * cap_in * 8);
        sc.gkey = (u64*)p;
        p += align256((size_t)KW * cap_in * 8);
        sc.rep = (u32*)p;
        p += align256(cap_in * 4);
        sc.cnt = (u32*)p;
        p += align256(cap_in * 4);
        sc.off = (u32*)p;
        p += align256(cap_in * 4);
        sc.fill = (u32*)p;
        p += align256(cap_in * 4);
        sc.order = (u32*)p;
        p += align256(cap_in * 4);
        sc.groups = (u32*)p;
        p += align256(cap_in * 4);
        sc.big = (u32*)p;
        p += align256(cap_in * 4);
        retry_list = (u32*)p;
        p += align256(cap_in * 4);
        nretry = (u32*)p;
        p += 256;
        sc.gcoef = (double*)p;
        p += align256(2 * cap_in * 8);
        sc.list2 = (u32*)p;
        p += align256(cap_in * 4);
        sc.gslots = (u64*)p;
        sc.gmask = hc - 1;
        sc.cap_in = cap_in;
        return sc;
    }

    // One orbit batch: rotations [g0, g0+k) of the batch gate table and the
    // batch-end truncation t (may be null).
    struct OrbitJob {
        int g0, k;
        const TruncArgs* t;
    };

    OrbitBatchArgs batch_args(const OrbitJob& j, int maxdeg) const {
        OrbitBatchArgs a{};
        a.gates = ctx->d_bgates + j.g0;
        a.k = j.k;
        a.maxdeg = maxdeg;
        a.thr = j.t ? j.t->thr : 0;
        a.tau = j.t ? j.t->tau : 0.0;
        a.max_xweight = j.t ? j.t->max_xweight : -1;
        a.route_big = ctx->orbit_route_big;
        if (ctx->batch) {
            a.inst_cs = ctx->batch->d_inst_cs + (size_t)j.g0 * ctx->batch->ninst;
            a.ninst = ctx->batch->ninst;
            a.inst_plane = ctx->batch->inst_plane;
            a.inst_shift = ctx->batch->inst_shift;
            a.inst_mask = ctx->batch->inst_mask;
            if (ctx->batch->d_active) {
                a.active = ctx->batch->d_active;
                a.active_words = ctx->batch->active_words;
                a.act_r0 = (int)ctx->batch->nrot - 1 - j.g0;
            }
        }
        a.cap = ctx->capture_dev;
        return a;
    }

    // Runs consecutive orbit batches on the (dense) live store.  Up to
    // orbit_window batches are enqueued back to back, ping-ponging between the
    // two store buffers sized for the window, with no host round trip: every
    // kernel reads its input size from the batch's counters (orbit_gate).  The
    // host then reads all counters once and walks the batches: completed ones
    // are committed; at a batch that overflowed (its input is still intact)
    // the capacity grows and the next window starts there; a batch that left
    // groups too large for shared memory is finished with global-memory
    // passes (the batches after it were skipped, so its scratch is intact).
    int exec_orbit_window(const OrbitJob* jobs, int njobs, int maxdeg) {
        constexpr int NWo = PAULI ? NW : 1;
        const size_t smem = sizeof(OrbitTable<KW, CPLX>) * kOrbitWarps;
        static u64 attr_devs = 0;  // devices whose function attributes are set
        if (!((attr_devs >> (ctx->device & 63)) & 1ull)) {
            CK(cudaFuncSetAttribute(orbit_process<NWo, CPLX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
            CK(cudaFuncSetAttribute(orbit_process<NWo, CPLX, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
            attr_devs |= 1ull << (ctx->device & 63);
        }
        const int G = ctx->num_sms * 8;
        // qubit -> gate indexes of every job (Pauli batches), uploaded once
        std::vector<size_t> qbase(njobs, 0);
        if (PAULI && !h_bgates.empty()) {
            std::vector<u32> qv;
            for (int j = 0; j < njobs; j++) {
                qbase[j] = qv.size();
                build_qidx(jobs[j].g0, jobs[j].k, qv);
            }
            int rc = upload(ctx->d_qidx, ctx->qidx_cap, qv);
            if (rc) return rc;
        }
        auto args_of = [&](int j) {
            OrbitBatchArgs a = batch_args(jobs[j], maxdeg);
            if (PAULI && !h_bgates.empty() && ctx->orbit_qidx) a.qidx = ctx->d_qidx + qbase[j];
            return a;
        };
        int i = 0, regrows = 0;
        u64 grow = 0;
        while (i < njobs) {
            const u64 n_cur = ctx->h_ctr->n;  // dense store: no dead entries
            if (n_cur == 0) return FFG_OK;  // every later batch is empty too
            const u64 wcap =
                std::max<u64>(std::max<u64>(cap, pow2_at_least((u64)ctx->store_headroom * n_cur)), grow);
            int rc = FFG_OK;
            if (cap < wcap) {
                rc = compact_into(1 - active, wcap);
                if (rc) return rc;
            }
            rc = ensure_buf(ctx, ctx->buf[1 - active], store_bytes(KW, CPLX, wcap));
            if (rc) return rc;
            Store S[2] = {cur, carve(ctx->buf[1 - active], KW, CPLX, wcap)};
            OrbitScratch sc = carve_scratch(wcap);
            if (!sc.amask) return set_err(ctx, FFG_ERR_CUDA, "orbit scratch allocation failed");
            const int m = std::min(std::max(1, std::min(ctx->orbit_window, kOrbitWindowMax)), njobs - i);
            {
                PhaseScope ps(ctx, PH_ROT);
                for (int j = 0; j < m; j++) {
                    const OrbitBatchArgs a = args_of(i + j);
                    OrbitCounters* oc = ctx->d_ocw + j;
                    const StoreView& in = S[j & 1].v;
                    const StoreView& out = S[(j + 1) & 1].v;
                    const bool pdl = ctx->pdl;
                    const OrbitCounters* prev = j ? oc - 1 : nullptr;
                    CK(launch_k(pdl, orbit_gate, 1, 32, 0, ctx->stream, oc, prev, n_cur, sc.gmask + 1, nretry));
                    if (a.active)
                        CK(launch_k(pdl, orbit_classify<NWo, CPLX, true>, G, kBlock, 0, ctx->stream, in, out, sc, oc,
                                    a));
                    else
                        CK(launch_k(pdl, orbit_classify<NWo, CPLX>, G, kBlock, 0, ctx->stream, in, out, sc, oc, a));
                    OSTEP("orbit_classify");
                    CK(launch_k(pdl, orbit_group<KW>, G, kBlock, 0, ctx->stream, sc, oc));
                    OSTEP("orbit_group");
                    CK(launch_k(pdl, orbit_offsets, G, kBlock, 0, ctx->stream, sc, oc));
                    OSTEP("orbit_offsets");
                    CK(launch_k(pdl, orbit_scatter<KW, CPLX>, G, kBlock, 0, ctx->stream, in, sc,
                                (const OrbitCounters*)oc));
                    OSTEP("orbit_scatter");
                    if (a.cap)
                        CK(launch_k(pdl, orbit_process<NWo, CPLX, true>, ctx->num_sms * 2, 32 * kOrbitWarps, smem,
                                    ctx->stream, in, out, sc, oc, a));
                    else
                        CK(launch_k(pdl, orbit_process<NWo, CPLX>, ctx->num_sms * 2, 32 * kOrbitWarps, smem,
                                    ctx->stream, in, out, sc, oc, a));
                    OSTEP("orbit_process");
                    ctx->prof.kernel_launches += 6;
                    rc = launch_big_tiers(in, out, sc, a, oc);
                    if (rc) return rc;
                }
            }
            CK(cudaGetLastError());
            u32 nleft = 0;
            CK(cudaMemcpyAsync(ctx->h_ocw, ctx->d_ocw, m * sizeof(OrbitCounters), cudaMemcpyDeviceToHost,
                               ctx->stream));
            CK(cudaMemcpyAsync(&nleft, nretry + 1, 4, cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaStreamSynchronize(ctx->stream));
            ctx->prof.syncs++;
            if (ctx->profiling) drain_events(ctx);
            int done = 0, live = 0;  // committed batches; S[live] holds the live store
            bool overflow = false;
            DevCounters h = *ctx->h_ctr;
            for (int j = 0; j < m; j++) {
                OrbitCounters& oc = ctx->h_ocw[j];
                if (oc.error) return set_err(ctx, FFG_ERR_STATE, "orbit grouping index overrun");
                if (oc.chk_code)
                    return set_err(ctx, FFG_ERR_STATE, "orbit self-check " + std::to_string(oc.chk_code) + " a=" +
                                                           std::to_string(oc.chk_a) + " b=" + std::to_string(oc.chk_b) +
                                                           " c=" + std::to_string(oc.chk_c));
                if (oc.overflow & 1u) {
                    grow = pow2_at_least(std::max<u64>(oc.n_out + oc.n_out / 4 + 1024, 2 * wcap));
                    overflow = true;
                    break;
                }
                if (oc.skip) break;
                const bool last = j == m - 1 || ctx->h_ocw[j + 1].skip;
                if (last && nleft) {
                    const OrbitBatchArgs a = args_of(i + j);
                    const int br = finish_big_groups(S[j & 1].v, S[(j + 1) & 1].v, sc, a, nleft, ctx->d_ocw + j, &oc);
                    if (br < 0) return br;
                    if (br == 2) {
                        grow = pow2_at_least(std::max<u64>(oc.n_out + oc.n_out / 4 + 1024, 2 * wcap));
                        overflow = true;
                        break;
                    }
                }
                // commit batch j
                const OrbitJob& jb = jobs[i + j];
                ctx->prof.orbit_fallbacks += oc.nbig;  // groups done by the block-level passes
                ctx->prof.orbit_max_group = std::max<int64_t>(ctx->prof.orbit_max_group, oc.max_members);
                ctx->prof.orbit_batches++;
                ctx->prof.orbit_groups += oc.ngroups;
                if (ctx->orbit_stats) {
                    fprintf(stderr, "batch k=%d n_in=%llu groups=%u big=%u wasted=%u out=%llu |", jb.k,
                            (unsigned long long)oc.n_in, oc.ngroups, oc.nbig, oc.wasted,
                            (unsigned long long)oc.n_out);
                    for (int b = 0; b < 16; b++) fprintf(stderr, " %u", oc.hist[b]);
                    fprintf(stderr, " | A:");
                    for (int b = 0; b < 16; b++) fprintf(stderr, " %u", oc.hist_a[b]);
                    fprintf(stderr, "\n");
                }
                h.apps += (u64)jb.k * oc.n_in + oc.xapps;
                h.emits += oc.emits;
                const u64 before_trunc = oc.n_in + oc.created;
                if (before_trunc > h.peak) h.peak = before_trunc;
                h.n = oc.n_out;
                h.alive = oc.n_out;
                live = (j + 1) & 1;
                done++;
                if (h.n == 0) break;
            }
            if (done) {
                cur = S[live];
                if (live == 1) active = 1 - active;
                cap = wcap;
                index_valid = false;
                *ctx->h_ctr = h;
                CK(cudaMemcpyAsync(ctx->d_ctr, ctx->h_ctr, sizeof(DevCounters), cudaMemcpyHostToDevice,
                                   ctx->stream));
                i += done;
                if (h.n == 0) return FFG_OK;
            } else {
                cap = wcap;  // the live store stays in place (S[0])
            }
            if (overflow) {
                ctx->prof.regrows++;
                if (++regrows > 64) return set_err(ctx, FFG_ERR_STATE, "orbit batch: output store kept overflowing");
            }
        }
        return FFG_OK;
    }

    // ---------------------------------------------------------------------
    // per-gate sort-and-reduce merge (option merge_sort; Pauli)
    // ---------------------------------------------------------------------
    int run_sortmerge(const std::vector<Op>& ops, const std::vector<TruncArgs>& truncs,
                      const std::vector<GArgs>& groups) {
        index_valid = false;
        for (size_t i = 0; i < ops.size(); i++) {
            const Op& o = ops[i];
            if (o.type == Op::GROUP) {
                const GArgs& ga = groups[o.idx];
                if (ga.ng != 1) return set_err(ctx, FFG_ERR_ARG, "merge_sort needs one rotation per pass");
                ffg_sm::SmGate g{};
                for (int w = 0; w < 4; w++) g.p[w] = ga.psub[1][w];
                g.c = ga.c[0];
                g.s = ga.s[0];
                g.yP = ga.yP[0];
                g.maxdeg = ga.maxdeg;
                const u64 n_in = ctx->h_ctr->n;
                u64 out_cap = std::max<u64>(cap, pow2_at_least(2 * n_in));
                for (int attempt = 0; attempt < 4; attempt++) {
                    int rc = ensure_buf(ctx, ctx->buf[1 - active], store_bytes(KW, CPLX, out_cap));
                    if (rc) return rc;
                    Store dst = carve(ctx->buf[1 - active], KW, CPLX, out_cap);
                    u64 n_out = 0, em = 0;
                    int e;
                    {
                        PhaseScope ps(ctx, PH_ROT);
                        e = ffg_sm::rotation(ctx->stream, KW, CPLX, cur.v.key, cur.v.re, CPLX ? cur.v.im : nullptr,
                                             n_in, cap, g, dst.v.key, dst.v.re, CPLX ? dst.v.im : nullptr, out_cap,
                                             &n_out, &em, &ctx->d_smscratch, &ctx->smscratch_bytes);
                    }
                    if (e) return set_err(ctx, FFG_ERR_CUDA, std::string("sort-merge pass: ") +
                                                                 cudaGetErrorString((cudaError_t)e));
                    ctx->prof.kernel_launches += 5;
                    ctx->prof.syncs++;
                    if (n_out > out_cap) {
                        out_cap = pow2_at_least(n_out);
                        continue;
                    }
                    CK(cudaMemsetAsync(dst.v.dead, 0, n_out, ctx->stream));
                    cur = dst;
                    cap = out_cap;
                    active = 1 - active;
                    DevCounters h = *ctx->h_ctr;
                    h.apps += n_in;
                    h.emits += em;
                    h.n = h.alive = n_out;
                    if (n_out > h.peak) h.peak = n_out;
                    *ctx->h_ctr = h;
                    CK(cudaMemcpyAsync(ctx->d_ctr, ctx->h_ctr, sizeof(DevCounters), cudaMemcpyHostToDevice,
                                       ctx->stream));
                    break;
                }
            } else if (o.type == Op::TRUNC) {
                if (o.topk > 0) return set_err(ctx, FFG_ERR_ARG, "merge_sort does not support top-k truncation");
                TruncArgs t = truncs[o.idx];
                t.op = (u32)i;
                if (t.thr || t.max_xweight >= 0) launch_trunc(t);
                int rc = sync_counters();
                if (rc) return rc;
                if (ctx->h_ctr->n != ctx->h_ctr->alive) {
                    rc = compact_into(1 - active, cap);
                    if (rc) return rc;
                    rc = sync_counters();
                    if (rc) return rc;
                }
            } else if (o.type == Op::CLIFF) {
                launch_cliff(o.begin, o.end, (u32)i);
                int rc = sync_counters();
                if (rc) return rc;
            } else {
                return set_err(ctx, FFG_ERR_ARG, "merge_sort: unexpected op");
            }
        }
        return finish();
    }

    // ---------------------------------------------------------------------
    // Majorana runs (batch-orbit path with the threshold after every gate)
    // ---------------------------------------------------------------------
    int upload_mgates(const std::vector<RotArgs>& rots) {
        std::vector<MBatchGate> mg(rots.size());
        for (size_t i = 0; i < rots.size(); i++) {
            MBatchGate g{};
            for (int w = 0; w < 4; w++) {
                g.p[w] = rots[i].p[w];
                g.mg[w] = rots[i].mg[w];
            }
            g.c = rots[i].c;
            g.fr = rots[i].fr;
            g.fi = rots[i].fi;
            g.odd = rots[i].gate_odd;
            mg[i] = g;
        }
        h_mgates = mg;
        return upload(ctx->d_mgates, ctx->mgates_cap, mg);
    }

    // Gates [g0, g0 + k) of the Majorana gate table (application order), all
    // mutually commuting, each followed by the threshold of t, on the dense
    // live store.
    std::vector<MBatchGate> h_mgates;  // host copy of the Majorana gate table

    // mode -> gate index of gates [g0, g0 + k) (MOrbitArgs::midx layout); empty
    // when some gate has odd degree
    bool build_midx(int g0, int k, std::vector<u32>& out) const {
        std::vector<std::vector<u32>> lists(256);
        for (int t = 0; t < k; t++) {
            const MBatchGate& G = h_mgates[g0 + t];
            if (G.odd) return false;
            for (int w = 0; w < 4; w++) {
                u64 sup = G.p[w];
                while (sup) {
                    lists[64 * w + __builtin_ctzll(sup)].push_back((u32)t);
                    sup &= sup - 1;
                }
            }
        }
        out.assign(257, 0);
        u32 e = 0;
        for (int i = 0; i < 256; i++) {
            out[i] = e;
            e += (u32)lists[i].size();
        }
        out[256] = e;
        for (int i = 0; i < 256; i++) out.insert(out.end(), lists[i].begin(), lists[i].end());
        return true;
    }

    int exec_morbit_batch(int g0, int k, const TruncArgs& t, int maxdeg) {
        const u64 n_in = ctx->h_ctr->n;
        if (n_in == 0) return FFG_OK;
        const u64 cap_in = std::max<u64>(n_in, 1024);
        OrbitScratch sc = carve_scratch(cap_in);
        if (!sc.amask) return set_err(ctx, FFG_ERR_CUDA, "orbit scratch allocation failed");
        MOrbitArgs a{};
        a.gates = ctx->d_mgates + g0;
        a.k = k;
        a.maxdeg = maxdeg;
        a.thr = t.thr;
        a.tau = t.tau;
        a.route_big = ctx->morbit_route_big;
        if (ctx->orbit_qidx) {
            std::vector<u32> mv;
            if (build_midx(g0, k, mv)) {
                int rc = upload(ctx->d_qidx, ctx->qidx_cap, mv);
                if (rc) return rc;
                a.midx = ctx->d_qidx;
            }
        }
        const size_t wsm = (size_t)kMWarps * mtable_bytes<KW>(kMWarpCap);
        const size_t tsm = mtable_bytes<KW>(kMTeamCap);
        const size_t ssm = (size_t)(32 * kMSubWarps / kMSubLanes) * mtable_bytes<KW>(kMSubCap);
        static u64 attr_devs = 0;  // devices whose function attributes are set
        static int team_per_sm = 1, sub_per_sm = 1;
        if (!((attr_devs >> (ctx->device & 63)) & 1ull)) {
            CK(cudaFuncSetAttribute(morbit_sub<KW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ssm));
            CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&sub_per_sm, morbit_sub<KW>, 32 * kMSubWarps, ssm));
            sub_per_sm = std::max(sub_per_sm, 1);
            CK(cudaFuncSetAttribute(morbit_warp<KW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)wsm));
            CK(cudaFuncSetAttribute(morbit_block<KW, 256, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)tsm));
            CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&team_per_sm, morbit_block<KW, 256, true>, 256, tsm));
            team_per_sm = std::max(team_per_sm, 1);
            attr_devs |= 1ull << (ctx->device & 63);
        }
        u64 out_cap = std::max<u64>(cap, pow2_at_least(4 * n_in));
        const int G = ctx->num_sms * 8;
        for (int attempt = 0; attempt < 8; attempt++) {
            int rc = ensure_buf(ctx, ctx->buf[1 - active], store_bytes(KW, true, out_cap));
            if (rc) return rc;
            Store dst = carve(ctx->buf[1 - active], KW, true, out_cap);
            OrbitCounters* oc = ctx->d_oc;
            {
                PhaseScope ps(ctx, PH_ROT);
                const bool pdl = ctx->pdl;
                const StoreView in = cur.v, ov = dst.v;
                CK(launch_k(pdl, orbit_gate, 1, 32, 0, ctx->stream, oc, (const OrbitCounters*)nullptr, n_in,
                            sc.gmask + 1, nretry));
                CK(launch_k(pdl, morbit_classify<KW>, G, kBlock, 0, ctx->stream, in, ov, sc, oc, a));
                OSTEP("morbit_classify");
                CK(launch_k(pdl, orbit_group<KW>, G, kBlock, 0, ctx->stream, sc, oc));
                CK(launch_k(pdl, orbit_offsets, G, kBlock, 0, ctx->stream, sc, oc));
                CK(launch_k(pdl, orbit_scatter<KW, true>, G, kBlock, 0, ctx->stream, in, sc, (const OrbitCounters*)oc));
                OSTEP("orbit_scatter");
                CK(launch_k(pdl, morbit_single<KW>, G, kBlock, 0, ctx->stream, in, ov, sc, oc, a));
                OSTEP("morbit_single");
                CK(launch_k(pdl, morbit_sub<KW>, ctx->num_sms * sub_per_sm, 32 * kMSubWarps, ssm, ctx->stream, in, ov,
                            sc, oc, a));
                OSTEP("morbit_sub");
                CK(launch_k(pdl, morbit_warp<KW>, ctx->num_sms * 2, 32 * kMWarps, wsm, ctx->stream, in, ov, sc, oc, a));
                OSTEP("morbit_warp");
                CK(launch_k(pdl, morbit_block<KW, 256, true>, ctx->num_sms * team_per_sm, 256, tsm, ctx->stream, in, ov,
                            sc, oc, a, (u32)kMTeamCap, (char*)nullptr, (u64)0, (const u32*)sc.big, 0u,
                            (const u32*)&oc->nbig, retry_list, nretry));
                OSTEP("morbit_block");
                ctx->prof.kernel_launches += 9;
            }
            u32 nleft = 0;
            CK(cudaMemcpyAsync(ctx->h_oc, oc, sizeof(OrbitCounters), cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaMemcpyAsync(&nleft, nretry, 4, cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaStreamSynchronize(ctx->stream));
            ctx->prof.syncs++;
            if (ctx->profiling) drain_events(ctx);
            if (ctx->h_oc->error) return set_err(ctx, FFG_ERR_STATE, "orbit grouping index overrun");
            bool overflow = (ctx->h_oc->overflow & 1u) != 0;
            u32* list = retry_list;
            u32* other = sc.big;
            u32 rcap = (u32)std::max<u64>(ctx->group_region_cap / 4, 64);
            while (!overflow && nleft > 0) {
                if (rcap > (1u << 22)) return set_err(ctx, FFG_ERR_STATE, "Majorana orbit group larger than 2^22 terms");
                const u32 grid = std::min<u32>(nleft, (u32)ctx->num_sms);
                const u64 region = mtable_bytes<KW>(rcap);
                rc = ensure_buf(ctx, ctx->bigpool, region * grid);
                if (rc) return rc;
                CK(cudaMemsetAsync(nretry + 1, 0, 4, ctx->stream));
                {
                    PhaseScope ps(ctx, PH_ROT);
                    morbit_block<KW, 1024, false><<<grid, 1024, 0, ctx->stream>>>(
                        cur.v, dst.v, sc, oc, a, rcap, ctx->bigpool.p, region, list, nleft, nullptr, other, nretry + 1);
                    OSTEP("morbit_block");
                    ctx->prof.kernel_launches++;
                }
                u32 hr = 0;
                CK(cudaMemcpyAsync(ctx->h_oc, oc, sizeof(OrbitCounters), cudaMemcpyDeviceToHost, ctx->stream));
                CK(cudaMemcpyAsync(&hr, nretry + 1, 4, cudaMemcpyDeviceToHost, ctx->stream));
                CK(cudaStreamSynchronize(ctx->stream));
                ctx->prof.syncs++;
                overflow = (ctx->h_oc->overflow & 1u) != 0;
                std::swap(list, other);
                nleft = hr;
                rcap *= 4;
            }
            const OrbitCounters oc_h = *ctx->h_oc;
            if (overflow) {
                out_cap = pow2_at_least(oc_h.n_out + oc_h.n_out / 4 + 1024);
                ctx->prof.regrows++;
                continue;
            }
            ctx->prof.orbit_batches++;
            ctx->prof.orbit_groups += oc_h.ngroups;
            ctx->prof.orbit_fallbacks += oc_h.nbig;
            cur = dst;
            cap = out_cap;
            active = 1 - active;
            index_valid = false;
            DevCounters h = *ctx->h_ctr;
            h.apps += oc_h.xapps;
            h.emits += oc_h.emits;
            if (oc_h.n_out > h.peak) h.peak = oc_h.n_out;
            h.n = oc_h.n_out;
            h.alive = oc_h.n_out;
            *ctx->h_ctr = h;
            CK(cudaMemcpyAsync(ctx->d_ctr, ctx->h_ctr, sizeof(DevCounters), cudaMemcpyHostToDevice, ctx->stream));
            return FFG_OK;
        }
        return set_err(ctx, FFG_ERR_STATE, "Majorana orbit batch: output store kept overflowing");
    }

    // Majorana circuit: commuting runs (gate ranges, application order) of at
    // least morbit_min_gates gates go through the orbit path, the rest (and
    // the first gate, so that every run starts from thresholded terms)
    // through the persistent per-gate kernel.
    int run_majorana(const std::vector<Op>& ops, const std::vector<RotArgs>& rots,
                     const std::vector<TruncArgs>& truncs, const std::vector<std::pair<int, int>>& runs,
                     int maxdeg) {
        int rc = prepare_persistent(ops, rots, truncs, {});
        if (rc) return rc;
        rc = upload_mgates(rots);
        if (rc) return rc;
        const bool thr = !truncs.empty() && truncs[0].thr;
        const size_t opg = thr ? 2 : 1;  // ops per gate: the rotation, then the threshold
        const TruncArgs t = thr ? truncs[0] : TruncArgs{};
        size_t p0 = 0, p1 = 0;           // pending persistent ops [p0, p1)
        auto flush = [&]() -> int {
            int r = FFG_OK;
            if (p1 > p0) r = exec_persistent(p0, p1);
            p0 = p1;
            return r;
        };
        for (const auto& run : runs) {
            int g = run.first;
            const int g1 = run.second;
            if (g == 0) g = 1;  // the first gate runs per gate (it also thresholds the input)
            if (g1 - g < ctx->morbit_min_gates) {
                p1 = (size_t)g1 * opg;
                continue;
            }
            p1 = (size_t)g * opg;
            rc = flush();
            if (rc) return rc;
            if (ctx->h_ctr->n != ctx->h_ctr->alive) {
                rc = compact_into(1 - active, cap);
                if (rc) return rc;
                rc = sync_counters();
                if (rc) return rc;
            }
            for (int done = g; done < g1;) {
                const int k = std::min(kMaxBatchGates, g1 - done);
                rc = exec_morbit_batch(done, k, t, maxdeg);
                if (rc) return rc;
                done += k;
            }
            p0 = p1 = (size_t)g1 * opg;
        }
        p1 = ops.size();
        rc = flush();
        if (rc) return rc;
        return finish();
    }

    // Batch gate table (one entry per GROUP op, in op order); gate_of_op maps an
    // op index to its entry.
    int upload_batch_gates(const std::vector<Op>& ops, const std::vector<GArgs>& groups,
                           std::vector<int>& gate_of_op) {
        std::vector<BatchGate> bg;
        gate_of_op.assign(ops.size(), -1);
        for (size_t o = 0; o < ops.size(); o++) {
            if (ops[o].type != Op::GROUP) continue;
            const GArgs& ga = groups[ops[o].idx];
            BatchGate b{};
            for (int w = 0; w < 4; w++) b.p[w] = ga.psub[1][w];
            b.c = ga.c[0];
            b.s = ga.s[0];
            b.yP = ga.yP[0];
            b.gidx = group_gate && ops[o].idx < (int)group_gate->size() ? (*group_gate)[ops[o].idx] : -1;
            gate_of_op[o] = (int)bg.size();
            bg.push_back(b);
        }
        h_bgates = bg;
        return upload(ctx->d_bgates, ctx->bgates_cap, bg);
    }

    std::vector<BatchGate> h_bgates;  // host copy of the batch gate table

    // qubit -> gate index of batch gates [g0, g0 + k) (layout of OrbitBatchArgs::qidx)
    void build_qidx(int g0, int k, std::vector<u32>& out) const {
        std::vector<std::vector<u32>> lists(128);
        for (int t = 0; t < k; t++) {
            const BatchGate& G = h_bgates[g0 + t];
            for (int w = 0; w < NW; w++) {
                u64 sup = G.p[w] | G.p[NW + w];
                while (sup) {
                    const int q = 64 * w + __builtin_ctzll(sup);
                    sup &= sup - 1;
                    lists[q].push_back((u32)t);
                }
            }
        }
        const size_t base = out.size();
        out.resize(base + 129);
        u32 e = 0;
        for (int q = 0; q < 128; q++) {
            out[base + q] = e;
            e += (u32)lists[q].size();
        }
        out[base + 128] = e;
        for (int q = 0; q < 128; q++) out.insert(out.end(), lists[q].begin(), lists[q].end());
    }

    // ---------------------------------------------------------------------
    // batched instances: the op list as a list of steps (AdjRecord)
    // ---------------------------------------------------------------------
    // Splits the schedule into steps: Clifford ranges between commuting runs
    // and orbit batches (every run goes through the orbit path).
    static int build_records(const std::vector<Op>& ops, const std::vector<TruncArgs>& truncs,
                             const std::vector<BatchInfo>& batches, const std::vector<int>& gate_of_op,
                             std::vector<AdjRecord>& recs, std::string& err) {
        recs.clear();
        size_t pos = 0;
        auto cliff = [&](size_t a, size_t b) -> bool {
            for (size_t o = a; o < b; o++)
                if (ops[o].type != Op::CLIFF) {
                    err = "batched propagation: unexpected op outside a commuting run";
                    return false;
                }
            if (a < b) {
                AdjRecord r{};
                r.type = AdjRecord::CLIFF;
                r.op_begin = a;
                r.op_end = b;
                recs.push_back(r);
            }
            return true;
        };
        for (const BatchInfo& b : batches) {
            if (b.trunc >= 0 && ops[b.trunc].topk > 0) {
                err = "batched propagation does not support top-k truncation";
                return -1;
            }
            const size_t end = b.trunc >= 0 ? (size_t)b.trunc + 1 : (size_t)(b.first + b.nrot);
            if (!cliff(pos, (size_t)b.first)) return -1;
            int done = 0;
            while (done < b.nrot) {
                const int k = std::min(kMaxBatchGates, b.nrot - done);
                AdjRecord r{};
                r.type = AdjRecord::ORBIT;
                r.g0 = gate_of_op[b.first + done];
                r.k = k;
                if (done + k == b.nrot && b.trunc >= 0) {
                    r.has_trunc = true;
                    r.trunc = truncs[ops[b.trunc].idx];
                }
                recs.push_back(r);
                done += k;
            }
            pos = end;
        }
        if (!cliff(pos, ops.size())) return -1;
        return 0;
    }

    // Copies the current (dense) store into a checkpoint of the step.
    int snapshot(AdjRecord& r) {
        const u64 n = ctx->h_ctr->n;
        if (n != ctx->h_ctr->alive) return set_err(ctx, FFG_ERR_STATE, "batched propagation: sparse store at a step");
        r.n_in = n;
        const size_t m = std::max<u64>(n, 1);
        CK(cudaMalloc(&r.key, (size_t)KW * m * 8));
        CK(cudaMalloc(&r.re, m * 8));
        for (int w = 0; w < KW; w++)
            CK(cudaMemcpyAsync(r.key + (size_t)w * n, cur.v.key + (size_t)w * cap, n * 8, cudaMemcpyDeviceToDevice,
                               ctx->stream));
        CK(cudaMemcpyAsync(r.re, cur.v.re, n * 8, cudaMemcpyDeviceToDevice, ctx->stream));
        return FFG_OK;
    }

    // Loads a checkpoint (store planes, dense) as the live store.
    int restore(const AdjRecord& r) {
        const u64 n = r.n_in;
        cap = pow2_at_least(std::max<u64>((u64)n * 4, ctx->min_capacity));
        int rc = ensure_buf(ctx, ctx->buf[0], store_bytes(KW, CPLX, cap));
        if (rc) return rc;
        active = 0;
        cur = carve(ctx->buf[0], KW, CPLX, cap);
        for (int w = 0; w < KW; w++)
            CK(cudaMemcpyAsync(cur.v.key + (size_t)w * cap, r.key + (size_t)w * n, n * 8, cudaMemcpyDeviceToDevice,
                               ctx->stream));
        CK(cudaMemcpyAsync(cur.v.re, r.re, n * 8, cudaMemcpyDeviceToDevice, ctx->stream));
        CK(cudaMemsetAsync(cur.v.dead, 0, cap, ctx->stream));
        DevCounters h = *ctx->h_ctr;
        h.n = n;
        h.alive = n;
        h.overflow = 0;
        h.error = 0;
        *ctx->h_ctr = h;
        CK(cudaMemcpyAsync(ctx->d_ctr, ctx->h_ctr, sizeof(DevCounters), cudaMemcpyHostToDevice, ctx->stream));
        reindex(cur, 0);
        index_valid = true;
        return sync_counters();
    }

    // Runs one step forward on the live store.
    int exec_record(const AdjRecord& r, int maxdeg) {
        if (r.type == AdjRecord::CLIFF) {
            int rc = exec_persistent(r.op_begin, r.op_end);
            if (!rc) rc = sync_counters();
            return rc;
        }
        const OrbitJob job{r.g0, r.k, r.has_trunc ? &r.trunc : nullptr};
        return exec_orbit_window(&job, 1, maxdeg);
    }

    // Pauli batched runs: long commuting runs go through the batch-orbit path,
    // everything else through persistent per-gate runs.
    int run_mixed(const std::vector<Op>& ops, const std::vector<RotArgs>& rots,
                  const std::vector<TruncArgs>& truncs, const std::vector<GArgs>& groups,
                  const std::vector<BatchInfo>& batches, int maxdeg) {
        int rc = prepare_persistent(ops, rots, truncs, groups);
        if (rc) return rc;
        std::vector<int> gate_of_op;
        rc = upload_batch_gates(ops, groups, gate_of_op);
        if (rc) return rc;
        size_t pos = 0;  // next op to execute
        std::vector<OrbitJob> jobs;  // consecutive orbit batches not yet run
        auto flush = [&]() -> int {
            if (jobs.empty()) return FFG_OK;
            const int r = exec_orbit_window(jobs.data(), (int)jobs.size(), maxdeg);
            jobs.clear();
            return r;
        };
        for (const BatchInfo& b : batches) {
            if (b.nrot < ctx->orbit_min_gates) continue;
            const int end = b.trunc >= 0 ? b.trunc + 1 : b.first + b.nrot;
            if (b.trunc >= 0 && ops[b.trunc].topk > 0) continue;
            // ops before this batch go through the persistent kernel
            if (pos < (size_t)b.first) {
                rc = flush();
                if (rc) return rc;
                rc = exec_persistent(pos, b.first);
                if (rc) return rc;
                // the orbit path reads a dense store (the host counters are
                // current after a persistent run)
                if (ctx->h_ctr->n != ctx->h_ctr->alive) {
                    rc = compact_into(1 - active, cap);
                    if (rc) return rc;
                    rc = sync_counters();
                    if (rc) return rc;
                }
            }
            // runs longer than the batch gate limit are split
            for (int done = 0; done < b.nrot;) {
                const int k = std::min(kMaxBatchGates, b.nrot - done);
                const bool last = done + k == b.nrot;
                jobs.push_back({gate_of_op[b.first + done], k, (last && b.trunc >= 0) ? &truncs[ops[b.trunc].idx] : nullptr});
                done += k;
            }
            pos = end;
        }
        rc = flush();
        if (rc) return rc;
        if (pos < ops.size()) {
            rc = exec_persistent(pos, ops.size());
            if (rc) return rc;
        }
        return finish();
    }

    int extract(ffg_result** out, int kind, bool deterministic) {
        const u64 n = ctx->h_ctr->n;
        ffg_result* r = new ffg_result();
        r->kind = kind;
        r->nplanes = KW;
        r->cplx = CPLX;
        r->n = n;
        r->ctx = ctx;
        r->deterministic = deterministic;
        r->device = ctx->device;
        const size_t m = std::max<u64>(n, 1);
        cudaError_t e = cudaMalloc(&r->key, (size_t)KW * m * 8);
        if (e == cudaSuccess) e = cudaMalloc(&r->re, m * 8);
        if (e == cudaSuccess && CPLX) e = cudaMalloc(&r->im, m * 8);
        if (e == cudaSuccess) e = cudaMalloc(&r->dead, m);
        if (e != cudaSuccess) {
            ffg_result_free(r);
            return set_err(ctx, FFG_ERR_CUDA, std::string("result allocation: ") + cudaGetErrorString(e));
        }
        for (int w = 0; w < KW; w++)
            CK(cudaMemcpyAsync(r->key + (size_t)w * n, cur.v.key + (size_t)w * cap, n * 8,
                               cudaMemcpyDeviceToDevice, ctx->stream));
        CK(cudaMemcpyAsync(r->re, cur.v.re, n * 8, cudaMemcpyDeviceToDevice, ctx->stream));
        if (CPLX) CK(cudaMemcpyAsync(r->im, cur.v.im, n * 8, cudaMemcpyDeviceToDevice, ctx->stream));
        CK(cudaMemsetAsync(r->dead, 0, m, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        *out = r;
        return FFG_OK;
    }
};

// ---------------------------------------------------------------------------
// schedule construction
// ---------------------------------------------------------------------------
bool pauli_commute(const ffg_pauli_gate& a, const ffg_pauli_gate& b) {
    int p = popc64(a.x[0] & b.z[0]) + popc64(a.x[1] & b.z[1]);
    int q = popc64(a.z[0] & b.x[0]) + popc64(a.z[1] & b.x[1]);
    return (p & 1) == (q & 1);
}

// Builds the op list; returns the batch sizes through `batches` when non-null.
// GF(2) independence of the group's axes (x and z words as one 256-bit vector)
struct Basis {
    u64 v[kGroupD][4];
    int piv[kGroupD];
    int n = 0;
    bool add(const u64* w4) {
        u64 r[4] = {w4[0], w4[1], w4[2], w4[3]};
        for (int b = 0; b < n; b++)
            if ((r[piv[b] >> 6] >> (piv[b] & 63)) & 1ull)
                for (int k = 0; k < 4; k++) r[k] ^= v[b][k];
        int p = -1;
        for (int k = 0; k < 4 && p < 0; k++)
            if (r[k]) p = 64 * k + __builtin_ctzll(r[k]);
        if (p < 0) return false;
        for (int k = 0; k < 4; k++) v[n][k] = r[k];
        piv[n++] = p;
        return true;
    }
};

// Splits a run of rotations (application order) into fused groups.
void add_groups(const ffg_pauli_gate* g, const std::vector<size_t>& run, const ffg_pauli_params& p,
                int nw, int dmax, std::vector<Op>& ops, std::vector<GArgs>& groups) {
    size_t s = 0;
    while (s < run.size()) {
        Basis B;
        size_t e = s;
        while (e < run.size() && (int)(e - s) < dmax) {
            const ffg_pauli_gate& G = g[run[e]];
            const u64 w4[4] = {G.x[0], G.x[1], G.z[0], G.z[1]};
            if (!B.add(w4)) break;
            e++;
        }
        if (e == s) e = s + 1;  // an identity axis: a group of its own
        GArgs a{};
        a.ng = (int)(e - s);
        a.maxdeg = p.maxdegree;
        u64 axes[kGroupD][4] = {};
        for (int t = 0; t < a.ng; t++) {
            const ffg_pauli_gate& G = g[run[s + t]];
            for (int w = 0; w < nw; w++) {
                axes[t][w] = G.x[w];
                axes[t][nw + w] = G.z[w];
            }
            a.c[t] = std::cos(G.theta);
            a.s[t] = std::sin(G.theta);
            a.yP[t] = popc64(G.x[0] & G.z[0]) + popc64(G.x[1] & G.z[1]);
        }
        for (int m = 0; m < (1 << kGroupD); m++)
            for (int w = 0; w < 4; w++) {
                u64 x = 0;
                for (int t = 0; t < a.ng; t++)
                    if ((m >> t) & 1) x ^= axes[t][w];
                a.psub[m][w] = x;
            }
        u32 need = 0;
        for (int t = 0; t < a.ng; t++)
            for (int w = 0; w < nw; w++) {
                if (axes[t][nw + w]) need |= 1u << w;          // z_P -> x_Q plane
                if (axes[t][w]) need |= 1u << (nw + w);        // x_P -> z_Q plane
            }
        a.need = need;
        groups.push_back(a);
        ops.push_back({Op::GROUP, (int)groups.size() - 1, 0, 0, 0});
        s = e;
    }
}

void build_pauli_ops(const ffg_pauli_gate* g, size_t ng, const ffg_pauli_params& p, int nw,
                     std::vector<Op>& ops, std::vector<RotArgs>& rots, std::vector<TruncArgs>& truncs,
                     std::vector<int64_t>* batches, std::vector<GArgs>* groups = nullptr,
                     int dmax = kGroupD, std::vector<BatchInfo>* binfo = nullptr,
                     std::vector<int>* rot_gates = nullptr) {
    // rot_gates: circuit index of every rotation in application order (with
    // dmax = 1 its position is the index of the rotation's group)
    int rot_count = 0;
    auto add_rot = [&](size_t i) {
        RotArgs a{};
        const ffg_pauli_gate& G = g[i];
        for (int w = 0; w < nw; w++) {
            a.p[w] = G.x[w];
            a.p[nw + w] = G.z[w];
        }
        a.c = std::cos(G.theta);
        a.s = std::sin(G.theta);
        a.maxdeg = p.maxdegree;
        a.yP = popc64(G.x[0] & G.z[0]) + popc64(G.x[1] & G.z[1]);
        rots.push_back(a);
        ops.push_back({Op::ROT, (int)rots.size() - 1, 0, 0, 0});
    };
    auto add_trunc = [&](int rc) {
        TruncArgs t{};
        t.thr = p.mincoeff > 0;
        t.tau = p.mincoeff;
        t.max_xweight = (p.max_xweight >= 0 && p.xtrunc_period > 0 && (rc + 1) % p.xtrunc_period == 0)
                            ? p.max_xweight
                            : -1;
        const int tk = p.topk > 0 ? p.topk : 0;
        if (!t.thr && t.max_xweight < 0 && tk == 0) return;
        truncs.push_back(t);
        ops.push_back({Op::TRUNC, (int)truncs.size() - 1, 0, 0, tk});
    };
    auto add_cliff = [&](long long begin, long long end) {
        ops.push_back({Op::CLIFF, 0, (int)begin, (int)end, 0});
    };
    long long cb = 0;
    bool pending = false;
    if (!p.batched) {
        for (long long i = (long long)ng - 1; i >= 0; i--) {
            if (g[i].kind != FFG_ROT) {
                if (!pending) {
                    cb = i;
                    pending = true;
                }
            } else {
                if (pending) {
                    add_cliff(i + 1, cb + 1);
                    pending = false;
                }
                const int first = (int)ops.size();
                if (groups)
                    add_groups(g, std::vector<size_t>{(size_t)i}, p, nw, dmax, ops, *groups);
                else
                    add_rot((size_t)i);
                if (rot_gates) rot_gates->push_back((int)i);
                const int nrot = (int)ops.size() - first;
                if (batches) batches->push_back(1);
                const size_t before = ops.size();
                add_trunc(rot_count);
                if (binfo) binfo->push_back({first, nrot, ops.size() > before ? (int)before : -1});
                rot_count++;
            }
        }
    } else {
        std::vector<size_t> buf;
        auto flush = [&]() {
            size_t s = 0;
            while (s < buf.size()) {
                size_t e = s + 1;
                while (e < buf.size()) {
                    bool ok = true;
                    for (size_t t = s; t < e && ok; t++)
                        if (!pauli_commute(g[buf[e]], g[buf[t]])) ok = false;
                    if (!ok) break;
                    e++;
                }
                const int first = (int)ops.size();
                if (groups)
                    add_groups(g, std::vector<size_t>(buf.begin() + s, buf.begin() + e), p, nw, dmax,
                               ops, *groups);
                else
                    for (size_t t = s; t < e; t++) add_rot(buf[t]);
                if (rot_gates)
                    for (size_t t = s; t < e; t++) rot_gates->push_back((int)buf[t]);
                const int nrot = (int)ops.size() - first;
                if (batches) batches->push_back((int64_t)(e - s));
                rot_count += (int)(e - s);
                const size_t before = ops.size();
                add_trunc(rot_count - 1);
                if (binfo) binfo->push_back({first, nrot, ops.size() > before ? (int)before : -1});
                s = e;
            }
            buf.clear();
        };
        for (long long i = (long long)ng - 1; i >= 0; i--) {
            if (g[i].kind != FFG_ROT) {
                flush();
                if (!pending) {
                    cb = i;
                    pending = true;
                }
            } else {
                if (pending) {
                    add_cliff(i + 1, cb + 1);
                    pending = false;
                }
                buf.push_back((size_t)i);
            }
        }
        flush();
    }
    if (pending) add_cliff(0, cb + 1);
}

// suffix-parity mask: bit t = parity of #{s in S : s > t}
void suffix_parity(const uint64_t* alpha, u64* mg) {
    int par = 0;
    u64 out[4] = {0, 0, 0, 0};
    for (int t = 255; t >= 0; t--) {
        if (par) out[t >> 6] |= 1ull << (t & 63);
        if ((alpha[t >> 6] >> (t & 63)) & 1ull) par ^= 1;
    }
    for (int w = 0; w < 4; w++) mg[w] = out[w];
}

template <int KW, bool CPLX, bool PAULI>
int run_engine(ffg_ctx* ctx, const uint64_t* keys, const double* re, const double* im, size_t n,
               int on_device, const std::vector<Op>& ops, const std::vector<RotArgs>& rots,
               const std::vector<TruncArgs>& truncs, const std::vector<GArgs>& groups,
               bool deterministic, ffg_result** out, const std::vector<BatchInfo>* binfo = nullptr,
               int maxdeg = 128, const std::vector<std::pair<int, int>>* mruns = nullptr,
               const std::vector<int>* rot_gates = nullptr) {
    Engine<KW, CPLX, PAULI> E(ctx);
    E.group_gate = rot_gates;
    int rc = E.load(keys, re, im, n, on_device, 0);
    if (rc) return rc;
    bool has_topk = false;
    for (const Op& o : ops) has_topk = has_topk || (o.type == Op::TRUNC && o.topk > 0);
    if (!PAULI && mruns && ctx->morbit && ctx->persistent)
        rc = E.run_majorana(ops, rots, truncs, *mruns, maxdeg);
    else if (PAULI && ctx->merge_sort && ctx->group_d == 1)
        rc = E.run_sortmerge(ops, truncs, groups);
    else if (has_topk)
        rc = E.run(ops, rots, truncs, groups);
    else if (PAULI && binfo && ctx->orbit && ctx->persistent && ctx->group_d == 1)
        rc = E.run_mixed(ops, rots, truncs, groups, *binfo, maxdeg);
    else if (ctx->persistent && ctx->group_d <= 2)
        rc = E.run_persistent(ops, rots, truncs, groups);
    else
        rc = E.run(ops, rots, truncs, groups);
    if (rc) return rc;
    ctx->prof.apps = (int64_t)ctx->h_ctr->apps;
    ctx->prof.emits = (int64_t)ctx->h_ctr->emits;
    ctx->prof.peak_terms = (int64_t)ctx->h_ctr->peak;
    ctx->prof.final_terms = (int64_t)ctx->h_ctr->n;
    return E.extract(out, PAULI ? 1 : 2, deterministic);
}

void reset_profile(ffg_ctx* ctx) {
    ctx->prof = ffg_profile{};
}

int upload_cliffords(ffg_ctx* ctx, const ffg_pauli_gate* g, size_t ng) {
    if (ctx->cliff_cap < ng) {
        if (ctx->d_cliff) CK(cudaFree(ctx->d_cliff));
        ctx->cliff_cap = std::max<size_t>(ng, 256);
        CK(cudaMalloc(&ctx->d_cliff, ctx->cliff_cap * sizeof(CliffordOp)));
    }
    std::vector<CliffordOp> h(ng);
    for (size_t i = 0; i < ng; i++) h[i] = {g[i].kind, g[i].q0, g[i].q1, 0};
    if (ng) CK(cudaMemcpyAsync(ctx->d_cliff, h.data(), ng * sizeof(CliffordOp), cudaMemcpyHostToDevice,
                               ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return FFG_OK;
}


void free_record(AdjRecord& r) {
    if (r.key) cudaFree(r.key);
    if (r.re) cudaFree(r.re);
    r.key = nullptr;
    r.re = nullptr;
}

// Forward pass of a batched propagation on encoded keys (caller layout).
template <int KW>
int batch_forward(ffg_batch* h, const uint64_t* keys, const double* re, size_t n, double* expect) {
    ffg_ctx* ctx = h->ctx;
    Engine<KW, false, true> E(ctx);
    int rc = E.load(keys, re, nullptr, n, 0, 0);
    if (rc) return rc;
    rc = E.prepare_persistent(h->ops, h->rots, h->truncs, h->groups);
    if (rc) return rc;
    std::vector<int> gate_of_op;
    rc = E.upload_batch_gates(h->ops, h->groups, gate_of_op);
    if (rc) return rc;
    std::string err;
    if (E.build_records(h->ops, h->truncs, h->binfo, gate_of_op, h->recs, err)) return set_err(ctx, FFG_ERR_ARG, err);
    ctx->batch = &h->bc;
    if (h->every > 0) {
        for (size_t r = 0; r < h->recs.size() && !rc; r++) {
            if (r % (size_t)h->every == 0) rc = E.snapshot(h->recs[r]);
            if (!rc) {
                h->recs[r].n_in = ctx->h_ctr->n;
                rc = E.exec_record(h->recs[r], h->maxdeg);
            }
        }
    } else {
        // no adjoint: consecutive orbit batches run in windows (one host round
        // trip per window), Clifford ranges through the persistent kernel
        std::vector<typename Engine<KW, false, true>::OrbitJob> jobs;
        auto flush = [&]() {
            int r2 = FFG_OK;
            if (!jobs.empty()) r2 = E.exec_orbit_window(jobs.data(), (int)jobs.size(), h->maxdeg);
            jobs.clear();
            return r2;
        };
        for (size_t r = 0; r < h->recs.size() && !rc; r++) {
            const AdjRecord& rec = h->recs[r];
            if (rec.type == AdjRecord::ORBIT) {
                jobs.push_back({rec.g0, rec.k, rec.has_trunc ? &rec.trunc : nullptr});
            } else {
                rc = flush();
                if (!rc) rc = E.exec_record(rec, h->maxdeg);
            }
        }
        if (!rc) rc = flush();
    }
    if (!rc) rc = E.finish();
    ctx->batch = nullptr;
    if (rc) return rc;
    ctx->prof.apps = (int64_t)ctx->h_ctr->apps;
    ctx->prof.emits = (int64_t)ctx->h_ctr->emits;
    ctx->prof.peak_terms = (int64_t)ctx->h_ctr->peak;
    ctx->prof.final_terms = (int64_t)ctx->h_ctr->n;
    // keep the final term set
    const u64 fn = ctx->h_ctr->n;
    const size_t m = std::max<u64>(fn, 1);
    h->fn = fn;
    CK(cudaMalloc(&h->fkey, (size_t)KW * m * 8));
    CK(cudaMalloc(&h->fre, m * 8));
    for (int w = 0; w < KW; w++)
        CK(cudaMemcpyAsync(h->fkey + (size_t)w * fn, E.cur.v.key + (size_t)w * E.cap, fn * 8,
                           cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaMemcpyAsync(h->fre, E.cur.v.re, fn * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    // per-instance <0|O|0>
    double* d_exp = nullptr;
    CK(cudaMalloc(&d_exp, h->ninst * 8));
    CK(cudaMemsetAsync(d_exp, 0, h->ninst * 8, ctx->stream));
    if (fn) {
        StoreView v{};
        v.key = h->fkey;
        v.re = h->fre;
        v.cap = fn;
        batch_expect<KW / 2><<<grid_for(ctx, fn), kBlock, 0, ctx->stream>>>(
            v, fn, h->xmask[0], h->xmask[1], h->bc.inst_plane, h->bc.inst_shift, h->bc.inst_mask, d_exp, nullptr,
            nullptr);
        ctx->prof.kernel_launches++;
    }
    cudaError_t e = cudaMemcpyAsync(expect, d_exp, h->ninst * 8, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(d_exp);
    if (e != cudaSuccess) return set_err(ctx, FFG_ERR_CUDA, cudaGetErrorString(e));
    return FFG_OK;
}

// Device buffers of the backward pass.
struct AdjBufs {
    double* abar_out = nullptr;
    u64* slots_out = nullptr;
    size_t slots_out_n = 0;
    double* abar_in = nullptr;
    u64* slots_in = nullptr;
    size_t slots_in_n = 0;
    double* grad = nullptr;
    double* w = nullptr;
    int2* segs = nullptr;
    u32* err = nullptr;
    ~AdjBufs() {
        for (void* p : {(void*)abar_out, (void*)slots_out, (void*)abar_in, (void*)slots_in, (void*)grad, (void*)w,
                        (void*)segs, (void*)err})
            if (p) cudaFree(p);
    }
};

// Index over a dense term set (kw planes of n keys, stride n) in `slots`.
template <int KW>
int index_dense(ffg_ctx* ctx, StoreView& v, u64*& slots, size_t& slots_n, u32* err) {
    const u64 n = v.cap;
    const size_t need = 2 * pow2_at_least(std::max<u64>(n, 16));
    if (slots_n < need) {
        if (slots) CK(cudaFree(slots));
        slots = nullptr;
        CK(cudaMalloc(&slots, need * 8));
        slots_n = need;
    }
    v.slots = slots;
    v.hmask = need - 1;
    clear_slots_kernel<<<grid_for(ctx, need), kBlock, 0, ctx->stream>>>(slots, need);
    if (n) adj_index<KW><<<grid_for(ctx, n), kBlock, 0, ctx->stream>>>(v, n, err);
    CK(cudaGetLastError());
    return FFG_OK;
}

template <int KW>
int batch_adjoint(ffg_batch* h, const double* weights, double* grad_theta, double* grad_coef) {
    constexpr int NW = KW / 2;
    ffg_ctx* ctx = h->ctx;
    CK(cudaSetDevice(ctx->device));
    if (h->every <= 0) return set_err(ctx, FFG_ERR_ARG, "the propagation kept no checkpoints (checkpoint_every = 0)");
    Engine<KW, false, true> E(ctx);
    int rc = upload_cliffords(ctx, h->gates.data(), h->gates.size());
    if (rc) return rc;
    rc = E.prepare_persistent(h->ops, h->rots, h->truncs, h->groups);
    if (rc) return rc;
    std::vector<int> gate_of_op;
    rc = E.upload_batch_gates(h->ops, h->groups, gate_of_op);
    if (rc) return rc;
    const size_t ninst = h->ninst;
    size_t nbg = 0;
    for (const Op& o : h->ops) nbg += o.type == Op::GROUP;
    AdjBufs B;
    CK(cudaMalloc(&B.err, 8));
    CK(cudaMemsetAsync(B.err, 0, 8, ctx->stream));
    CK(cudaMalloc(&B.w, ninst * 8));
    CK(cudaMemcpyAsync(B.w, weights, ninst * 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMalloc(&B.grad, std::max<size_t>(nbg * ninst, 1) * 8));
    CK(cudaMemsetAsync(B.grad, 0, std::max<size_t>(nbg * ninst, 1) * 8, ctx->stream));
    // abar of the final term set
    StoreView out{};
    out.key = h->fkey;
    out.re = h->fre;
    out.cap = h->fn;
    // abar buffers sized once for the largest term set of any step
    u64 nmax = std::max<u64>(h->fn, 1);
    for (const AdjRecord& q : h->recs) nmax = std::max<u64>(nmax, q.n_in);
    CK(cudaMalloc(&B.abar_out, nmax * 8));
    CK(cudaMalloc(&B.abar_in, nmax * 8));
    rc = index_dense<KW>(ctx, out, B.slots_out, B.slots_out_n, B.err);
    if (rc) return rc;
    if (h->fn)
        batch_expect<NW><<<grid_for(ctx, h->fn), kBlock, 0, ctx->stream>>>(
            out, h->fn, h->xmask[0], h->xmask[1], h->bc.inst_plane, h->bc.inst_shift, h->bc.inst_mask, nullptr, B.w,
            B.abar_out);
    const size_t warp_smem = (size_t)kAdjWarps * adj_table_bytes<KW>(kAdjWarpCap, kAdjWarpGates);
    CK(cudaFuncSetAttribute(adj_orbit_warp<NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)warp_smem));
    ctx->batch = &h->bc;
    const int R = (int)h->recs.size();
    for (int r = R - 1; r >= 0 && !rc; r--) {
        AdjRecord& rec = h->recs[r];
        if (!rec.key) {
            // recompute the segment from the last checkpoint before r
            int c = r;
            while (c > 0 && !h->recs[c].key) c--;
            if (!h->recs[c].key) return set_err(ctx, FFG_ERR_STATE, "adjoint: no checkpoint before step");
            rc = E.restore(h->recs[c]);
            for (int q = c; q < r && !rc; q++) {
                if (q > c) {
                    rc = E.snapshot(h->recs[q]);
                    h->recs[q].temp = true;
                }
                if (!rc) rc = E.exec_record(h->recs[q], h->maxdeg);
            }
            if (!rc) rc = E.sync_counters();
            if (!rc) {
                rc = E.snapshot(rec);
                rec.temp = true;
            }
            if (rc) break;
        }
        const u64 n_in = rec.n_in;
        StoreView in{};
        in.key = rec.key;
        in.re = rec.re;
        in.cap = n_in;
        if (n_in > nmax) return set_err(ctx, FFG_ERR_STATE, "adjoint: step larger than recorded");
        if (n_in && rec.type == AdjRecord::CLIFF) {
            std::vector<int2> segs;
            for (size_t o = rec.op_begin; o < rec.op_end; o++) segs.push_back(make_int2(h->ops[o].begin, h->ops[o].end));
            CK(cudaMalloc(&B.segs, segs.size() * sizeof(int2)));
            CK(cudaMemcpyAsync(B.segs, segs.data(), segs.size() * sizeof(int2), cudaMemcpyHostToDevice, ctx->stream));
            adj_clifford<NW><<<grid_for(ctx, n_in), kBlock, 0, ctx->stream>>>(
                in, n_in, ctx->d_cliff, B.segs, (int)segs.size(), out, B.abar_out, B.abar_in, B.err);
            CK(cudaGetLastError());
            CK(cudaStreamSynchronize(ctx->stream));
            CK(cudaFree(B.segs));
            B.segs = nullptr;
        } else if (n_in) {
            const u64 cap_in = std::max<u64>(n_in, 1024);
            OrbitScratch sc = E.carve_scratch(cap_in);
            if (!sc.amask) return set_err(ctx, FFG_ERR_CUDA, "adjoint: orbit scratch allocation failed");
            // classification needs an output store for the untouched terms (discarded here)
            const u64 dcap = pow2_at_least(std::max<u64>(n_in, 1024));
            rc = ensure_buf(ctx, ctx->buf[0], store_bytes(KW, false, dcap));
            if (rc) break;
            Store dummy = carve(ctx->buf[0], KW, false, dcap);
            AdjArgs A{};
            OrbitBatchArgs& a = A.a;
            a.gates = ctx->d_bgates + rec.g0;
            a.k = rec.k;
            a.maxdeg = h->maxdeg;
            a.thr = rec.has_trunc ? rec.trunc.thr : 0;
            a.tau = rec.has_trunc ? rec.trunc.tau : 0.0;
            a.max_xweight = rec.has_trunc ? rec.trunc.max_xweight : -1;
            a.route_big = (int)kAdjWarpGates + 1;  // the warp tier takes every group its tables hold
            a.inst_cs = h->bc.d_inst_cs + (size_t)rec.g0 * ninst;
            a.ninst = (u32)ninst;
            a.inst_plane = h->bc.inst_plane;
            a.inst_shift = h->bc.inst_shift;
            a.inst_mask = h->bc.inst_mask;
            A.out = out;
            A.abar_out = B.abar_out;
            A.abar_in = B.abar_in;
            A.grad = B.grad + (size_t)rec.g0 * ninst;
            A.err = B.err;
            const int g = grid_for(ctx, n_in);
            orbit_gate<<<1, 32, 0, ctx->stream>>>(ctx->d_oc, nullptr, n_in, sc.gmask + 1, E.nretry);
            orbit_classify<NW, false><<<g, kBlock, 0, ctx->stream>>>(in, dummy.v, sc, ctx->d_oc, a);
            orbit_group<KW><<<g, kBlock, 0, ctx->stream>>>(sc, ctx->d_oc);
            orbit_offsets<<<g, kBlock, 0, ctx->stream>>>(sc, ctx->d_oc);
            orbit_scatter<KW, false><<<g, kBlock, 0, ctx->stream>>>(in, sc, ctx->d_oc);
            adj_passthrough<KW><<<g, kBlock, 0, ctx->stream>>>(in, n_in, sc, A);
            adj_orbit_warp<NW><<<ctx->num_sms * 2, 32 * kAdjWarps, warp_smem, ctx->stream>>>(in, sc, ctx->d_oc, A);
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(ctx->h_oc, ctx->d_oc, sizeof(OrbitCounters), cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaStreamSynchronize(ctx->stream));
            if (ctx->h_oc->error) return set_err(ctx, FFG_ERR_STATE, "adjoint: orbit grouping index overrun");
            u32 nbig = ctx->h_oc->nbig;
            u32* list = sc.big;
            u32* other = E.retry_list;
            u32 tcap = 4096;
            while (nbig > 0) {
                if (tcap > (1u << 22)) return set_err(ctx, FFG_ERR_STATE, "adjoint: orbit group larger than 2^22 terms");
                const u32 grid = std::min<u32>(nbig, (u32)ctx->num_sms);
                const u64 region = adj_table_bytes<KW>(tcap, (u32)rec.k);
                rc = ensure_buf(ctx, ctx->bigpool, region * grid);
                if (rc) return rc;
                CK(cudaMemsetAsync(E.nretry, 0, 4, ctx->stream));
                adj_orbit_block<NW><<<grid, 1024, 0, ctx->stream>>>(in, sc, A, ctx->bigpool.p, region, tcap,
                                                                    (u32)rec.k, list, nbig, other, E.nretry);
                CK(cudaGetLastError());
                u32 hr = 0;
                CK(cudaMemcpyAsync(&hr, E.nretry, 4, cudaMemcpyDeviceToHost, ctx->stream));
                CK(cudaStreamSynchronize(ctx->stream));
                std::swap(list, other);
                nbig = hr;
                tcap *= 4;
            }
        }
        // this step's input becomes the next step's output side
        rc = index_dense<KW>(ctx, in, B.slots_in, B.slots_in_n, B.err);
        if (rc) break;
        CK(cudaStreamSynchronize(ctx->stream));
        std::swap(B.abar_out, B.abar_in);
        std::swap(B.slots_out, B.slots_in);
        std::swap(B.slots_out_n, B.slots_in_n);
        out = in;
        // recomputed checkpoints after this step are no longer needed (this
        // step's own checkpoint is the output side of the next one)
        for (int q = r + 1; q < R; q++)
            if (h->recs[q].temp) {
                free_record(h->recs[q]);
                h->recs[q].temp = false;
            }
    }
    ctx->batch = nullptr;
    for (AdjRecord& q : h->recs)
        if (q.temp) {
            free_record(q);
            q.temp = false;
        }
    if (rc) return rc;
    u32 herr[2] = {0, 0};
    CK(cudaMemcpy(herr, B.err, 8, cudaMemcpyDeviceToHost));
    if (herr[0] & 2u) return set_err(ctx, FFG_ERR_STATE, "adjoint: index probe overrun");
    if (grad_coef && h->n_input) {
        if (out.cap != h->n_input) return set_err(ctx, FFG_ERR_STATE, "adjoint: input term count mismatch");
        CK(cudaMemcpy(grad_coef, B.abar_out, h->n_input * 8, cudaMemcpyDeviceToHost));
    }
    std::vector<double> g(nbg * ninst);
    if (!g.empty()) CK(cudaMemcpy(g.data(), B.grad, g.size() * 8, cudaMemcpyDeviceToHost));
    // batch gate b is the b-th rotation in application order = rotation nrot-1-b in circuit order
    for (size_t i = 0; i < ninst; i++)
        for (size_t b = 0; b < nbg; b++) grad_theta[i * h->nrot + (h->nrot - 1 - b)] = g[b * ninst + i];
    return FFG_OK;
}

}  // namespace

namespace {
// host copy in caller layout ([4][n]) and, when deterministic, sorted order
int result_to_host(const ffg_result* r, std::vector<uint64_t>& k4, std::vector<double>& re,
                   std::vector<double>& im) {
    ffg_ctx* ctx = r->ctx;
    const size_t n = r->n;
    k4.assign(4 * n, 0);
    re.assign(n, 0.0);
    im.assign(n, 0.0);
    std::vector<uint64_t> planes((size_t)r->nplanes * n);
    if (n) {
        CK(cudaMemcpy(planes.data(), r->key, planes.size() * 8, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(re.data(), r->re, n * 8, cudaMemcpyDeviceToHost));
        if (r->cplx) CK(cudaMemcpy(im.data(), r->im, n * 8, cudaMemcpyDeviceToHost));
    }
    for (int w = 0; w < r->nplanes; w++) {
        int dst = w;
        if (r->kind == 1) {
            const int nw = r->nplanes / 2;
            dst = (w < nw) ? w : 2 + (w - nw);
        }
        std::memcpy(&k4[(size_t)dst * n], &planes[(size_t)w * n], n * 8);
    }
    if (r->deterministic && n > 1) {
        std::vector<size_t> ord(n);
        for (size_t i = 0; i < n; i++) ord[i] = i;
        std::sort(ord.begin(), ord.end(), [&](size_t a, size_t b) {
            for (int w = 0; w < 4; w++)
                if (k4[(size_t)w * n + a] != k4[(size_t)w * n + b]) return k4[(size_t)w * n + a] < k4[(size_t)w * n + b];
            return false;
        });
        std::vector<uint64_t> k2(4 * n);
        std::vector<double> r2(n), i2(n);
        for (size_t t = 0; t < n; t++) {
            for (int w = 0; w < 4; w++) k2[(size_t)w * n + t] = k4[(size_t)w * n + ord[t]];
            r2[t] = re[ord[t]];
            i2[t] = im[ord[t]];
        }
        k4.swap(k2);
        re.swap(r2);
        im.swap(i2);
    }
    return FFG_OK;
}
}  // namespace

