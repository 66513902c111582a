/*
 * ffg.h -- C ABI of libffg, the GB300 (sm_103a) implementation of truncated
 * Heisenberg-picture propagation of Pauli and Majorana polynomials.
 *
 * Plain C: integers, doubles and pointers only; every call returns FFG_OK (0)
 * or a negative status, and ffg_last_error() gives the message.  One context
 * owns one CUDA stream on one device and must not be used from two threads at
 * once.  Device memory is pooled in the context and reused across calls.
 * Results (ffg_result) and batches (ffg_batch) use their context's stream and
 * scratch buffers: free them before destroying that context.
 *
 * Key layout (all entry points): uint64 arrays of shape [4][n] (plane-major).
 *   Pauli:    plane 0 = xory bits of qubits 0..63, plane 1 = xory of 64..127,
 *             plane 2 = yorz bits of qubits 0..63, plane 3 = yorz of 64..127
 *             (I=(0,0) X=(1,0) Y=(1,1) Z=(0,1), src/pauli/algebra.h:30-33)
 *   Majorana: planes 0..3 = bits of Majorana indices 0..255
 *             (src/majorana_algebra.h:30-33)
 * Coefficients: separate re[n] and im[n] arrays of doubles (im may be NULL on
 * input, meaning all-zero imaginary parts).  Input keys must be distinct.
 *
 * Reference interfaces replaced (paths relative to the fastfermion project):
 *   ffg_pauli_propagate     pauli_gates::propagate, src/pauli/propagate.h:297-493,
 *                           as bound in src/python_bind.cpp:392-425
 *   ffg_majorana_propagate  majorana_gates::propagate, src/majorana_propagation.h:35-55,
 *                           as bound in src/python_bind.cpp:490-527
 *   ffg_result_overlapwithzero  PauliPolynomial::overlapwithzero, src/pauli/algebra.h:549-557
 *   ffg_result_qubit_state  QubitProductState::operator(), src/qubitproductstate.h:73-88
 *   ffg_result_fock_state   FockState::operator() on Majorana, src/fockstate.h:95-114
 *   ffg_profile_get         prop_profile()/profile_get, src/pauli/propagate.h:34-65,
 *                           src/python_bind.cpp:428-446
 */
#ifndef FFG_H_
#define FFG_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FFG_OK 0
#define FFG_ERR_ARG -1     /* invalid argument (bad gate, duplicate key, ...) */
#define FFG_ERR_CUDA -2    /* CUDA runtime error (no device, out of memory, ...) */
#define FFG_ERR_STATE -3   /* internal consistency check failed */

/* gate kinds of the Pauli circuit table (src/pauli/gates.h:260-269) */
#define FFG_ROT 0
#define FFG_H 1
#define FFG_S 2
#define FFG_CNOT 3
#define FFG_SWAP 4
#define FFG_CZ 5

typedef struct ffg_ctx ffg_ctx;
typedef struct ffg_result ffg_result;

/* One gate of a Pauli circuit, in circuit order (index 0 is applied to the
 * state first, i.e. last in the Heisenberg picture). */
typedef struct {
    int32_t kind;    /* FFG_ROT, FFG_H, FFG_S, FFG_CNOT, FFG_SWAP, FFG_CZ */
    int32_t q0, q1;  /* qubits of a Clifford gate (q1 unused for H and S) */
    int32_t pad;
    uint64_t x[2];   /* ROT axis: xory words */
    uint64_t z[2];   /* ROT axis: yorz words */
    double theta;    /* ROT: U = exp(-i theta/2 P) */
} ffg_pauli_gate;

/* One Majorana rotation U = exp(-i theta/2 * i^r gamma_S)
 * (src/majorana_gates.h:17-60; theta already includes the monomial coefficient). */
typedef struct {
    uint64_t alpha[4];
    double theta;
    int32_t r;       /* 1 when gamma_S is not Hermitian (|S| mod 4 in {2,3}) */
    int32_t pad;
} ffg_majorana_gate;

/* Truncation parameters; the defaults of the reference binding are
 * maxdegree = 128, mincoeff = 0, topk = 0, max_xweight = -1,
 * xtrunc_period = 1, batched = 1 (src/python_bind.cpp:413-416). */
typedef struct {
    int32_t maxdegree;      /* partner filter: emitted strings must have weight <= maxdegree */
    int32_t topk;           /* > 0: keep the topk largest |c| after each truncation point */
    double mincoeff;        /* > 0: erase |c| <= mincoeff */
    int32_t max_xweight;    /* >= 0: erase X/Y weight > max_xweight every xtrunc_period rotations */
    int32_t xtrunc_period;
    int32_t batched;        /* 1: truncate once per maximal run of commuting rotations */
    int32_t deterministic;  /* 1: expectation sums run in sorted-key order */
} ffg_pauli_params;

typedef struct {
    int32_t has_maxdegree;  /* 0: no degree filter */
    int32_t maxdegree;
    double mincoeff;        /* > 0: erase |c| <= mincoeff after every gate */
    int32_t deterministic;
    int32_t pad;
} ffg_majorana_params;

/* Counters and per-phase device times of the most recent propagation. */
typedef struct {
    double seconds_total;     /* wall time of the call */
    double seconds_rotations; /* device time in rotation kernels (profiling on) */
    double seconds_truncate;  /* device time in truncation passes (profiling on) */
    double seconds_clifford;  /* device time in Clifford segments + re-indexing */
    double seconds_compact;   /* device time in compaction + re-indexing */
    double seconds_h2d;       /* host-to-device input transfer */
    double seconds_d2h;       /* device-to-host result transfer (ffg_result_copy) */
    int64_t n_gates;          /* rotation gates applied */
    int64_t apps;             /* sum over rotations of live terms entering the gate */
    int64_t emits;            /* partners emitted that passed the degree filter */
    int64_t peak_terms;       /* largest live-term count after any gate */
    int64_t final_terms;
    int64_t syncs;            /* host synchronisation points */
    int64_t regrows;          /* capacity growths (each replays the pending gates) */
    int64_t compactions;
    int64_t kernel_launches;  /* kernels launched by the propagation */
    int64_t orbit_batches;    /* commuting runs processed orbit by orbit */
    int64_t orbit_fallbacks;  /* groups too large for a warp table (done by the block-level pass) */
    int64_t orbit_groups;     /* groups processed */
    int64_t orbit_max_group;  /* largest group (members) */
} ffg_profile;

/* -------------------------------------------------------------------------- */
int ffg_create(ffg_ctx** ctx, int device);
int ffg_destroy(ffg_ctx* ctx);
const char* ffg_last_error(const ffg_ctx* ctx);
/* 1: record per-phase device times with CUDA events (adds synchronisation). */
int ffg_set_profiling(ffg_ctx* ctx, int enabled);
int ffg_profile_get(const ffg_ctx* ctx, ffg_profile* out);
/* The context's CUDA stream (a cudaStream_t), for callers that time or order
 * work around the library's launches. */
void* ffg_stream(const ffg_ctx* ctx);

/* Engine options (no counterpart in the reference): runtime knobs of the
 * orbit engine, tuned by fastfermion_gb300.autotune.  Names:
 *   orbit_route_big   |A| from which a Pauli group skips the warp tier (default 8)
 *   orbit_team        1: team tier (1024-member tables) before the block tier (1)
 *   orbit_team_threads   threads per team-tier group: 128 or 256 (256)
 *   orbit_block_threads  threads per block-tier group: 512 or 1024 (1024)
 *   orbit_window      orbit batches per host round trip, 1..16 (16)
 *   orbit_min_gates   shortest commuting run sent to the orbit path (4)
 *   orbit_qidx        1: classify against the gates on each term's support (1)
 *   pdl               1: programmatic dependent launch of the orbit kernels (1)
 *   morbit            1: orbit path for commuting Majorana runs (1)
 *   morbit_min_gates  shortest Majorana run sent to the orbit path (2)
 *   morbit_route_big  |A| from which a Majorana group skips the warp tier (12)
 *   merge_sort        1: Pauli rotations one at a time with a radix sort and a
 *                     segmented reduce instead of the hash index / orbit paths (0)
 *   orbit             1: batch-orbit path for commuting Pauli runs (1)
 *   persistent        1: one cooperative launch per run of per-gate ops; 0: one
 *                     launch per op (1)
 *   persist_blocks_per_sm  blocks per SM of the persistent kernel, 1..8 (2)
 *   group_d           rotations fused per pass of the per-gate paths, 1..4 (1)
 *   orbit_stats       1: per-batch group statistics on stderr (0)
 *   min_capacity      smallest term-store capacity, a power of two >= 64 (65536)
 *   store_headroom    orbit windows size their output stores for this many times
 *                     the entering terms, 1..64 (4); a batch that outgrows its
 *                     store runs again after the store grows
 *   barrier_limit_kcycles  thousands of clock cycles a block of the persistent
 *                     kernel waits at a grid barrier before the launch gives up
 *                     and the call returns FFG_ERR_STATE, 1..4000000 (4000000,
 *                     about 2 s); the context stays usable
 *   group_region_cap  members of the first global-memory region of a group too
 *                     large for shared memory, a power of two >= 64 (16384; the
 *                     Majorana path starts at a quarter); regions grow x4 on
 *                     overflow and the group runs again
 * Results do not depend on the options (only speed does). */
int ffg_set_option(ffg_ctx* ctx, const char* name, int64_t value);
int ffg_get_option(const ffg_ctx* ctx, const char* name, int64_t* value);

/* Truncated Heisenberg propagation of a Pauli polynomial through a circuit.
 * keys/re/im are host pointers when on_device == 0, device pointers of the
 * context's device otherwise.  The result stays on the device until copied. */
int ffg_pauli_propagate(ffg_ctx* ctx, const uint64_t* keys, const double* re, const double* im,
                        size_t n, const ffg_pauli_gate* gates, size_t ngates,
                        const ffg_pauli_params* params, int on_device, ffg_result** out);

/* Majorana propagation: gates applied last to first, threshold after every gate. */
int ffg_majorana_propagate(ffg_ctx* ctx, const uint64_t* keys, const double* re, const double* im,
                           size_t n, const ffg_majorana_gate* gates, size_t ngates,
                           const ffg_majorana_params* params, int on_device, ffg_result** out);

/* -------------------------------------------------------------------------- */
size_t ffg_result_size(const ffg_result* r);
/* 1 for a Pauli result, 2 for a Majorana result */
int ffg_result_kind(const ffg_result* r);
/* Copies the terms to host arrays: keys [4][n], re[n], im[n] (im may be NULL).
 * With the deterministic parameter set, terms come sorted lexicographically by
 * (plane 0, plane 1, plane 2, plane 3); otherwise in store order. */
int ffg_result_copy(const ffg_result* r, uint64_t* keys, double* re, double* im);
/* Device pointers of the result (valid until ffg_result_free).  Key plane w of
 * the n entries starts at keys + w * stride, w < *nplanes.  Pauli results use
 * nplanes = 2*NW with the NW xory planes first (NW = 1 when every qubit index
 * is below 64, else 2); Majorana results use one plane per 64 indices.  *im is
 * NULL when the coefficients are real. */
int ffg_result_device(const ffg_result* r, const uint64_t** keys, size_t* stride, int* nplanes,
                      const double** re, const double** im);
int ffg_result_overlapwithzero(const ffg_result* r, double* re, double* im);
int ffg_result_qubit_state(const ffg_result* r, const uint64_t* b /* [2] */, double* re, double* im);
int ffg_result_fock_state(const ffg_result* r, const uint64_t* b /* [2] */, double* re, double* im);
void ffg_result_free(ffg_result* r);

/* -------------------------------------------------------------------------- */
/* Conversions of polynomials, computed on the GPU.
 *
 * ffg_majorana_to_pauli: Jordan-Wigner map of a Majorana polynomial
 * (keys [4][n] Majorana bits, re/im; host or device pointers as in
 * ffg_pauli_propagate) to a Pauli polynomial result; terms whose mapped
 * coefficient is exactly zero are dropped.  Replaces jordan_wigner /
 * majorana_to_pauli, src/transforms.h:124-151, bound as `jw` in
 * src/python_bind.cpp:172-175.
 *
 * ffg_result_sparse: the 2^n x 2^n CSC matrix of a Pauli result (qubit 0 is
 * the most significant bit of the row/column index; qubits >= n are ignored),
 * 0 <= n <= 30.  indptr has 2^n + 1 entries and is always written, with *nnz;
 * indices/data_re/data_im (capacity cap) are written when they are non-NULL
 * and cap >= *nnz (call once with indices = NULL to size them).  Within a
 * column the entries come in increasing order of the bit-reversed X mask, as
 * in the reference.  Replaces PauliPolynomial::sparse, src/pauli/sparse.h:20-131
 * (bound in src/python_bind.cpp:127-140; the fixed-particle-number subspace
 * variant is not provided). */
int ffg_majorana_to_pauli(ffg_ctx* ctx, const uint64_t* keys, const double* re, const double* im, size_t n,
                          int on_device, ffg_result** out);
int ffg_result_sparse(const ffg_result* r, int n, int64_t* indptr, int64_t* indices, double* data_re,
                      double* data_im, size_t cap, size_t* nnz);

/* -------------------------------------------------------------------------- */
/* Batched instances and gradients.  No counterpart in the reference: its
 * propagate runs one observable through one circuit and has no derivatives.
 *
 * ffg_pauli_propagate_batched propagates ninst observables through circuits
 * that share the gate axes and Clifford gates of `gates` but have their own
 * rotation angles, in one term store and one set of launches.  The terms of
 * instance i are keys/re[offsets[i] .. offsets[i+1]) (caller layout [4][n],
 * real coefficients; keys distinct within an instance).  Row i of thetas
 * ([ninst][nrot], nrot = number of FFG_ROT gates, circuit order) holds
 * instance i's angles; thetas == NULL uses gates[].theta for every instance.
 * Truncation follows params exactly as ffg_pauli_propagate would for each
 * instance alone (every instance's term set is bit-identical to that), except
 * that top-k and X-weight truncation are not supported (FFG_ERR_ARG).
 * expect[i] receives <0|O_i|0> (summation order not fixed).
 * checkpoint_every = k >= 1 keeps the term set entering every k-th step
 * (Clifford segment or commuting run) on the device so that
 * ffg_batch_adjoint can run; the steps in between are recomputed during the
 * backward pass.  out may be NULL when no handle is wanted. */
typedef struct ffg_batch ffg_batch;

typedef struct {
    size_t ninst;
    const int64_t* offsets;    /* [ninst + 1], offsets[0] = 0, offsets[ninst] = n */
    const double* thetas;      /* [ninst][nrot] or NULL */
    int32_t checkpoint_every;  /* 0: no adjoint */
    int32_t pad;
} ffg_batch_params;

int ffg_pauli_propagate_batched(ffg_ctx* ctx, const uint64_t* keys, const double* re, size_t n,
                                const ffg_pauli_gate* gates, size_t ngates, const ffg_pauli_params* params,
                                const ffg_batch_params* bparams, double* expect, ffg_batch** out);
/* ffg_pauli_propagate_instances: ffg_pauli_propagate_batched with, in
 * addition, a per-instance choice of the rotations that act.  active is NULL
 * (every rotation acts on every instance) or an array [ninst][W], W =
 * max(1, ceil(nrot / 64)) words: rotation r (the r-th FFG_ROT gate in circuit
 * order) acts on instance i iff bit r % 64 of active[i * W + r / 64] is set.
 * An inactive rotation leaves the instance's terms as they are; Clifford gates
 * act on every instance, and the truncation points are those of the whole
 * circuit (after each commuting run of its rotations), so each instance's term
 * set is that of the whole circuit with its inactive rotations skipped.  Not
 * combinable with the adjoint (checkpoint_every must be 0 when active is set).
 * The learned correction uses it to propagate every dropped partner from the
 * gate that created it, all partners in one launch. */
int ffg_pauli_propagate_instances(ffg_ctx* ctx, const uint64_t* keys, const double* re, size_t n,
                                  const ffg_pauli_gate* gates, size_t ngates, const ffg_pauli_params* params,
                                  const ffg_batch_params* bparams, const uint64_t* active, double* expect,
                                  ffg_batch** out);
/* Terms left over all instances. */
size_t ffg_batch_size(const ffg_batch* b);
/* Final terms: keys [4][n] (caller layout, instance code removed), re[n],
 * inst[n] = instance of each term (may be NULL). */
int ffg_batch_copy(const ffg_batch* b, uint64_t* keys, double* re, int64_t* inst);
/* Reverse-mode derivative of F = sum_i weights[i] <0|O_i|0> with the
 * truncation pattern of the forward pass held fixed:
 * grad_theta[i * nrot + r] = dF / dthetas[i][r]; grad_coef[t] (may be NULL) =
 * dF / d re[t] for the input terms.  Uses the context the handle was made
 * with; may run any number of times. */
int ffg_batch_adjoint(ffg_batch* b, const double* weights, double* grad_theta, double* grad_coef);
void ffg_batch_free(ffg_batch* b);

/* -------------------------------------------------------------------------- */
/* Dropped partners (training data of the learned correction).  No counterpart
 * in the reference, whose conjugate (src/pauli/propagate.h:71-89) discards
 * them.  ffg_pauli_propagate_capture runs ffg_pauli_propagate (batched mode
 * without top-k; the result is identical) and also records every partner that
 * the degree filter drops whose degree is at most capdeg (> maxdegree) and
 * whose |value| exceeds min_abs (min_abs = 0: every one, exact zeros
 * included): its key, its value c (i sin theta) phase(P Q),
 * and the index in gates[] of the rotation that created it (the gates still
 * to be applied to it are gates[0 .. gate)).  Each (key, gate) is recorded
 * once.  *drops stays valid until ffg_drops_free; ffg_drops_copy returns the
 * records sorted by gate, then key (keys [4][n] caller layout). */
typedef struct ffg_drops ffg_drops;
int ffg_pauli_propagate_capture(ffg_ctx* ctx, const uint64_t* keys, const double* re, const double* im,
                                size_t n, const ffg_pauli_gate* gates, size_t ngates,
                                const ffg_pauli_params* params, int on_device, int32_t capdeg, double min_abs,
                                ffg_result** out, ffg_drops** drops);
size_t ffg_drops_size(const ffg_drops* d);
int ffg_drops_copy(const ffg_drops* d, uint64_t* keys, double* re, double* im, int32_t* gate);
/* Device arrays of the records, in no particular order: key plane w at
 * keys + w * stride (stride = size), re, im, gate. */
int ffg_drops_device(const ffg_drops* d, const uint64_t** keys, size_t* stride, const double** re,
                     const double** im, const int32_t** gate);
void ffg_drops_free(ffg_drops* d);

/* -------------------------------------------------------------------------- */
/* Learned truncation correction: the surrogate network and the features of
 * dropped partners.  No counterpart in the reference.
 *
 * The network maps the 32 features of a dropped partner to its transfer t,
 * the value at the end of the circuit of the partner with unit coefficient:
 * 32 -> 128 -> 128 -> 128 -> 1, GELU after each hidden layer.  The three
 * hidden GEMMs run on the tensor cores (tcgen05, BF16 operands, FP32
 * accumulation in tensor memory); the output layer, biases, activations and
 * the optimizer are FP32.  Parameters (FP32, FFG_MLP_NPARAMS values) are laid
 * out as W1[128][32], b1[128], W2[128][128], b2[128], W3[128][128], b3[128],
 * w4[128], b4 (weights as [out][in]).  A network uses its context's stream;
 * create it with the context's device current.  x arrays are device BF16
 * (uint16 bit patterns) [n][32], row-major, 16-byte aligned; target, weight
 * and y are device FP32 [n].  The training loss is
 * L = sum_r weight[r] (y[r] - target[r])^2. */
#define FFG_MLP_IN 32
#define FFG_MLP_HIDDEN 128
#define FFG_MLP_NPARAMS 37377
typedef struct ffg_mlp ffg_mlp;
int ffg_mlp_create(ffg_ctx* ctx, ffg_mlp** out);
void ffg_mlp_free(ffg_mlp* m);
const char* ffg_mlp_last_error(const ffg_mlp* m);
/* Host FP32 parameters in and out (set_params also resets the optimizer). */
int ffg_mlp_set_params(ffg_mlp* m, const float* params);
int ffg_mlp_get_params(const ffg_mlp* m, float* params);
/* y = f(x) for n rows. */
int ffg_mlp_forward(ffg_mlp* m, const uint16_t* x, size_t n, float* y);
/* dL/dparams over n rows into the host array grad, and L (may be NULL). */
int ffg_mlp_gradient(ffg_mlp* m, const uint16_t* x, const float* target, const float* weight, size_t n,
                     float* grad, double* loss);
/* One Adam step on L over n rows; *loss (may be NULL: no synchronisation)
 * receives L before the step. */
int ffg_mlp_adam_step(ffg_mlp* m, const uint16_t* x, const float* target, const float* weight, size_t n,
                      float lr, float beta1, float beta2, float eps, double* loss);
/* Predicted correction sum_r coef[r] t[r] (coef device FP64 [n]); t receives
 * the n transfers. */
int ffg_mlp_correction(ffg_mlp* m, const uint16_t* x, const double* coef, size_t n, float* t, double* out);
/* Set-level targets: rows seg[s] .. seg[s+1] (device int64 [nseg+1], seg[0] =
 * 0, seg[nseg] = n) are the dropped partners of one circuit, whose total
 * correction should be delta[s] (device FP64 [nseg]).  Writes device target and
 * weight [n] such that one ffg_mlp_adam_step on (x, target, weight) is a step
 * on
 *   L = sum_s (sum_{r in s} coef_r y_r - delta_s)^2
 *       + sum_r label_weight_r (y_r - label_r)^2
 * (label / label_weight: device FP32 [n], or both NULL for the first term
 * alone); loss (host [2], may be NULL) receives the two terms at the current
 * parameters. */
int ffg_mlp_set_targets(ffg_mlp* m, const uint16_t* x, size_t n, const double* coef, const int64_t* seg,
                        const double* delta, size_t nseg, const float* label, const float* label_weight,
                        float* target, float* weight, double* loss);
/* Self-test of the tensor-core path: D[128][N] = A[128][K] B[N][K]^T with host
 * BF16 A, B and FP32 D (K in 16..128, N in 16..256, multiples of 16). */
int ffg_mlp_selftest_gemm(ffg_mlp* m, int N, int K, const uint16_t* a, const uint16_t* b, float* d);
/* Features of n dropped partners (device keys [4][stride], coef = real parts,
 * gate = creating gate) of the circuit gates[0..ngates) (host): batch_of_gate
 * (host, [ngates]) is the commuting run of each gate in application order
 * (nbatches runs), coords (host, [2][128]) the lattice coordinates of the
 * qubits, obs_qubit the observable's site, maxdegree the cutoff that dropped
 * them.  Writes FP32 features feat[n][32] and/or the BF16 network input
 * x[n][32] = (feature - shift) * scale (device, either may be NULL; shift and
 * scale are host [32] arrays, both NULL for no standardisation). */
int ffg_drop_features(ffg_ctx* ctx, const uint64_t* keys, size_t stride, const double* coef, const int32_t* gate,
                      size_t n, const ffg_pauli_gate* gates, size_t ngates, const int32_t* batch_of_gate,
                      int32_t nbatches, const float* coords, int32_t obs_qubit, int32_t maxdegree,
                      const float* shift, const float* scale, float* feat, uint16_t* x);

/* -------------------------------------------------------------------------- */
/* Allocation-free rotations.  No counterpart in the reference: this entry
 * point exists for callers that cannot allocate device memory when they call
 * it -- processes in which a framework's caching allocator already holds
 * (nearly) all device memory, so a library cudaMalloc fails or fragments that
 * pool, and latency-critical loops that share the GPU with other streams and
 * cannot accept cudaFree's implicit device-wide synchronisation.  It creates
 * no context and calls no allocating CUDA or library routine: the term store
 * lives in a fixed 65536-term device array inside libffg (about 4.3 MB, held
 * by every GPU that loads the library until the process exits).
 *
 * Applies the FFG_ROT gates of gates[0..ngates) last to first, one reference
 * conjugation each (partners of weight > maxdegree are not emitted), with no
 * truncation, on the device polynomial keys_in [4][n] / re_in / im_in (im_in
 * may be NULL), and writes the result to caller-allocated device arrays:
 * key plane w at keys_out + w * out_cap, re_out[0..*n_out), im_out[0..*n_out).
 * Work is issued on `stream` (a cudaStream_t; NULL = legacy default stream)
 * and the call returns after it completes.
 *   - n must be at most 32768 and the polynomial may not outgrow 65536 terms:
 *     larger sizes return FFG_ERR_ARG with a message in errbuf (may be NULL)
 *     naming the gates[] index at which it outgrew the array;
 *   - *n_out receives the result size even when out_cap is too small;
 *   - duplicate input keys return FFG_ERR_ARG;
 *   - the first call on a device looks up the device address of the array
 *     (once per device, with that device current) and keeps it; make that
 *     first call before any stream capture begins.  A cudaDeviceReset of the
 *     device invalidates the kept address;
 *   - all calls share the one array and each leaves its contents behind; calls
 *     whose GPU work overlaps (e.g. on two streams) race and give wrong results.
 */
int ffg_pauli_rotations_noalloc(void* stream, const uint64_t* keys_in, const double* re_in,
                                const double* im_in, size_t n, const ffg_pauli_gate* gates,
                                size_t ngates, int32_t maxdegree, uint64_t* keys_out,
                                double* re_out, double* im_out, size_t out_cap, size_t* n_out,
                                char* errbuf, size_t errlen);

/* -------------------------------------------------------------------------- */
/* Host-side helpers exposed for tests (no device work). */
/* 1 when hypot(re, im) <= tau under round-to-nearest (the truncation rule). */
int ffg_abs_le(double re, double im, double tau);
/* Number of commuting batches the reference schedule forms for the rotations
 * of a Pauli circuit (src/pauli/propagate.h:272-291 applied between Clifford
 * segments); writes up to cap batch sizes in application order. */
int64_t ffg_pauli_schedule(const ffg_pauli_gate* gates, size_t ngates, int batched, int64_t* sizes,
                           int64_t cap);

#ifdef __cplusplus
}
#endif
#endif
