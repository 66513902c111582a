/*
 * ffo.h -- CPU oracle for truncated Heisenberg-picture propagation of Pauli and
 * Majorana polynomials.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (fastfermion `propagate`), used by the test-suite as the checker
 * and by bench.py as the timed CPU baseline.  The product library never links,
 * loads or calls it.
 *
 * Key layout (one term): four 64-bit words.
 *   Pauli:    k[0] = xory word 0, k[1] = xory word 1, k[2] = yorz word 0,
 *             k[3] = yorz word 1   (qubits 0..127, I=(0,0) X=(1,0) Y=(1,1)
 *             Z=(0,1) as in src/pauli/algebra.h:30)
 *   Majorana: k[0..3] = alpha words (Majorana indices 0..255,
 *             src/majorana_algebra.h:30-33)
 */
#ifndef FFO_ORACLE_H_
#define FFO_ORACLE_H_
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { FFO_ROT = 0, FFO_H = 1, FFO_S = 2, FFO_CNOT = 3, FFO_SWAP = 4, FFO_CZ = 5 };

typedef struct {
    int32_t kind;      /* FFO_* */
    int32_t q0, q1;    /* Clifford qubits */
    int32_t pad;
    uint64_t x[2];     /* ROT axis xory words */
    uint64_t z[2];     /* ROT axis yorz words */
    double theta;      /* ROT angle */
} ffo_pauli_gate;

typedef struct {
    uint64_t alpha[4]; /* Majorana string */
    double theta;      /* already folded with the monomial coefficient */
    int32_t r;         /* 1 when the string is not Hermitian (deg % 4 in {2,3}) */
    int32_t pad;
} ffo_majorana_gate;

typedef struct {
    int32_t maxdegree;
    int32_t topk;
    double mincoeff;
    int32_t max_xweight;
    int32_t xtrunc_period;
    int32_t batched;
    int32_t n_threads;  /* > 1 selects the sharded OpenMP strategy */
} ffo_pauli_params;

typedef struct ffo_poly ffo_poly;

/* Pauli propagation (src/pauli/propagate.h:297-493).  Returns NULL on bad input. */
ffo_poly* ffo_pauli_propagate(const ffo_pauli_gate* gates, int64_t ngates,
                              const uint64_t* keys /* [4][n] */, const double* re,
                              const double* im, int64_t n, const ffo_pauli_params* p);

/* Partners that the degree filter drops (not a reference feature: training
 * data of the learned-correction form).  ffo_pauli_propagate_capture runs the
 * serial strategy (n_threads is ignored) and records, in creation order, every
 * partner whose degree is above maxdegree and at most capdeg: its key, its
 * coefficient c (i sin) phase, and the index of the gate that created it.  The
 * part of the circuit still to be applied to it is gates [0, gate). */
typedef struct ffo_drops ffo_drops;
ffo_poly* ffo_pauli_propagate_capture(const ffo_pauli_gate* gates, int64_t ngates,
                                      const uint64_t* keys, const double* re, const double* im,
                                      int64_t n, const ffo_pauli_params* p, int32_t capdeg,
                                      ffo_drops** dropped);
/* Propagation with some rotations skipped (not a reference feature: the
 * semantics of one instance of the GPU's per-instance active rotations).
 * Rotation r (circuit order among the ROT gates) acts iff bit r % 64 of
 * active[r / 64] is set; an inactive rotation leaves the terms as they are,
 * while batching and truncation points stay those of the whole circuit.
 * Serial and sharded strategies as in ffo_pauli_propagate. */
ffo_poly* ffo_pauli_propagate_masked(const ffo_pauli_gate* gates, int64_t ngates,
                                     const uint64_t* keys, const double* re, const double* im,
                                     int64_t n, const ffo_pauli_params* p, const uint64_t* active);
int64_t ffo_drops_size(const ffo_drops* d);
void ffo_drops_copy(const ffo_drops* d, uint64_t* keys /* [4][n] */, double* re, double* im,
                    int64_t* gate);
void ffo_drops_free(ffo_drops* d);
/* Majorana propagation (src/majorana_propagation.h:18-55). */
ffo_poly* ffo_majorana_propagate(const ffo_majorana_gate* gates, int64_t ngates,
                                 const uint64_t* keys, const double* re, const double* im,
                                 int64_t n, int32_t has_maxdegree, int32_t maxdegree,
                                 double mincoeff);

int64_t ffo_size(const ffo_poly* p);
/* Copies the terms in the oracle's iteration order (keys as [4][n]). */
void ffo_copy(const ffo_poly* p, uint64_t* keys, double* re, double* im);
void ffo_free(ffo_poly* p);
/* Sum over rotation gates of the live terms entering each gate. */
int64_t ffo_apps(const ffo_poly* p);
/* Largest live-term count seen at any point. */
int64_t ffo_peak(const ffo_poly* p);

/* <0|O|0> in iteration order (src/pauli/algebra.h:549-557). */
void ffo_overlapwithzero(const ffo_poly* p, double* re, double* im);
/* QubitProductState(b)(O) (src/qubitproductstate.h:73-88). */
void ffo_qubit_state(const ffo_poly* p, const uint64_t* b /* [2] */, double* re, double* im);
/* FockState(b)(O) for Majorana polynomials (src/fockstate.h:95-114). */
void ffo_fock_state(const ffo_poly* p, const uint64_t* b /* [2] */, double* re, double* im);

/* glibc-compatible |c| used by the truncation rules (exposed for tests). */
double ffo_abs(double re, double im);

#ifdef __cplusplus
}
#endif
#endif
