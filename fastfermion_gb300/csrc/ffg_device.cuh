// Device-side building blocks shared by the propagation kernels: term-store
// layout, key hashing, exact complex arithmetic and the truncation predicate.
//
// Exactness: every coefficient update of the reference is a single IEEE
// rounding (src/pauli/propagate.h:71-89, src/majorana_gates.h:86-102), so the
// kernels reproduce it bit for bit as long as (a) cos/sin come from the host C
// library, (b) no multiply-add is contracted.  All coefficient arithmetic below
// therefore uses the explicit round-to-nearest intrinsics.
#pragma once
#include <cstdint>

namespace ffg {

typedef unsigned long long u64;
typedef unsigned int u32;

constexpr u64 kEmptySlot = ~0ull;
constexpr int kBlock = 256;

// ---------------------------------------------------------------------------
// Counters that live in device memory and let consecutive kernels agree on the
// term-store size without any host round trip.  Each kernel reads n/alive at
// entry, accumulates its changes in the d_* fields, and the last block to
// finish folds them in (threadfence-reduction pattern).
// ---------------------------------------------------------------------------
struct DevCounters {
    u64 n;         // entries in [0, n): live or dead
    u64 alive;     // live entries
    u64 apps;      // sum over rotation gates of the live terms entering the gate
    u64 peak;      // largest live count seen after a gate
    u64 emits;     // partners emitted that passed the degree filter
    u64 d_app;     // entries appended by the running kernel
    u64 d_apps;    // fused passes: live terms created inside the pass that enter later gates
    long long d_alive;  // live-count change of the running kernel
    u32 done;      // blocks finished in the running kernel
    u32 overflow;  // 1 + op index that found the store too small (0 = none)
    u32 error;     // nonzero: inconsistent input (duplicate key) or probe overrun
    u32 pad;
    double sum_re[2];  // reduction scratch (expectation values)
    double sum_im[2];
};

// ---------------------------------------------------------------------------
// Term store view (structure of arrays in HBM)
//   key  : KW planes of u64, plane w at key[w * cap + i]
//          Pauli:    planes [0, NW) are xory words, [NW, 2NW) are yorz words
//          Majorana: planes [0, KW) are alpha words
//   re/im: FP64 coefficients (im unused in real mode)
//   dead : 1 when the entry has been truncated away (kept in place until the
//          next compaction so that indices stay stable)
//   slots: open-addressing index, entry = (fingerprint << 32) | position
// ---------------------------------------------------------------------------
struct StoreView {
    u64* key;
    double* re;
    double* im;
    unsigned char* dead;
    u64* slots;
    u64 hmask;
    u64 cap;
};

__host__ __device__ inline u64 mix64(u64 x) {
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}

template <int KW>
__device__ __forceinline__ u64 hash_key(const u64 (&k)[KW]) {
    u64 h = mix64(k[0] ^ 0x9e3779b97f4a7c15ull);
#pragma unroll
    for (int w = 1; w < KW; w++) h = mix64(h ^ k[w]);
    return h;
}

template <int KW>
__device__ __forceinline__ void load_key(const StoreView& s, u64 i, u64 (&k)[KW]) {
#pragma unroll
    for (int w = 0; w < KW; w++) k[w] = s.key[(u64)w * s.cap + i];
}

// L2-coherent load: entries appended by other SMs during the same kernel are
// visible once their slot has been published.
template <int KW>
__device__ __forceinline__ bool key_equals_cg(const StoreView& s, u64 i, const u64 (&k)[KW]) {
#pragma unroll
    for (int w = 0; w < KW; w++)
        if (__ldcg(&s.key[(u64)w * s.cap + i]) != k[w]) return false;
    return true;
}

// Returns the position of key k, or -1; *slot_at receives the index slot that
// holds it.  Entries are never removed from the index (dead ones stay until
// compaction), so the probe chain of a key present before the kernel started is
// never interrupted by an empty slot.
template <int KW>
__device__ __forceinline__ long long lookup(const StoreView& s, const u64 (&k)[KW], u32* err,
                                            u64* slot_at = nullptr) {
    const u64 h = hash_key<KW>(k);
    const u32 fp = (u32)(h >> 32);
    u64 pos = h & s.hmask;
    for (u64 probe = 0; probe <= s.hmask; probe++) {
        const u64 e = __ldcg(&s.slots[pos]);
        if (e == kEmptySlot) return -1;
        if ((u32)(e >> 32) == fp) {
            const u32 idx = (u32)e;
            if (key_equals_cg<KW>(s, idx, k)) {
                if (slot_at) *slot_at = pos;
                return (long long)idx;
            }
        }
        pos = (pos + 1) & s.hmask;
    }
    atomicOr(err, 2u);
    return -1;
}

// Publishes position idx (whose key words are already written) for key k.
// When check_dup is set an equal key already in the index is reported as an
// error (used when loading caller input, which must have distinct keys).
template <int KW>
__device__ __forceinline__ void insert(const StoreView& s, const u64 (&k)[KW], u32 idx, u32* err,
                                       bool check_dup) {
    const u64 h = hash_key<KW>(k);
    const u32 fp = (u32)(h >> 32);
    const u64 entry = ((u64)fp << 32) | idx;
    u64 pos = h & s.hmask;
    for (u64 probe = 0; probe <= s.hmask; probe++) {
        u64 e = __ldcg(&s.slots[pos]);
        if (e == kEmptySlot) {
            e = atomicCAS(&s.slots[pos], kEmptySlot, entry);
            if (e == kEmptySlot) return;
        }
        if (check_dup && (u32)(e >> 32) == fp && key_equals_cg<KW>(s, (u32)e, k)) {
            atomicOr(err, 1u);
            return;
        }
        pos = (pos + 1) & s.hmask;
    }
    atomicOr(err, 2u);
}

// ---------------------------------------------------------------------------
// exact complex arithmetic (std::complex<double> as GCC evaluates it)
// ---------------------------------------------------------------------------
struct cplx {
    double re, im;
};

__device__ __forceinline__ cplx cmul(cplx a, cplx b) {
    const double ac = __dmul_rn(a.re, b.re), bd = __dmul_rn(a.im, b.im);
    const double ad = __dmul_rn(a.re, b.im), bc = __dmul_rn(a.im, b.re);
    return {__dsub_rn(ac, bd), __dadd_rn(ad, bc)};
}

__device__ __forceinline__ cplx cscale(cplx a, double c) { return {__dmul_rn(a.re, c), __dmul_rn(a.im, c)}; }
__device__ __forceinline__ cplx cadd(cplx a, cplx b) { return {__dadd_rn(a.re, b.re), __dadd_rn(a.im, b.im)}; }

// i^m for any integer m (src/common.h:61-66)
__device__ __forceinline__ cplx ipow(int m) {
    switch (m & 3) {
        case 0: return {1.0, 0.0};
        case 1: return {0.0, 1.0};
        case 2: return {-1.0, 0.0};
        default: return {0.0, -1.0};
    }
}

// Rotation update terms with a real-mode specialisation.  With imaginary parts
// zero, the complex expressions of the reference reduce exactly (same IEEE
// result up to the sign of zero) to:
//   keep:    (a, 0) * c                          -> a*c
//   partner: (b, 0) * (0, s) * i^j               -> -(b*s) for j = 1 mod 4,
//                                                   +(b*s) for j = 3 mod 4,
//                                                   (+-)0 for even j
//   sum:     x + y                               -> one rounding of the real parts
// (the partner product is b*s + 0 then a sign flip, both exact).  Real mode is
// used only for finite inputs: with an infinite coefficient the complex form
// produces NaN where the reduced form would not.
template <bool CPLX>
__device__ __forceinline__ cplx rot_keep(cplx a, double c) {
    if (CPLX) return cscale(a, c);
    return {__dmul_rn(a.re, c), 0.0};
}

template <bool CPLX>
__device__ __forceinline__ cplx rot_partner(cplx b, double s, int j) {
    if (CPLX) return cmul(cmul(b, {0.0, s}), ipow(j));
    const double p = __dmul_rn(b.re, s);
    switch (j & 3) {
        case 1: return {-p, 0.0};
        case 3: return {p, 0.0};
        default: return {0.0, 0.0};
    }
}

template <bool CPLX>
__device__ __forceinline__ cplx rot_add(cplx a, cplx b) {
    if (CPLX) return cadd(a, b);
    return {__dadd_rn(a.re, b.re), 0.0};
}

// GB300 runs FP64 instructions at a small fraction of the FP32 rate, and the
// orbit kernels meet a burst of them after every gate barrier; these tests
// therefore run on the integer pipes, on IEEE bit patterns (non-negative
// doubles order like their bit patterns).
// |s| == 1 exactly.
__device__ __forceinline__ bool unit_sine(double s) {
    return ((unsigned long long)__double_as_longlong(s) & 0x7fffffffffffffffull) == 0x3ff0000000000000ull;
}
// fabs(x) <= tau, with the floating-point comparison's result for every x
// and tau (false when either is NaN; tau = -0 admits only zeros).
__device__ __forceinline__ bool abs_le_bits(double x, double tau) {
    const unsigned long long ax = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
    const unsigned long long t = (unsigned long long)__double_as_longlong(tau);
    const unsigned long long at = t & 0x7fffffffffffffffull;
    if (ax > 0x7ff0000000000000ull || at > 0x7ff0000000000000ull) return false;
    if (t >> 63) return ax == 0 && at == 0;
    return ax <= at;
}

// The partner value when |s| = 1 (sin theta = +-1, e.g. RZZ(-pi/2)), real
// mode: b*s is exact, so the product is b with its sign flipped when s < 0,
// then the sign of i^j as in rot_partner -- the same value with no FP64
// instruction (GB300 issues FP64 at a small fraction of the FP32 rate).
template <bool CPLX>
__device__ __forceinline__ cplx rot_partner_unit(cplx b, double s, int j) {
    if (CPLX) return rot_partner<true>(b, s, j);
    if (!(j & 1)) return {0.0, 0.0};
    const bool neg = ((unsigned long long)__double_as_longlong(s) >> 63) != (unsigned long long)((j & 3) == 1);
    return {__longlong_as_double(__double_as_longlong(b.re) ^ (neg ? (long long)0x8000000000000000ull : 0ll)), 0.0};
}

// The value of a new entry, 0 + v (the reference adds a partner into a
// value-initialised coefficient): in real mode (finite v) that is v with a
// negative zero made positive, without an FP64 addition.
template <bool CPLX>
__device__ __forceinline__ cplx rot_new(cplx v) {
    if (CPLX) return rot_add<true>({0.0, 0.0}, v);
    return {__double_as_longlong(v.re) == (long long)0x8000000000000000ull ? 0.0 : v.re, 0.0};
}

// ---------------------------------------------------------------------------
// Truncation predicate |c| <= tau with |c| = hypot(re, im) correctly rounded
// (the reference uses std::abs on std::complex<double>, i.e. libm hypot).
// RN(sqrt(S)) <= tau  <=>  S < M, or S == M and tau has an even significand,
// where S = re^2 + im^2 and M = (tau + ulp(tau)/2)^2.  The sign of S - M is
// obtained exactly from a nonoverlapping expansion of the eight partial
// products (two-sum accumulation, Shewchuk 1997).
// ---------------------------------------------------------------------------
__host__ __device__ inline void two_sum(double a, double b, double& s, double& e) {
#ifdef __CUDA_ARCH__
    s = __dadd_rn(a, b);
    const double bb = __dsub_rn(s, a);
    e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
#else
    volatile double vs = a + b;
    s = vs;
    volatile double bb = s - a;
    volatile double t1 = s - bb;
    volatile double t2 = a - t1;
    volatile double t3 = b - bb;
    e = t2 + t3;
#endif
}

__host__ __device__ inline double exact_prod(double a, double b, double& lo) {
    const double p = a * b;
#ifdef __CUDA_ARCH__
    lo = __fma_rn(a, b, -p);
#else
    lo = __builtin_fma(a, b, -p);
#endif
    return p;
}

__host__ __device__ inline int sign_of_sum(const double* t, int n) {
    // grow-expansion: e holds a nonoverlapping expansion, increasing magnitude
    double e[16];
    int m = 0;
    for (int i = 0; i < n; i++) {
        double q = t[i];
        int k = 0;
        for (int j = 0; j < m; j++) {
            double s, err;
            two_sum(q, e[j], s, err);
            q = s;
            if (err != 0.0) e[k++] = err;
        }
        if (q != 0.0) e[k++] = q;
        m = k;
    }
    if (m == 0) return 0;
    return e[m - 1] > 0.0 ? 1 : -1;
}

__host__ __device__ inline double fabs_hd(double x) { return x < 0 ? -x : x; }

// true when hypot(re, im) <= tau (tau > 0)
__host__ __device__ inline bool abs_le(double re, double im, double tau) {
    double x = fabs_hd(re), y = fabs_hd(im);
    if (x < y) {
        double t = x;
        x = y;
        y = t;
    }
    if (!(x == x) || !(y == y)) return false;  // NaN: comparison is false
    if (y == 0.0) return x <= tau;
    if (x > 2.0 * tau) return false;
    if (x + y < 0.70 * tau) return true;  // sqrt(x^2+y^2) <= x + y < tau
    // scale so that every square is a normal number (powers of two are exact)
    double sc = 1.0;
    if (tau < 0x1p-400) sc = 0x1p600;
    if (tau > 0x1p400) sc = 0x1p-600;
    x *= sc;
    y *= sc;
    double t = tau * sc;
    // ulp(t)/2 for a normal t
    int ex;
#ifdef __CUDA_ARCH__
    ex = (int)((__double_as_longlong(t) >> 52) & 0x7ff) - 1075;
    const double half_ulp = __longlong_as_double((long long)(ex + 1023 - 1 + 0) << 52);
#else
    union {
        double d;
        long long i;
    } u;
    u.d = t;
    ex = (int)((u.i >> 52) & 0x7ff) - 1075;
    u.i = (long long)(ex + 1023 - 1) << 52;
    const double half_ulp = u.d;
#endif
    // S - M = x^2 + y^2 - t^2 - t*ulp - ulp^2/4
    double parts[8];
    double lo;
    parts[0] = exact_prod(x, x, lo);
    parts[1] = lo;
    parts[2] = exact_prod(y, y, lo);
    parts[3] = lo;
    parts[4] = -exact_prod(t, t, lo);
    parts[5] = -lo;
    parts[6] = -(t * (2.0 * half_ulp));      // exact: power-of-two factor
    parts[7] = -(half_ulp * half_ulp);       // exact: power of two
    const int sg = sign_of_sum(parts, 8);
    if (sg < 0) return true;
    if (sg > 0) return false;
#ifdef __CUDA_ARCH__
    const long long bits = __double_as_longlong(t);
#else
    u.d = t;
    const long long bits = u.i;
#endif
    return (bits & 1) == 0;  // tie: rounds to even
}

// ---------------------------------------------------------------------------
// block-level helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long block_sum_ll(long long v, long long* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    long long r = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) r += sh[w];
    return r;  // valid in thread 0
}

// Warp-aggregated append: returns a slot in [base + 0, ...) for every lane
// that has want == true.  All lanes of the warp that reach this call must pass.
__device__ __forceinline__ u64 warp_append(bool want, u64* counter) {
    const u32 mask = __activemask();
    const u32 vote = __ballot_sync(mask, want);
    if (!vote) return 0;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(vote) - 1;
    u64 base = 0;
    if (lane == leader) base = atomicAdd(counter, (u64)__popc(vote));
    base = __shfl_sync(mask, base, leader);
    return base + __popc(vote & ((1u << lane) - 1u));
}

}  // namespace ffg
