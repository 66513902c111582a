/*
 * ffo.c -- CPU oracle: plain-C restatement of fastfermion's truncated
 * Heisenberg-picture propagation.
 *
 * TEST INFRASTRUCTURE ONLY.  Only the test-suite, the smoke check and the
 * CPU-baseline leg of bench.py load this file's shared library; the product
 * (libffg) never does.
 *
 * The serial strategy mirrors the reference term store's iteration order
 * exactly: new keys are appended, erase moves the last entry into the erased
 * position, and erase_if walks back to front, as the vendored ankerl
 * unordered_dense v4.5.0 map does (src/hashmap/unordered_dense.h:1052-1085 and
 * :1983-2000).  Because of that, order-dependent outputs (overlapwithzero,
 * top-k tie trimming) agree with the reference's serial path bit for bit.
 * The sharded strategy (OpenMP, n_threads > 1) follows the reference's
 * hash-partitioned scheme (src/pauli/propagate.h:157-264) and produces the
 * same term set and coefficients in a different order.
 *
 * Build with -ffp-contract=off: every coefficient update is one IEEE
 * rounding, as in the reference.
 */
#include "ffo.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    uint64_t k[4];
    double re, im;
} term_t;

typedef struct {
    term_t* v;
    int64_t n, cap;
} vec_t;

typedef struct {
    vec_t d;          /* dense, insertion-ordered entries */
    int64_t* slot;    /* open-addressing index into d (-1 = empty) */
    uint64_t hmask;
} map_t;

struct ffo_poly {
    map_t m;
    int64_t apps;
    int64_t peak;
};

/* ------------------------------------------------------------------------- */
/* small helpers                                                             */
/* ------------------------------------------------------------------------- */

static inline int popc(uint64_t x) { return __builtin_popcountll(x); }

static inline uint64_t mix64(uint64_t x) {
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ULL;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebULL;
    x ^= x >> 31;
    return x;
}

static inline uint64_t hkey(const uint64_t* k) {
    uint64_t h = mix64(k[0] ^ 0x9e3779b97f4a7c15ULL);
    h = mix64(h ^ k[1]);
    h = mix64(h ^ k[2]);
    return mix64(h ^ k[3]);
}

static inline int keq(const uint64_t* a, const uint64_t* b) {
    return a[0] == b[0] && a[1] == b[1] && a[2] == b[2] && a[3] == b[3];
}

/* std::complex<double> product as GCC evaluates it for finite operands:
 * (ac - bd, ad + bc), each product and sum rounded once. */
static inline void cmul(double a, double b, double c, double d, double* re, double* im) {
    double ac = a * c, bd = b * d, ad = a * d, bc = b * c;
    *re = ac - bd;
    *im = ad + bc;
}

/* i^m, src/common.h:61-66 */
static inline void ipow(int m, double* re, double* im) {
    switch (m & 3) {
        case 0: *re = 1.0; *im = 0.0; break;
        case 1: *re = 0.0; *im = 1.0; break;
        case 2: *re = -1.0; *im = 0.0; break;
        default: *re = 0.0; *im = -1.0; break;
    }
}

double ffo_abs(double re, double im) { return hypot(re, im); }

static void vec_push(vec_t* v, const term_t* t) {
    if (v->n == v->cap) {
        v->cap = v->cap ? v->cap * 2 : 64;
        v->v = (term_t*)realloc(v->v, (size_t)v->cap * sizeof(term_t));
    }
    v->v[v->n++] = *t;
}

/* ------------------------------------------------------------------------- */
/* insertion-ordered map                                                     */
/* ------------------------------------------------------------------------- */

static void map_reindex(map_t* m, int64_t want) {
    uint64_t hcap = 16;
    while (hcap < (uint64_t)(2 * want)) hcap <<= 1;
    free(m->slot);
    m->slot = (int64_t*)malloc(hcap * sizeof(int64_t));
    memset(m->slot, 0xff, hcap * sizeof(int64_t));
    m->hmask = hcap - 1;
    for (int64_t i = 0; i < m->d.n; i++) {
        uint64_t p = hkey(m->d.v[i].k) & m->hmask;
        while (m->slot[p] >= 0) p = (p + 1) & m->hmask;
        m->slot[p] = i;
    }
}

static void map_init(map_t* m) {
    memset(m, 0, sizeof(*m));
    map_reindex(m, 8);
}

static void map_release(map_t* m) {
    free(m->d.v);
    free(m->slot);
    memset(m, 0, sizeof(*m));
}

static int64_t map_find(const map_t* m, const uint64_t* k) {
    uint64_t p = hkey(k) & m->hmask;
    for (;;) {
        int64_t s = m->slot[p];
        if (s < 0) return -1;
        if (keq(m->d.v[s].k, k)) return s;
        p = (p + 1) & m->hmask;
    }
}

/* terms[k] += (re, im): an absent key starts from complex zero, as
 * operator[] does in the reference map. */
static void map_add(map_t* m, const uint64_t* k, double re, double im) {
    int64_t s = map_find(m, k);
    if (s >= 0) {
        m->d.v[s].re = m->d.v[s].re + re;
        m->d.v[s].im = m->d.v[s].im + im;
        return;
    }
    term_t t;
    memcpy(t.k, k, sizeof(t.k));
    t.re = 0.0 + re;
    t.im = 0.0 + im;
    vec_push(&m->d, &t);
    if ((uint64_t)(2 * m->d.n) > m->hmask + 1) {
        map_reindex(m, m->d.n);
    } else {
        uint64_t p = hkey(k) & m->hmask;
        while (m->slot[p] >= 0) p = (p + 1) & m->hmask;
        m->slot[p] = m->d.n - 1;
    }
}

/* std::erase_if on the reference map: back to front, erase moves the last
 * entry into the hole. */
typedef int (*pred_fn)(const term_t*, const void*);

static int64_t map_erase_if(map_t* m, pred_fn pred, const void* ctx) {
    int64_t old = m->d.n;
    for (int64_t i = m->d.n - 1; i >= 0; i--) {
        if (pred(&m->d.v[i], ctx)) {
            m->d.v[i] = m->d.v[m->d.n - 1];
            m->d.n--;
        }
    }
    if (m->d.n != old) map_reindex(m, m->d.n);
    return old - m->d.n;
}

/* ------------------------------------------------------------------------- */
/* Pauli algebra (src/pauli/algebra.h)                                       */
/* ------------------------------------------------------------------------- */

/* PauliString::commutes, algebra.h:209-211 */
static inline int pauli_anticommutes(const uint64_t* q, const uint64_t* px, const uint64_t* pz) {
    int a = popc(q[0] & pz[0]) + popc(q[1] & pz[1]);
    int b = popc(q[2] & px[0]) + popc(q[3] & px[1]);
    return (a & 1) != (b & 1);
}

/* P * Q with the phase exponent of pauli_string_multiply, algebra.h:227-233 */
static inline int pauli_mul(const uint64_t* px, const uint64_t* pz, const uint64_t* q, uint64_t* out) {
    int jpow = popc(px[0] & pz[0]) + popc(px[1] & pz[1]) + popc(q[0] & q[2]) + popc(q[1] & q[3]) +
               2 * (popc(pz[0] & q[0]) + popc(pz[1] & q[1]));
    out[0] = px[0] ^ q[0];
    out[1] = px[1] ^ q[1];
    out[2] = pz[0] ^ q[2];
    out[3] = pz[1] ^ q[3];
    jpow -= popc(out[0] & out[2]) + popc(out[1] & out[3]);
    return jpow;
}

static inline int pauli_degree(const uint64_t* k) { return popc(k[0] | k[2]) + popc(k[1] | k[3]); }

/* ------------------------------------------------------------------------- */
/* Clifford maps (src/pauli/gates.h:15-69)                                   */
/* ------------------------------------------------------------------------- */

static inline uint64_t getbit(const uint64_t* w, int i) { return (w[i >> 6] >> (i & 63)) & 1ULL; }
static inline void setbit(uint64_t* w, int i, uint64_t b) {
    w[i >> 6] = (w[i >> 6] & ~(1ULL << (i & 63))) | (b << (i & 63));
}

/* Applies one Clifford gate to key k (x = k[0..1], z = k[2..3]); returns 1
 * when the sign flips.  Each branch evaluates the reference's bit formulas on
 * the bits before the update, including for coincident qubits. */
static int clifford_apply(const ffo_pauli_gate* g, uint64_t* k) {
    uint64_t* x = k;
    uint64_t* z = k + 2;
    int i = g->q0, j = g->q1;
    switch (g->kind) {
        case FFO_H: {
            uint64_t xi = getbit(x, i), zi = getbit(z, i);
            setbit(x, i, zi);
            setbit(z, i, xi);
            return (int)(xi & zi);
        }
        case FFO_S: {
            uint64_t xi = getbit(x, i), zi = getbit(z, i);
            setbit(z, i, xi ^ zi);
            return (int)(xi & (zi ^ 1));
        }
        case FFO_CNOT: {
            uint64_t xi = getbit(x, i), xj = getbit(x, j), zi = getbit(z, i), zj = getbit(z, j);
            /* x_j <- x_i ^ x_j ; z_i <- z_i ^ z_j (gates.h:40-53) */
            setbit(x, j, xi ^ xj);
            setbit(z, i, zi ^ zj);
            return (int)(xi & zj & ((zi ^ xj) ^ 1));
        }
        case FFO_SWAP: {
            uint64_t xi = getbit(x, i), xj = getbit(x, j), zi = getbit(z, i), zj = getbit(z, j);
            setbit(x, i, xj);
            setbit(x, j, xi);
            setbit(z, i, zj);
            setbit(z, j, zi);
            return 0;
        }
        case FFO_CZ: {
            uint64_t xi = getbit(x, i), xj = getbit(x, j), zi = getbit(z, i), zj = getbit(z, j);
            int flip = (int)(xi & xj & (zi ^ zj));
            /* yorz ^= (x_j at i) | (x_i at j) (gates.h:61-69) */
            uint64_t m[2] = {0, 0};
            m[i >> 6] |= xj << (i & 63);
            m[j >> 6] |= xi << (j & 63);
            z[0] ^= m[0];
            z[1] ^= m[1];
            return flip;
        }
        default:
            return 0;
    }
}

/* ------------------------------------------------------------------------- */
/* Pauli rotation, serial (src/pauli/propagate.h:71-89)                      */
/* ------------------------------------------------------------------------- */

/* Partners dropped by the degree filter, recorded for the learned-correction
 * form's training data (not a reference feature): key, coefficient and the
 * index of the gate that created them, for degrees up to capdeg. */
struct ffo_drops {
    vec_t t;
    int64_t* gate;
    int64_t gcap;
    int capdeg;
};

static void drops_push(ffo_drops* d, const term_t* p, int64_t gi) {
    vec_push(&d->t, p);
    if (d->t.n > d->gcap) {
        d->gcap = d->t.cap;
        d->gate = (int64_t*)realloc(d->gate, (size_t)d->gcap * sizeof(int64_t));
    }
    d->gate[d->t.n - 1] = gi;
}

static void pauli_conjugate(map_t* m, const ffo_pauli_gate* g, int maxdeg, vec_t* nb, ffo_drops* drops,
                            int64_t gi) {
    const double c = cos(g->theta);
    const double s = sin(g->theta);
    nb->n = 0;
    for (int64_t i = 0; i < m->d.n; i++) {
        term_t* t = &m->d.v[i];
        if (!pauli_anticommutes(t->k, g->x, g->z)) continue;
        term_t p;
        int jpow = pauli_mul(g->x, g->z, t->k, p.k);
        const int deg = pauli_degree(p.k);
        if (deg <= maxdeg || (drops && deg <= drops->capdeg)) {
            double tr, ti, fr, fi;
            cmul(t->re, t->im, 0.0, s, &tr, &ti); /* coeff * (i sin) */
            ipow(jpow, &fr, &fi);
            cmul(tr, ti, fr, fi, &p.re, &p.im); /* ... * phase(P*Q) */
            if (deg <= maxdeg)
                vec_push(nb, &p);
            else
                drops_push(drops, &p, gi);
        }
        t->re = t->re * c;
        t->im = t->im * c;
    }
    for (int64_t i = 0; i < nb->n; i++) map_add(m, nb->v[i].k, nb->v[i].re, nb->v[i].im);
}

static void pauli_clifford(map_t* m, const ffo_pauli_gate* gates, int64_t begin, int64_t end) {
    map_t out;
    map_init(&out);
    for (int64_t i = 0; i < m->d.n; i++) {
        term_t t = m->d.v[i];
        double mr = 1.0, mi = 0.0;
        for (int64_t j = end - 1; j >= begin; j--) {
            if (clifford_apply(&gates[j], t.k)) {
                mr = mr * -1.0;
                mi = mi * -1.0;
            }
        }
        double r, im;
        cmul(mr, mi, t.re, t.im, &r, &im);
        map_add(&out, t.k, r, im);
    }
    map_release(m);
    *m = out;
}

/* ------------------------------------------------------------------------- */
/* truncation (src/pauli/truncate.h)                                         */
/* ------------------------------------------------------------------------- */

static int pred_small(const term_t* t, const void* ctx) {
    return ffo_abs(t->re, t->im) <= *(const double*)ctx;
}
static int pred_below(const term_t* t, const void* ctx) {
    return ffo_abs(t->re, t->im) < *(const double*)ctx;
}
static int pred_xweight(const term_t* t, const void* ctx) {
    return popc(t->k[0]) + popc(t->k[1]) > *(const int*)ctx;
}

static int cmp_desc(const void* a, const void* b) {
    double x = *(const double*)a, y = *(const double*)b;
    return (x < y) - (x > y);
}

static void truncate_top_k(map_t* m, int k) {
    if (k <= 0 || m->d.n <= k) return;
    double* mags = (double*)malloc((size_t)m->d.n * sizeof(double));
    for (int64_t i = 0; i < m->d.n; i++) mags[i] = ffo_abs(m->d.v[i].re, m->d.v[i].im);
    qsort(mags, (size_t)m->d.n, sizeof(double), cmp_desc);
    double cutoff = mags[k];
    free(mags);
    map_erase_if(m, pred_below, &cutoff);
    /* trim exact ties in iteration order (truncate.h:31-37) */
    while (m->d.n > k) {
        int64_t i = 0;
        while (i < m->d.n && ffo_abs(m->d.v[i].re, m->d.v[i].im) > cutoff) i++;
        if (i == m->d.n) break;
        m->d.v[i] = m->d.v[m->d.n - 1];
        m->d.n--;
    }
    map_reindex(m, m->d.n);
}

static void truncate_all(map_t* m, double mincoeff, int topk, int max_xweight, int period,
                         int rot_count) {
    if (mincoeff > 0) map_erase_if(m, pred_small, &mincoeff);
    if (topk > 0) truncate_top_k(m, topk);
    if (max_xweight >= 0 && period > 0 && (rot_count + 1) % period == 0)
        map_erase_if(m, pred_xweight, &max_xweight);
}

/* ------------------------------------------------------------------------- */
/* sharded strategy (src/pauli/propagate.h:157-264)                          */
/* ------------------------------------------------------------------------- */

typedef struct {
    int T;
    map_t* sh;
    vec_t* out; /* out[src*T + dst] */
} shards_t;

static inline int shard_of(const uint64_t* k, int T) { return (int)(mix64(hkey(k)) % (uint64_t)T); }

static void shards_from(shards_t* S, const map_t* m) {
    for (int t = 0; t < S->T; t++) map_init(&S->sh[t]);
    for (int64_t i = 0; i < m->d.n; i++) {
        const term_t* e = &m->d.v[i];
        map_add(&S->sh[shard_of(e->k, S->T)], e->k, e->re, e->im);
    }
}

static void shards_to(shards_t* S, map_t* m) {
    map_init(m);
    for (int t = 0; t < S->T; t++) {
        for (int64_t i = 0; i < S->sh[t].d.n; i++) {
            const term_t* e = &S->sh[t].d.v[i];
            map_add(m, e->k, e->re, e->im);
        }
        map_release(&S->sh[t]);
    }
}

static int64_t shards_size(const shards_t* S) {
    int64_t n = 0;
    for (int t = 0; t < S->T; t++) n += S->sh[t].d.n;
    return n;
}

static void pauli_conjugate_sharded(shards_t* S, const ffo_pauli_gate* g, int maxdeg) {
    const int T = S->T;
    const double c = cos(g->theta);
    const double s = sin(g->theta);
#pragma omp parallel num_threads(T)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        map_t* m = &S->sh[tid];
        vec_t local = {0};
        for (int d = 0; d < T; d++) S->out[tid * T + d].n = 0;
        for (int64_t i = 0; i < m->d.n; i++) {
            term_t* t = &m->d.v[i];
            if (!pauli_anticommutes(t->k, g->x, g->z)) continue;
            term_t p;
            int jpow = pauli_mul(g->x, g->z, t->k, p.k);
            if (pauli_degree(p.k) <= maxdeg) {
                double tr, ti, fr, fi;
                cmul(t->re, t->im, 0.0, s, &tr, &ti);
                ipow(jpow, &fr, &fi);
                cmul(tr, ti, fr, fi, &p.re, &p.im);
                int dst = shard_of(p.k, T);
                if (dst == tid)
                    vec_push(&local, &p);
                else
                    vec_push(&S->out[tid * T + dst], &p);
            }
            t->re = t->re * c;
            t->im = t->im * c;
        }
        for (int64_t i = 0; i < local.n; i++) map_add(m, local.v[i].k, local.v[i].re, local.v[i].im);
        free(local.v);
    }
#pragma omp parallel num_threads(T)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        map_t* m = &S->sh[tid];
        for (int src = 0; src < T; src++) {
            vec_t* in = &S->out[src * T + tid];
            for (int64_t i = 0; i < in->n; i++) map_add(m, in->v[i].k, in->v[i].re, in->v[i].im);
        }
    }
}

static void truncate_sharded(shards_t* S, double mincoeff, int topk, int max_xweight, int period,
                             int rot_count) {
    if (topk > 0) {
        map_t m;
        shards_to(S, &m);
        truncate_all(&m, mincoeff, topk, max_xweight, period, rot_count);
        shards_from(S, &m);
        map_release(&m);
        return;
    }
#pragma omp parallel for num_threads(S->T) schedule(static, 1)
    for (int t = 0; t < S->T; t++) truncate_all(&S->sh[t], mincoeff, 0, max_xweight, period, rot_count);
}

/* ------------------------------------------------------------------------- */
/* Pauli driver (src/pauli/propagate.h:297-493)                              */
/* ------------------------------------------------------------------------- */

typedef struct {
    const ffo_pauli_gate* gates;
    const ffo_pauli_params* p;
    map_t* m;        /* serial */
    shards_t* S;     /* sharded (NULL when serial) */
    vec_t nb;
    int rot_count;
    int64_t apps, peak;
    ffo_drops* drops; /* serial strategy only */
    const uint64_t* active;  /* per-rotation mask (NULL: every rotation acts) */
    const int64_t* rot_of;   /* circuit gate index -> rotation index */
} pdrv_t;

static int64_t drv_size(pdrv_t* D) { return D->S ? shards_size(D->S) : D->m->d.n; }

static void drv_rot(pdrv_t* D, int64_t gi) {
    if (D->active) { /* an inactive rotation leaves the terms as they are */
        const int64_t r = D->rot_of[gi];
        if (!((D->active[r >> 6] >> (r & 63)) & 1ULL)) return;
    }
    D->apps += drv_size(D);
    if (D->S)
        pauli_conjugate_sharded(D->S, &D->gates[gi], D->p->maxdegree);
    else
        pauli_conjugate(D->m, &D->gates[gi], D->p->maxdegree, &D->nb, D->drops, gi);
    int64_t n = drv_size(D);
    if (n > D->peak) D->peak = n;
}

static void drv_trunc(pdrv_t* D, int rc) {
    const ffo_pauli_params* p = D->p;
    if (D->S)
        truncate_sharded(D->S, p->mincoeff, p->topk, p->max_xweight, p->xtrunc_period, rc);
    else
        truncate_all(D->m, p->mincoeff, p->topk, p->max_xweight, p->xtrunc_period, rc);
}

static void drv_clifford(pdrv_t* D, int64_t begin, int64_t end) {
    if (D->S) {
        shards_to(D->S, D->m);
        pauli_clifford(D->m, D->gates, begin, end);
        shards_from(D->S, D->m);
        map_release(D->m);
        map_init(D->m);
    } else {
        pauli_clifford(D->m, D->gates, begin, end);
    }
}

/* batch_commuting_gates, propagate.h:272-291 */
static void drv_flush(pdrv_t* D, int64_t* buf, int64_t* nbuf) {
    int64_t start = 0;
    while (start < *nbuf) {
        int64_t end = start + 1;
        while (end < *nbuf) {
            const ffo_pauli_gate* g = &D->gates[buf[end]];
            int ok = 1;
            for (int64_t j = start; j < end && ok; j++) {
                const ffo_pauli_gate* h = &D->gates[buf[j]];
                uint64_t k[4] = {g->x[0], g->x[1], g->z[0], g->z[1]};
                if (pauli_anticommutes(k, h->x, h->z)) ok = 0;
            }
            if (!ok) break;
            end++;
        }
        for (int64_t j = start; j < end; j++) drv_rot(D, buf[j]);
        D->rot_count += (int)(end - start);
        drv_trunc(D, D->rot_count - 1);
        start = end;
    }
    *nbuf = 0;
}

static int valid_qubit(int q) { return q >= 0 && q < 128; }

static ffo_poly* pauli_propagate(const ffo_pauli_gate* gates, int64_t ngates, const uint64_t* keys,
                                 const double* re, const double* im, int64_t n, const ffo_pauli_params* p,
                                 ffo_drops* drops, const uint64_t* active) {
    for (int64_t i = 0; i < ngates; i++) {
        const ffo_pauli_gate* g = &gates[i];
        if (g->kind < 0 || g->kind > FFO_CZ) return NULL;
        if (g->kind != FFO_ROT) {
            if (!valid_qubit(g->q0)) return NULL;
            if (g->kind != FFO_H && g->kind != FFO_S && !valid_qubit(g->q1)) return NULL;
        }
    }
    ffo_poly* out = (ffo_poly*)calloc(1, sizeof(ffo_poly));
    map_init(&out->m);
    for (int64_t i = 0; i < n; i++) {
        uint64_t k[4] = {keys[i], keys[n + i], keys[2 * n + i], keys[3 * n + i]};
        map_add(&out->m, k, re[i], im ? im[i] : 0.0);
    }
    int T = p->n_threads > 1 && !drops ? p->n_threads : 1;
    shards_t S = {0};
    pdrv_t D = {0};
    D.gates = gates;
    D.p = p;
    D.drops = drops;
    D.active = active;
    int64_t* rot_of = NULL;
    if (active) {
        rot_of = (int64_t*)malloc((size_t)(ngates > 0 ? ngates : 1) * sizeof(int64_t));
        int64_t r = 0;
        for (int64_t i = 0; i < ngates; i++) rot_of[i] = gates[i].kind == FFO_ROT ? r++ : -1;
        D.rot_of = rot_of;
    }
    D.m = &out->m;
    D.peak = out->m.d.n;
    if (T > 1) {
        S.T = T;
        S.sh = (map_t*)calloc((size_t)T, sizeof(map_t));
        S.out = (vec_t*)calloc((size_t)T * T, sizeof(vec_t));
        shards_from(&S, &out->m);
        map_release(&out->m);
        map_init(&out->m);
        D.S = &S;
    }
    int64_t cb = 0;
    int pending = 0;
    if (!p->batched) {
        for (int64_t i = ngates - 1; i >= 0; i--) {
            if (gates[i].kind != FFO_ROT) {
                if (!pending) {
                    cb = i;
                    pending = 1;
                }
            } else {
                if (pending) {
                    drv_clifford(&D, i + 1, cb + 1);
                    pending = 0;
                }
                drv_rot(&D, i);
                drv_trunc(&D, D.rot_count);
                D.rot_count++;
            }
        }
    } else {
        int64_t* buf = (int64_t*)malloc((size_t)(ngates > 0 ? ngates : 1) * sizeof(int64_t));
        int64_t nbuf = 0;
        for (int64_t i = ngates - 1; i >= 0; i--) {
            if (gates[i].kind != FFO_ROT) {
                drv_flush(&D, buf, &nbuf);
                if (!pending) {
                    cb = i;
                    pending = 1;
                }
            } else {
                if (pending) {
                    drv_clifford(&D, i + 1, cb + 1);
                    pending = 0;
                }
                buf[nbuf++] = i;
            }
        }
        drv_flush(&D, buf, &nbuf);
        free(buf);
    }
    if (pending) drv_clifford(&D, 0, cb + 1);
    if (T > 1) {
        map_release(&out->m);
        shards_to(&S, &out->m);
        for (int i = 0; i < T * T; i++) free(S.out[i].v);
        free(S.out);
        free(S.sh);
    }
    free(D.nb.v);
    free(rot_of);
    out->apps = D.apps;
    out->peak = D.peak;
    return out;
}

ffo_poly* ffo_pauli_propagate(const ffo_pauli_gate* gates, int64_t ngates, const uint64_t* keys,
                              const double* re, const double* im, int64_t n,
                              const ffo_pauli_params* p) {
    return pauli_propagate(gates, ngates, keys, re, im, n, p, NULL, NULL);
}

ffo_poly* ffo_pauli_propagate_masked(const ffo_pauli_gate* gates, int64_t ngates, const uint64_t* keys,
                                     const double* re, const double* im, int64_t n,
                                     const ffo_pauli_params* p, const uint64_t* active) {
    return pauli_propagate(gates, ngates, keys, re, im, n, p, NULL, active);
}

ffo_poly* ffo_pauli_propagate_capture(const ffo_pauli_gate* gates, int64_t ngates, const uint64_t* keys,
                                      const double* re, const double* im, int64_t n,
                                      const ffo_pauli_params* p, int32_t capdeg, ffo_drops** dropped) {
    ffo_drops* d = (ffo_drops*)calloc(1, sizeof(ffo_drops));
    d->capdeg = capdeg;
    ffo_poly* r = pauli_propagate(gates, ngates, keys, re, im, n, p, d, NULL);
    if (!r) {
        ffo_drops_free(d);
        d = NULL;
    }
    *dropped = d;
    return r;
}

int64_t ffo_drops_size(const ffo_drops* d) { return d ? d->t.n : 0; }

void ffo_drops_copy(const ffo_drops* d, uint64_t* keys, double* re, double* im, int64_t* gate) {
    const int64_t n = d->t.n;
    for (int64_t i = 0; i < n; i++) {
        const term_t* t = &d->t.v[i];
        for (int w = 0; w < 4; w++) keys[w * n + i] = t->k[w];
        re[i] = t->re;
        im[i] = t->im;
        gate[i] = d->gate[i];
    }
}

void ffo_drops_free(ffo_drops* d) {
    if (!d) return;
    free(d->t.v);
    free(d->gate);
    free(d);
}

/* ------------------------------------------------------------------------- */
/* Majorana propagation (src/majorana_gates.h:67-103,                        */
/* src/majorana_propagation.h:18-33)                                         */
/* ------------------------------------------------------------------------- */

/* merge_parity(term, gate): parity of #{(t, g) : t in term, g in gate, t < g}
 * (src/bits_utils.h:14-38): for each set bit g of the gate, the term bits
 * below it are counted. */
static int merge_parity(const uint64_t* term, const uint64_t* gate) {
    int tot = 0;
    for (int wg = 0; wg < 4; wg++) {
        for (uint64_t gb = gate[wg]; gb; gb &= gb - 1) {
            const int b = __builtin_ctzll(gb);
            for (int w = 0; w < wg; w++) tot += popc(term[w]);
            tot += popc(term[wg] & ((1ULL << b) - 1));
        }
    }
    return tot & 1;
}

static int pred_small_maj(const term_t* t, const void* ctx) {
    return ffo_abs(t->re, t->im) <= *(const double*)ctx;
}

ffo_poly* ffo_majorana_propagate(const ffo_majorana_gate* gates, int64_t ngates,
                                 const uint64_t* keys, const double* re, const double* im,
                                 int64_t n, int32_t has_maxdegree, int32_t maxdegree,
                                 double mincoeff) {
    ffo_poly* out = (ffo_poly*)calloc(1, sizeof(ffo_poly));
    map_t* m = &out->m;
    map_init(m);
    for (int64_t i = 0; i < n; i++) {
        uint64_t k[4] = {keys[i], keys[n + i], keys[2 * n + i], keys[3 * n + i]};
        map_add(m, k, re[i], im ? im[i] : 0.0);
    }
    out->peak = m->d.n;
    vec_t nb = {0};
    for (int64_t gi = ngates - 1; gi >= 0; gi--) {
        const ffo_majorana_gate* g = &gates[gi];
        const double c = cos(g->theta);
        const double s = sin(g->theta);
        /* i * i^r * sin(theta) (majorana_gates.h:86-88) */
        double fr = g->r ? -s : 0.0, fi = g->r ? 0.0 : s;
        int nbits = popc(g->alpha[0]) + popc(g->alpha[1]) + popc(g->alpha[2]) + popc(g->alpha[3]);
        out->apps += m->d.n;
        nb.n = 0;
        for (int64_t i = 0; i < m->d.n; i++) {
            term_t* t = &m->d.v[i];
            int na = popc(t->k[0]) + popc(t->k[1]) + popc(t->k[2]) + popc(t->k[3]);
            int nab = popc(t->k[0] & g->alpha[0]) + popc(t->k[1] & g->alpha[1]) +
                      popc(t->k[2] & g->alpha[2]) + popc(t->k[3] & g->alpha[3]);
            if ((na * nbits - nab) % 2 == 0) continue;
            term_t p;
            for (int w = 0; w < 4; w++) p.k[w] = g->alpha[w] ^ t->k[w];
            int deg = popc(p.k[0]) + popc(p.k[1]) + popc(p.k[2]) + popc(p.k[3]);
            if (!has_maxdegree || deg <= maxdegree) {
                double sg = merge_parity(t->k, g->alpha) ? -1.0 : 1.0;
                double tr, ti;
                cmul(t->re, t->im, fr, fi, &tr, &ti);
                cmul(tr, ti, sg, 0.0, &p.re, &p.im);
                vec_push(&nb, &p);
            }
            t->re = t->re * c;
            t->im = t->im * c;
        }
        for (int64_t i = 0; i < nb.n; i++) map_add(m, nb.v[i].k, nb.v[i].re, nb.v[i].im);
        if (m->d.n > out->peak) out->peak = m->d.n;
        if (mincoeff > 0) map_erase_if(m, pred_small_maj, &mincoeff);
    }
    free(nb.v);
    return out;
}

/* ------------------------------------------------------------------------- */
/* results and expectations                                                  */
/* ------------------------------------------------------------------------- */

int64_t ffo_size(const ffo_poly* p) { return p->m.d.n; }
int64_t ffo_apps(const ffo_poly* p) { return p->apps; }
int64_t ffo_peak(const ffo_poly* p) { return p->peak; }

void ffo_copy(const ffo_poly* p, uint64_t* keys, double* re, double* im) {
    int64_t n = p->m.d.n;
    for (int64_t i = 0; i < n; i++) {
        const term_t* t = &p->m.d.v[i];
        for (int w = 0; w < 4; w++) keys[w * n + i] = t->k[w];
        re[i] = t->re;
        im[i] = t->im;
    }
}

void ffo_free(ffo_poly* p) {
    if (!p) return;
    map_release(&p->m);
    free(p);
}

void ffo_overlapwithzero(const ffo_poly* p, double* re, double* im) {
    double r = 0.0, i = 0.0;
    for (int64_t j = 0; j < p->m.d.n; j++) {
        const term_t* t = &p->m.d.v[j];
        if (t->k[0] == 0 && t->k[1] == 0) {
            r = r + t->re;
            i = i + t->im;
        }
    }
    *re = r;
    *im = i;
}

void ffo_qubit_state(const ffo_poly* p, const uint64_t* b, double* re, double* im) {
    double r = 0.0, i = 0.0;
    for (int64_t j = 0; j < p->m.d.n; j++) {
        const term_t* t = &p->m.d.v[j];
        double vr = 0.0, vi = 0.0;
        if (t->k[0] == 0 && t->k[1] == 0) vr = ((popc(t->k[2] & b[0]) + popc(t->k[3] & b[1])) & 1) ? -1.0 : 1.0;
        double xr, xi;
        cmul(t->re, t->im, vr, vi, &xr, &xi);
        r = r + xr;
        i = i + xi;
    }
    *re = r;
    *im = i;
}

/* bits 2j and 2j+1 both set -> bit j of the result (pair set J) */
static uint64_t pairs64(uint64_t w) {
    uint64_t ev = w & 0x5555555555555555ULL, od = (w >> 1) & 0x5555555555555555ULL;
    uint64_t both = ev & od, out = 0;
    for (int j = 0; j < 32; j++) out |= ((both >> (2 * j)) & 1ULL) << j;
    return out;
}

void ffo_fock_state(const ffo_poly* p, const uint64_t* b, double* re, double* im) {
    double r = 0.0, i = 0.0;
    for (int64_t j = 0; j < p->m.d.n; j++) {
        const term_t* t = &p->m.d.v[j];
        int paired = 1;
        for (int w = 0; w < 4; w++) {
            uint64_t ev = t->k[w] & 0x5555555555555555ULL, od = (t->k[w] >> 1) & 0x5555555555555555ULL;
            if (ev != od) paired = 0;
        }
        double vr = 0.0, vi = 0.0;
        if (paired) {
            /* J as a 128-bit set: word w of alpha holds modes 32w..32w+31 */
            uint64_t J0 = pairs64(t->k[0]) | (pairs64(t->k[1]) << 32);
            uint64_t J1 = pairs64(t->k[2]) | (pairs64(t->k[3]) << 32);
            int e = popc(J0) + popc(J1) + 2 * (popc(J0 & b[0]) + popc(J1 & b[1]));
            ipow(e, &vr, &vi);
        }
        double xr, xi;
        cmul(t->re, t->im, vr, vi, &xr, &xi);
        r = r + xr;
        i = i + xi;
    }
    *re = r;
    *im = i;
}
