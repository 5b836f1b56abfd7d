/*
 * bn254_oracle.c -- CPU restatement of pyZKP's hot-path algorithms.
 *
 * ORACLE / TEST INFRASTRUCTURE. Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py may load this library, and
 * only as the checker or the timed CPU baseline -- never as the product path.
 *
 * What it restates (reference files, paths within fzybravery/pyZKP):
 *   - Fr field r = curve_order (crypto/field/fr.py:7), Fq field q
 *     (runtime/metal/msm.py:9); Montgomery form with R = 2^256 as in
 *     runtime/kernels/cpu/kernels.py:46-50,135-141.
 *   - ntt_inplace / intt_inplace (crypto/poly/ntt.py:42-89): bit-reversal
 *     permutation then radix-2 DIT with wlen = omega^(n/len) per level;
 *     iNTT = NTT with omega^-1 then multiply by n^-1.
 *   - evals_from_coeffs_on_roots / coeffs_from_evals_on_roots /
 *     evals_from_coeffs_on_coset / coeffs_from_evals_on_coset
 *     (crypto/poly/ntt.py:103-146): pad/truncate to n, coset scale by shift^i,
 *     inverse coset scale by shift^-i (0 when shift == 0).
 *   - msm_pippenger (crypto/msm/pippenger.py:10-64): unsigned windows of w bits,
 *     k descending over range(0, 254, w), list buckets when 2^w <= 1024 else the
 *     sparse "dict" path with gap multiplications, Horner acc = acc*2^w + sum.
 *   - the G1 group law of py_ecc.optimized_bn128 (crypto/ecc/bn254.py:9-28) in
 *     Jacobian coordinates, complete w.r.t. infinity / P == Q / P == -Q.
 *   - the G2 group law (crypto/ecc/bn254.py g2_add / g2_mul over py_ecc's FQ2 with
 *     u^2 = -1) in Jacobian coordinates over Fq2, and MSM_G2 as the plain sum of
 *     scalar multiples (_msm_g2_impl, runtime/kernels/cpu/kernels.py:574-582).
 *
 * Layout at the ABI: field elements are 4 little-endian uint64 limbs of the
 * canonical value; affine G1 points are 8 limbs (x then y), the point at
 * infinity is (0, 0) (not on y^2 = x^3 + 3). Affine G2 points are 16 limbs
 * (x.c0, x.c1, y.c0, y.c1 for x = x.c0 + x.c1 u), infinity all zero.
 *
 * Portable C11 + pthreads + unsigned __int128 (gcc on x86_64 and aarch64).
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

typedef unsigned __int128 u128;

typedef struct {
    uint64_t p[4];
    uint64_t inv;    /* -p^-1 mod 2^64 */
    uint64_t one[4]; /* R mod p */
    uint64_t r2[4];  /* R^2 mod p */
} field_t;

static field_t FR, FQ;
static int g_init = 0;

static const uint64_t FR_P[4] = {0x43e1f593f0000001ULL, 0x2833e84879b97091ULL, 0xb85045b68181585dULL,
                                 0x30644e72e131a029ULL};
static const uint64_t FQ_P[4] = {0x3c208c16d87cfd47ULL, 0x97816a916871ca8dULL, 0xb85045b68181585dULL,
                                 0x30644e72e131a029ULL};

static int geq(const uint64_t a[4], const uint64_t b[4]) {
    for (int i = 3; i >= 0; i--) {
        if (a[i] != b[i]) return a[i] > b[i];
    }
    return 1;
}

static uint64_t sub4(uint64_t r[4], const uint64_t a[4], const uint64_t b[4]) {
    uint64_t borrow = 0;
    for (int i = 0; i < 4; i++) {
        u128 d = (u128)a[i] - b[i] - borrow;
        r[i] = (uint64_t)d;
        borrow = (uint64_t)(d >> 64) & 1;
    }
    return borrow;
}

static uint64_t add4(uint64_t r[4], const uint64_t a[4], const uint64_t b[4]) {
    u128 c = 0;
    for (int i = 0; i < 4; i++) {
        c += (u128)a[i] + b[i];
        r[i] = (uint64_t)c;
        c >>= 64;
    }
    return (uint64_t)c;
}

static void fadd(const field_t *F, uint64_t r[4], const uint64_t a[4], const uint64_t b[4]) {
    uint64_t t[4];
    uint64_t c = add4(t, a, b);
    if (c || geq(t, F->p)) sub4(t, t, F->p);
    memcpy(r, t, 32);
}

static void fsub(const field_t *F, uint64_t r[4], const uint64_t a[4], const uint64_t b[4]) {
    uint64_t t[4];
    if (sub4(t, a, b)) add4(t, t, F->p);
    memcpy(r, t, 32);
}

/* CIOS Montgomery multiplication: r = a*b*R^-1 mod p, inputs and output < p. */
static void fmul(const field_t *F, uint64_t r[4], const uint64_t a[4], const uint64_t b[4]) {
    uint64_t t[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < 4; i++) {
        uint64_t c = 0;
        for (int j = 0; j < 4; j++) {
            u128 x = (u128)a[j] * b[i] + t[j] + c;
            t[j] = (uint64_t)x;
            c = (uint64_t)(x >> 64);
        }
        u128 s = (u128)t[4] + c;
        t[4] = (uint64_t)s;
        t[5] = (uint64_t)(s >> 64);
        uint64_t m = t[0] * F->inv;
        u128 x = (u128)m * F->p[0] + t[0];
        c = (uint64_t)(x >> 64);
        for (int j = 1; j < 4; j++) {
            x = (u128)m * F->p[j] + t[j] + c;
            t[j - 1] = (uint64_t)x;
            c = (uint64_t)(x >> 64);
        }
        s = (u128)t[4] + c;
        t[3] = (uint64_t)s;
        t[4] = t[5] + (uint64_t)(s >> 64);
    }
    if (t[4] || geq(t, F->p)) sub4(t, t, F->p);
    memcpy(r, t, 32);
}

static int is_zero4(const uint64_t a[4]) { return (a[0] | a[1] | a[2] | a[3]) == 0; }

static void field_setup(field_t *F, const uint64_t p[4]) {
    memcpy(F->p, p, 32);
    /* inv = -p^-1 mod 2^64 by Newton iteration */
    uint64_t x = 1;
    for (int i = 0; i < 7; i++) x *= 2 - p[0] * x;
    F->inv = (uint64_t)0 - x;
    /* one = 2^256 mod p: start from 1 and double 256 times */
    uint64_t t[4] = {1, 0, 0, 0};
    for (int i = 0; i < 256; i++) fadd(F, t, t, t);
    memcpy(F->one, t, 32);
    /* r2 = 2^512 mod p: double 256 more times */
    for (int i = 0; i < 256; i++) fadd(F, t, t, t);
    memcpy(F->r2, t, 32);
}

static void init_once(void) {
    if (g_init) return;
    field_setup(&FR, FR_P);
    field_setup(&FQ, FQ_P);
    g_init = 1;
}

/* canonical (any 256-bit value) -> Montgomery; values >= p are reduced first */
static void to_mont(const field_t *F, uint64_t r[4], const uint64_t a[4]) {
    uint64_t t[4];
    memcpy(t, a, 32);
    while (geq(t, F->p)) sub4(t, t, F->p);
    fmul(F, r, t, F->r2);
}

static void from_mont(const field_t *F, uint64_t r[4], const uint64_t a[4]) {
    const uint64_t one[4] = {1, 0, 0, 0};
    fmul(F, r, a, one);
}

static void fpow(const field_t *F, uint64_t r[4], const uint64_t a[4], const uint64_t e[4]) {
    uint64_t acc[4], base[4];
    memcpy(acc, F->one, 32);
    memcpy(base, a, 32);
    for (int i = 0; i < 4; i++) {
        uint64_t w = e[i];
        for (int b = 0; b < 64; b++) {
            if (w & 1) fmul(F, acc, acc, base);
            fmul(F, base, base, base);
            w >>= 1;
        }
    }
    memcpy(r, acc, 32);
}

static void fpow_u64(const field_t *F, uint64_t r[4], const uint64_t a[4], uint64_t e) {
    const uint64_t ee[4] = {e, 0, 0, 0};
    fpow(F, r, a, ee);
}

static void finv(const field_t *F, uint64_t r[4], const uint64_t a[4]) {
    uint64_t e[4];
    const uint64_t two[4] = {2, 0, 0, 0};
    sub4(e, F->p, two);
    fpow(F, r, a, e);
}

/* ------------------------------------------------------------------------- */
/* threading helper                                                           */
/* ------------------------------------------------------------------------- */
typedef void (*range_fn)(void *ctx, size_t lo, size_t hi);
typedef struct {
    range_fn fn;
    void *ctx;
    size_t lo, hi;
} range_job;

static void *range_thread(void *arg) {
    range_job *j = (range_job *)arg;
    j->fn(j->ctx, j->lo, j->hi);
    return NULL;
}

static int resolve_threads(int nthreads) {
    if (nthreads > 0) return nthreads;
    long c = sysconf(_SC_NPROCESSORS_ONLN);
    return c > 0 ? (int)c : 1;
}

static void parallel_for(size_t total, int nthreads, range_fn fn, void *ctx) {
    nthreads = resolve_threads(nthreads);
    if (nthreads <= 1 || total < 2) {
        fn(ctx, 0, total);
        return;
    }
    if ((size_t)nthreads > total) nthreads = (int)total;
    pthread_t th[256];
    range_job jobs[256];
    if (nthreads > 256) nthreads = 256;
    size_t chunk = (total + nthreads - 1) / nthreads;
    int started = 0;
    for (int t = 0; t < nthreads; t++) {
        size_t lo = (size_t)t * chunk, hi = lo + chunk;
        if (lo >= total) break;
        if (hi > total) hi = total;
        jobs[t].fn = fn;
        jobs[t].ctx = ctx;
        jobs[t].lo = lo;
        jobs[t].hi = hi;
        if (pthread_create(&th[t], NULL, range_thread, &jobs[t]) != 0) {
            fn(ctx, lo, hi);
            jobs[t].fn = NULL;
        }
        started = t + 1;
    }
    for (int t = 0; t < started; t++)
        if (jobs[t].fn) pthread_join(th[t], NULL);
}

/* ------------------------------------------------------------------------- */
/* Fr vector helpers                                                          */
/* ------------------------------------------------------------------------- */
typedef struct {
    uint64_t *a;
    const uint64_t *in;
    int dir; /* 1 = to mont, 0 = from mont */
    const field_t *F;
} conv_ctx;

static void conv_range(void *c, size_t lo, size_t hi) {
    conv_ctx *x = (conv_ctx *)c;
    for (size_t i = lo; i < hi; i++) {
        if (x->dir)
            to_mont(x->F, x->a + 4 * i, x->in + 4 * i);
        else
            from_mont(x->F, x->a + 4 * i, x->in + 4 * i);
    }
}

/* ------------------------------------------------------------------------- */
/* NTT, crypto/poly/ntt.py:42-89                                              */
/* ------------------------------------------------------------------------- */
typedef struct {
    uint64_t *a; /* Montgomery */
    size_t n, half, len;
    uint64_t wlen[4];
} stage_ctx;

static void stage_range(void *c, size_t lo, size_t hi) {
    /* butterflies b in [lo, hi): group i = b / half, j = b % half */
    stage_ctx *s = (stage_ctx *)c;
    uint64_t w[4];
    size_t j0 = lo % s->half;
    fpow_u64(&FR, w, s->wlen, (uint64_t)j0);
    for (size_t b = lo; b < hi; b++) {
        size_t j = b % s->half;
        size_t base = (b / s->half) * s->len;
        if (j == 0 && b != lo) memcpy(w, FR.one, 32);
        uint64_t *u = s->a + 4 * (base + j);
        uint64_t *v = s->a + 4 * (base + j + s->half);
        uint64_t t[4], uu[4];
        fmul(&FR, t, v, w);
        memcpy(uu, u, 32);
        fadd(&FR, u, uu, t);
        fsub(&FR, v, uu, t);
        fmul(&FR, w, w, s->wlen);
    }
}

/* a: n Montgomery elements, omega Montgomery; in-place forward transform. */
static void ntt_inplace_mont(uint64_t *a, size_t n, const uint64_t omega_m[4], int nthreads) {
    if (n <= 1) return;
    /* bit-reversal permutation, the exact index walk of ntt.py:50-57 */
    size_t j = 0;
    for (size_t i = 1; i < n; i++) {
        size_t bit = n >> 1;
        while (j & bit) {
            j ^= bit;
            bit >>= 1;
        }
        j ^= bit;
        if (i < j) {
            uint64_t t[4];
            memcpy(t, a + 4 * i, 32);
            memcpy(a + 4 * i, a + 4 * j, 32);
            memcpy(a + 4 * j, t, 32);
        }
    }
    for (size_t len = 2; len <= n; len <<= 1) {
        stage_ctx s;
        s.a = a;
        s.n = n;
        s.len = len;
        s.half = len >> 1;
        fpow_u64(&FR, s.wlen, omega_m, (uint64_t)(n / len));
        int nt = (n >= (1u << 14)) ? nthreads : 1;
        parallel_for(n / 2, nt, stage_range, &s);
    }
}

static int is_pow2(size_t n) { return n && !(n & (n - 1)); }

/*
 * mode: 0 evals_from_coeffs_on_roots, 1 coeffs_from_evals_on_roots,
 *       2 evals_from_coeffs_on_coset, 3 coeffs_from_evals_on_coset.
 * in: in_len canonical elements; out: n canonical elements. For modes 1 and 3
 * the reference requires in_len == n (a power of two).
 */
int orc_ntt_op(int mode, const uint64_t *in, size_t in_len, uint64_t *out, size_t n, const uint64_t omega[4],
               const uint64_t shift[4], int nthreads) {
    init_once();
    if (!is_pow2(n)) return -1;
    if ((mode == 1 || mode == 3) && in_len != n) return -2;
    uint64_t *a = (uint64_t *)calloc(n, 32);
    if (!a) return -3;
    size_t m = in_len < n ? in_len : n;
    conv_ctx cc = {a, in, 1, &FR};
    parallel_for(m, nthreads, conv_range, &cc);
    uint64_t om[4];
    to_mont(&FR, om, omega);
    if (mode == 2) {
        uint64_t s[4], ps[4];
        to_mont(&FR, s, shift);
        memcpy(ps, FR.one, 32);
        for (size_t i = 0; i < m; i++) {
            fmul(&FR, a + 4 * i, a + 4 * i, ps);
            fmul(&FR, ps, ps, s);
        }
    }
    if (mode == 0 || mode == 2) {
        ntt_inplace_mont(a, n, om, nthreads);
    } else {
        uint64_t iom[4], ninv[4], nn[4] = {(uint64_t)n, 0, 0, 0}, nm[4];
        finv(&FR, iom, om);
        ntt_inplace_mont(a, n, iom, nthreads);
        to_mont(&FR, nm, nn);
        finv(&FR, ninv, nm);
        for (size_t i = 0; i < n; i++) fmul(&FR, a + 4 * i, a + 4 * i, ninv);
        if (mode == 3) {
            uint64_t s[4], is[4], p[4];
            to_mont(&FR, s, shift);
            if (is_zero4(s)) {
                memset(is, 0, 32);
            } else {
                finv(&FR, is, s);
            }
            memcpy(p, FR.one, 32);
            for (size_t i = 0; i < n; i++) {
                fmul(&FR, a + 4 * i, a + 4 * i, p);
                fmul(&FR, p, p, is);
            }
        }
    }
    conv_ctx cd = {out, a, 0, &FR};
    parallel_for(n, nthreads, conv_range, &cd);
    free(a);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* G1 in Jacobian coordinates over Fq (Montgomery), crypto/ecc/bn254.py        */
/* ------------------------------------------------------------------------- */
typedef struct {
    uint64_t X[4], Y[4], Z[4];
} jac;

static void jac_set_inf(jac *p) {
    memcpy(p->X, FQ.one, 32);
    memcpy(p->Y, FQ.one, 32);
    memset(p->Z, 0, 32);
}

static int jac_is_inf(const jac *p) { return is_zero4(p->Z); }

static void jac_dbl(jac *r, const jac *p) {
    if (jac_is_inf(p)) {
        *r = *p;
        return;
    }
    uint64_t A[4], B[4], C[4], S[4], M[4], t[4], X3[4], Y3[4], Z3[4];
    fmul(&FQ, A, p->X, p->X);
    fmul(&FQ, B, p->Y, p->Y);
    fmul(&FQ, C, B, B);
    fmul(&FQ, S, p->X, B);
    fadd(&FQ, S, S, S);
    fadd(&FQ, S, S, S); /* S = 4 X B */
    fadd(&FQ, M, A, A);
    fadd(&FQ, M, M, A); /* M = 3 A */
    fmul(&FQ, X3, M, M);
    fsub(&FQ, X3, X3, S);
    fsub(&FQ, X3, X3, S);
    fsub(&FQ, t, S, X3);
    fmul(&FQ, Y3, M, t);
    fadd(&FQ, C, C, C);
    fadd(&FQ, C, C, C);
    fadd(&FQ, C, C, C); /* 8 C */
    fsub(&FQ, Y3, Y3, C);
    fmul(&FQ, Z3, p->Y, p->Z);
    fadd(&FQ, Z3, Z3, Z3);
    memcpy(r->X, X3, 32);
    memcpy(r->Y, Y3, 32);
    memcpy(r->Z, Z3, 32);
}

static void jac_add(jac *r, const jac *p, const jac *q) {
    if (jac_is_inf(p)) {
        *r = *q;
        return;
    }
    if (jac_is_inf(q)) {
        *r = *p;
        return;
    }
    uint64_t Z1Z1[4], Z2Z2[4], U1[4], U2[4], S1[4], S2[4], H[4], R[4], t[4];
    fmul(&FQ, Z1Z1, p->Z, p->Z);
    fmul(&FQ, Z2Z2, q->Z, q->Z);
    fmul(&FQ, U1, p->X, Z2Z2);
    fmul(&FQ, U2, q->X, Z1Z1);
    fmul(&FQ, t, q->Z, Z2Z2);
    fmul(&FQ, S1, p->Y, t);
    fmul(&FQ, t, p->Z, Z1Z1);
    fmul(&FQ, S2, q->Y, t);
    fsub(&FQ, H, U2, U1);
    fsub(&FQ, R, S2, S1);
    if (is_zero4(H)) {
        if (is_zero4(R)) {
            jac_dbl(r, p);
        } else {
            jac_set_inf(r);
        }
        return;
    }
    uint64_t HH[4], HHH[4], V[4], X3[4], Y3[4], Z3[4];
    fmul(&FQ, HH, H, H);
    fmul(&FQ, HHH, H, HH);
    fmul(&FQ, V, U1, HH);
    fmul(&FQ, X3, R, R);
    fsub(&FQ, X3, X3, HHH);
    fsub(&FQ, X3, X3, V);
    fsub(&FQ, X3, X3, V);
    fsub(&FQ, t, V, X3);
    fmul(&FQ, Y3, R, t);
    fmul(&FQ, t, S1, HHH);
    fsub(&FQ, Y3, Y3, t);
    fmul(&FQ, Z3, p->Z, q->Z);
    fmul(&FQ, Z3, Z3, H);
    memcpy(r->X, X3, 32);
    memcpy(r->Y, Y3, 32);
    memcpy(r->Z, Z3, 32);
}

/* r = p + (x, y) with (x, y) affine Montgomery, not infinity */
static void jac_madd(jac *r, const jac *p, const uint64_t x[4], const uint64_t y[4]) {
    if (jac_is_inf(p)) {
        memcpy(r->X, x, 32);
        memcpy(r->Y, y, 32);
        memcpy(r->Z, FQ.one, 32);
        return;
    }
    uint64_t Z1Z1[4], U2[4], S2[4], H[4], R[4], t[4];
    fmul(&FQ, Z1Z1, p->Z, p->Z);
    fmul(&FQ, U2, x, Z1Z1);
    fmul(&FQ, t, p->Z, Z1Z1);
    fmul(&FQ, S2, y, t);
    fsub(&FQ, H, U2, p->X);
    fsub(&FQ, R, S2, p->Y);
    if (is_zero4(H)) {
        if (is_zero4(R)) {
            jac q;
            memcpy(q.X, x, 32);
            memcpy(q.Y, y, 32);
            memcpy(q.Z, FQ.one, 32);
            jac_dbl(r, &q);
        } else {
            jac_set_inf(r);
        }
        return;
    }
    uint64_t HH[4], HHH[4], V[4], X3[4], Y3[4], Z3[4];
    fmul(&FQ, HH, H, H);
    fmul(&FQ, HHH, H, HH);
    fmul(&FQ, V, p->X, HH);
    fmul(&FQ, X3, R, R);
    fsub(&FQ, X3, X3, HHH);
    fsub(&FQ, X3, X3, V);
    fsub(&FQ, X3, X3, V);
    fsub(&FQ, t, V, X3);
    fmul(&FQ, Y3, R, t);
    fmul(&FQ, t, p->Y, HHH);
    fsub(&FQ, Y3, Y3, t);
    fmul(&FQ, Z3, p->Z, H);
    memcpy(r->X, X3, 32);
    memcpy(r->Y, Y3, 32);
    memcpy(r->Z, Z3, 32);
}

static void jac_mul_u64(jac *r, const jac *p, uint64_t k) {
    jac acc;
    jac_set_inf(&acc);
    for (int b = 63; b >= 0; b--) {
        jac_dbl(&acc, &acc);
        if ((k >> b) & 1) jac_add(&acc, &acc, p);
    }
    *r = acc;
}

/* affine canonical out (x, y) or (0, 0) for infinity */
static void jac_to_affine(uint64_t out[8], const jac *p) {
    if (jac_is_inf(p)) {
        memset(out, 0, 64);
        return;
    }
    uint64_t zi[4], zi2[4], zi3[4], x[4], y[4];
    finv(&FQ, zi, p->Z);
    fmul(&FQ, zi2, zi, zi);
    fmul(&FQ, zi3, zi2, zi);
    fmul(&FQ, x, p->X, zi2);
    fmul(&FQ, y, p->Y, zi3);
    from_mont(&FQ, out, x);
    from_mont(&FQ, out + 4, y);
}

/* ------------------------------------------------------------------------- */
/* msm_pippenger, crypto/msm/pippenger.py:10-64                               */
/* ------------------------------------------------------------------------- */
typedef struct {
    const uint64_t *bx; /* Montgomery affine x, y per point (8 limbs) */
    const uint8_t *inf;
    const uint64_t *s; /* canonical reduced scalars */
    size_t n;
    int w;
    int nwin;
    jac *win_sums; /* per window, index by window number (k / w) */
} pip_ctx;

static uint32_t digit_at(const uint64_t s[4], int k, int w) {
    /* (s >> k) & (2^w - 1) for w <= 20 */
    int limb = k >> 6, off = k & 63;
    uint64_t v = s[limb] >> off;
    if (off + w > 64 && limb + 1 < 4) v |= s[limb + 1] << (64 - off);
    return (uint32_t)(v & ((1ULL << w) - 1));
}

static void pip_window_range(void *c, size_t lo, size_t hi) {
    pip_ctx *x = (pip_ctx *)c;
    size_t bn = (size_t)1 << x->w;
    jac *buckets = (jac *)malloc(bn * sizeof(jac));
    uint8_t *used = (uint8_t *)malloc(bn);
    for (size_t wi = lo; wi < hi; wi++) {
        int k = (int)wi * x->w;
        for (size_t d = 0; d < bn; d++) jac_set_inf(&buckets[d]);
        memset(used, 0, bn);
        for (size_t i = 0; i < x->n; i++) {
            uint32_t d = digit_at(x->s + 4 * i, k, x->w);
            if (d == 0) continue;
            used[d] = 1; /* the dict path keeps a key even when the added point is Z1 */
            if (x->inf[i]) continue;
            jac_madd(&buckets[d], &buckets[d], x->bx + 8 * i, x->bx + 8 * i + 4);
        }
        jac running, wsum;
        jac_set_inf(&running);
        jac_set_inf(&wsum);
        if (bn <= 1024) {
            for (size_t d = bn - 1; d > 0; d--) {
                jac_add(&running, &running, &buckets[d]);
                jac_add(&wsum, &wsum, &running);
            }
        } else {
            size_t prev = bn - 1;
            for (size_t d = bn - 1; d > 0; d--) {
                if (!used[d]) continue;
                size_t gap = prev - d - 1;
                if (gap > 0 && !jac_is_inf(&running)) {
                    jac t;
                    jac_mul_u64(&t, &running, gap);
                    jac_add(&wsum, &wsum, &t);
                }
                jac_add(&running, &running, &buckets[d]);
                jac_add(&wsum, &wsum, &running);
                prev = d;
            }
            if (prev > 1 && !jac_is_inf(&running)) {
                jac t;
                jac_mul_u64(&t, &running, prev - 1);
                jac_add(&wsum, &wsum, &t);
            }
        }
        x->win_sums[wi] = wsum;
    }
    free(buckets);
    free(used);
}

typedef struct {
    uint64_t *bx;
    uint8_t *inf;
    uint64_t *s;
    const uint64_t *bases;
    const uint64_t *scalars;
} prep_ctx;

static void prep_range(void *c, size_t lo, size_t hi) {
    prep_ctx *x = (prep_ctx *)c;
    for (size_t i = lo; i < hi; i++) {
        const uint64_t *b = x->bases + 8 * i;
        x->inf[i] = is_zero4(b) && is_zero4(b + 4);
        if (!x->inf[i]) {
            to_mont(&FQ, x->bx + 8 * i, b);
            to_mont(&FQ, x->bx + 8 * i + 4, b + 4);
        }
        uint64_t t[4];
        memcpy(t, x->scalars + 4 * i, 32);
        while (geq(t, FR.p)) sub4(t, t, FR.p); /* ss = int(s) % FR_MODULUS */
        memcpy(x->s + 4 * i, t, 32);
    }
}

/*
 * bases: n affine canonical points (8 limbs, (0,0) = infinity);
 * scalars: n canonical 256-bit values (reduced mod r like pippenger.py:28).
 * window_bits in [1, 20] (pippenger.py:15-17). out: affine canonical (8 limbs).
 */
int orc_msm_pippenger(const uint64_t *bases, const uint64_t *scalars, size_t n, int window_bits, uint64_t out[8],
                      int nthreads) {
    init_once();
    if (window_bits <= 0 || window_bits > 20) return -1;
    if (n == 0) {
        memset(out, 0, 64);
        return 0;
    }
    prep_ctx pc;
    pc.bx = (uint64_t *)malloc(n * 64);
    pc.inf = (uint8_t *)malloc(n);
    pc.s = (uint64_t *)malloc(n * 32);
    pc.bases = bases;
    pc.scalars = scalars;
    if (!pc.bx || !pc.inf || !pc.s) return -3;
    parallel_for(n, nthreads, prep_range, &pc);
    int max_bits = 254;
    int nwin = (max_bits + window_bits - 1) / window_bits;
    pip_ctx x;
    x.bx = pc.bx;
    x.inf = pc.inf;
    x.s = pc.s;
    x.n = n;
    x.w = window_bits;
    x.nwin = nwin;
    x.win_sums = (jac *)malloc(sizeof(jac) * nwin);
    parallel_for((size_t)nwin, nthreads, pip_window_range, &x);
    jac acc;
    jac_set_inf(&acc);
    for (int wi = nwin - 1; wi >= 0; wi--) {
        for (int d = 0; d < window_bits; d++) jac_dbl(&acc, &acc); /* g1_mul(acc, 1 << w) */
        jac_add(&acc, &acc, &x.win_sums[wi]);
    }
    jac_to_affine(out, &acc);
    free(x.win_sums);
    free(pc.bx);
    free(pc.inf);
    free(pc.s);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* scalar multiplication (bases [k_i]P for known-answer checks)               */
/* ------------------------------------------------------------------------- */
typedef struct {
    const uint64_t *k;
    uint64_t *out;
    jac *table; /* table[j * 256 + d] = d * 2^(8 j) * P, j < 32 */
} fb_ctx;

static void fb_range(void *c, size_t lo, size_t hi) {
    fb_ctx *x = (fb_ctx *)c;
    size_t m = hi - lo;
    if (!m) return;
    jac *acc = (jac *)malloc(m * sizeof(jac));
    for (size_t i = lo; i < hi; i++) {
        jac a;
        jac_set_inf(&a);
        uint64_t kk[4];
        memcpy(kk, x->k + 4 * i, 32);
        while (geq(kk, FR.p)) sub4(kk, kk, FR.p);
        for (int j = 0; j < 32; j++) {
            uint32_t d = (uint32_t)((kk[j >> 3] >> (8 * (j & 7))) & 0xff);
            if (d) jac_add(&a, &a, &x->table[j * 256 + d]);
        }
        acc[i - lo] = a;
    }
    /* batch-normalise with Montgomery's trick */
    uint64_t *pref = (uint64_t *)malloc(m * 32);
    uint64_t run[4];
    memcpy(run, FQ.one, 32);
    for (size_t i = 0; i < m; i++) {
        memcpy(pref + 4 * i, run, 32);
        if (!jac_is_inf(&acc[i])) fmul(&FQ, run, run, acc[i].Z);
    }
    uint64_t inv[4];
    finv(&FQ, inv, run);
    for (size_t ii = m; ii-- > 0;) {
        uint64_t *o = x->out + 8 * (lo + ii);
        if (jac_is_inf(&acc[ii])) {
            memset(o, 0, 64);
            continue;
        }
        uint64_t zi[4], zi2[4], zi3[4], t[4];
        fmul(&FQ, zi, inv, pref + 4 * ii);
        fmul(&FQ, inv, inv, acc[ii].Z);
        fmul(&FQ, zi2, zi, zi);
        fmul(&FQ, zi3, zi2, zi);
        fmul(&FQ, t, acc[ii].X, zi2);
        from_mont(&FQ, o, t);
        fmul(&FQ, t, acc[ii].Y, zi3);
        from_mont(&FQ, o + 4, t);
    }
    free(pref);
    free(acc);
}

/* out[i] = [k_i] P (affine canonical), P affine canonical; k reduced mod r. */
int orc_g1_fixed_base_mul(const uint64_t P[8], const uint64_t *k, size_t n, uint64_t *out, int nthreads) {
    init_once();
    jac *table = (jac *)malloc(sizeof(jac) * 32 * 256);
    if (!table) return -3;
    jac base;
    if (is_zero4(P) && is_zero4(P + 4)) {
        memset(out, 0, n * 64);
        free(table);
        return 0;
    }
    to_mont(&FQ, base.X, P);
    to_mont(&FQ, base.Y, P + 4);
    memcpy(base.Z, FQ.one, 32);
    for (int j = 0; j < 32; j++) {
        jac_set_inf(&table[j * 256]);
        for (int d = 1; d < 256; d++) jac_add(&table[j * 256 + d], &table[j * 256 + d - 1], &base);
        for (int b = 0; b < 8; b++) jac_dbl(&base, &base);
    }
    fb_ctx x = {k, out, table};
    /* chunks of 4096 points so that each thread batch-normalises its own slice */
    size_t chunks = (n + 4095) / 4096;
    int nt = resolve_threads(nthreads);
    for (size_t c0 = 0; c0 < chunks; c0 += (size_t)nt) {
        size_t c1 = c0 + (size_t)nt;
        if (c1 > chunks) c1 = chunks;
        /* run chunks [c0, c1) in parallel: one thread per chunk */
        pthread_t th[256];
        range_job jobs[256];
        int started = 0;
        for (size_t c = c0; c < c1 && started < 256; c++) {
            size_t lo = c * 4096, hi = lo + 4096;
            if (hi > n) hi = n;
            jobs[started].fn = fb_range;
            jobs[started].ctx = &x;
            jobs[started].lo = lo;
            jobs[started].hi = hi;
            if (pthread_create(&th[started], NULL, range_thread, &jobs[started]) != 0) {
                fb_range(&x, lo, hi);
                jobs[started].fn = NULL;
            }
            started++;
        }
        for (int t = 0; t < started; t++)
            if (jobs[t].fn) pthread_join(th[t], NULL);
    }
    free(table);
    return 0;
}

/* out = [k] P for one point (double-and-add over the 256-bit k, reduced mod r). */
int orc_g1_mul(const uint64_t P[8], const uint64_t k[4], uint64_t out[8]) {
    init_once();
    if (is_zero4(P) && is_zero4(P + 4)) {
        memset(out, 0, 64);
        return 0;
    }
    jac base, acc;
    to_mont(&FQ, base.X, P);
    to_mont(&FQ, base.Y, P + 4);
    memcpy(base.Z, FQ.one, 32);
    jac_set_inf(&acc);
    for (int i = 255; i >= 0; i--) {
        jac_dbl(&acc, &acc);
        if ((k[i >> 6] >> (i & 63)) & 1) jac_add(&acc, &acc, &base);
    }
    jac_to_affine(out, &acc);
    return 0;
}

/* out = P + Q on affine canonical points */
int orc_g1_add(const uint64_t P[8], const uint64_t Q[8], uint64_t out[8]) {
    init_once();
    jac a, b;
    if (is_zero4(P) && is_zero4(P + 4)) {
        jac_set_inf(&a);
    } else {
        to_mont(&FQ, a.X, P);
        to_mont(&FQ, a.Y, P + 4);
        memcpy(a.Z, FQ.one, 32);
    }
    if (is_zero4(Q) && is_zero4(Q + 4)) {
        jac_set_inf(&b);
    } else {
        to_mont(&FQ, b.X, Q);
        to_mont(&FQ, b.Y, Q + 4);
        memcpy(b.Z, FQ.one, 32);
    }
    jac_add(&a, &a, &b);
    jac_to_affine(out, &a);
    return 0;
}

/* out = sum_i a_i * b_i mod r (canonical in and out) */
int orc_fr_dot(const uint64_t *a, const uint64_t *b, size_t n, uint64_t out[4]) {
    init_once();
    uint64_t acc[4] = {0, 0, 0, 0};
    for (size_t i = 0; i < n; i++) {
        uint64_t x[4], y[4], t[4];
        to_mont(&FR, x, a + 4 * i);
        to_mont(&FR, y, b + 4 * i);
        fmul(&FR, t, x, y);
        fadd(&FR, acc, acc, t);
    }
    from_mont(&FR, out, acc);
    return 0;
}

/* Montgomery conversions of Fr / Fq vectors: which = 0 Fr, 1 Fq; dir = 1 to, 0 from */
int orc_to_from_mont(int which, int dir, const uint64_t *in, uint64_t *out, size_t n, int nthreads) {
    init_once();
    conv_ctx c = {out, in, dir, which ? &FQ : &FR};
    parallel_for(n, nthreads, conv_range, &c);
    return 0;
}

int orc_num_threads(void) { return resolve_threads(0); }

/* ------------------------------------------------------------------------- */
/* G2 over Fq2 = Fq[u] / (u^2 + 1), Jacobian coordinates (Montgomery)          */
/* ------------------------------------------------------------------------- */
typedef struct {
    uint64_t a[4], b[4]; /* a + b u */
} fq2_t;

typedef struct {
    fq2_t X, Y, Z;
} jac2;

static void f2add(fq2_t *r, const fq2_t *x, const fq2_t *y) {
    fadd(&FQ, r->a, x->a, y->a);
    fadd(&FQ, r->b, x->b, y->b);
}

static void f2sub(fq2_t *r, const fq2_t *x, const fq2_t *y) {
    fsub(&FQ, r->a, x->a, y->a);
    fsub(&FQ, r->b, x->b, y->b);
}

/* (xa + xb u)(ya + yb u) = (xa ya - xb yb) + (xa yb + xb ya) u (schoolbook, 4 products) */
static void f2mul(fq2_t *r, const fq2_t *x, const fq2_t *y) {
    uint64_t t0[4], t1[4], t2[4], t3[4];
    fmul(&FQ, t0, x->a, y->a);
    fmul(&FQ, t1, x->b, y->b);
    fmul(&FQ, t2, x->a, y->b);
    fmul(&FQ, t3, x->b, y->a);
    fsub(&FQ, r->a, t0, t1);
    fadd(&FQ, r->b, t2, t3);
}

static int f2is_zero(const fq2_t *x) { return is_zero4(x->a) && is_zero4(x->b); }

/* 1 / (a + b u) = (a - b u) / (a^2 + b^2) */
static void f2inv(fq2_t *r, const fq2_t *x) {
    uint64_t t0[4], t1[4], z[4] = {0, 0, 0, 0};
    fmul(&FQ, t0, x->a, x->a);
    fmul(&FQ, t1, x->b, x->b);
    fadd(&FQ, t0, t0, t1);
    finv(&FQ, t1, t0);
    fmul(&FQ, r->a, x->a, t1);
    fmul(&FQ, t0, x->b, t1);
    fsub(&FQ, r->b, z, t0);
}

static void jac2_set_inf(jac2 *p) {
    memcpy(p->X.a, FQ.one, 32);
    memset(p->X.b, 0, 32);
    memcpy(p->Y.a, FQ.one, 32);
    memset(p->Y.b, 0, 32);
    memset(&p->Z, 0, sizeof(fq2_t));
}

static int jac2_is_inf(const jac2 *p) { return f2is_zero(&p->Z); }

static void jac2_dbl(jac2 *r, const jac2 *p) {
    if (jac2_is_inf(p)) {
        *r = *p;
        return;
    }
    fq2_t A, B, C, S, M, t, X3, Y3, Z3;
    f2mul(&A, &p->X, &p->X);
    f2mul(&B, &p->Y, &p->Y);
    f2mul(&C, &B, &B);
    f2mul(&S, &p->X, &B);
    f2add(&S, &S, &S);
    f2add(&S, &S, &S); /* 4 X B */
    f2add(&M, &A, &A);
    f2add(&M, &M, &A); /* 3 A */
    f2mul(&X3, &M, &M);
    f2sub(&X3, &X3, &S);
    f2sub(&X3, &X3, &S);
    f2sub(&t, &S, &X3);
    f2mul(&Y3, &M, &t);
    f2add(&C, &C, &C);
    f2add(&C, &C, &C);
    f2add(&C, &C, &C); /* 8 C */
    f2sub(&Y3, &Y3, &C);
    f2mul(&Z3, &p->Y, &p->Z);
    f2add(&Z3, &Z3, &Z3);
    r->X = X3;
    r->Y = Y3;
    r->Z = Z3;
}

static void jac2_add(jac2 *r, const jac2 *p, const jac2 *q) {
    if (jac2_is_inf(p)) {
        *r = *q;
        return;
    }
    if (jac2_is_inf(q)) {
        *r = *p;
        return;
    }
    fq2_t Z1Z1, Z2Z2, U1, U2, S1, S2, H, R, t;
    f2mul(&Z1Z1, &p->Z, &p->Z);
    f2mul(&Z2Z2, &q->Z, &q->Z);
    f2mul(&U1, &p->X, &Z2Z2);
    f2mul(&U2, &q->X, &Z1Z1);
    f2mul(&t, &q->Z, &Z2Z2);
    f2mul(&S1, &p->Y, &t);
    f2mul(&t, &p->Z, &Z1Z1);
    f2mul(&S2, &q->Y, &t);
    f2sub(&H, &U2, &U1);
    f2sub(&R, &S2, &S1);
    if (f2is_zero(&H)) {
        if (f2is_zero(&R)) {
            jac2_dbl(r, p);
        } else {
            jac2_set_inf(r);
        }
        return;
    }
    fq2_t HH, HHH, V, X3, Y3, Z3;
    f2mul(&HH, &H, &H);
    f2mul(&HHH, &H, &HH);
    f2mul(&V, &U1, &HH);
    f2mul(&X3, &R, &R);
    f2sub(&X3, &X3, &HHH);
    f2sub(&X3, &X3, &V);
    f2sub(&X3, &X3, &V);
    f2sub(&t, &V, &X3);
    f2mul(&Y3, &R, &t);
    f2mul(&t, &S1, &HHH);
    f2sub(&Y3, &Y3, &t);
    f2mul(&Z3, &p->Z, &q->Z);
    f2mul(&Z3, &Z3, &H);
    r->X = X3;
    r->Y = Y3;
    r->Z = Z3;
}

static void jac2_from_affine(jac2 *r, const uint64_t P[16]) {
    if (is_zero4(P) && is_zero4(P + 4) && is_zero4(P + 8) && is_zero4(P + 12)) {
        jac2_set_inf(r);
        return;
    }
    to_mont(&FQ, r->X.a, P);
    to_mont(&FQ, r->X.b, P + 4);
    to_mont(&FQ, r->Y.a, P + 8);
    to_mont(&FQ, r->Y.b, P + 12);
    memcpy(r->Z.a, FQ.one, 32);
    memset(r->Z.b, 0, 32);
}

static void jac2_to_affine(uint64_t out[16], const jac2 *p) {
    if (jac2_is_inf(p)) {
        memset(out, 0, 128);
        return;
    }
    fq2_t zi, zi2, zi3, x, y;
    f2inv(&zi, &p->Z);
    f2mul(&zi2, &zi, &zi);
    f2mul(&zi3, &zi2, &zi);
    f2mul(&x, &p->X, &zi2);
    f2mul(&y, &p->Y, &zi3);
    from_mont(&FQ, out, x.a);
    from_mont(&FQ, out + 4, x.b);
    from_mont(&FQ, out + 8, y.a);
    from_mont(&FQ, out + 12, y.b);
}

static void jac2_mul(jac2 *r, const jac2 *p, const uint64_t k[4]) {
    uint64_t kk[4];
    memcpy(kk, k, 32);
    while (geq(kk, FR.p)) sub4(kk, kk, FR.p);
    jac2 acc;
    jac2_set_inf(&acc);
    for (int i = 255; i >= 0; i--) {
        jac2_dbl(&acc, &acc);
        if ((kk[i >> 6] >> (i & 63)) & 1) jac2_add(&acc, &acc, p);
    }
    *r = acc;
}

/* out = [k] P on affine canonical G2 points (k reduced mod r). */
int orc_g2_mul(const uint64_t P[16], const uint64_t k[4], uint64_t out[16]) {
    init_once();
    jac2 base, acc;
    jac2_from_affine(&base, P);
    jac2_mul(&acc, &base, k);
    jac2_to_affine(out, &acc);
    return 0;
}

/* out = P + Q on affine canonical G2 points */
int orc_g2_add(const uint64_t P[16], const uint64_t Q[16], uint64_t out[16]) {
    init_once();
    jac2 a, b;
    jac2_from_affine(&a, P);
    jac2_from_affine(&b, Q);
    jac2_add(&a, &a, &b);
    jac2_to_affine(out, &a);
    return 0;
}

typedef struct {
    const uint64_t *bases; /* msm: n affine canonical G2 points (16 limbs each) */
    const uint64_t *k;     /* n scalars */
    uint64_t *out;         /* fixed-base: n affine canonical results */
    const jac2 *table;     /* fixed-base: table[j * 16 + d] = d * 2^(4 j) * P, j < 64 */
    jac2 *total;           /* msm: running sum of the per-thread partial sums */
    pthread_mutex_t mu;
} g2_ctx;

static void g2_fb_range(void *c, size_t lo, size_t hi) {
    g2_ctx *x = (g2_ctx *)c;
    for (size_t i = lo; i < hi; i++) {
        uint64_t kk[4];
        memcpy(kk, x->k + 4 * i, 32);
        while (geq(kk, FR.p)) sub4(kk, kk, FR.p);
        jac2 a;
        jac2_set_inf(&a);
        for (int j = 0; j < 64; j++) {
            uint32_t d = (uint32_t)((kk[j >> 4] >> (4 * (j & 15))) & 0xf);
            if (d) jac2_add(&a, &a, &x->table[j * 16 + d]);
        }
        jac2_to_affine(x->out + 16 * i, &a);
    }
}

/* out[i] = [k_i] P (affine canonical G2), from a table of 4-bit windows. */
int orc_g2_fixed_base_mul(const uint64_t P[16], const uint64_t *k, size_t n, uint64_t *out, int nthreads) {
    init_once();
    jac2 *table = (jac2 *)malloc(sizeof(jac2) * 64 * 16);
    if (!table) return -3;
    jac2 base;
    jac2_from_affine(&base, P);
    for (int j = 0; j < 64; j++) {
        jac2_set_inf(&table[j * 16]);
        for (int d = 1; d < 16; d++) jac2_add(&table[j * 16 + d], &table[j * 16 + d - 1], &base);
        for (int b = 0; b < 4; b++) jac2_dbl(&base, &base);
    }
    g2_ctx x;
    memset(&x, 0, sizeof(x));
    x.k = k;
    x.out = out;
    x.table = table;
    parallel_for(n, nthreads, g2_fb_range, &x);
    free(table);
    return 0;
}

static void g2_msm_range(void *c, size_t lo, size_t hi) {
    g2_ctx *x = (g2_ctx *)c;
    jac2 acc;
    jac2_set_inf(&acc);
    for (size_t i = lo; i < hi; i++) {
        jac2 p, t;
        jac2_from_affine(&p, x->bases + 16 * i);
        jac2_mul(&t, &p, x->k + 4 * i);
        jac2_add(&acc, &acc, &t);
    }
    pthread_mutex_lock(&x->mu);
    jac2_add(x->total, x->total, &acc);
    pthread_mutex_unlock(&x->mu);
}

/* MSM_G2 as sum_i [s_i] P_i (runtime/kernels/cpu/kernels.py:574-582; every result is the
 * same unique point whatever the method). bases: n affine canonical G2 points. */
int orc_g2_msm(const uint64_t *bases, const uint64_t *scalars, size_t n, uint64_t out[16], int nthreads) {
    init_once();
    g2_ctx x;
    jac2 total;
    memset(&x, 0, sizeof(x));
    jac2_set_inf(&total);
    x.bases = bases;
    x.k = scalars;
    x.total = &total;
    pthread_mutex_init(&x.mu, NULL);
    parallel_for(n, nthreads, g2_msm_range, &x);
    pthread_mutex_destroy(&x.mu);
    jac2_to_affine(out, &total);
    return 0;
}
