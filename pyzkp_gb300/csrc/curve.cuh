// curve.cuh -- BN254 point arithmetic for the MSM kernels: G1 (y^2 = x^3 + 3 over Fq)
// and G2 (the sextic twist y^2 = x^3 + 3/(9 + u) over Fq2 = Fq[u]/(u^2 + 1)).
//
// Bases are affine (x, y) in Montgomery form (64 bytes for G1, 128 for G2); the point at
// infinity is stored as all-zero coordinates, which is on neither curve. Bucket
// accumulators use XYZZ coordinates (x = X/ZZ, y = Y/ZZZ, ZZ^3 = ZZZ^2), infinity is
// ZZ == 0. The formulas are the published short-Weierstrass a = 0 XYZZ formulas
// (madd-2008-s, add-2008-s, dbl-2008-s-1, mdbl-2008-s-1 of the Explicit-Formulas
// Database); they do not involve b, so one generic version serves both groups. They are
// made complete by handling infinity, P == Q (doubling) and P == -Q (infinity)
// explicitly -- the same cases the reference's Jacobian code handles
// (runtime/metal/ecc_source.py:206-293; G2 in crypto/ecc/bn254.py via py_ecc).
#pragma once
#include "field.cuh"

namespace zk {

// ---- Fq2 = Fq[u] / (u^2 + 1) ------------------------------------------------------------
struct __align__(16) fq2 {
    fe c0, c1;  // c0 + c1 u
};

// ---- coordinate operations, overloaded for Fq (fe) and Fq2 (fq2) ------------------------
__device__ __forceinline__ fe c_add(const fe& a, const fe& b) { return fe_add<FqP>(a, b); }
__device__ __forceinline__ fe c_sub(const fe& a, const fe& b) { return fe_sub<FqP>(a, b); }
__device__ __forceinline__ fe c_dbl(const fe& a) { return fe_dbl<FqP>(a); }
__device__ __forceinline__ fe c_neg(const fe& a) { return fe_neg<FqP>(a); }
__device__ __forceinline__ fe c_mul(const fe& a, const fe& b) { return fe_mul<FqP>(a, b); }
__device__ __forceinline__ fe c_sqr(const fe& a) { return fe_sqr<FqP>(a); }
// a b - c d with one reduction (field.cuh, separated forms)
__device__ __forceinline__ fe c_mul_sub(const fe& a, const fe& b, const fe& c, const fe& d) {
    return fe_mul_sub<FqP>(a, b, c, d);
}
// zero mod q: the curve formulas keep Fq values lazy in [0, 2q) (field.cuh)
__device__ __forceinline__ bool c_is_zero(const fe& a) { return fe_is_zero_mod<FqP, true>(a); }
__device__ __forceinline__ void c_set_zero(fe& a) { a = fe_zero(); }
__device__ __forceinline__ void c_set_one(fe& a) { a = fe_one<FqP>(); }
__device__ __forceinline__ fe c_ldg(const fe* p) { return fe_ldg(p); }
__device__ __forceinline__ fe c_load(const fe* p) { return fe_load(p); }
__device__ __forceinline__ void c_store(fe* p, const fe& a) { fe_store(p, a); }

template <class T>
struct c_pair {
    T x, y;
};

// Two independent products; for Fq they go through fe_mul2 (one interleaved pair when
// ZK_USE_MUL2 is set).
__device__ __forceinline__ c_pair<fe> c_mul2(const fe& a, const fe& b, const fe& c, const fe& d) {
    const fe2 r = fe_mul2<FqP>(a, b, c, d);
    return {r.x, r.y};
}

__device__ __forceinline__ fq2 c_add(const fq2& a, const fq2& b) { return {c_add(a.c0, b.c0), c_add(a.c1, b.c1)}; }
__device__ __forceinline__ fq2 c_sub(const fq2& a, const fq2& b) { return {c_sub(a.c0, b.c0), c_sub(a.c1, b.c1)}; }
__device__ __forceinline__ fq2 c_dbl(const fq2& a) { return {c_dbl(a.c0), c_dbl(a.c1)}; }
__device__ __forceinline__ fq2 c_neg(const fq2& a) { return {c_neg(a.c0), c_neg(a.c1)}; }
// (a0 + a1 u)(b0 + b1 u) = (a0 b0 - a1 b1) + (a0 b1 + a1 b0) u, Karatsuba: the u coefficient
// is (a0 + a1)(b0 + b1) - a0 b0 - a1 b1. ZK_FQ2_SCHOOLBOOK selects a0 b0 - a1 b1, a0 b1 + a1 b0
// with one reduction each instead (4 partial products): measured on GB300 against full
// Karatsuba products, accumulation 12.1 / 10.5 ms at 2^20, whole MSM 14.8 / 13.4 ms.
#ifdef ZK_FQ2_SCHOOLBOOK
constexpr bool kFq2Schoolbook = true;
#else
constexpr bool kFq2Schoolbook = false;
#endif
// Default: Karatsuba with lazy reduction (fe2_mul_lazy: 3 unreduced 512-bit products, 2
// reductions; ZK_FQ2_FULL keeps 3 full products). Measured on GB300 (G2 MSM): 2.03 / 2.45 ms
// at 2^16, 4.55 / 5.27 ms at 2^18, 12.71 / 13.35 ms at 2^20 (accumulation -2%, window
// reduction and fixup kernels -18 to -28%).
#ifdef ZK_FQ2_FULL
constexpr bool kFq2Lazy = false;
#else
constexpr bool kFq2Lazy = true;
#endif
__device__ __forceinline__ fq2 c_mul(const fq2& a, const fq2& b) {
    if constexpr (use_sos<FqP>() && kFq2Lazy) {
        const fe_pair r = fe2_mul_lazy_call<FqP>(a.c0, a.c1, b.c0, b.c1);
        return {r.c0, r.c1};
    } else if constexpr (use_sos<FqP>() && kFq2Schoolbook) {
        return {fe_mul_sub<FqP>(a.c0, b.c0, a.c1, b.c1), fe_mul_add<FqP>(a.c0, b.c1, a.c1, b.c0)};
    } else {
        const fe t0 = c_mul(a.c0, b.c0);
        const fe t1 = c_mul(a.c1, b.c1);
        const fe t2 = c_mul(c_add(a.c0, a.c1), c_add(b.c0, b.c1));
        return {c_sub(t0, t1), c_sub(c_sub(t2, t0), t1)};
    }
}
// (a0 + a1 u)^2 = (a0 + a1)(a0 - a1) + 2 a0 a1 u: 2 products
__device__ __forceinline__ fq2 c_sqr(const fq2& a) {
    const fe t0 = c_mul(c_add(a.c0, a.c1), c_sub(a.c0, a.c1));
    const fe t1 = c_mul(a.c0, a.c1);
    return {t0, c_dbl(t1)};
}
__device__ __forceinline__ bool c_is_zero(const fq2& a) {
    return fe_is_zero_mod<FqP>(a.c0) && fe_is_zero_mod<FqP>(a.c1);
}
__device__ __forceinline__ void c_set_zero(fq2& a) {
    a.c0 = fe_zero();
    a.c1 = fe_zero();
}
__device__ __forceinline__ void c_set_one(fq2& a) {
    a.c0 = fe_one<FqP>();
    a.c1 = fe_zero();
}
__device__ __forceinline__ fq2 c_ldg(const fq2* p) { return {fe_ldg(&p->c0), fe_ldg(&p->c1)}; }
__device__ __forceinline__ fq2 c_load(const fq2* p) { return {fe_load(&p->c0), fe_load(&p->c1)}; }
__device__ __forceinline__ void c_store(fq2* p, const fq2& a) {
    fe_store(&p->c0, a.c0);
    fe_store(&p->c1, a.c1);
}
__device__ __forceinline__ c_pair<fq2> c_mul2(const fq2& a, const fq2& b, const fq2& c, const fq2& d) {
    return {c_mul(a, b), c_mul(c, d)};
}

// Pairs with squares, {a^2, b^2} and {a^2, c d}: over Fq a square has its own product form
// (field.cuh) when the separated forms are on; over Fq2 a square takes 2 Fq products
// instead of 3. c_mul_sub(a, b, c, d) = a b - c d, one reduction over Fq.
__device__ __forceinline__ c_pair<fe> c_sqr2(const fe& a, const fe& b) {
    if constexpr (use_sos<FqP>()) return {c_sqr(a), c_sqr(b)};
    else return c_mul2(a, a, b, b);
}
__device__ __forceinline__ c_pair<fe> c_sqr_mul(const fe& a, const fe& c, const fe& d) {
    if constexpr (use_sos<FqP>()) return {c_sqr(a), c_mul(c, d)};
    else return c_mul2(a, a, c, d);
}
__device__ __forceinline__ fq2 c_mul_sub(const fq2& a, const fq2& b, const fq2& c, const fq2& d) {
    return c_sub(c_mul(a, b), c_mul(c, d));
}
__device__ __forceinline__ c_pair<fq2> c_sqr2(const fq2& a, const fq2& b) { return {c_sqr(a), c_sqr(b)}; }
__device__ __forceinline__ c_pair<fq2> c_sqr_mul(const fq2& a, const fq2& c, const fq2& d) {
    return {c_sqr(a), c_mul(c, d)};
}

// ---- points -------------------------------------------------------------------------------
template <class T>
struct __align__(16) AffineT {
    T x, y;
};

template <class T>
struct __align__(16) XyzzT {
    T X, Y, ZZ, ZZZ;
};

using affine_t = AffineT<fe>;
using xyzz_t = XyzzT<fe>;
using affine2_t = AffineT<fq2>;
using xyzz2_t = XyzzT<fq2>;

template <class T>
__device__ __forceinline__ bool affine_is_inf(const AffineT<T>& p) {
    return c_is_zero(p.x) && c_is_zero(p.y);
}

// OR of every limb of a coordinate
__device__ __forceinline__ uint32_t c_bits_or(const fe& a) {
    return a.v[0] | a.v[1] | a.v[2] | a.v[3] | a.v[4] | a.v[5] | a.v[6] | a.v[7];
}
__device__ __forceinline__ uint32_t c_bits_or(const fq2& a) { return c_bits_or(a.c0) | c_bits_or(a.c1); }

// The stored form of infinity in a base array: all bits zero. Exact for stored bases: the
// Montgomery conversion keeps 0 at 0, and no point of either curve has x = y = 0.
template <class T>
__device__ __forceinline__ bool affine_is_zero_bits(const AffineT<T>& p) {
    return (c_bits_or(p.x) | c_bits_or(p.y)) == 0;
}

template <class T = fe>
__device__ __forceinline__ XyzzT<T> xyzz_inf() {
    XyzzT<T> r;
    c_set_zero(r.X);
    c_set_zero(r.Y);
    c_set_zero(r.ZZ);
    c_set_zero(r.ZZZ);
    return r;
}

template <class T>
__device__ __forceinline__ bool xyzz_is_inf(const XyzzT<T>& p) {
    return c_is_zero(p.ZZ);
}

template <class T>
__device__ __forceinline__ XyzzT<T> xyzz_neg(const XyzzT<T>& p) {
    XyzzT<T> r = p;
    r.Y = c_neg(p.Y);
    return r;
}

// The formulas below issue their multiplications in independent pairs (c_mul2), so the
// two carry-chain sequences of a pair can overlap.

// 2 * (x, y) for an affine point that is not infinity (y != 0 on these curves).
template <class T>
__device__ __forceinline__ XyzzT<T> xyzz_dbl_affine(const T& x, const T& y) {
    const T U = c_dbl(y);
    const c_pair<T> vx = c_sqr2(U, x);              // V = U^2, x^2
    const c_pair<T> ws = c_mul2(U, vx.x, x, vx.x);  // W = U V, S = x V
    const T M = c_add(c_dbl(vx.y), vx.y);
    const T MM = c_sqr(M);
    XyzzT<T> r;
    r.X = c_sub(MM, c_dbl(ws.y));
    r.Y = c_mul_sub(M, c_sub(ws.y, r.X), ws.x, y);
    r.ZZ = vx.x;
    r.ZZZ = ws.x;
    return r;
}

template <class T>
__device__ __forceinline__ XyzzT<T> xyzz_dbl(const XyzzT<T>& p) {
    if (xyzz_is_inf(p)) return p;
    const T U = c_dbl(p.Y);
    const c_pair<T> vx = c_sqr2(U, p.X);              // V = U^2, X^2
    const c_pair<T> ws = c_mul2(U, vx.x, p.X, vx.x);  // W = U V, S = X V
    const T M = c_add(c_dbl(vx.y), vx.y);
    const c_pair<T> mz = c_sqr_mul(M, vx.x, p.ZZ);  // M^2, ZZ3 = V ZZ
    XyzzT<T> r;
    r.X = c_sub(mz.x, c_dbl(ws.y));
    r.Y = c_mul_sub(M, c_sub(ws.y, r.X), ws.x, p.Y);
    r.ZZ = mz.y;
    r.ZZZ = c_mul(ws.x, p.ZZZ);
    return r;
}

// acc + (x, y), (x, y) affine and not infinity.
template <class T>
__device__ __forceinline__ XyzzT<T> xyzz_madd(const XyzzT<T>& acc, const T& x, const T& y) {
    if (xyzz_is_inf(acc)) {
        XyzzT<T> r;
        r.X = x;
        r.Y = y;
        c_set_one(r.ZZ);
        c_set_one(r.ZZZ);
        return r;
    }
    const c_pair<T> us = c_mul2(x, acc.ZZ, y, acc.ZZZ);  // U2, S2
    const T P = c_sub(us.x, acc.X);
    const T R = c_sub(us.y, acc.Y);
    if (c_is_zero(P)) {
        if (c_is_zero(R)) return xyzz_dbl_affine(x, y);
        return xyzz_inf<T>();
    }
    const c_pair<T> pr = c_sqr2(P, R);                  // PP, R^2
    const c_pair<T> pq = c_mul2(P, pr.x, acc.X, pr.x);  // PPP, Q
    XyzzT<T> r;
    r.X = c_sub(c_sub(pr.y, pq.x), c_dbl(pq.y));
    const c_pair<T> zz = c_mul2(acc.ZZ, pr.x, acc.ZZZ, pq.x);
    r.Y = c_mul_sub(R, c_sub(pq.y, r.X), acc.Y, pq.x);
    r.ZZ = zz.x;
    r.ZZZ = zz.y;
    return r;
}

template <class T>
__device__ __forceinline__ XyzzT<T> xyzz_add(const XyzzT<T>& p, const XyzzT<T>& q) {
    if (xyzz_is_inf(p)) return q;
    if (xyzz_is_inf(q)) return p;
    const c_pair<T> u = c_mul2(p.X, q.ZZ, q.X, p.ZZ);    // U1, U2
    const c_pair<T> s = c_mul2(p.Y, q.ZZZ, q.Y, p.ZZZ);  // S1, S2
    const T P = c_sub(u.y, u.x);
    const T R = c_sub(s.y, s.x);
    if (c_is_zero(P)) {
        if (c_is_zero(R)) return xyzz_dbl(p);
        return xyzz_inf<T>();
    }
    const c_pair<T> pr = c_sqr2(P, R);                // PP, R^2
    const c_pair<T> pq = c_mul2(P, pr.x, u.x, pr.x);  // PPP, Q
    const c_pair<T> zz = c_mul2(p.ZZ, q.ZZ, p.ZZZ, q.ZZZ);
    XyzzT<T> r;
    r.X = c_sub(c_sub(pr.y, pq.x), c_dbl(pq.y));
    const c_pair<T> z3 = c_mul2(zz.x, pr.x, zz.y, pq.x);
    r.Y = c_mul_sub(R, c_sub(pq.y, r.X), s.x, pq.x);
    r.ZZ = z3.x;
    r.ZZZ = z3.y;
    return r;
}

template <class T>
__device__ __forceinline__ AffineT<T> affine_load(const AffineT<T>* p) {
    AffineT<T> r;
    r.x = c_ldg(&p->x);
    r.y = c_ldg(&p->y);
    return r;
}

template <class T>
__device__ __forceinline__ XyzzT<T> xyzz_load(const XyzzT<T>* p) {
    XyzzT<T> r;
    r.X = c_load(&p->X);
    r.Y = c_load(&p->Y);
    r.ZZ = c_load(&p->ZZ);
    r.ZZZ = c_load(&p->ZZZ);
    return r;
}

// The same through L2 only (points written earlier in the same launch by other CTAs).
__device__ __forceinline__ fe c_ldcg(const fe* p) { return fe_ldcg(p); }
__device__ __forceinline__ fq2 c_ldcg(const fq2* p) { return {fe_ldcg(&p->c0), fe_ldcg(&p->c1)}; }

template <class T>
__device__ __forceinline__ XyzzT<T> xyzz_ldcg(const XyzzT<T>* p) {
    XyzzT<T> r;
    r.X = c_ldcg(&p->X);
    r.Y = c_ldcg(&p->Y);
    r.ZZ = c_ldcg(&p->ZZ);
    r.ZZZ = c_ldcg(&p->ZZZ);
    return r;
}

// xyzz_load, or xyzz_ldcg when kL2 (inputs produced in the same launch)
template <bool kL2, class T>
__device__ __forceinline__ XyzzT<T> xyzz_get(const XyzzT<T>* p) {
    if constexpr (kL2) return xyzz_ldcg(p);
    else return xyzz_load(p);
}

template <class T>
__device__ __forceinline__ void xyzz_store(XyzzT<T>* p, const XyzzT<T>& a) {
    c_store(&p->X, a.X);
    c_store(&p->Y, a.Y);
    c_store(&p->ZZ, a.ZZ);
    c_store(&p->ZZZ, a.ZZZ);
}

// The two groups as template arguments of the MSM kernels.
// Minimum resident 128-thread CTAs per SM asked of the G1 accumulation: 4 caps it at 128
// registers (no spills), 16 warps per SM; measured on GB300 against no cap (130 registers,
// 12 warps): 3.26 / 3.29 ms at 2^20, 12.80 / 12.92 ms at 2^22.
#ifndef ZK_ACC_MINB
#define ZK_ACC_MINB 4
#endif
#ifndef ZK_ACC_MINB_G2
#define ZK_ACC_MINB_G2 1
#endif
// Threads of the CTA that sums one long bucket's pieces (strided partial sums, then a
// shared-memory tree of the threads' partials); G2 points (256 B) keep it at 128 so that
// the tree fits 32 KB of static shared memory. G1 runs 128 threads with four CTAs per SM
// (a grid of as many): since huge buckets are summed in chunks by many CTAs, the CTA size
// serves the long buckets of small pipelines, whose few pieces leave most of a wide CTA
// idle. Measured on GB300 against 256 threads at two CTAs per SM: single MSMs 2^14 / 2^16
// 0.476 / 0.758 -> 0.466 / 0.713 ms, 64 instances of 2^10..2^14 4.41 -> 4.28 ms; 2^18
// +0.5%, witness-like 2^20 fixup 0.139 -> 0.158 ms. (Before the chunks, 256 threads had
// won: one CTA summed the ~1600-segment bucket that witness-like 0/1 values make at 2^20.)
#ifndef ZK_FIXUP_LONG_G1
#define ZK_FIXUP_LONG_G1 128
#endif
// Minimum resident 128-thread CTAs per SM asked of the G1 merge and fixup kernels (G2 keeps
// 1: its points need the registers).
#ifndef ZK_RED_MINB
#define ZK_RED_MINB 1
#endif
#ifndef ZK_FIXUP_LONG_MINB_G1
#define ZK_FIXUP_LONG_MINB_G1 4
#endif
struct CurveG1 {
    using T = fe;
    using A = affine_t;
    using P = xyzz_t;
    static constexpr int kTargetThreads = 256;
    static constexpr int kAccMinBlocks = ZK_ACC_MINB;
    static constexpr int kFixupLongThreads = ZK_FIXUP_LONG_G1;
    static constexpr int kFixupLongMinBlocks = ZK_FIXUP_LONG_MINB_G1;
    static constexpr int kRedMinBlocks = ZK_RED_MINB;
};

struct CurveG2 {
    using T = fq2;
    using A = affine2_t;
    using P = xyzz2_t;
    static constexpr int kTargetThreads = 128;  // 128 x 256-byte points of shared memory
    static constexpr int kAccMinBlocks = ZK_ACC_MINB_G2;
    static constexpr int kFixupLongThreads = 128;
    static constexpr int kFixupLongMinBlocks = 1;
    static constexpr int kRedMinBlocks = 1;
};

}  // namespace zk
