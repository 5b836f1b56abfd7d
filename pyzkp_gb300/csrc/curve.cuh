// curve.cuh -- BN254 G1 (y^2 = x^3 + 3 over Fq) point arithmetic for the MSM kernels.
//
// Bases are affine (x, y) in Montgomery form, 64 bytes; the point at infinity is
// stored as (0, 0), which is not on the curve. Bucket accumulators use XYZZ
// coordinates (x = X/ZZ, y = Y/ZZZ, ZZ^3 = ZZZ^2), infinity is ZZ == 0. The formulas
// are the published short-Weierstrass a = 0 XYZZ formulas (madd-2008-s, add-2008-s,
// dbl-2008-s-1, mdbl-2008-s-1 of the Explicit-Formulas Database), made complete here
// by handling infinity, P == Q (doubling) and P == -Q (infinity) explicitly -- the
// same cases the reference's Jacobian code handles (runtime/metal/ecc_source.py:206-293).
#pragma once
#include "field.cuh"

namespace zk {

struct __align__(16) affine_t {
    fe x, y;
};

struct __align__(16) xyzz_t {
    fe X, Y, ZZ, ZZZ;
};

__device__ __forceinline__ bool affine_is_inf(const affine_t& p) { return fe_is_zero(p.x) && fe_is_zero(p.y); }

__device__ __forceinline__ xyzz_t xyzz_inf() {
    xyzz_t r;
    r.X = fe_zero();
    r.Y = fe_zero();
    r.ZZ = fe_zero();
    r.ZZZ = fe_zero();
    return r;
}

__device__ __forceinline__ bool xyzz_is_inf(const xyzz_t& p) { return fe_is_zero(p.ZZ); }

__device__ __forceinline__ affine_t affine_neg(const affine_t& p) {
    affine_t r;
    r.x = p.x;
    r.y = fe_neg<FqP>(p.y);
    return r;
}

__device__ __forceinline__ xyzz_t xyzz_neg(const xyzz_t& p) {
    xyzz_t r = p;
    r.Y = fe_neg<FqP>(p.Y);
    return r;
}

// The formulas below issue their multiplications in independent pairs (fe_mul2), so the
// two carry-chain sequences of a pair overlap.

// 2 * (x, y) for an affine point that is not infinity (y != 0 on this curve).
__device__ __forceinline__ xyzz_t xyzz_dbl_affine(const fe& x, const fe& y) {
    using F = FqP;
    const fe U = fe_dbl<F>(y);
    const fe2 vx = fe_mul2<F>(U, U, x, x);  // V = U^2, x^2
    const fe2 ws = fe_mul2<F>(U, vx.x, x, vx.x);  // W = U V, S = x V
    const fe M = fe_add<F>(fe_dbl<F>(vx.y), vx.y);
    const fe MM = fe_sqr<F>(M);
    xyzz_t r;
    r.X = fe_sub<F>(MM, fe_dbl<F>(ws.y));
    const fe2 t = fe_mul2<F>(M, fe_sub<F>(ws.y, r.X), ws.x, y);
    r.Y = fe_sub<F>(t.x, t.y);
    r.ZZ = vx.x;
    r.ZZZ = ws.x;
    return r;
}

__device__ __forceinline__ xyzz_t xyzz_dbl(const xyzz_t& p) {
    using F = FqP;
    if (xyzz_is_inf(p)) return p;
    const fe U = fe_dbl<F>(p.Y);
    const fe2 vx = fe_mul2<F>(U, U, p.X, p.X);    // V = U^2, X^2
    const fe2 ws = fe_mul2<F>(U, vx.x, p.X, vx.x);  // W = U V, S = X V
    const fe M = fe_add<F>(fe_dbl<F>(vx.y), vx.y);
    const fe2 mz = fe_mul2<F>(M, M, vx.x, p.ZZ);  // M^2, ZZ3 = V ZZ
    xyzz_t r;
    r.X = fe_sub<F>(mz.x, fe_dbl<F>(ws.y));
    const fe2 t = fe_mul2<F>(M, fe_sub<F>(ws.y, r.X), ws.x, p.Y);
    r.Y = fe_sub<F>(t.x, t.y);
    r.ZZ = mz.y;
    r.ZZZ = fe_mul<F>(ws.x, p.ZZZ);
    return r;
}

// acc + (x, y), (x, y) affine and not infinity.
__device__ __forceinline__ xyzz_t xyzz_madd(const xyzz_t& acc, const fe& x, const fe& y) {
    using F = FqP;
    if (xyzz_is_inf(acc)) {
        xyzz_t r;
        r.X = x;
        r.Y = y;
        r.ZZ = fe_one<F>();
        r.ZZZ = fe_one<F>();
        return r;
    }
    const fe2 us = fe_mul2<F>(x, acc.ZZ, y, acc.ZZZ);  // U2, S2
    const fe P = fe_sub<F>(us.x, acc.X);
    const fe R = fe_sub<F>(us.y, acc.Y);
    if (fe_is_zero(P)) {
        if (fe_is_zero(R)) return xyzz_dbl_affine(x, y);
        return xyzz_inf();
    }
    const fe2 pr = fe_mul2<F>(P, P, R, R);          // PP, R^2
    const fe2 pq = fe_mul2<F>(P, pr.x, acc.X, pr.x);  // PPP, Q
    xyzz_t r;
    r.X = fe_sub<F>(fe_sub<F>(pr.y, pq.x), fe_dbl<F>(pq.y));
    const fe2 zz = fe_mul2<F>(acc.ZZ, pr.x, acc.ZZZ, pq.x);
    const fe2 t = fe_mul2<F>(R, fe_sub<F>(pq.y, r.X), acc.Y, pq.x);
    r.Y = fe_sub<F>(t.x, t.y);
    r.ZZ = zz.x;
    r.ZZZ = zz.y;
    return r;
}

__device__ __forceinline__ xyzz_t xyzz_add(const xyzz_t& p, const xyzz_t& q) {
    using F = FqP;
    if (xyzz_is_inf(p)) return q;
    if (xyzz_is_inf(q)) return p;
    const fe2 u = fe_mul2<F>(p.X, q.ZZ, q.X, p.ZZ);    // U1, U2
    const fe2 s = fe_mul2<F>(p.Y, q.ZZZ, q.Y, p.ZZZ);  // S1, S2
    const fe P = fe_sub<F>(u.y, u.x);
    const fe R = fe_sub<F>(s.y, s.x);
    if (fe_is_zero(P)) {
        if (fe_is_zero(R)) return xyzz_dbl(p);
        return xyzz_inf();
    }
    const fe2 pr = fe_mul2<F>(P, P, R, R);           // PP, R^2
    const fe2 pq = fe_mul2<F>(P, pr.x, u.x, pr.x);   // PPP, Q
    const fe2 zz = fe_mul2<F>(p.ZZ, q.ZZ, p.ZZZ, q.ZZZ);
    xyzz_t r;
    r.X = fe_sub<F>(fe_sub<F>(pr.y, pq.x), fe_dbl<F>(pq.y));
    const fe2 z3 = fe_mul2<F>(zz.x, pr.x, zz.y, pq.x);
    const fe2 t = fe_mul2<F>(R, fe_sub<F>(pq.y, r.X), s.x, pq.x);
    r.Y = fe_sub<F>(t.x, t.y);
    r.ZZ = z3.x;
    r.ZZZ = z3.y;
    return r;
}

__device__ __forceinline__ affine_t affine_load(const affine_t* p) {
    affine_t r;
    r.x = fe_ldg(&p->x);
    r.y = fe_ldg(&p->y);
    return r;
}

__device__ __forceinline__ xyzz_t xyzz_load(const xyzz_t* p) {
    xyzz_t r;
    r.X = fe_load(&p->X);
    r.Y = fe_load(&p->Y);
    r.ZZ = fe_load(&p->ZZ);
    r.ZZZ = fe_load(&p->ZZZ);
    return r;
}

__device__ __forceinline__ void xyzz_store(xyzz_t* p, const xyzz_t& a) {
    fe_store(&p->X, a.X);
    fe_store(&p->Y, a.Y);
    fe_store(&p->ZZ, a.ZZ);
    fe_store(&p->ZZZ, a.ZZZ);
}

}  // namespace zk
