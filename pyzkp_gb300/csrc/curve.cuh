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

// 2 * (x, y) for an affine point that is not infinity (y != 0 on this curve).
__device__ __forceinline__ xyzz_t xyzz_dbl_affine(const fe& x, const fe& y) {
    using F = FqP;
    fe U = fe_dbl<F>(y);
    fe V = fe_sqr<F>(U);
    fe W = fe_mul<F>(U, V);
    fe S = fe_mul<F>(x, V);
    fe x2 = fe_sqr<F>(x);
    fe M = fe_add<F>(fe_dbl<F>(x2), x2);
    xyzz_t r;
    r.X = fe_sub<F>(fe_sqr<F>(M), fe_dbl<F>(S));
    r.Y = fe_sub<F>(fe_mul<F>(M, fe_sub<F>(S, r.X)), fe_mul<F>(W, y));
    r.ZZ = V;
    r.ZZZ = W;
    return r;
}

__device__ __forceinline__ xyzz_t xyzz_dbl(const xyzz_t& p) {
    using F = FqP;
    if (xyzz_is_inf(p)) return p;
    fe U = fe_dbl<F>(p.Y);
    fe V = fe_sqr<F>(U);
    fe W = fe_mul<F>(U, V);
    fe S = fe_mul<F>(p.X, V);
    fe x2 = fe_sqr<F>(p.X);
    fe M = fe_add<F>(fe_dbl<F>(x2), x2);
    xyzz_t r;
    r.X = fe_sub<F>(fe_sqr<F>(M), fe_dbl<F>(S));
    r.Y = fe_sub<F>(fe_mul<F>(M, fe_sub<F>(S, r.X)), fe_mul<F>(W, p.Y));
    r.ZZ = fe_mul<F>(V, p.ZZ);
    r.ZZZ = fe_mul<F>(W, p.ZZZ);
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
    fe U2 = fe_mul<F>(x, acc.ZZ);
    fe S2 = fe_mul<F>(y, acc.ZZZ);
    fe P = fe_sub<F>(U2, acc.X);
    fe R = fe_sub<F>(S2, acc.Y);
    if (fe_is_zero(P)) {
        if (fe_is_zero(R)) return xyzz_dbl_affine(x, y);
        return xyzz_inf();
    }
    fe PP = fe_sqr<F>(P);
    fe PPP = fe_mul<F>(P, PP);
    fe Q = fe_mul<F>(acc.X, PP);
    xyzz_t r;
    r.X = fe_sub<F>(fe_sub<F>(fe_sqr<F>(R), PPP), fe_dbl<F>(Q));
    r.Y = fe_sub<F>(fe_mul<F>(R, fe_sub<F>(Q, r.X)), fe_mul<F>(acc.Y, PPP));
    r.ZZ = fe_mul<F>(acc.ZZ, PP);
    r.ZZZ = fe_mul<F>(acc.ZZZ, PPP);
    return r;
}

__device__ __forceinline__ xyzz_t xyzz_add(const xyzz_t& p, const xyzz_t& q) {
    using F = FqP;
    if (xyzz_is_inf(p)) return q;
    if (xyzz_is_inf(q)) return p;
    fe U1 = fe_mul<F>(p.X, q.ZZ);
    fe U2 = fe_mul<F>(q.X, p.ZZ);
    fe S1 = fe_mul<F>(p.Y, q.ZZZ);
    fe S2 = fe_mul<F>(q.Y, p.ZZZ);
    fe P = fe_sub<F>(U2, U1);
    fe R = fe_sub<F>(S2, S1);
    if (fe_is_zero(P)) {
        if (fe_is_zero(R)) return xyzz_dbl(p);
        return xyzz_inf();
    }
    fe PP = fe_sqr<F>(P);
    fe PPP = fe_mul<F>(P, PP);
    fe Q = fe_mul<F>(U1, PP);
    xyzz_t r;
    r.X = fe_sub<F>(fe_sub<F>(fe_sqr<F>(R), PPP), fe_dbl<F>(Q));
    r.Y = fe_sub<F>(fe_mul<F>(R, fe_sub<F>(Q, r.X)), fe_mul<F>(S1, PPP));
    r.ZZ = fe_mul<F>(fe_mul<F>(p.ZZ, q.ZZ), PP);
    r.ZZZ = fe_mul<F>(fe_mul<F>(p.ZZZ, q.ZZZ), PPP);
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
