// host_field.hpp -- host-side BN254 field, G1 and G2 arithmetic used by the library's
// host code: NTT twiddle/scale tables, omega checks, and the final combination of
// MSM window sums into one affine point. 4 x 64-bit limbs, Montgomery R = 2^256
// (byte-identical to the device's 8 x 32-bit form). Portable C++ (unsigned __int128).
#pragma once
#include <cstdint>
#include <cstring>

namespace zkh {

typedef unsigned __int128 u128;

struct Field {
    uint64_t p[4];
    uint64_t inv;  // -p^-1 mod 2^64
    uint64_t one[4];
    uint64_t r2[4];
    uint64_t r3[4];  // R^3 mod p (turns a plain inverse of a Montgomery form into a Montgomery form)
};

struct F4 {
    uint64_t v[4];
};

inline bool geq(const uint64_t a[4], const uint64_t b[4]) {
    if (a[3] != b[3]) return a[3] > b[3];
    if (a[2] != b[2]) return a[2] > b[2];
    if (a[1] != b[1]) return a[1] > b[1];
    return a[0] >= b[0];
}

// r = a - b, returns the borrow (unrolled: the loops were not unrolled at -O2)
inline uint64_t sub4(uint64_t r[4], const uint64_t a[4], const uint64_t b[4]) {
    u128 d = (u128)a[0] - b[0];
    r[0] = (uint64_t)d;
    d = (u128)a[1] - b[1] - (uint64_t)((d >> 64) & 1);
    r[1] = (uint64_t)d;
    d = (u128)a[2] - b[2] - (uint64_t)((d >> 64) & 1);
    r[2] = (uint64_t)d;
    d = (u128)a[3] - b[3] - (uint64_t)((d >> 64) & 1);
    r[3] = (uint64_t)d;
    return (uint64_t)((d >> 64) & 1);
}

// r = a + b, returns the carry
inline uint64_t add4(uint64_t r[4], const uint64_t a[4], const uint64_t b[4]) {
    u128 c = (u128)a[0] + b[0];
    r[0] = (uint64_t)c;
    c = (u128)a[1] + b[1] + (uint64_t)(c >> 64);
    r[1] = (uint64_t)c;
    c = (u128)a[2] + b[2] + (uint64_t)(c >> 64);
    r[2] = (uint64_t)c;
    c = (u128)a[3] + b[3] + (uint64_t)(c >> 64);
    r[3] = (uint64_t)c;
    return (uint64_t)(c >> 64);
}

inline bool is_zero(const F4& a) { return (a.v[0] | a.v[1] | a.v[2] | a.v[3]) == 0; }
inline bool eq(const F4& a, const F4& b) { return std::memcmp(a.v, b.v, 32) == 0; }

inline F4 add(const Field& F, const F4& a, const F4& b) {
    F4 r;
    uint64_t c = add4(r.v, a.v, b.v);
    if (c || geq(r.v, F.p)) sub4(r.v, r.v, F.p);
    return r;
}

inline F4 sub(const Field& F, const F4& a, const F4& b) {
    F4 r;
    if (sub4(r.v, a.v, b.v)) add4(r.v, r.v, F.p);
    return r;
}

inline F4 neg(const Field& F, const F4& a) {
    F4 z = {{0, 0, 0, 0}};
    return sub(F, z, a);
}

// Montgomery product a b 2^-256 mod p for a, b below 2p: CIOS with its rows unrolled and no
// carry words beyond the 4 limbs -- both moduli are below 2^254, so every row's running value
// (below 3p) fits 256 bits and the final value is below 2p (one conditional subtraction).
// Measured on x86-64 at -O2: 64 -> ~20 ns per product against the looped form.
inline void mac_row(uint64_t& t0, uint64_t& t1, uint64_t& t2, uint64_t& t3, const uint64_t a[4], uint64_t bi,
                    const Field& F) {
    u128 x = (u128)a[0] * bi + t0;
    uint64_t A = (uint64_t)(x >> 64);
    const uint64_t s0 = (uint64_t)x;
    const uint64_t m = s0 * F.inv;
    u128 y = (u128)m * F.p[0] + s0;
    uint64_t C = (uint64_t)(y >> 64);
    x = (u128)a[1] * bi + t1 + A;
    A = (uint64_t)(x >> 64);
    y = (u128)m * F.p[1] + (uint64_t)x + C;
    C = (uint64_t)(y >> 64);
    t0 = (uint64_t)y;
    x = (u128)a[2] * bi + t2 + A;
    A = (uint64_t)(x >> 64);
    y = (u128)m * F.p[2] + (uint64_t)x + C;
    C = (uint64_t)(y >> 64);
    t1 = (uint64_t)y;
    x = (u128)a[3] * bi + t3 + A;
    A = (uint64_t)(x >> 64);
    y = (u128)m * F.p[3] + (uint64_t)x + C;
    C = (uint64_t)(y >> 64);
    t2 = (uint64_t)y;
    t3 = C + A;
}

inline F4 mul(const Field& F, const F4& a, const F4& b) {
    uint64_t t0 = 0, t1 = 0, t2 = 0, t3 = 0;
    mac_row(t0, t1, t2, t3, a.v, b.v[0], F);
    mac_row(t0, t1, t2, t3, a.v, b.v[1], F);
    mac_row(t0, t1, t2, t3, a.v, b.v[2], F);
    mac_row(t0, t1, t2, t3, a.v, b.v[3], F);
    F4 r = {{t0, t1, t2, t3}};
    if (geq(r.v, F.p)) sub4(r.v, r.v, F.p);
    return r;
}

inline Field make_field(const uint64_t p[4]) {
    Field F;
    std::memcpy(F.p, p, 32);
    uint64_t x = 1;
    for (int i = 0; i < 7; i++) x *= 2 - p[0] * x;
    F.inv = (uint64_t)0 - x;
    F4 t = {{1, 0, 0, 0}};
    for (int i = 0; i < 256; i++) t = add(F, t, t);
    std::memcpy(F.one, t.v, 32);
    for (int i = 0; i < 256; i++) t = add(F, t, t);
    std::memcpy(F.r2, t.v, 32);
    t = mul(F, t, t);  // R^2 R^2 / R
    std::memcpy(F.r3, t.v, 32);
    return F;
}

inline const Field& fr() {
    static const uint64_t P[4] = {0x43e1f593f0000001ULL, 0x2833e84879b97091ULL, 0xb85045b68181585dULL,
                                  0x30644e72e131a029ULL};
    static const Field F = make_field(P);
    return F;
}

inline const Field& fq() {
    static const uint64_t P[4] = {0x3c208c16d87cfd47ULL, 0x97816a916871ca8dULL, 0xb85045b68181585dULL,
                                  0x30644e72e131a029ULL};
    static const Field F = make_field(P);
    return F;
}

inline F4 one(const Field& F) {
    F4 r;
    std::memcpy(r.v, F.one, 32);
    return r;
}

inline F4 to_mont(const Field& F, const F4& canon) {
    F4 a = canon;
    while (geq(a.v, F.p)) sub4(a.v, a.v, F.p);
    F4 r2;
    std::memcpy(r2.v, F.r2, 32);
    return mul(F, a, r2);
}

inline F4 from_mont(const Field& F, const F4& a) {
    F4 o = {{1, 0, 0, 0}};
    return mul(F, a, o);
}

inline F4 pow(const Field& F, const F4& a, const uint64_t e[4]) {
    F4 acc = one(F), base = a;
    for (int i = 0; i < 4; i++) {
        uint64_t w = e[i];
        for (int b = 0; b < 64; b++) {
            if (w & 1) acc = mul(F, acc, base);
            base = mul(F, base, base);
            w >>= 1;
        }
    }
    return acc;
}

inline F4 pow_u64(const Field& F, const F4& a, uint64_t e) {
    uint64_t ee[4] = {e, 0, 0, 0};
    return pow(F, a, ee);
}

inline bool is_one4(const uint64_t a[4]) { return a[0] == 1 && (a[1] | a[2] | a[3]) == 0; }

// a >> 1 with `top` shifted into bit 255
inline void shr1(uint64_t a[4], uint64_t top) {
    a[0] = (a[0] >> 1) | (a[1] << 63);
    a[1] = (a[1] >> 1) | (a[2] << 63);
    a[2] = (a[2] >> 1) | (a[3] << 63);
    a[3] = (a[3] >> 1) | (top << 63);
}

// x / 2 mod p for x < p (x + p < 2^255: no carry out of the 4 limbs)
inline void half_mod(const Field& F, uint64_t x[4]) {
    if (x[0] & 1) {
        add4(x, x, F.p);
        shr1(x, 0);
    } else {
        shr1(x, 0);
    }
}

// Inverse of a Montgomery form a = A R: the Montgomery form R / A = R^2 a^-1 of A^-1 (zero for
// zero). Binary extended Euclid on (a, p) with x1 a = u, x2 a = v (mod p) kept throughout;
// variable time (the inputs are public values: MSM results, roots of unity, sizes).
inline F4 inv(const Field& F, const F4& a) {
    uint64_t u[4], v[4], x1[4] = {1, 0, 0, 0}, x2[4] = {0, 0, 0, 0};
    std::memcpy(u, a.v, 32);
    while (geq(u, F.p)) sub4(u, u, F.p);
    if ((u[0] | u[1] | u[2] | u[3]) == 0) return F4{{0, 0, 0, 0}};
    std::memcpy(v, F.p, 32);
    while (!is_one4(u) && !is_one4(v)) {
        while (!(u[0] & 1)) {
            shr1(u, 0);
            half_mod(F, x1);
        }
        while (!(v[0] & 1)) {
            shr1(v, 0);
            half_mod(F, x2);
        }
        if (geq(u, v)) {
            sub4(u, u, v);
            if (sub4(x1, x1, x2)) add4(x1, x1, F.p);
        } else {
            sub4(v, v, u);
            if (sub4(x2, x2, x1)) add4(x2, x2, F.p);
        }
    }
    F4 r, r3;
    std::memcpy(r.v, is_one4(u) ? x1 : x2, 32);
    std::memcpy(r3.v, F.r3, 32);
    return mul(F, r, r3);  // a^-1 R^3 / R
}

// Fermat form of the same inverse, a^(p-2) (checks the binary form)
inline F4 inv_pow(const Field& F, const F4& a) {
    uint64_t e[4];
    const uint64_t two[4] = {2, 0, 0, 0};
    sub4(e, F.p, two);
    return pow(F, a, e);
}

// ---- coordinate fields of G1 (Fq) and G2 (Fq2 = Fq[u] / (u^2 + 1)), Montgomery ---------
struct F2 {
    F4 c0, c1;  // c0 + c1 u
};

inline F4 cadd(const F4& a, const F4& b) { return add(fq(), a, b); }
inline F4 csub(const F4& a, const F4& b) { return sub(fq(), a, b); }
inline F4 cmul(const F4& a, const F4& b) { return mul(fq(), a, b); }
inline bool cis_zero(const F4& a) { return is_zero(a); }
inline F4 cinv(const F4& a) { return inv(fq(), a); }
inline F4 cfrom_mont(const F4& a) { return from_mont(fq(), a); }
inline F4 cto_mont(const F4& a) { return to_mont(fq(), a); }

inline F2 cadd(const F2& a, const F2& b) { return {cadd(a.c0, b.c0), cadd(a.c1, b.c1)}; }
inline F2 csub(const F2& a, const F2& b) { return {csub(a.c0, b.c0), csub(a.c1, b.c1)}; }
inline F2 cmul(const F2& a, const F2& b) {
    const F4 t0 = cmul(a.c0, b.c0), t1 = cmul(a.c1, b.c1);
    const F4 t2 = cmul(cadd(a.c0, a.c1), cadd(b.c0, b.c1));
    return {csub(t0, t1), csub(csub(t2, t0), t1)};
}
// squares: a a for Fq; (a0 + a1 u)^2 = (a0 + a1)(a0 - a1) + 2 a0 a1 u for Fq2 (2 products
// instead of 3)
inline F4 csqr(const F4& a) { return cmul(a, a); }
inline F2 csqr(const F2& a) {
    const F4 t = cmul(a.c0, a.c1);
    return {cmul(cadd(a.c0, a.c1), csub(a.c0, a.c1)), cadd(t, t)};
}
inline bool cis_zero(const F2& a) { return is_zero(a.c0) && is_zero(a.c1); }
// 1 / (a0 + a1 u) = (a0 - a1 u) / (a0^2 + a1^2)
inline F2 cinv(const F2& a) {
    const F4 t = inv(fq(), cadd(cmul(a.c0, a.c0), cmul(a.c1, a.c1)));
    return {cmul(a.c0, t), csub(F4{{0, 0, 0, 0}}, cmul(a.c1, t))};
}
inline F2 cfrom_mont(const F2& a) { return {cfrom_mont(a.c0), cfrom_mont(a.c1)}; }
inline F2 cto_mont(const F2& a) { return {cto_mont(a.c0), cto_mont(a.c1)}; }

// Montgomery one of a coordinate field
template <class T>
inline T cone();
template <>
inline F4 cone<F4>() {
    return one(fq());
}
template <>
inline F2 cone<F2>() {
    return {one(fq()), F4{{0, 0, 0, 0}}};
}

// Device Fq values may be lazy in [0, 2p): one conditional subtraction makes them canonical.
inline F4 cnorm(const F4& a) {
    F4 r = a;
    if (geq(r.v, fq().p)) sub4(r.v, r.v, fq().p);
    return r;
}
inline F2 cnorm(const F2& a) { return {cnorm(a.c0), cnorm(a.c1)}; }

// ---- XYZZ points over either coordinate field --------------------------------------------
template <class T>
struct XyzzT {
    T X, Y, ZZ, ZZZ;  // infinity: ZZ == 0
};
using Xyzz = XyzzT<F4>;
using Xyzz2 = XyzzT<F2>;

template <class T = F4>
inline XyzzT<T> xyzz_inf() {
    XyzzT<T> r;
    std::memset(&r, 0, sizeof(r));
    return r;
}

template <class T>
inline XyzzT<T> xyzz_dbl(const XyzzT<T>& p) {
    if (cis_zero(p.ZZ)) return p;
    T U = cadd(p.Y, p.Y);
    T V = csqr(U);
    T W = cmul(U, V);
    T S = cmul(p.X, V);
    T x2 = csqr(p.X);
    T M = cadd(cadd(x2, x2), x2);
    XyzzT<T> r;
    r.X = csub(csqr(M), cadd(S, S));
    r.Y = csub(cmul(M, csub(S, r.X)), cmul(W, p.Y));
    r.ZZ = cmul(V, p.ZZ);
    r.ZZZ = cmul(W, p.ZZZ);
    return r;
}

template <class T>
inline XyzzT<T> xyzz_add(const XyzzT<T>& p, const XyzzT<T>& q) {
    if (cis_zero(p.ZZ)) return q;
    if (cis_zero(q.ZZ)) return p;
    T U1 = cmul(p.X, q.ZZ);
    T U2 = cmul(q.X, p.ZZ);
    T S1 = cmul(p.Y, q.ZZZ);
    T S2 = cmul(q.Y, p.ZZZ);
    T P = csub(U2, U1);
    T R = csub(S2, S1);
    if (cis_zero(P)) {
        if (cis_zero(R)) return xyzz_dbl(p);
        return xyzz_inf<T>();
    }
    T PP = csqr(P);
    T PPP = cmul(P, PP);
    T Q = cmul(U1, PP);
    XyzzT<T> r;
    r.X = csub(csub(csqr(R), PPP), cadd(Q, Q));
    r.Y = csub(cmul(R, csub(Q, r.X)), cmul(S1, PPP));
    r.ZZ = cmul(cmul(p.ZZ, q.ZZ), PP);
    r.ZZZ = cmul(cmul(p.ZZZ, q.ZZZ), PPP);
    return r;
}

// affine canonical (x, y); infinity -> all zero and returns true
template <class T>
inline bool xyzz_to_affine_canonical(const XyzzT<T>& p, T* x, T* y) {
    if (cis_zero(p.ZZ)) {
        std::memset(x, 0, sizeof(T));
        std::memset(y, 0, sizeof(T));
        return true;
    }
    // one inversion: 1/ZZ = ZZZ / (ZZ ZZZ), 1/ZZZ = ZZ / (ZZ ZZZ)
    const T t = cinv(cmul(p.ZZ, p.ZZZ));
    *x = cfrom_mont(cmul(p.X, cmul(t, p.ZZZ)));
    *y = cfrom_mont(cmul(p.Y, cmul(t, p.ZZ)));
    return false;
}

}  // namespace zkh
