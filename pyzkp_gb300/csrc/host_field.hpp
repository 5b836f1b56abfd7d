// host_field.hpp -- host-side BN254 field and G1 arithmetic used by the library's
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
};

struct F4 {
    uint64_t v[4];
};

inline bool geq(const uint64_t a[4], const uint64_t b[4]) {
    for (int i = 3; i >= 0; i--)
        if (a[i] != b[i]) return a[i] > b[i];
    return true;
}

inline uint64_t sub4(uint64_t r[4], const uint64_t a[4], const uint64_t b[4]) {
    uint64_t br = 0;
    for (int i = 0; i < 4; i++) {
        u128 d = (u128)a[i] - b[i] - br;
        r[i] = (uint64_t)d;
        br = (uint64_t)(d >> 64) & 1;
    }
    return br;
}

inline uint64_t add4(uint64_t r[4], const uint64_t a[4], const uint64_t b[4]) {
    u128 c = 0;
    for (int i = 0; i < 4; i++) {
        c += (u128)a[i] + b[i];
        r[i] = (uint64_t)c;
        c >>= 64;
    }
    return (uint64_t)c;
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

inline F4 mul(const Field& F, const F4& a, const F4& b) {
    uint64_t t[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < 4; i++) {
        uint64_t c = 0;
        for (int j = 0; j < 4; j++) {
            u128 x = (u128)a.v[j] * b.v[i] + t[j] + c;
            t[j] = (uint64_t)x;
            c = (uint64_t)(x >> 64);
        }
        u128 s = (u128)t[4] + c;
        t[4] = (uint64_t)s;
        t[5] = (uint64_t)(s >> 64);
        uint64_t m = t[0] * F.inv;
        u128 x = (u128)m * F.p[0] + t[0];
        c = (uint64_t)(x >> 64);
        for (int j = 1; j < 4; j++) {
            x = (u128)m * F.p[j] + t[j] + c;
            t[j - 1] = (uint64_t)x;
            c = (uint64_t)(x >> 64);
        }
        s = (u128)t[4] + c;
        t[3] = (uint64_t)s;
        t[4] = t[5] + (uint64_t)(s >> 64);
    }
    F4 r;
    std::memcpy(r.v, t, 32);
    if (t[4] || geq(r.v, F.p)) sub4(r.v, r.v, F.p);
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

inline F4 inv(const Field& F, const F4& a) {
    uint64_t e[4];
    const uint64_t two[4] = {2, 0, 0, 0};
    sub4(e, F.p, two);
    return pow(F, a, e);
}

// ---- G1 over Fq (Montgomery) ----------------------------------------------
struct Xyzz {
    F4 X, Y, ZZ, ZZZ;  // infinity: ZZ == 0
};

inline Xyzz xyzz_inf() {
    Xyzz r;
    std::memset(&r, 0, sizeof(r));
    return r;
}

inline Xyzz xyzz_dbl(const Xyzz& p) {
    const Field& F = fq();
    if (is_zero(p.ZZ)) return p;
    F4 U = add(F, p.Y, p.Y);
    F4 V = mul(F, U, U);
    F4 W = mul(F, U, V);
    F4 S = mul(F, p.X, V);
    F4 x2 = mul(F, p.X, p.X);
    F4 M = add(F, add(F, x2, x2), x2);
    Xyzz r;
    r.X = sub(F, mul(F, M, M), add(F, S, S));
    r.Y = sub(F, mul(F, M, sub(F, S, r.X)), mul(F, W, p.Y));
    r.ZZ = mul(F, V, p.ZZ);
    r.ZZZ = mul(F, W, p.ZZZ);
    return r;
}

inline Xyzz xyzz_add(const Xyzz& p, const Xyzz& q) {
    const Field& F = fq();
    if (is_zero(p.ZZ)) return q;
    if (is_zero(q.ZZ)) return p;
    F4 U1 = mul(F, p.X, q.ZZ);
    F4 U2 = mul(F, q.X, p.ZZ);
    F4 S1 = mul(F, p.Y, q.ZZZ);
    F4 S2 = mul(F, q.Y, p.ZZZ);
    F4 P = sub(F, U2, U1);
    F4 R = sub(F, S2, S1);
    if (is_zero(P)) {
        if (is_zero(R)) return xyzz_dbl(p);
        return xyzz_inf();
    }
    F4 PP = mul(F, P, P);
    F4 PPP = mul(F, P, PP);
    F4 Q = mul(F, U1, PP);
    Xyzz r;
    r.X = sub(F, sub(F, mul(F, R, R), PPP), add(F, Q, Q));
    r.Y = sub(F, mul(F, R, sub(F, Q, r.X)), mul(F, S1, PPP));
    r.ZZ = mul(F, mul(F, p.ZZ, q.ZZ), PP);
    r.ZZZ = mul(F, mul(F, p.ZZZ, q.ZZZ), PPP);
    return r;
}

// affine canonical (x, y); infinity -> (0, 0) and returns true
inline bool xyzz_to_affine_canonical(const Xyzz& p, F4* x, F4* y) {
    const Field& F = fq();
    if (is_zero(p.ZZ)) {
        std::memset(x, 0, sizeof(F4));
        std::memset(y, 0, sizeof(F4));
        return true;
    }
    F4 izz = inv(F, p.ZZ);
    F4 izzz = inv(F, p.ZZZ);
    *x = from_mont(F, mul(F, p.X, izz));
    *y = from_mont(F, mul(F, p.Y, izzz));
    return false;
}

}  // namespace zkh
