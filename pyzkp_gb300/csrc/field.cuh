// field.cuh -- BN254 Fr / Fq arithmetic for sm_103a, 8 x 32-bit limbs, Montgomery R = 2^256.
//
// The Montgomery form uses R = 2^256, the same as the reference's 4 x u64 packing
// (runtime/kernels/cpu/kernels.py:46-50,135-141; runtime/metal/runtime.py:30-40 and
// runtime/metal/ecc_source.py:14-25 hold the same moduli), so the bytes of a device
// element are the bytes of the reference's "fr_mont_u64x4" element.
//
// Multiplication is CIOS (coarsely integrated operand scanning): per limb b_i of
// the multiplier, one carry chain adds the low halves a_j*b_i into t_j and one adds
// the high halves into t_{j+1}; then m = t_0 * (-p^-1) and two chains add m*p and
// shift one limb. Every carry chain is one inline-PTX block (mad.lo.cc / madc.hi.cc
// map to IMAD with carry in/out), so carries stay in the condition-code register.
// Both moduli are below 2^254, so the running value stays below 2^288 (9 limbs)
// and below 2p after each row; one conditional subtraction yields the canonical
// representative in [0, p).
//
// Fr values are always fully reduced (equal values have equal bits: NTT outputs are
// stored and compared). Fq values inside the curve formulas are kept "lazy", in [0, 2p)
// (F::LAZY): since 4p < 2^256, a product of inputs below 2p is already below 2p without
// the final subtraction, sums subtract 2p when >= 2p, differences add 2p on a borrow, and
// zero tests accept 0 and p. fe_from_mont returns the canonical value; host code that
// reads device Fq values reduces them once more.
#pragma once
#include <cstdint>

namespace zk {

// Modulus, Montgomery one (2^256 mod p) and R^2 mod p as constexpr limb accessors, so
// unrolled code folds them into immediates.
struct FrP {
    __host__ __device__ static constexpr uint32_t P(int i) { return i == 0 ? 0xf0000001u : i == 1 ? 0x43e1f593u : i == 2 ? 0x79b97091u : i == 3 ? 0x2833e848u : i == 4 ? 0x8181585du : i == 5 ? 0xb85045b6u : i == 6 ? 0xe131a029u : 0x30644e72u; }
    static constexpr uint32_t INV = 0xefffffffu  /* -r^-1 mod 2^32 */;
    static constexpr int MUL_STYLE = 4;
    static constexpr bool LAZY = false;
    __host__ __device__ static constexpr uint32_t ONE(int i) { return i == 0 ? 0x4ffffffbu : i == 1 ? 0xac96341cu : i == 2 ? 0x9f60cd29u : i == 3 ? 0x36fc7695u : i == 4 ? 0x7879462eu : i == 5 ? 0x666ea36fu : i == 6 ? 0x9a07df2fu : 0x0e0a77c1u; }
    __host__ __device__ static constexpr uint32_t R2(int i) { return i == 0 ? 0xae216da7u : i == 1 ? 0x1bb8e645u : i == 2 ? 0xe35c59e3u : i == 3 ? 0x53fe3ab1u : i == 4 ? 0x53bb8085u : i == 5 ? 0x8c49833du : i == 6 ? 0x7f4e44a5u : 0x0216d0b1u; }
};

struct FqP {
    __host__ __device__ static constexpr uint32_t P(int i) { return i == 0 ? 0xd87cfd47u : i == 1 ? 0x3c208c16u : i == 2 ? 0x6871ca8du : i == 3 ? 0x97816a91u : i == 4 ? 0x8181585du : i == 5 ? 0xb85045b6u : i == 6 ? 0xe131a029u : 0x30644e72u; }
    static constexpr uint32_t INV = 0xe4866389u  /* -q^-1 mod 2^32 */;
    static constexpr int MUL_STYLE = 3;
#ifdef ZK_FQ_STRICT
    static constexpr bool LAZY = false;
#else
    static constexpr bool LAZY = true;
#endif
    __host__ __device__ static constexpr uint32_t ONE(int i) { return i == 0 ? 0xc58f0d9du : i == 1 ? 0xd35d438du : i == 2 ? 0xf5c70b3du : i == 3 ? 0x0a78eb28u : i == 4 ? 0x7879462cu : i == 5 ? 0x666ea36fu : i == 6 ? 0x9a07df2fu : 0x0e0a77c1u; }
    // 4 q^2 as 16 limbs (the offset that keeps a difference of two products below 4q^2 each
    // non-negative)
    __host__ __device__ static constexpr uint32_t FOUR_P_SQ(int i) {
        constexpr uint32_t v[16] = {0x9d75a6c4u, 0xed516288u, 0x27ab0404u, 0x98081cb4u, 0xb65b2b72u, 0x29406271u,
                                    0xe8490b21u, 0x11a27a55u, 0xd31ace34u, 0x9bb7e970u, 0x58dd5818u, 0xc02e1544u,
                                    0x0d234872u, 0x6669bdf0u, 0xd8f2fe71u, 0x249712e1u};
        return v[i];
    }
    __host__ __device__ static constexpr uint32_t R2(int i) { return i == 0 ? 0x538afa89u : i == 1 ? 0xf32cfc5bu : i == 2 ? 0xd44501fbu : i == 3 ? 0xb5e71911u : i == 4 ? 0x0a417ff6u : i == 5 ? 0x47ab1effu : i == 6 ? 0xcab8351fu : 0x06d89f71u; }
};

// Fr with lazy values in [0, 2r): for the NTT pass kernel only, whose last pass reduces
// every output once more (all other Fr code sees canonical values).
struct FrLazyP : FrP {
#ifdef ZK_NTT_STRICT
    static constexpr bool LAZY = false;
#else
    static constexpr bool LAZY = true;
#endif
};

// Fr with one non-inlined copy of the product, for kernels whose loop bodies hold many
// products (inlined, they overflow the instruction cache).
struct FrCallP : FrP {
    static constexpr int MUL_STYLE = 3;
};

// One field element: 8 little-endian 32-bit limbs (32 bytes, 32-byte aligned in memory).
struct __align__(16) fe {
    uint32_t v[8];
};

template <class F>
__device__ __forceinline__ fe fe_one() {
    fe r;
#pragma unroll
    for (int i = 0; i < 8; i++) r.v[i] = F::ONE(i);
    return r;
}

__device__ __forceinline__ fe fe_zero() {
    fe r;
#pragma unroll
    for (int i = 0; i < 8; i++) r.v[i] = 0;
    return r;
}

__device__ __forceinline__ bool fe_is_zero(const fe& a) {
    uint32_t x = a.v[0] | a.v[1] | a.v[2] | a.v[3] | a.v[4] | a.v[5] | a.v[6] | a.v[7];
    return x == 0;
}

__device__ __forceinline__ bool fe_eq(const fe& a, const fe& b) {
    uint32_t x = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) x |= a.v[i] ^ b.v[i];
    return x == 0;
}

// limb i of 2p
template <class F>
__host__ __device__ constexpr uint32_t p2_limb(int i) {
    return (F::P(i) << 1) | (i ? (F::P(i - 1) >> 31) : 0u);
}

// the modulus of the field's representation: 2p when lazy (values in [0, 2p)), else p
template <class F>
__host__ __device__ constexpr uint32_t mod_limb(int i) {
    return F::LAZY ? p2_limb<F>(i) : F::P(i);
}

// a == 0 mod p for a value of the field's representation ([0, p), or [0, 2p) when lazy).
// kEarly: limb 0 first (0 or p's limb 0 for either zero form): almost every value fails
// there, so a test costs a compare and a branch instead of 16 logic ops. Measured on GB300:
// G1 accumulation -0.4% / -0.6% at 2^20 / 2^22 with it, G2 +0.5% (its pairs of tests), so
// the G1 coordinates take it and the Fq2 ones do not.
template <class F, bool kEarly = false>
__device__ __forceinline__ bool fe_is_zero_mod(const fe& a) {
    if constexpr (kEarly) {
        if (a.v[0] != 0u && (!F::LAZY || a.v[0] != F::P(0))) return false;
    }
    if constexpr (F::LAZY) {
        uint32_t z = 0, e = 0;
#pragma unroll
        for (int i = 0; i < 8; i++) {
            z |= a.v[i];
            e |= a.v[i] ^ F::P(i);
        }
        return z == 0 || e == 0;
    } else {
        return fe_is_zero(a);
    }
}

// r = t - 2p if t >= 2p else t, for t < 4p (< 2^256).
template <class F>
__device__ __forceinline__ fe fe_reduce_2p(const fe& t) {
    fe s;
    uint32_t borrow;
    asm("sub.cc.u32  %0, %9, %17;\n\t"
        "subc.cc.u32 %1, %10, %18;\n\t"
        "subc.cc.u32 %2, %11, %19;\n\t"
        "subc.cc.u32 %3, %12, %20;\n\t"
        "subc.cc.u32 %4, %13, %21;\n\t"
        "subc.cc.u32 %5, %14, %22;\n\t"
        "subc.cc.u32 %6, %15, %23;\n\t"
        "subc.cc.u32 %7, %16, %24;\n\t"
        "subc.u32    %8, 0, 0;"
        : "=r"(s.v[0]), "=r"(s.v[1]), "=r"(s.v[2]), "=r"(s.v[3]), "=r"(s.v[4]), "=r"(s.v[5]), "=r"(s.v[6]),
          "=r"(s.v[7]), "=r"(borrow)
        : "r"(t.v[0]), "r"(t.v[1]), "r"(t.v[2]), "r"(t.v[3]), "r"(t.v[4]), "r"(t.v[5]), "r"(t.v[6]), "r"(t.v[7]),
          "n"(p2_limb<F>(0)), "n"(p2_limb<F>(1)), "n"(p2_limb<F>(2)), "n"(p2_limb<F>(3)), "n"(p2_limb<F>(4)),
          "n"(p2_limb<F>(5)), "n"(p2_limb<F>(6)), "n"(p2_limb<F>(7)));
    fe r;
#pragma unroll
    for (int i = 0; i < 8; i++) r.v[i] = borrow ? t.v[i] : s.v[i];
    return r;
}

// limb i of 4p (4p < 2^256 for both moduli)
template <class F>
__host__ __device__ constexpr uint32_t p4_limb(int i) {
    return (F::P(i) << 2) | (i ? (F::P(i - 1) >> 30) : 0u);
}

// r = t - 4p if t >= 4p else t, for any t < 2^256: r < 4p (2^256 < 6p), so fe_reduce_2p
// after it brings any 256-bit value into [0, 2p).
template <class F>
__device__ __forceinline__ fe fe_reduce_4p(const fe& t) {
    fe s;
    uint32_t borrow;
    asm("sub.cc.u32  %0, %9, %17;\n\t"
        "subc.cc.u32 %1, %10, %18;\n\t"
        "subc.cc.u32 %2, %11, %19;\n\t"
        "subc.cc.u32 %3, %12, %20;\n\t"
        "subc.cc.u32 %4, %13, %21;\n\t"
        "subc.cc.u32 %5, %14, %22;\n\t"
        "subc.cc.u32 %6, %15, %23;\n\t"
        "subc.cc.u32 %7, %16, %24;\n\t"
        "subc.u32    %8, 0, 0;"
        : "=r"(s.v[0]), "=r"(s.v[1]), "=r"(s.v[2]), "=r"(s.v[3]), "=r"(s.v[4]), "=r"(s.v[5]), "=r"(s.v[6]),
          "=r"(s.v[7]), "=r"(borrow)
        : "r"(t.v[0]), "r"(t.v[1]), "r"(t.v[2]), "r"(t.v[3]), "r"(t.v[4]), "r"(t.v[5]), "r"(t.v[6]), "r"(t.v[7]),
          "n"(p4_limb<F>(0)), "n"(p4_limb<F>(1)), "n"(p4_limb<F>(2)), "n"(p4_limb<F>(3)), "n"(p4_limb<F>(4)),
          "n"(p4_limb<F>(5)), "n"(p4_limb<F>(6)), "n"(p4_limb<F>(7)));
    fe r;
#pragma unroll
    for (int i = 0; i < 8; i++) r.v[i] = borrow ? t.v[i] : s.v[i];
    return r;
}

// r = t - p if t >= p else t, for t < 2p (< 2^255).
template <class F>
__device__ __forceinline__ fe fe_reduce_once(const fe& t) {
    fe s;
    uint32_t borrow;
    asm("sub.cc.u32  %0, %9, %17;\n\t"
        "subc.cc.u32 %1, %10, %18;\n\t"
        "subc.cc.u32 %2, %11, %19;\n\t"
        "subc.cc.u32 %3, %12, %20;\n\t"
        "subc.cc.u32 %4, %13, %21;\n\t"
        "subc.cc.u32 %5, %14, %22;\n\t"
        "subc.cc.u32 %6, %15, %23;\n\t"
        "subc.cc.u32 %7, %16, %24;\n\t"
        "subc.u32    %8, 0, 0;"
        : "=r"(s.v[0]), "=r"(s.v[1]), "=r"(s.v[2]), "=r"(s.v[3]), "=r"(s.v[4]), "=r"(s.v[5]), "=r"(s.v[6]),
          "=r"(s.v[7]), "=r"(borrow)
        : "r"(t.v[0]), "r"(t.v[1]), "r"(t.v[2]), "r"(t.v[3]), "r"(t.v[4]), "r"(t.v[5]), "r"(t.v[6]), "r"(t.v[7]),
          "n"(F::P(0)), "n"(F::P(1)), "n"(F::P(2)), "n"(F::P(3)), "n"(F::P(4)), "n"(F::P(5)), "n"(F::P(6)),
          "n"(F::P(7)));
    fe r;
#pragma unroll
    for (int i = 0; i < 8; i++) r.v[i] = borrow ? t.v[i] : s.v[i];
    return r;
}

template <class F>
__device__ __forceinline__ fe fe_add(const fe& a, const fe& b) {
    fe t;
    asm("add.cc.u32  %0, %8, %16;\n\t"
        "addc.cc.u32 %1, %9, %17;\n\t"
        "addc.cc.u32 %2, %10, %18;\n\t"
        "addc.cc.u32 %3, %11, %19;\n\t"
        "addc.cc.u32 %4, %12, %20;\n\t"
        "addc.cc.u32 %5, %13, %21;\n\t"
        "addc.cc.u32 %6, %14, %22;\n\t"
        "addc.u32    %7, %15, %23;"
        : "=r"(t.v[0]), "=r"(t.v[1]), "=r"(t.v[2]), "=r"(t.v[3]), "=r"(t.v[4]), "=r"(t.v[5]), "=r"(t.v[6]),
          "=r"(t.v[7])
        : "r"(a.v[0]), "r"(a.v[1]), "r"(a.v[2]), "r"(a.v[3]), "r"(a.v[4]), "r"(a.v[5]), "r"(a.v[6]), "r"(a.v[7]),
          "r"(b.v[0]), "r"(b.v[1]), "r"(b.v[2]), "r"(b.v[3]), "r"(b.v[4]), "r"(b.v[5]), "r"(b.v[6]), "r"(b.v[7]));
    if constexpr (F::LAZY) return fe_reduce_2p<F>(t);
    else return fe_reduce_once<F>(t);
}

template <class F>
__device__ __forceinline__ fe fe_sub(const fe& a, const fe& b) {
    fe t;
    uint32_t m;
    asm("sub.cc.u32  %0, %9, %17;\n\t"
        "subc.cc.u32 %1, %10, %18;\n\t"
        "subc.cc.u32 %2, %11, %19;\n\t"
        "subc.cc.u32 %3, %12, %20;\n\t"
        "subc.cc.u32 %4, %13, %21;\n\t"
        "subc.cc.u32 %5, %14, %22;\n\t"
        "subc.cc.u32 %6, %15, %23;\n\t"
        "subc.cc.u32 %7, %16, %24;\n\t"
        "subc.u32    %8, 0, 0;"
        : "=r"(t.v[0]), "=r"(t.v[1]), "=r"(t.v[2]), "=r"(t.v[3]), "=r"(t.v[4]), "=r"(t.v[5]), "=r"(t.v[6]),
          "=r"(t.v[7]), "=r"(m)
        : "r"(a.v[0]), "r"(a.v[1]), "r"(a.v[2]), "r"(a.v[3]), "r"(a.v[4]), "r"(a.v[5]), "r"(a.v[6]), "r"(a.v[7]),
          "r"(b.v[0]), "r"(b.v[1]), "r"(b.v[2]), "r"(b.v[3]), "r"(b.v[4]), "r"(b.v[5]), "r"(b.v[6]), "r"(b.v[7]));
    fe r;
    asm("add.cc.u32  %0, %8, %16;\n\t"
        "addc.cc.u32 %1, %9, %17;\n\t"
        "addc.cc.u32 %2, %10, %18;\n\t"
        "addc.cc.u32 %3, %11, %19;\n\t"
        "addc.cc.u32 %4, %12, %20;\n\t"
        "addc.cc.u32 %5, %13, %21;\n\t"
        "addc.cc.u32 %6, %14, %22;\n\t"
        "addc.u32    %7, %15, %23;"
        : "=r"(r.v[0]), "=r"(r.v[1]), "=r"(r.v[2]), "=r"(r.v[3]), "=r"(r.v[4]), "=r"(r.v[5]), "=r"(r.v[6]),
          "=r"(r.v[7])
        : "r"(t.v[0]), "r"(t.v[1]), "r"(t.v[2]), "r"(t.v[3]), "r"(t.v[4]), "r"(t.v[5]), "r"(t.v[6]), "r"(t.v[7]),
          "r"(mod_limb<F>(0) & m), "r"(mod_limb<F>(1) & m), "r"(mod_limb<F>(2) & m), "r"(mod_limb<F>(3) & m),
          "r"(mod_limb<F>(4) & m), "r"(mod_limb<F>(5) & m), "r"(mod_limb<F>(6) & m), "r"(mod_limb<F>(7) & m));
    return r;
}

template <class F>
__device__ __forceinline__ fe fe_neg(const fe& a) {
    return fe_sub<F>(fe_zero(), a);
}

template <class F>
__device__ __forceinline__ fe fe_dbl(const fe& a) {
    return fe_add<F>(a, a);
}

// One CIOS row: t += a * bi, then t += m * p with m = t0 * (-p^-1), then shift one limb.
#define ZK_MUL_ROW(F, bi)                                                                                      \
    do {                                                                                                       \
        asm("mad.lo.cc.u32  %0, %9, %17, %0;\n\t"                                                              \
            "madc.lo.cc.u32 %1, %10, %17, %1;\n\t"                                                             \
            "madc.lo.cc.u32 %2, %11, %17, %2;\n\t"                                                             \
            "madc.lo.cc.u32 %3, %12, %17, %3;\n\t"                                                             \
            "madc.lo.cc.u32 %4, %13, %17, %4;\n\t"                                                             \
            "madc.lo.cc.u32 %5, %14, %17, %5;\n\t"                                                             \
            "madc.lo.cc.u32 %6, %15, %17, %6;\n\t"                                                             \
            "madc.lo.cc.u32 %7, %16, %17, %7;\n\t"                                                             \
            "addc.u32       %8, %8, 0;"                                                                        \
            : "+r"(t0), "+r"(t1), "+r"(t2), "+r"(t3), "+r"(t4), "+r"(t5), "+r"(t6), "+r"(t7), "+r"(t8)        \
            : "r"(a.v[0]), "r"(a.v[1]), "r"(a.v[2]), "r"(a.v[3]), "r"(a.v[4]), "r"(a.v[5]), "r"(a.v[6]),      \
              "r"(a.v[7]), "r"(bi));                                                                           \
        asm("mad.hi.cc.u32  %0, %8, %16, %0;\n\t"                                                              \
            "madc.hi.cc.u32 %1, %9, %16, %1;\n\t"                                                              \
            "madc.hi.cc.u32 %2, %10, %16, %2;\n\t"                                                             \
            "madc.hi.cc.u32 %3, %11, %16, %3;\n\t"                                                             \
            "madc.hi.cc.u32 %4, %12, %16, %4;\n\t"                                                             \
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"                                                             \
            "madc.hi.cc.u32 %6, %14, %16, %6;\n\t"                                                             \
            "madc.hi.u32    %7, %15, %16, %7;"                                                                 \
            : "+r"(t1), "+r"(t2), "+r"(t3), "+r"(t4), "+r"(t5), "+r"(t6), "+r"(t7), "+r"(t8)                   \
            : "r"(a.v[0]), "r"(a.v[1]), "r"(a.v[2]), "r"(a.v[3]), "r"(a.v[4]), "r"(a.v[5]), "r"(a.v[6]),      \
              "r"(a.v[7]), "r"(bi));                                                                           \
        const uint32_t m_ = t0 * F::INV;                                                                       \
        asm("mad.lo.cc.u32  %0, %9, %10, %0;\n\t"                                                              \
            "madc.lo.cc.u32 %1, %9, %11, %1;\n\t"                                                              \
            "madc.lo.cc.u32 %2, %9, %12, %2;\n\t"                                                              \
            "madc.lo.cc.u32 %3, %9, %13, %3;\n\t"                                                              \
            "madc.lo.cc.u32 %4, %9, %14, %4;\n\t"                                                              \
            "madc.lo.cc.u32 %5, %9, %15, %5;\n\t"                                                              \
            "madc.lo.cc.u32 %6, %9, %16, %6;\n\t"                                                              \
            "madc.lo.cc.u32 %7, %9, %17, %7;\n\t"                                                              \
            "addc.u32       %8, %8, 0;"                                                                        \
            : "+r"(t0), "+r"(t1), "+r"(t2), "+r"(t3), "+r"(t4), "+r"(t5), "+r"(t6), "+r"(t7), "+r"(t8)        \
            : "r"(m_), "n"(F::P(0)), "n"(F::P(1)), "n"(F::P(2)), "n"(F::P(3)), "n"(F::P(4)), "n"(F::P(5)),   \
              "n"(F::P(6)), "n"(F::P(7)));                                                                     \
        asm("mad.hi.cc.u32  %0, %8, %9, %0;\n\t"                                                               \
            "madc.hi.cc.u32 %1, %8, %10, %1;\n\t"                                                              \
            "madc.hi.cc.u32 %2, %8, %11, %2;\n\t"                                                              \
            "madc.hi.cc.u32 %3, %8, %12, %3;\n\t"                                                              \
            "madc.hi.cc.u32 %4, %8, %13, %4;\n\t"                                                              \
            "madc.hi.cc.u32 %5, %8, %14, %5;\n\t"                                                              \
            "madc.hi.cc.u32 %6, %8, %15, %6;\n\t"                                                              \
            "madc.hi.u32    %7, %8, %16, %7;"                                                                  \
            : "+r"(t1), "+r"(t2), "+r"(t3), "+r"(t4), "+r"(t5), "+r"(t6), "+r"(t7), "+r"(t8)                   \
            : "r"(m_), "n"(F::P(0)), "n"(F::P(1)), "n"(F::P(2)), "n"(F::P(3)), "n"(F::P(4)), "n"(F::P(5)),   \
              "n"(F::P(6)), "n"(F::P(7)));                                                                     \
        t0 = t1;                                                                                               \
        t1 = t2;                                                                                               \
        t2 = t3;                                                                                               \
        t3 = t4;                                                                                               \
        t4 = t5;                                                                                               \
        t5 = t6;                                                                                               \
        t6 = t7;                                                                                               \
        t7 = t8;                                                                                               \
        t8 = 0;                                                                                                \
    } while (0)

// Code-size strategy of the multiplication, per field (F::MUL_STYLE; ZK_MUL_STYLE overrides
// both at compile time for measurements):
//   0: the 8 rows fully unrolled and inlined at every call site (largest code);
//   1: one non-inlined copy of the unrolled body, called from every site;
//   2: inlined, but the row loop kept rolled (b's limbs rotate through one register);
//   3: like 1 on full-width products (fe_mul_wide_unrolled: mul.wide + add chains);
//   4: like 0 on full-width products.
// The curve formulas hold 10-14 multiplications per loop body, so inlining them all
// overflows the instruction cache (the MSM accumulation stalled on "no instruction");
// measured on GB300 at n = 2^20: MSM 125 / 160 / 147 / 179 / 143 Mpts/s and 2^22 NTT
// 3013 / 2966 / 2643 / 3098 / 3136 Melem/s for styles 0 / 1 / 2 / 3 / 4.
// Fq (curve) uses 3, Fr (NTT butterflies) uses 4.

template <class F>
__device__ __forceinline__ fe fe_mul_unrolled(const fe& a, const fe& b) {
    uint32_t t0 = 0, t1 = 0, t2 = 0, t3 = 0, t4 = 0, t5 = 0, t6 = 0, t7 = 0, t8 = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) ZK_MUL_ROW(F, b.v[i]);
    fe t;
    t.v[0] = t0;
    t.v[1] = t1;
    t.v[2] = t2;
    t.v[3] = t3;
    t.v[4] = t4;
    t.v[5] = t5;
    t.v[6] = t6;
    t.v[7] = t7;
    if constexpr (F::LAZY) return t;
    else return fe_reduce_once<F>(t);
}

template <class F>
__device__ __forceinline__ fe fe_mul_rolled(const fe& a, const fe& b) {
    uint32_t t0 = 0, t1 = 0, t2 = 0, t3 = 0, t4 = 0, t5 = 0, t6 = 0, t7 = 0, t8 = 0;
    uint32_t b0 = b.v[0], b1 = b.v[1], b2 = b.v[2], b3 = b.v[3], b4 = b.v[4], b5 = b.v[5], b6 = b.v[6],
             b7 = b.v[7];
#pragma unroll 1
    for (int i = 0; i < 8; i++) {
        ZK_MUL_ROW(F, b0);
        b0 = b1;
        b1 = b2;
        b2 = b3;
        b3 = b4;
        b4 = b5;
        b5 = b6;
        b6 = b7;
    }
    fe t;
    t.v[0] = t0;
    t.v[1] = t1;
    t.v[2] = t2;
    t.v[3] = t3;
    t.v[4] = t4;
    t.v[5] = t5;
    t.v[6] = t6;
    t.v[7] = t7;
    if constexpr (F::LAZY) return t;
    else return fe_reduce_once<F>(t);
}

// CIOS on full-width products: mul.wide.u32 (IMAD.WIDE) yields lo and hi of a_j * b_i
// in one instruction -- measured on GB300 at twice the rate of a mad.lo + mad.hi pair,
// whose hi half issues at half rate -- and two add-with-carry chains fold the halves
// into t (lo(P_j) into t_j, hi(P_j) into t_{j+1}). Same bounds as ZK_MUL_ROW.
#define ZK_ADD_LO_CHAIN(p0, p1, p2, p3, p4, p5, p6, p7)                                                         \
    asm("add.cc.u32  %0, %0, %9;\n\t"                                                                          \
        "addc.cc.u32 %1, %1, %10;\n\t"                                                                         \
        "addc.cc.u32 %2, %2, %11;\n\t"                                                                         \
        "addc.cc.u32 %3, %3, %12;\n\t"                                                                         \
        "addc.cc.u32 %4, %4, %13;\n\t"                                                                         \
        "addc.cc.u32 %5, %5, %14;\n\t"                                                                         \
        "addc.cc.u32 %6, %6, %15;\n\t"                                                                         \
        "addc.cc.u32 %7, %7, %16;\n\t"                                                                         \
        "addc.u32    %8, %8, 0;"                                                                               \
        : "+r"(t0), "+r"(t1), "+r"(t2), "+r"(t3), "+r"(t4), "+r"(t5), "+r"(t6), "+r"(t7), "+r"(t8)            \
        : "r"((uint32_t)(p0)), "r"((uint32_t)(p1)), "r"((uint32_t)(p2)), "r"((uint32_t)(p3)),                 \
          "r"((uint32_t)(p4)), "r"((uint32_t)(p5)), "r"((uint32_t)(p6)), "r"((uint32_t)(p7)))
#define ZK_ADD_HI_CHAIN(p0, p1, p2, p3, p4, p5, p6, p7)                                                         \
    asm("add.cc.u32  %0, %0, %8;\n\t"                                                                          \
        "addc.cc.u32 %1, %1, %9;\n\t"                                                                          \
        "addc.cc.u32 %2, %2, %10;\n\t"                                                                         \
        "addc.cc.u32 %3, %3, %11;\n\t"                                                                         \
        "addc.cc.u32 %4, %4, %12;\n\t"                                                                         \
        "addc.cc.u32 %5, %5, %13;\n\t"                                                                         \
        "addc.cc.u32 %6, %6, %14;\n\t"                                                                         \
        "addc.u32    %7, %7, %15;"                                                                             \
        : "+r"(t1), "+r"(t2), "+r"(t3), "+r"(t4), "+r"(t5), "+r"(t6), "+r"(t7), "+r"(t8)                       \
        : "r"((uint32_t)((p0) >> 32)), "r"((uint32_t)((p1) >> 32)), "r"((uint32_t)((p2) >> 32)),              \
          "r"((uint32_t)((p3) >> 32)), "r"((uint32_t)((p4) >> 32)), "r"((uint32_t)((p5) >> 32)),              \
          "r"((uint32_t)((p6) >> 32)), "r"((uint32_t)((p7) >> 32)))

// Rows (bit i = row i) whose reduction half m * p uses mad.lo.cc / madc.hi.cc chains
// (IMAD pipe) instead of mul.wide + add chains (IMAD.WIDE + ALU pipe).
#ifndef ZK_MIX_ROWS
#define ZK_MIX_ROWS 0
#endif
#define ZK_RED_MAD_ROW(F, m_)                                                                                  \
    do {                                                                                                       \
        asm("mad.lo.cc.u32  %0, %9, %10, %0;\n\t"                                                              \
            "madc.lo.cc.u32 %1, %9, %11, %1;\n\t"                                                              \
            "madc.lo.cc.u32 %2, %9, %12, %2;\n\t"                                                              \
            "madc.lo.cc.u32 %3, %9, %13, %3;\n\t"                                                              \
            "madc.lo.cc.u32 %4, %9, %14, %4;\n\t"                                                              \
            "madc.lo.cc.u32 %5, %9, %15, %5;\n\t"                                                              \
            "madc.lo.cc.u32 %6, %9, %16, %6;\n\t"                                                              \
            "madc.lo.cc.u32 %7, %9, %17, %7;\n\t"                                                              \
            "addc.u32       %8, %8, 0;"                                                                        \
            : "+r"(t0), "+r"(t1), "+r"(t2), "+r"(t3), "+r"(t4), "+r"(t5), "+r"(t6), "+r"(t7), "+r"(t8)        \
            : "r"(m_), "n"(F::P(0)), "n"(F::P(1)), "n"(F::P(2)), "n"(F::P(3)), "n"(F::P(4)), "n"(F::P(5)),   \
              "n"(F::P(6)), "n"(F::P(7)));                                                                     \
        asm("mad.hi.cc.u32  %0, %8, %9, %0;\n\t"                                                               \
            "madc.hi.cc.u32 %1, %8, %10, %1;\n\t"                                                              \
            "madc.hi.cc.u32 %2, %8, %11, %2;\n\t"                                                              \
            "madc.hi.cc.u32 %3, %8, %12, %3;\n\t"                                                              \
            "madc.hi.cc.u32 %4, %8, %13, %4;\n\t"                                                              \
            "madc.hi.cc.u32 %5, %8, %14, %5;\n\t"                                                              \
            "madc.hi.cc.u32 %6, %8, %15, %6;\n\t"                                                              \
            "madc.hi.u32    %7, %8, %16, %7;"                                                                  \
            : "+r"(t1), "+r"(t2), "+r"(t3), "+r"(t4), "+r"(t5), "+r"(t6), "+r"(t7), "+r"(t8)                   \
            : "r"(m_), "n"(F::P(0)), "n"(F::P(1)), "n"(F::P(2)), "n"(F::P(3)), "n"(F::P(4)), "n"(F::P(5)),   \
              "n"(F::P(6)), "n"(F::P(7)));                                                                     \
    } while (0)

// Row of the carry-save form: x_j = a_j * b + t_j as one 64-bit multiply-add each
// (mul.wide with a 64-bit addend: (2^32 - 1)^2 + (2^32 - 1) < 2^64, no overflow), then a
// single add-carry chain t_j = lo(x_j) + hi(x_{j-1}), t_8 += hi(x_7): one ALU addition per
// partial product instead of two (the low halves ride in the multiply).
#define ZK_ROW_ACC(a0, a1, a2, a3, a4, a5, a6, a7, bi)                                                          \
    do {                                                                                                       \
        const uint64_t x0 = (uint64_t)(a0) * (bi) + t0, x1 = (uint64_t)(a1) * (bi) + t1,                      \
                       x2 = (uint64_t)(a2) * (bi) + t2, x3 = (uint64_t)(a3) * (bi) + t3,                      \
                       x4 = (uint64_t)(a4) * (bi) + t4, x5 = (uint64_t)(a5) * (bi) + t5,                      \
                       x6 = (uint64_t)(a6) * (bi) + t6, x7 = (uint64_t)(a7) * (bi) + t7;                      \
        t0 = (uint32_t)x0;                                                                                     \
        asm("add.cc.u32  %0, %8, %15;\n\t"                                                                      \
            "addc.cc.u32 %1, %9, %16;\n\t"                                                                      \
            "addc.cc.u32 %2, %10, %17;\n\t"                                                                     \
            "addc.cc.u32 %3, %11, %18;\n\t"                                                                     \
            "addc.cc.u32 %4, %12, %19;\n\t"                                                                     \
            "addc.cc.u32 %5, %13, %20;\n\t"                                                                     \
            "addc.cc.u32 %6, %14, %21;\n\t"                                                                     \
            "addc.u32    %7, %7, %22;"                                                                         \
            : "=r"(t1), "=r"(t2), "=r"(t3), "=r"(t4), "=r"(t5), "=r"(t6), "=r"(t7), "+r"(t8)                   \
            : "r"((uint32_t)x1), "r"((uint32_t)x2), "r"((uint32_t)x3), "r"((uint32_t)x4), "r"((uint32_t)x5),   \
              "r"((uint32_t)x6), "r"((uint32_t)x7), "r"((uint32_t)(x0 >> 32)), "r"((uint32_t)(x1 >> 32)),     \
              "r"((uint32_t)(x2 >> 32)), "r"((uint32_t)(x3 >> 32)), "r"((uint32_t)(x4 >> 32)),                 \
              "r"((uint32_t)(x5 >> 32)), "r"((uint32_t)(x6 >> 32)), "r"((uint32_t)(x7 >> 32)));                \
    } while (0)

// CIOS on the carry-save rows: per row 16 multiply-adds and two 8-long carry chains.
template <class F>
__device__ __forceinline__ fe fe_mul_acc_unrolled(const fe& a, const fe& b) {
    uint32_t t0 = 0, t1 = 0, t2 = 0, t3 = 0, t4 = 0, t5 = 0, t6 = 0, t7 = 0, t8 = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        ZK_ROW_ACC(a.v[0], a.v[1], a.v[2], a.v[3], a.v[4], a.v[5], a.v[6], a.v[7], b.v[i]);
        const uint32_t m = t0 * F::INV;
        ZK_ROW_ACC(F::P(0), F::P(1), F::P(2), F::P(3), F::P(4), F::P(5), F::P(6), F::P(7), m);
        // t0 == 0 now (m was chosen so); shift one limb
        t0 = t1;
        t1 = t2;
        t2 = t3;
        t3 = t4;
        t4 = t5;
        t5 = t6;
        t6 = t7;
        t7 = t8;
        t8 = 0;
    }
    fe t;
    t.v[0] = t0;
    t.v[1] = t1;
    t.v[2] = t2;
    t.v[3] = t3;
    t.v[4] = t4;
    t.v[5] = t5;
    t.v[6] = t6;
    t.v[7] = t7;
    if constexpr (F::LAZY) return t;
    else return fe_reduce_once<F>(t);
}

template <class F>
__device__ __forceinline__ fe fe_mul_wide_unrolled(const fe& a, const fe& b) {
    uint32_t t0 = 0, t1 = 0, t2 = 0, t3 = 0, t4 = 0, t5 = 0, t6 = 0, t7 = 0, t8 = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const uint32_t bi = b.v[i];
        const uint64_t p0 = (uint64_t)a.v[0] * bi, p1 = (uint64_t)a.v[1] * bi, p2 = (uint64_t)a.v[2] * bi,
                       p3 = (uint64_t)a.v[3] * bi, p4 = (uint64_t)a.v[4] * bi, p5 = (uint64_t)a.v[5] * bi,
                       p6 = (uint64_t)a.v[6] * bi, p7 = (uint64_t)a.v[7] * bi;
        ZK_ADD_LO_CHAIN(p0, p1, p2, p3, p4, p5, p6, p7);
        ZK_ADD_HI_CHAIN(p0, p1, p2, p3, p4, p5, p6, p7);
        const uint32_t m = t0 * F::INV;
        if ((ZK_MIX_ROWS >> i) & 1) {
            // this row's m * p on the IMAD pipe (multiply-add with carry), balancing the ALU pipe
            ZK_RED_MAD_ROW(F, m);
        } else {
            const uint64_t q0 = (uint64_t)m * F::P(0), q1 = (uint64_t)m * F::P(1), q2 = (uint64_t)m * F::P(2),
                           q3 = (uint64_t)m * F::P(3), q4 = (uint64_t)m * F::P(4), q5 = (uint64_t)m * F::P(5),
                           q6 = (uint64_t)m * F::P(6), q7 = (uint64_t)m * F::P(7);
            ZK_ADD_LO_CHAIN(q0, q1, q2, q3, q4, q5, q6, q7);
            ZK_ADD_HI_CHAIN(q0, q1, q2, q3, q4, q5, q6, q7);
        }
        t0 = t1;
        t1 = t2;
        t2 = t3;
        t3 = t4;
        t4 = t5;
        t5 = t6;
        t6 = t7;
        t7 = t8;
        t8 = 0;
    }
    fe t;
    t.v[0] = t0;
    t.v[1] = t1;
    t.v[2] = t2;
    t.v[3] = t3;
    t.v[4] = t4;
    t.v[5] = t5;
    t.v[6] = t6;
    t.v[7] = t7;
    if constexpr (F::LAZY) return t;
    else return fe_reduce_once<F>(t);
}

// Two independent products a*b and c*d with their rows interleaved: the carry chains of
// one product fill the latency of the other's (a thread's carry flag serialises each chain).
#define ZK_LO_CHAIN_R(r0, r1, r2, r3, r4, r5, r6, r7, r8, p0, p1, p2, p3, p4, p5, p6, p7)                     \
    asm("add.cc.u32  %0, %0, %9;\n\t"                                                                          \
        "addc.cc.u32 %1, %1, %10;\n\t"                                                                         \
        "addc.cc.u32 %2, %2, %11;\n\t"                                                                         \
        "addc.cc.u32 %3, %3, %12;\n\t"                                                                         \
        "addc.cc.u32 %4, %4, %13;\n\t"                                                                         \
        "addc.cc.u32 %5, %5, %14;\n\t"                                                                         \
        "addc.cc.u32 %6, %6, %15;\n\t"                                                                         \
        "addc.cc.u32 %7, %7, %16;\n\t"                                                                         \
        "addc.u32    %8, %8, 0;"                                                                               \
        : "+r"(r0), "+r"(r1), "+r"(r2), "+r"(r3), "+r"(r4), "+r"(r5), "+r"(r6), "+r"(r7), "+r"(r8)            \
        : "r"((uint32_t)(p0)), "r"((uint32_t)(p1)), "r"((uint32_t)(p2)), "r"((uint32_t)(p3)),                 \
          "r"((uint32_t)(p4)), "r"((uint32_t)(p5)), "r"((uint32_t)(p6)), "r"((uint32_t)(p7)))
#define ZK_HI_CHAIN_R(r1, r2, r3, r4, r5, r6, r7, r8, p0, p1, p2, p3, p4, p5, p6, p7)                         \
    asm("add.cc.u32  %0, %0, %8;\n\t"                                                                          \
        "addc.cc.u32 %1, %1, %9;\n\t"                                                                          \
        "addc.cc.u32 %2, %2, %10;\n\t"                                                                         \
        "addc.cc.u32 %3, %3, %11;\n\t"                                                                         \
        "addc.cc.u32 %4, %4, %12;\n\t"                                                                         \
        "addc.cc.u32 %5, %5, %13;\n\t"                                                                         \
        "addc.cc.u32 %6, %6, %14;\n\t"                                                                         \
        "addc.u32    %7, %7, %15;"                                                                             \
        : "+r"(r1), "+r"(r2), "+r"(r3), "+r"(r4), "+r"(r5), "+r"(r6), "+r"(r7), "+r"(r8)                       \
        : "r"((uint32_t)((p0) >> 32)), "r"((uint32_t)((p1) >> 32)), "r"((uint32_t)((p2) >> 32)),              \
          "r"((uint32_t)((p3) >> 32)), "r"((uint32_t)((p4) >> 32)), "r"((uint32_t)((p5) >> 32)),              \
          "r"((uint32_t)((p6) >> 32)), "r"((uint32_t)((p7) >> 32)))

struct fe2 {
    fe x, y;
};

template <class F>
__device__ __forceinline__ fe2 fe_mul2_wide_unrolled(const fe& a, const fe& b, const fe& c, const fe& d) {
    uint32_t t0 = 0, t1 = 0, t2 = 0, t3 = 0, t4 = 0, t5 = 0, t6 = 0, t7 = 0, t8 = 0;
    uint32_t u0 = 0, u1 = 0, u2 = 0, u3 = 0, u4 = 0, u5 = 0, u6 = 0, u7 = 0, u8 = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const uint32_t bi = b.v[i], di = d.v[i];
        const uint64_t p0 = (uint64_t)a.v[0] * bi, p1 = (uint64_t)a.v[1] * bi, p2 = (uint64_t)a.v[2] * bi,
                       p3 = (uint64_t)a.v[3] * bi, p4 = (uint64_t)a.v[4] * bi, p5 = (uint64_t)a.v[5] * bi,
                       p6 = (uint64_t)a.v[6] * bi, p7 = (uint64_t)a.v[7] * bi;
        const uint64_t r0 = (uint64_t)c.v[0] * di, r1 = (uint64_t)c.v[1] * di, r2 = (uint64_t)c.v[2] * di,
                       r3 = (uint64_t)c.v[3] * di, r4 = (uint64_t)c.v[4] * di, r5 = (uint64_t)c.v[5] * di,
                       r6 = (uint64_t)c.v[6] * di, r7 = (uint64_t)c.v[7] * di;
        ZK_LO_CHAIN_R(t0, t1, t2, t3, t4, t5, t6, t7, t8, p0, p1, p2, p3, p4, p5, p6, p7);
        ZK_LO_CHAIN_R(u0, u1, u2, u3, u4, u5, u6, u7, u8, r0, r1, r2, r3, r4, r5, r6, r7);
        ZK_HI_CHAIN_R(t1, t2, t3, t4, t5, t6, t7, t8, p0, p1, p2, p3, p4, p5, p6, p7);
        ZK_HI_CHAIN_R(u1, u2, u3, u4, u5, u6, u7, u8, r0, r1, r2, r3, r4, r5, r6, r7);
        const uint32_t m = t0 * F::INV, mu = u0 * F::INV;
        const uint64_t q0 = (uint64_t)m * F::P(0), q1 = (uint64_t)m * F::P(1), q2 = (uint64_t)m * F::P(2),
                       q3 = (uint64_t)m * F::P(3), q4 = (uint64_t)m * F::P(4), q5 = (uint64_t)m * F::P(5),
                       q6 = (uint64_t)m * F::P(6), q7 = (uint64_t)m * F::P(7);
        const uint64_t s0 = (uint64_t)mu * F::P(0), s1 = (uint64_t)mu * F::P(1), s2 = (uint64_t)mu * F::P(2),
                       s3 = (uint64_t)mu * F::P(3), s4 = (uint64_t)mu * F::P(4), s5 = (uint64_t)mu * F::P(5),
                       s6 = (uint64_t)mu * F::P(6), s7 = (uint64_t)mu * F::P(7);
        ZK_LO_CHAIN_R(t0, t1, t2, t3, t4, t5, t6, t7, t8, q0, q1, q2, q3, q4, q5, q6, q7);
        ZK_LO_CHAIN_R(u0, u1, u2, u3, u4, u5, u6, u7, u8, s0, s1, s2, s3, s4, s5, s6, s7);
        ZK_HI_CHAIN_R(t1, t2, t3, t4, t5, t6, t7, t8, q0, q1, q2, q3, q4, q5, q6, q7);
        ZK_HI_CHAIN_R(u1, u2, u3, u4, u5, u6, u7, u8, s0, s1, s2, s3, s4, s5, s6, s7);
        t0 = t1, t1 = t2, t2 = t3, t3 = t4, t4 = t5, t5 = t6, t6 = t7, t7 = t8, t8 = 0;
        u0 = u1, u1 = u2, u2 = u3, u3 = u4, u4 = u5, u5 = u6, u6 = u7, u7 = u8, u8 = 0;
    }
    fe x, y;
    x.v[0] = t0, x.v[1] = t1, x.v[2] = t2, x.v[3] = t3, x.v[4] = t4, x.v[5] = t5, x.v[6] = t6, x.v[7] = t7;
    y.v[0] = u0, y.v[1] = u1, y.v[2] = u2, y.v[3] = u3, y.v[4] = u4, y.v[5] = u5, y.v[6] = u6, y.v[7] = u7;
    fe2 r;
    if constexpr (F::LAZY) {
        r.x = x;
        r.y = y;
    } else {
        r.x = fe_reduce_once<F>(x);
        r.y = fe_reduce_once<F>(y);
    }
    return r;
}

template <class F>
__device__ __noinline__ fe2 fe_mul2_call(const fe a, const fe b, const fe c, const fe d) {
    return fe_mul2_wide_unrolled<F>(a, b, c, d);
}

// (a*b, c*d): two calls of fe_mul, or (with ZK_USE_MUL2 and style 3) one call of the
// interleaved product.
template <class F>
__device__ __forceinline__ fe2 fe_mul2(const fe& a, const fe& b, const fe& c, const fe& d);

template <class F>
__device__ __noinline__ fe fe_mul_call(const fe a, const fe b) {
    return fe_mul_unrolled<F>(a, b);
}

template <class F>
__host__ __device__ __forceinline__ fe fe_mul_sos(const fe& a, const fe& b);

template <class F>
__device__ __noinline__ fe fe_mul_wide_call(const fe a, const fe b) {
#ifdef ZK_WIDE_ACC
    return fe_mul_acc_unrolled<F>(a, b);
#elif defined(ZK_SOS_MUL)
    if constexpr (F::LAZY) return fe_mul_sos<F>(a, b);
    else return fe_mul_wide_unrolled<F>(a, b);
#else
    return fe_mul_wide_unrolled<F>(a, b);
#endif
}

// r = a * b * 2^-256 mod p (CIOS, see the file header).
template <class F>
__device__ __forceinline__ fe fe_mul(const fe& a, const fe& b) {
#ifdef ZK_MUL_STYLE
    constexpr int style = ZK_MUL_STYLE;
#else
    constexpr int style = F::MUL_STYLE;
#endif
    if constexpr (style == 0) {
        return fe_mul_unrolled<F>(a, b);
    } else if constexpr (style == 1) {
        return fe_mul_call<F>(a, b);
    } else if constexpr (style == 3) {
        return fe_mul_wide_call<F>(a, b);
    } else if constexpr (style == 4) {
#ifdef ZK_WIDE_ACC
        return fe_mul_acc_unrolled<F>(a, b);
#else
        return fe_mul_wide_unrolled<F>(a, b);
#endif
    } else {
        return fe_mul_rolled<F>(a, b);
    }
}

template <class F>
__device__ __forceinline__ fe2 fe_mul2(const fe& a, const fe& b, const fe& c, const fe& d) {
#ifdef ZK_USE_MUL2
#ifdef ZK_MUL_STYLE
    constexpr int style = ZK_MUL_STYLE;
#else
    constexpr int style = F::MUL_STYLE;
#endif
    // measured on GB300 (MSM 2^20): 179 Mpts/s with the interleaved pair, 180 without
    if constexpr (style == 3) return fe_mul2_call<F>(a, b, c, d);
#endif
    fe2 r;
    r.x = fe_mul<F>(a, b);
    r.y = fe_mul<F>(c, d);
    return r;
}

// ---- separated forms: a 512-bit product, then one Montgomery reduction -------------------
//
// Splitting the product from the reduction lets a square skip the 28 repeated cross
// products (36 instead of 64 partial products) and lets a difference of two products
// a b - c d share one reduction. They serve the lazy Fq of the curve formulas only.
//
// Reduction: for T = T_lo + 2^256 T_hi, the m_i of the Montgomery rows depend on T_lo alone,
// so (T + M p) / 2^256 = T_hi + (T_lo + M p) / 2^256; the second term is a CIOS reduction of
// the low 8 limbs (a 9-limb window, no carry beyond it) and is at most p. With T < 4p^2
// (a product of two values below 2p) T_hi < 0.76 p, so the result stays below 2p; with
// T < 8p^2 (a sum of two such products) it is below 2.52 p and one conditional subtraction
// of 2p brings it below 2p (both moduli are below 0.19 * 2^256).
//
// The carry flag primitives are one PTX instruction each on the device (asm volatile keeps
// their order, so the flag flows from one to the next as in a single asm block); on the
// host they emulate the flag, so the same code runs in a host-side check of the arithmetic.
#ifndef __CUDA_ARCH__
inline uint32_t& host_carry_flag() {
    static thread_local uint32_t cc = 0;
    return cc;
}
#endif

__host__ __device__ __forceinline__ uint32_t u_add_cc(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
    uint32_t r;
    asm volatile("add.cc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    return r;
#else
    const uint64_t s = (uint64_t)a + b;
    host_carry_flag() = (uint32_t)(s >> 32);
    return (uint32_t)s;
#endif
}

__host__ __device__ __forceinline__ uint32_t u_addc_cc(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
    uint32_t r;
    asm volatile("addc.cc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    return r;
#else
    const uint64_t s = (uint64_t)a + b + host_carry_flag();
    host_carry_flag() = (uint32_t)(s >> 32);
    return (uint32_t)s;
#endif
}

__host__ __device__ __forceinline__ uint32_t u_addc(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
    uint32_t r;
    asm volatile("addc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    return r;
#else
    return (uint32_t)((uint64_t)a + b + host_carry_flag());
#endif
}

__host__ __device__ __forceinline__ uint32_t u_sub_cc(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
    uint32_t r;
    asm volatile("sub.cc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    return r;
#else
    host_carry_flag() = a < b ? 1u : 0u;
    return a - b;
#endif
}

__host__ __device__ __forceinline__ uint32_t u_subc_cc(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
    uint32_t r;
    asm volatile("subc.cc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    return r;
#else
    const uint64_t d = (uint64_t)a - b - host_carry_flag();
    host_carry_flag() = (uint32_t)(d >> 63);
    return (uint32_t)d;
#endif
}

__host__ __device__ __forceinline__ uint32_t u_subc(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
    uint32_t r;
    asm volatile("subc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    return r;
#else
    return (uint32_t)((uint64_t)a - b - host_carry_flag());
#endif
}

__host__ __device__ __forceinline__ uint32_t lo32(uint64_t x) { return (uint32_t)x; }
__host__ __device__ __forceinline__ uint32_t hi32(uint64_t x) { return (uint32_t)(x >> 32); }

// Row I of t += a * b_I with a below 2^255: the low halves of a_j b_I into t_{I+j} (carry
// into t_{I+8}), the high halves into t_{I+j+1}. FIRST: t_{I..I+8} are not yet written
// (the first product's rows). Two products accumulated row by row stay below
// 2 * 2^255 * 2^(32(I+1)) = 2^(32(I+9)), so nothing carries out of t_{I+8}.
template <int I, bool FIRST>
__host__ __device__ __forceinline__ void sos_row(uint32_t* t, const uint32_t* a, uint32_t bi) {
    uint64_t p[8];
#pragma unroll
    for (int j = 0; j < 8; j++) p[j] = (uint64_t)a[j] * bi;
    if constexpr (FIRST && I == 0) {
#pragma unroll
        for (int j = 0; j < 8; j++) t[j] = lo32(p[j]);
        t[1] = u_add_cc(t[1], hi32(p[0]));
#pragma unroll
        for (int j = 1; j < 7; j++) t[j + 1] = u_addc_cc(t[j + 1], hi32(p[j]));
        t[8] = u_addc(0u, hi32(p[7]));
        return;
    }
    t[I] = u_add_cc(t[I], lo32(p[0]));
#pragma unroll
    for (int j = 1; j < 8; j++) t[I + j] = u_addc_cc(t[I + j], lo32(p[j]));
    if constexpr (FIRST) t[I + 8] = u_addc(0u, 0u);
    else t[I + 8] = u_addc(t[I + 8], 0u);
    t[I + 1] = u_add_cc(t[I + 1], hi32(p[0]));
#pragma unroll
    for (int j = 1; j < 7; j++) t[I + j + 1] = u_addc_cc(t[I + j + 1], hi32(p[j]));
    t[I + 8] = u_addc(t[I + 8], hi32(p[7]));
}

// Row I of the cross products a_I a_j (j > I) into t_{I+j}: 7 - I products.
template <int I>
__host__ __device__ __forceinline__ void sqr_cross_row(uint32_t* t, const uint32_t* a) {
    constexpr int L = 7 - I;
    uint64_t p[8];
#pragma unroll
    for (int j = I + 1; j < 8; j++) p[j] = (uint64_t)a[I] * a[j];
    if constexpr (I == 0) {
#pragma unroll
        for (int j = 1; j < 8; j++) t[j] = lo32(p[j]);
        t[2] = u_add_cc(t[2], hi32(p[1]));
#pragma unroll
        for (int j = 2; j < 7; j++) t[j + 1] = u_addc_cc(t[j + 1], hi32(p[j]));
        t[8] = u_addc(0u, hi32(p[7]));
        return;
    }
    // low halves: t_{2I+1} .. t_{I+7}, carry into t_{I+8} (not yet written)
    t[2 * I + 1] = u_add_cc(t[2 * I + 1], lo32(p[I + 1]));
#pragma unroll
    for (int j = I + 2; j < 8; j++) t[I + j] = u_addc_cc(t[I + j], lo32(p[j]));
    t[I + 8] = u_addc(0u, 0u);
    // high halves: t_{2I+2} .. t_{I+8}
    if constexpr (L == 1) {
        t[I + 8] = t[I + 8] + hi32(p[7]);
    } else {
        t[2 * I + 2] = u_add_cc(t[2 * I + 2], hi32(p[I + 1]));
#pragma unroll
        for (int j = I + 2; j < 7; j++) t[I + j + 1] = u_addc_cc(t[I + j + 1], hi32(p[j]));
        t[I + 8] = u_addc(t[I + 8], hi32(p[7]));
    }
}

// t[0..15] = a * a: the cross products once, doubled, plus the squares a_i^2 at limb 2i.
__host__ __device__ __forceinline__ void sos_sqr_wide(uint32_t* t, const uint32_t* a) {
    sqr_cross_row<0>(t, a);
    sqr_cross_row<1>(t, a);
    sqr_cross_row<2>(t, a);
    sqr_cross_row<3>(t, a);
    sqr_cross_row<4>(t, a);
    sqr_cross_row<5>(t, a);
    sqr_cross_row<6>(t, a);
    // t_1 .. t_14 hold the cross sum (below a^2 / 2 < 2^511); double it into t_1 .. t_15
    t[1] = u_add_cc(t[1], t[1]);
#pragma unroll
    for (int j = 2; j < 15; j++) t[j] = u_addc_cc(t[j], t[j]);
    t[15] = u_addc(0u, 0u);
    uint64_t d[8];
#pragma unroll
    for (int i = 0; i < 8; i++) d[i] = (uint64_t)a[i] * a[i];
    t[0] = lo32(d[0]);
    t[1] = u_add_cc(t[1], hi32(d[0]));
#pragma unroll
    for (int i = 1; i < 7; i++) {
        t[2 * i] = u_addc_cc(t[2 * i], lo32(d[i]));
        t[2 * i + 1] = u_addc_cc(t[2 * i + 1], hi32(d[i]));
    }
    t[14] = u_addc_cc(t[14], lo32(d[7]));
    t[15] = u_addc(t[15], hi32(d[7]));
}

// r = T_hi + (T_lo + M p) / 2^256 for t = T (16 limbs): T * 2^-256 mod p, below T_hi + p + 1.
template <class F>
__host__ __device__ __forceinline__ fe sos_redc(const uint32_t* t) {
    uint32_t w[9];
#pragma unroll
    for (int j = 0; j < 8; j++) w[j] = t[j];
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const uint32_t m = w[0] * F::INV;
        uint64_t q[8];
#pragma unroll
        for (int j = 0; j < 8; j++) q[j] = (uint64_t)m * F::P(j);
        w[0] = u_add_cc(w[0], lo32(q[0]));
#pragma unroll
        for (int j = 1; j < 8; j++) w[j] = u_addc_cc(w[j], lo32(q[j]));
        w[8] = u_addc(0u, 0u);
        w[1] = u_add_cc(w[1], hi32(q[0]));
#pragma unroll
        for (int j = 1; j < 7; j++) w[j + 1] = u_addc_cc(w[j + 1], hi32(q[j]));
        w[8] = u_addc(w[8], hi32(q[7]));
        // w_0 == 0 now (m was chosen so); shift one limb
#pragma unroll
        for (int j = 0; j < 8; j++) w[j] = w[j + 1];
    }
    fe r;
    r.v[0] = u_add_cc(w[0], t[8]);
#pragma unroll
    for (int j = 1; j < 7; j++) r.v[j] = u_addc_cc(w[j], t[j + 8]);
    r.v[7] = u_addc(w[7], t[15]);
    return r;
}

// 2p - c for c in [0, 2p): in (0, 2p], congruent to -c
template <class F>
__host__ __device__ __forceinline__ fe sos_neg2p(const fe& c) {
    fe r;
    r.v[0] = u_sub_cc(p2_limb<F>(0), c.v[0]);
#pragma unroll
    for (int j = 1; j < 7; j++) r.v[j] = u_subc_cc(p2_limb<F>(j), c.v[j]);
    r.v[7] = u_subc(p2_limb<F>(7), c.v[7]);
    return r;
}

// r = t - 2p if t >= 2p else t, for t < 4p (the host-and-device twin of fe_reduce_2p)
template <class F>
__host__ __device__ __forceinline__ fe sos_reduce_2p(const fe& t) {
    fe s;
    s.v[0] = u_sub_cc(t.v[0], p2_limb<F>(0));
#pragma unroll
    for (int j = 1; j < 8; j++) s.v[j] = u_subc_cc(t.v[j], p2_limb<F>(j));
    const uint32_t borrow = u_subc(0u, 0u);
    fe r;
#pragma unroll
    for (int j = 0; j < 8; j++) r.v[j] = borrow ? t.v[j] : s.v[j];
    return r;
}

// a^2 * 2^-256 mod p in [0, 2p) for a in [0, 2p)
template <class F>
__host__ __device__ __forceinline__ fe fe_sqr_sos(const fe& a) {
    static_assert(F::LAZY, "the separated forms keep lazy values");
    uint32_t t[16];
    sos_sqr_wide(t, a.v);
    return sos_redc<F>(t);
}

// a b * 2^-256 mod p in [0, 2p) for a, b in [0, 2p): product rows, then the reduction
template <class F>
__host__ __device__ __forceinline__ fe fe_mul_sos(const fe& a, const fe& b) {
    static_assert(F::LAZY, "the separated forms keep lazy values");
    uint32_t t[16];
    sos_row<0, true>(t, a.v, b.v[0]);
    sos_row<1, true>(t, a.v, b.v[1]);
    sos_row<2, true>(t, a.v, b.v[2]);
    sos_row<3, true>(t, a.v, b.v[3]);
    sos_row<4, true>(t, a.v, b.v[4]);
    sos_row<5, true>(t, a.v, b.v[5]);
    sos_row<6, true>(t, a.v, b.v[6]);
    sos_row<7, true>(t, a.v, b.v[7]);
    return sos_redc<F>(t);
}

// (a b + c d) * 2^-256 mod p in [0, 2p) for inputs in [0, 2p] (one reduction)
template <class F>
__host__ __device__ __forceinline__ fe fe_mul_add_sos(const fe& a, const fe& b, const fe& c, const fe& d) {
    static_assert(F::LAZY, "the separated forms keep lazy values");
    uint32_t t[16];
    sos_row<0, true>(t, a.v, b.v[0]);
    sos_row<0, false>(t, c.v, d.v[0]);
    sos_row<1, true>(t, a.v, b.v[1]);
    sos_row<1, false>(t, c.v, d.v[1]);
    sos_row<2, true>(t, a.v, b.v[2]);
    sos_row<2, false>(t, c.v, d.v[2]);
    sos_row<3, true>(t, a.v, b.v[3]);
    sos_row<3, false>(t, c.v, d.v[3]);
    sos_row<4, true>(t, a.v, b.v[4]);
    sos_row<4, false>(t, c.v, d.v[4]);
    sos_row<5, true>(t, a.v, b.v[5]);
    sos_row<5, false>(t, c.v, d.v[5]);
    sos_row<6, true>(t, a.v, b.v[6]);
    sos_row<6, false>(t, c.v, d.v[6]);
    sos_row<7, true>(t, a.v, b.v[7]);
    sos_row<7, false>(t, c.v, d.v[7]);
    return sos_reduce_2p<F>(sos_redc<F>(t));
}

// (a b - c d) * 2^-256 mod p in [0, 2p) for inputs in [0, 2p): a b + (2p - c) d
template <class F>
__host__ __device__ __forceinline__ fe fe_mul_sub_sos(const fe& a, const fe& b, const fe& c, const fe& d) {
    return fe_mul_add_sos<F>(a, b, sos_neg2p<F>(c), d);
}

// Fq2 product with lazy reduction (Karatsuba): T0 = a0 b0, T1 = a1 b1, T2 = (a0 + a1)(b0 + b1)
// as 512-bit products, c0 = redc(T0 + (4q^2 - T1)), c1 = redc(T2 - T0 - T1) = redc(a0 b1 + a1 b0):
// 3 products and 2 reductions instead of 3 full products. Inputs in [0, 2q): the sums a0 + a1
// stay below 4q < 2^256 unreduced (one product row stays inside its 9 limbs for any 256-bit
// operand), both arguments of the reductions are below 8q^2, results in [0, 2q).
struct fe_pair {
    fe c0, c1;
};

template <class F>
__host__ __device__ __forceinline__ fe_pair fe2_mul_lazy(const fe& a0, const fe& a1, const fe& b0, const fe& b1) {
    static_assert(F::LAZY, "the separated forms keep lazy values");
    uint32_t t0[16], t1[16];
    sos_row<0, true>(t0, a0.v, b0.v[0]);
    sos_row<1, true>(t0, a0.v, b0.v[1]);
    sos_row<2, true>(t0, a0.v, b0.v[2]);
    sos_row<3, true>(t0, a0.v, b0.v[3]);
    sos_row<4, true>(t0, a0.v, b0.v[4]);
    sos_row<5, true>(t0, a0.v, b0.v[5]);
    sos_row<6, true>(t0, a0.v, b0.v[6]);
    sos_row<7, true>(t0, a0.v, b0.v[7]);
    sos_row<0, true>(t1, a1.v, b1.v[0]);
    sos_row<1, true>(t1, a1.v, b1.v[1]);
    sos_row<2, true>(t1, a1.v, b1.v[2]);
    sos_row<3, true>(t1, a1.v, b1.v[3]);
    sos_row<4, true>(t1, a1.v, b1.v[4]);
    sos_row<5, true>(t1, a1.v, b1.v[5]);
    sos_row<6, true>(t1, a1.v, b1.v[6]);
    sos_row<7, true>(t1, a1.v, b1.v[7]);
    // u = T0 + (4q^2 - T1) in (0, 8q^2); s = T0 + T1 (below 8q^2)
    uint32_t u[16], s[16];
    u[0] = u_sub_cc(F::FOUR_P_SQ(0), t1[0]);
#pragma unroll
    for (int j = 1; j < 15; j++) u[j] = u_subc_cc(F::FOUR_P_SQ(j), t1[j]);
    u[15] = u_subc(F::FOUR_P_SQ(15), t1[15]);
    u[0] = u_add_cc(u[0], t0[0]);
#pragma unroll
    for (int j = 1; j < 15; j++) u[j] = u_addc_cc(u[j], t0[j]);
    u[15] = u_addc(u[15], t0[15]);
    s[0] = u_add_cc(t0[0], t1[0]);
#pragma unroll
    for (int j = 1; j < 15; j++) s[j] = u_addc_cc(t0[j], t1[j]);
    s[15] = u_addc(t0[15], t1[15]);
    fe_pair r;
    r.c0 = sos_reduce_2p<F>(sos_redc<F>(u));
    // T2 - s with a0 + a1, b0 + b1 as plain 256-bit sums
    fe sa, sb;
    sa.v[0] = u_add_cc(a0.v[0], a1.v[0]);
#pragma unroll
    for (int j = 1; j < 7; j++) sa.v[j] = u_addc_cc(a0.v[j], a1.v[j]);
    sa.v[7] = u_addc(a0.v[7], a1.v[7]);
    sb.v[0] = u_add_cc(b0.v[0], b1.v[0]);
#pragma unroll
    for (int j = 1; j < 7; j++) sb.v[j] = u_addc_cc(b0.v[j], b1.v[j]);
    sb.v[7] = u_addc(b0.v[7], b1.v[7]);
    uint32_t t2[16];
    sos_row<0, true>(t2, sa.v, sb.v[0]);
    sos_row<1, true>(t2, sa.v, sb.v[1]);
    sos_row<2, true>(t2, sa.v, sb.v[2]);
    sos_row<3, true>(t2, sa.v, sb.v[3]);
    sos_row<4, true>(t2, sa.v, sb.v[4]);
    sos_row<5, true>(t2, sa.v, sb.v[5]);
    sos_row<6, true>(t2, sa.v, sb.v[6]);
    sos_row<7, true>(t2, sa.v, sb.v[7]);
    t2[0] = u_sub_cc(t2[0], s[0]);
#pragma unroll
    for (int j = 1; j < 15; j++) t2[j] = u_subc_cc(t2[j], s[j]);
    t2[15] = u_subc(t2[15], s[15]);
    r.c1 = sos_reduce_2p<F>(sos_redc<F>(t2));
    return r;
}

template <class F>
__device__ __noinline__ fe_pair fe2_mul_lazy_call(const fe a0, const fe a1, const fe b0, const fe b1) {
    return fe2_mul_lazy<F>(a0, a1, b0, b1);
}

template <class F>
__device__ __noinline__ fe fe_sqr_sos_call(const fe a) {
    return fe_sqr_sos<F>(a);
}

template <class F>
__device__ __noinline__ fe fe_mul_add_sos_call(const fe a, const fe b, const fe c, const fe d) {
    return fe_mul_add_sos<F>(a, b, c, d);
}

template <class F>
__device__ __noinline__ fe fe_mul_sub_sos_call(const fe a, const fe b, const fe c, const fe d) {
    return fe_mul_sub_sos<F>(a, b, c, d);
}

// The separated forms are used for the lazy fields with the called multiplication (style
// 3: the curve formulas over Fq); ZK_NO_SOS keeps every product on fe_mul for comparison.
template <class F>
__device__ __forceinline__ constexpr bool use_sos() {
#if defined(ZK_NO_SOS)
    return false;
#else
#ifdef ZK_MUL_STYLE
    constexpr int style = ZK_MUL_STYLE;
#else
    constexpr int style = F::MUL_STYLE;
#endif
    return F::LAZY && style == 3;
#endif
}

template <class F>
__device__ __forceinline__ fe fe_sqr(const fe& a) {
    if constexpr (use_sos<F>()) return fe_sqr_sos_call<F>(a);
    else return fe_mul<F>(a, a);
}

// a b - c d, and a b + c d (inputs in the field's representation)
template <class F>
__device__ __forceinline__ fe fe_mul_sub(const fe& a, const fe& b, const fe& c, const fe& d) {
    if constexpr (use_sos<F>()) return fe_mul_sub_sos_call<F>(a, b, c, d);
    else return fe_sub<F>(fe_mul<F>(a, b), fe_mul<F>(c, d));
}

template <class F>
__device__ __forceinline__ fe fe_mul_add(const fe& a, const fe& b, const fe& c, const fe& d) {
    if constexpr (use_sos<F>()) return fe_mul_add_sos_call<F>(a, b, c, d);
    else return fe_add<F>(fe_mul<F>(a, b), fe_mul<F>(c, d));
}

// canonical value (any 256-bit input, reduced mod p first) -> Montgomery form
template <class F>
__device__ __forceinline__ fe fe_to_mont(fe a) {
    // at most floor((2^256 - 1) / p) = 5 subtractions for both BN254 moduli
#pragma unroll 1
    for (int k = 0; k < 5; k++) {
        fe s;
        uint32_t br;
        asm("sub.cc.u32  %0, %9, %17;\n\t"
            "subc.cc.u32 %1, %10, %18;\n\t"
            "subc.cc.u32 %2, %11, %19;\n\t"
            "subc.cc.u32 %3, %12, %20;\n\t"
            "subc.cc.u32 %4, %13, %21;\n\t"
            "subc.cc.u32 %5, %14, %22;\n\t"
            "subc.cc.u32 %6, %15, %23;\n\t"
            "subc.cc.u32 %7, %16, %24;\n\t"
            "subc.u32    %8, 0, 0;"
            : "=r"(s.v[0]), "=r"(s.v[1]), "=r"(s.v[2]), "=r"(s.v[3]), "=r"(s.v[4]), "=r"(s.v[5]), "=r"(s.v[6]),
              "=r"(s.v[7]), "=r"(br)
            : "r"(a.v[0]), "r"(a.v[1]), "r"(a.v[2]), "r"(a.v[3]), "r"(a.v[4]), "r"(a.v[5]), "r"(a.v[6]),
              "r"(a.v[7]), "n"(F::P(0)), "n"(F::P(1)), "n"(F::P(2)), "n"(F::P(3)), "n"(F::P(4)), "n"(F::P(5)),
              "n"(F::P(6)), "n"(F::P(7)));
        if (br) break;  // a < p
        a = s;
    }
    fe r2;
#pragma unroll
    for (int i = 0; i < 8; i++) r2.v[i] = F::R2(i);
    return fe_mul<F>(a, r2);
}

// Montgomery -> canonical in [0, p) (also for lazy inputs below 2p: a * 1 * 2^-256 <= p).
template <class F>
__device__ __forceinline__ fe fe_from_mont(const fe& a) {
    fe one;
#pragma unroll
    for (int i = 0; i < 8; i++) one.v[i] = i == 0 ? 1u : 0u;
    const fe r = fe_mul<F>(a, one);
    if constexpr (F::LAZY) return fe_reduce_once<F>(r);
    else return r;
}

// 32-byte element loads / stores as two 16-byte vector accesses
__device__ __forceinline__ fe fe_load(const fe* p) {
    const uint4* q = reinterpret_cast<const uint4*>(p);
    uint4 lo = q[0], hi = q[1];
    fe r;
    r.v[0] = lo.x;
    r.v[1] = lo.y;
    r.v[2] = lo.z;
    r.v[3] = lo.w;
    r.v[4] = hi.x;
    r.v[5] = hi.y;
    r.v[6] = hi.z;
    r.v[7] = hi.w;
    return r;
}

__device__ __forceinline__ fe fe_ldg(const fe* p) {
    const uint4* q = reinterpret_cast<const uint4*>(p);
    uint4 lo = __ldg(q), hi = __ldg(q + 1);
    fe r;
    r.v[0] = lo.x;
    r.v[1] = lo.y;
    r.v[2] = lo.z;
    r.v[3] = lo.w;
    r.v[4] = hi.x;
    r.v[5] = hi.y;
    r.v[6] = hi.z;
    r.v[7] = hi.w;
    return r;
}

// A 32-byte element through L2 only (ld.global.cg): for data that other CTAs wrote earlier
// in the same launch, which the non-coherent read-only path is not guaranteed to see.
__device__ __forceinline__ fe fe_ldcg(const fe* p) {
    const uint4* q = reinterpret_cast<const uint4*>(p);
    uint4 lo = __ldcg(q), hi = __ldcg(q + 1);
    fe r;
    r.v[0] = lo.x;
    r.v[1] = lo.y;
    r.v[2] = lo.z;
    r.v[3] = lo.w;
    r.v[4] = hi.x;
    r.v[5] = hi.y;
    r.v[6] = hi.z;
    r.v[7] = hi.w;
    return r;
}

__device__ __forceinline__ void fe_store(fe* p, const fe& a) {
    uint4* q = reinterpret_cast<uint4*>(p);
    q[0] = make_uint4(a.v[0], a.v[1], a.v[2], a.v[3]);
    q[1] = make_uint4(a.v[4], a.v[5], a.v[6], a.v[7]);
}

}  // namespace zk
