// plonk.cu -- the PLONK quotient step on the device: BATCH_INV and the fused
// PLONK_T_QUOTIENT_EVALS op.
//
// BATCH_INV (runtime/kernels/cpu/kernels.py:_batch_inv -> crypto/field/batch.py:8-38):
// out[i] = in[i]^-1, and 0 where in[i] == 0. Each thread inverts a chunk of kInvChunk
// elements with Montgomery's trick (prefix products, one Fermat inversion, a backward
// pass), so an element costs about three multiplications plus 1/kInvChunk of an inversion.
//
// PLONK_T_QUOTIENT_EVALS (runtime/kernels/cpu/kernels.py:_plonk_t_quotient_evals, used by
// protocols/plonk/prove.py:395-416): at x_i = shift * omega_m^i, i < m, from the
// extended-coset evaluations of a, b, c, z, pi, ql, qr, qm, qo, qc, s1, s2, s3, z(omega x)
// and L1, with u = omega_m^n:
//   gate  = ql a + qr b + qm a b + qo c + qc + pi
//   perm  = (a + beta x + gamma)(b + beta k1 x + gamma)(c + beta k2 x + gamma) z
//         - (a + beta s1 + gamma)(b + beta s2 + gamma)(c + beta s3 + gamma) z(omega x)
//   num_i = gate + alpha perm + alpha^2 (z - 1) L1
//   zh_i  = shift_n u^i - 1
// One thread per kQChunk points, 32 apart (a warp covers 32 * kQChunk consecutive points, so
// its loads are contiguous), the powers of omega_m and u carried from the thread's first
// point (computed by square-and-multiply) in steps of omega_m^32 and u^32.
#include <cstring>
#include <vector>

#include "zk_internal.cuh"

namespace zk {

static constexpr uint32_t kInvChunk = 32;
static constexpr uint32_t kQChunk = 16;

template <class F>
__device__ fe fe_pow_fermat_inv(const fe& a) {
    // a^(p - 2), left-to-right over the constant exponent
    fe r = fe_one<F>();
    for (int limb = 7; limb >= 0; limb--) {
        const uint32_t e = limb == 0 ? F::P(0) - 2u : F::P(limb);
        for (int b = 31; b >= 0; b--) {
            r = fe_sqr<F>(r);
            if ((e >> b) & 1) r = fe_mul<F>(r, a);
        }
    }
    return r;
}

// out must not alias in: the backward pass reads in[] again (out holds the prefixes).
__global__ void fr_batch_inv_kernel(fe* __restrict__ out, const fe* __restrict__ in, size_t n) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t i0 = t * kInvChunk;
    if (i0 >= n) return;
    const size_t i1 = i0 + kInvChunk < n ? i0 + kInvChunk : n;
    fe acc = fe_one<FrP>();
    for (size_t i = i0; i < i1; i++) {
        fe_store(out + i, acc);  // product of the non-zero inputs before i
        const fe x = fe_ldg(in + i);
        if (!fe_is_zero(x)) acc = fe_mul<FrP>(acc, x);
    }
    fe inv = fe_pow_fermat_inv<FrP>(acc);  // acc != 0: a product of non-zero field elements
    for (size_t i = i1; i-- > i0;) {
        const fe x = fe_ldg(in + i);
        if (fe_is_zero(x)) {
            fe_store(out + i, fe_zero());
        } else {
            fe_store(out + i, fe_mul<FrP>(fe_load(out + i), inv));
            inv = fe_mul<FrP>(inv, x);
        }
    }
}

// The quotient kernel holds ~23 products per element: Fr with the non-inlined product
using FrQ = FrCallP;

struct QuotientIn {
    const fe* v[15];  // a b c z pi ql qr qm qo qc s1 s2 s3 zshift l1 (Montgomery)
};

struct QuotientK {  // Montgomery constants
    fe omega_m, u, shift, shift_n, alpha, alpha2, beta, gamma, beta_k1, beta_k2, one;
    fe omega_step, u_step;  // omega_m^32, u^32: a lane's step
};

// Starting powers of a lane, from tables (Montgomery): with i0 = 512 g + l (warp g, lane l),
// v^i0 = v^l * v^(512 (g mod 64)) * v^(32768 (g / 64)) for v = omega_m and v = u:
//   pw[l], pw[32 + l]              omega_m^l, u^l                        (l < 32)
//   pw[64 + j], pw[128 + j]        omega_m^(512 j), u^(512 j)           (j < 64)
//   pw[192 + h], pw[192 + H + h]   omega_m^(32768 h), u^(32768 h)       (h < H)
// 4 products per thread instead of ~2 log2(i0) by square-and-multiply for each of the two.
static constexpr uint32_t kQWarpPoints = 32 * kQChunk;

__global__ void plonk_quotient_kernel(QuotientIn in, QuotientK K, size_t m, const fe* __restrict__ pw, uint32_t H,
                                      fe* __restrict__ num, fe* __restrict__ zh) {
    // a warp covers 32 * kQChunk consecutive points, lane l the points base + l + 32 k (each
    // load of the warp reads 32 consecutive elements)
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t lane = t & 31;
    const size_t i0 = (t - lane) * kQChunk + lane;
    if (i0 >= m) return;
    const size_t g = i0 / kQWarpPoints;
    const uint32_t glo = (uint32_t)(g & 63), ghi = (uint32_t)(g >> 6);
    fe x = fe_mul<FrQ>(fe_mul<FrQ>(fe_ldg(pw + lane), fe_ldg(pw + 64 + glo)), fe_ldg(pw + 192 + ghi));
    x = fe_mul<FrQ>(K.shift, x);
    fe un = fe_mul<FrQ>(fe_mul<FrQ>(fe_ldg(pw + 32 + lane), fe_ldg(pw + 128 + glo)), fe_ldg(pw + 192 + H + ghi));
    for (size_t i = i0, k = 0; k < kQChunk && i < m; k++, i += 32) {
        const fe a = fe_ldg(in.v[0] + i), b = fe_ldg(in.v[1] + i), c = fe_ldg(in.v[2] + i);
        const fe z = fe_ldg(in.v[3] + i);
        fe gate = fe_add<FrQ>(fe_mul<FrQ>(fe_ldg(in.v[5] + i), a), fe_mul<FrQ>(fe_ldg(in.v[6] + i), b));
        gate = fe_add<FrQ>(gate, fe_mul<FrQ>(fe_mul<FrQ>(fe_ldg(in.v[7] + i), a), b));
        gate = fe_add<FrQ>(gate, fe_mul<FrQ>(fe_ldg(in.v[8] + i), c));
        gate = fe_add<FrQ>(gate, fe_add<FrQ>(fe_ldg(in.v[9] + i), fe_ldg(in.v[4] + i)));
        const fe t1 = fe_add<FrQ>(fe_add<FrQ>(a, fe_mul<FrQ>(K.beta, x)), K.gamma);
        const fe t2 = fe_add<FrQ>(fe_add<FrQ>(b, fe_mul<FrQ>(K.beta_k1, x)), K.gamma);
        const fe t3 = fe_add<FrQ>(fe_add<FrQ>(c, fe_mul<FrQ>(K.beta_k2, x)), K.gamma);
        const fe left = fe_mul<FrQ>(fe_mul<FrQ>(fe_mul<FrQ>(t1, t2), t3), z);
        const fe u1 = fe_add<FrQ>(fe_add<FrQ>(a, fe_mul<FrQ>(K.beta, fe_ldg(in.v[10] + i))), K.gamma);
        const fe u2 = fe_add<FrQ>(fe_add<FrQ>(b, fe_mul<FrQ>(K.beta, fe_ldg(in.v[11] + i))), K.gamma);
        const fe u3 = fe_add<FrQ>(fe_add<FrQ>(c, fe_mul<FrQ>(K.beta, fe_ldg(in.v[12] + i))), K.gamma);
        const fe right = fe_mul<FrQ>(fe_mul<FrQ>(fe_mul<FrQ>(u1, u2), u3), fe_ldg(in.v[13] + i));
        const fe perm = fe_sub<FrQ>(left, right);
        const fe boundary = fe_mul<FrQ>(fe_sub<FrQ>(z, K.one), fe_ldg(in.v[14] + i));
        const fe v = fe_add<FrQ>(gate, fe_add<FrQ>(fe_mul<FrQ>(K.alpha, perm), fe_mul<FrQ>(K.alpha2, boundary)));
        fe_store(num + i, v);
        fe_store(zh + i, fe_sub<FrQ>(fe_mul<FrQ>(K.shift_n, un), K.one));
        un = fe_mul<FrQ>(un, K.u_step);
        x = fe_mul<FrQ>(x, K.omega_step);
    }
}

static fe mont_fr(const uint8_t canonical[32]) {
    zkh::F4 v;
    std::memcpy(v.v, canonical, 32);
    const zkh::F4 m = zkh::to_mont(zkh::fr(), v);
    fe r;
    std::memcpy(r.v, m.v, 32);
    return r;
}

static fe mont_of(const zkh::F4& m) {
    fe r;
    std::memcpy(r.v, m.v, 32);
    return r;
}

}  // namespace zk

using zk::fe;

extern "C" {

int zk_fr_batch_inv(zk_ctx* ctx, void* out, const void* in, size_t n) {
    if (ctx == nullptr) {
        zk::set_error("null zk_ctx");
        return ZK_EINVAL;
    }
    if (n == 0) return ZK_OK;
    if (!out || !in) {
        zk::set_error("null buffer");
        return ZK_EINVAL;
    }
    ZK_TRY_CUDA(cudaSetDevice(ctx->impl.device));
    zk::Ctx* c = &ctx->impl;
    const fe* src = static_cast<const fe*>(in);
    void* copy = nullptr;
    if (out == in) {  // the kernel keeps its prefixes in out and re-reads in: copy the input
        int rc = zk::scratch_alloc(c, n * 32, &copy);
        if (rc != ZK_OK) return rc;
        ZK_TRY_CUDA(cudaMemcpyAsync(copy, in, n * 32, cudaMemcpyDeviceToDevice, c->stream));
        src = static_cast<const fe*>(copy);
    }
    const size_t chunks = (n + zk::kInvChunk - 1) / zk::kInvChunk;
    ZK_LAUNCH(c, "fr_batch_inv", zk::fr_batch_inv_kernel, (unsigned)((chunks + 127) / 128), 128, 0,
              static_cast<fe*>(out), src, n);
    ZK_TRY_CUDA(cudaGetLastError());
    if (copy) zk::scratch_free(c, copy);
    return ZK_OK;
}

int zk_plonk_quotient_evals(zk_ctx* ctx, const void* const* inputs, size_t m, uint64_t n, const uint8_t omega_m[32],
                            const uint8_t shift[32], const uint8_t shift_n[32], const uint8_t alpha[32],
                            const uint8_t beta[32], const uint8_t gamma[32], const uint8_t k1[32],
                            const uint8_t k2[32], void* num_out, void* zh_out) {
    if (ctx == nullptr) {
        zk::set_error("null zk_ctx");
        return ZK_EINVAL;
    }
    if (m == 0) return ZK_OK;
    if (!inputs || !num_out || !zh_out || !omega_m || !shift || !shift_n || !alpha || !beta || !gamma || !k1 || !k2) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    ZK_TRY_CUDA(cudaSetDevice(ctx->impl.device));
    zk::QuotientIn in;
    for (int i = 0; i < 15; i++) {
        if (inputs[i] == nullptr) {
            zk::set_error("null input vector");
            return ZK_EINVAL;
        }
        in.v[i] = static_cast<const fe*>(inputs[i]);
    }
    const zkh::Field& F = zkh::fr();
    zk::QuotientK K;
    K.omega_m = zk::mont_fr(omega_m);
    zkh::F4 om;
    std::memcpy(om.v, omega_m, 32);
    K.u = zk::mont_of(zkh::pow_u64(F, zkh::to_mont(F, om), n));
    K.shift = zk::mont_fr(shift);
    K.shift_n = zk::mont_fr(shift_n);
    K.alpha = zk::mont_fr(alpha);
    zkh::F4 a;
    std::memcpy(a.v, alpha, 32);
    const zkh::F4 am = zkh::to_mont(F, a);
    K.alpha2 = zk::mont_of(zkh::mul(F, am, am));
    K.beta = zk::mont_fr(beta);
    K.gamma = zk::mont_fr(gamma);
    zkh::F4 b, kk1, kk2;
    std::memcpy(b.v, beta, 32);
    std::memcpy(kk1.v, k1, 32);
    std::memcpy(kk2.v, k2, 32);
    const zkh::F4 bm = zkh::to_mont(F, b);
    K.beta_k1 = zk::mont_of(zkh::mul(F, bm, zkh::to_mont(F, kk1)));
    K.beta_k2 = zk::mont_of(zkh::mul(F, bm, zkh::to_mont(F, kk2)));
    K.one = zk::mont_of(zkh::one(F));
    K.omega_step = zk::mont_of(zkh::pow_u64(F, zkh::to_mont(F, om), 32));
    K.u_step = zk::mont_of(zkh::pow_u64(F, zkh::pow_u64(F, zkh::to_mont(F, om), n), 32));
    zk::Ctx* c = &ctx->impl;
    // the starting-power tables of the kernel (see plonk_quotient_kernel)
    const uint64_t warps = (m + zk::kQWarpPoints - 1) / zk::kQWarpPoints;
    const uint32_t H = (uint32_t)((warps + 63) / 64);
    std::vector<zkh::F4> pw(192 + 2 * (size_t)H);
    const zkh::F4 om_m = zkh::to_mont(F, om);
    const zkh::F4 u_m = zkh::pow_u64(F, om_m, n);
    struct Run {
        size_t at;
        zkh::F4 base;
        size_t count;
    };
    const Run runs[6] = {{0, om_m, 32},
                         {32, u_m, 32},
                         {64, zkh::pow_u64(F, om_m, zk::kQWarpPoints), 64},
                         {128, zkh::pow_u64(F, u_m, zk::kQWarpPoints), 64},
                         {192, zkh::pow_u64(F, om_m, 64ull * zk::kQWarpPoints), H},
                         {192 + (size_t)H, zkh::pow_u64(F, u_m, 64ull * zk::kQWarpPoints), H}};
    for (const Run& r : runs) {
        zkh::F4 cur = zkh::one(F);
        for (size_t i = 0; i < r.count; i++) {
            pw[r.at + i] = cur;
            cur = zkh::mul(F, cur, r.base);
        }
    }
    void* d_pw = nullptr;
    int rc = zk::scratch_alloc(c, pw.size() * 32, &d_pw);
    if (rc != ZK_OK) return rc;
    ZK_TRY_CUDA(cudaMemcpyAsync(d_pw, pw.data(), pw.size() * 32, cudaMemcpyHostToDevice, c->stream));
    const size_t chunks = (m + zk::kQChunk - 1) / zk::kQChunk;
    ZK_LAUNCH(c, "plonk_quotient", zk::plonk_quotient_kernel, (unsigned)((chunks + 127) / 128), 128, 0, in, K, m,
              static_cast<const fe*>(d_pw), H, static_cast<fe*>(num_out), static_cast<fe*>(zh_out));
    ZK_TRY_CUDA(cudaGetLastError());
    zk::scratch_free(c, d_pw);
    return ZK_OK;
}

}  // extern "C"
