// qap.cu -- Fr vector kernels of the Groth16 prover and setup, DIV_XN_MINUS_1, and host
// G1/G2 scalar multiplication for proof assembly.
//
// Reference: protocols/groth16/prove.py:80-126 (eval_r1cs_vectors, the QAP quotient, the
// proof A, B, C), protocols/groth16/r1cs.py:84-92 (R1CS rows times the witness),
// protocols/groth16/qap.py:53-101 (H = (A B - C) / (X^n - 1), ValueError on a non-zero
// remainder), crypto/poly/fast.py:8-37 (poly_div_by_xn_minus_1).
//
// The quotient is computed on the coset 5 * <omega> where X^n - 1 is the non-zero
// constant 5^n - 1: H = coset_iNTT((A B - C)(5 omega^i) / (5^n - 1)). It equals the
// reference's unique quotient (degree <= n - 2) whenever the remainder is zero, which
// zk_fr_r1cs_check establishes first: A(omega^i) B(omega^i) == C(omega^i) for every i is
// exactly divisibility by X^n - 1.
#include <cstring>
#include <vector>

#include "zk_internal.cuh"

namespace zk {

static unsigned grid_of(size_t n, int threads, int num_sms) {
    size_t blocks = (n + threads - 1) / threads;
    size_t cap = (size_t)num_sms * 16;
    if (blocks > cap) blocks = cap;
    return (unsigned)(blocks ? blocks : 1);
}

static fe host_mont_fr(const uint8_t canonical[32]) {
    zkh::F4 v;
    std::memcpy(v.v, canonical, 32);
    const zkh::F4 m = zkh::to_mont(zkh::fr(), v);
    fe r;
    std::memcpy(r.v, m.v, 32);
    return r;
}

// out[i] = sum_{j in row i} coeffs[j] * x[cols[j]] (Montgomery), one thread per row.
__global__ void fr_spmv_kernel(uint32_t nrows, const uint32_t* __restrict__ row_ptr,
                               const uint32_t* __restrict__ cols, const fe* __restrict__ coeffs,
                               const fe* __restrict__ x, fe* __restrict__ out) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nrows; i += (size_t)gridDim.x * blockDim.x) {
        fe acc = fe_zero();
        for (uint32_t j = row_ptr[i]; j < row_ptr[i + 1]; j++)
            acc = fe_add<FrP>(acc, fe_mul<FrP>(fe_ldg(coeffs + j), fe_ldg(x + cols[j])));
        fe_store(out + i, acc);
    }
}

__global__ void fr_r1cs_check_kernel(const fe* __restrict__ a, const fe* __restrict__ b, const fe* __restrict__ c,
                                     size_t n, unsigned long long* __restrict__ bad) {
    unsigned long long local = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const fe ab = fe_mul<FrP>(fe_ldg(a + i), fe_ldg(b + i));
        const fe cc = fe_ldg(c + i);
        bool eq = true;
#pragma unroll
        for (int k = 0; k < 8; k++) eq &= ab.v[k] == cc.v[k];
        local += eq ? 0 : 1;
    }
    if (local) atomicAdd(bad, local);
}

__global__ void fr_qap_quotient_kernel(fe* __restrict__ out, const fe* __restrict__ a, const fe* __restrict__ b,
                                       const fe* __restrict__ c, size_t n, fe zinv) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const fe ab = fe_mul<FrP>(fe_ldg(a + i), fe_ldg(b + i));
        fe_store(out + i, fe_mul<FrP>(fe_sub<FrP>(ab, fe_ldg(c + i)), zinv));
    }
}

__global__ void fr_gather_kernel(fe* __restrict__ out, const fe* __restrict__ in, const uint32_t* __restrict__ idx,
                                 size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        fe_store(out + i, fe_ldg(in + idx[i]));
}

__global__ void fr_scale_kernel(fe* __restrict__ out, const fe* __restrict__ in, size_t n, fe s) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        fe_store(out + i, fe_mul<FrP>(fe_ldg(in + i), s));
}

// out[i] = base^i (Montgomery): chunk t of kPowChunk consecutive powers starts from
// base^(t * kPowChunk), by square-and-multiply over the (at most 64-bit) exponent.
static constexpr uint32_t kPowChunk = 64;

__global__ void fr_powers_kernel(fe* __restrict__ out, size_t n, fe base) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t i0 = t * kPowChunk;
    if (i0 >= n) return;
    fe acc = fe_one<FrP>();
    fe sq = base;
    for (uint64_t e = i0; e; e >>= 1) {
        if (e & 1) acc = fe_mul<FrP>(acc, sq);
        sq = fe_mul<FrP>(sq, sq);
    }
    const size_t i1 = i0 + kPowChunk < n ? i0 + kPowChunk : n;
    for (size_t i = i0; i < i1; i++) {
        fe_store(out + i, acc);
        acc = fe_mul<FrP>(acc, base);
    }
}

// q[j] = sum_{t >= 1, j + t n < len} a[j + t n] for j < qlen = len - n (the quotient of
// a / (X^n - 1)), r[i] = a[i] + q[i] for i < n (q[i] = 0 past qlen) (crypto/poly/fast.py:20-31).
__global__ void fr_div_xn_kernel(const fe* __restrict__ a, size_t len, size_t n, fe* __restrict__ q,
                                 size_t qlen, fe* __restrict__ r) {
    const size_t span = n > qlen ? n : qlen;
    for (size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x; j < span; j += (size_t)gridDim.x * blockDim.x) {
        fe acc = fe_zero();
        for (size_t k = j + n; k < len; k += n) acc = fe_add<FrP>(acc, fe_ldg(a + k));
        if (j < qlen) fe_store(q + j, acc);
        if (j < n) {
            const fe aj = j < len ? fe_ldg(a + j) : fe_zero();
            fe_store(r + j, fe_add<FrP>(aj, acc));
        }
    }
}

static int count_bad(Ctx* c, const fe* a, const fe* b, const fe* cc, size_t n, uint64_t* bad) {
    unsigned long long* d = nullptr;
    int rc = scratch_alloc(c, sizeof(unsigned long long), reinterpret_cast<void**>(&d));
    if (rc != ZK_OK) return rc;
    ZK_TRY_CUDA(cudaMemsetAsync(d, 0, sizeof(unsigned long long), c->stream));
    ZK_LAUNCH(c, "fr_r1cs_check", fr_r1cs_check_kernel, grid_of(n, 256, c->num_sms), 256, 0, a, b, cc, n, d);
    ZK_TRY_CUDA(cudaGetLastError());
    unsigned long long h = 0;
    ZK_TRY_CUDA(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    ZK_TRY_CUDA(cudaStreamSynchronize(c->stream));
    scratch_free(c, d);
    *bad = h;
    return ZK_OK;
}

int trimmed_len(Ctx* c, const void* a, size_t n, size_t* out);

// ---- host scalar multiplication and addition (proof assembly) ------------------------------
template <class H>
void host_point_mul(const uint8_t* p, const uint8_t k[32], uint8_t* out) {
    H x, y;
    std::memcpy(&x, p, sizeof(H));
    std::memcpy(&y, p + sizeof(H), sizeof(H));
    zkh::XyzzT<H> acc = zkh::xyzz_inf<H>();
    if (!(zkh::cis_zero(x) && zkh::cis_zero(y))) {
        zkh::XyzzT<H> base;
        base.X = zkh::cto_mont(x);
        base.Y = zkh::cto_mont(y);
        base.ZZ = zkh::cone<H>();
        base.ZZZ = zkh::cone<H>();
        zkh::F4 kk;
        std::memcpy(kk.v, k, 32);
        const zkh::Field& R = zkh::fr();
        while (zkh::geq(kk.v, R.p)) zkh::sub4(kk.v, kk.v, R.p);
        for (int i = 255; i >= 0; i--) {
            acc = zkh::xyzz_dbl(acc);
            if ((kk.v[i >> 6] >> (i & 63)) & 1) acc = zkh::xyzz_add(acc, base);
        }
    }
    H ox, oy;
    zkh::xyzz_to_affine_canonical(acc, &ox, &oy);
    std::memcpy(out, &ox, sizeof(H));
    std::memcpy(out + sizeof(H), &oy, sizeof(H));
}

template <class H>
void host_point_add(const uint8_t* p, const uint8_t* q, uint8_t* out) {
    zkh::XyzzT<H> acc[2];
    const uint8_t* src[2] = {p, q};
    for (int t = 0; t < 2; t++) {
        H x, y;
        std::memcpy(&x, src[t], sizeof(H));
        std::memcpy(&y, src[t] + sizeof(H), sizeof(H));
        acc[t] = zkh::xyzz_inf<H>();
        if (!(zkh::cis_zero(x) && zkh::cis_zero(y))) {
            acc[t].X = zkh::cto_mont(x);
            acc[t].Y = zkh::cto_mont(y);
            acc[t].ZZ = zkh::cone<H>();
            acc[t].ZZZ = zkh::cone<H>();
        }
    }
    const zkh::XyzzT<H> s = zkh::xyzz_add(acc[0], acc[1]);
    H ox, oy;
    zkh::xyzz_to_affine_canonical(s, &ox, &oy);
    std::memcpy(out, &ox, sizeof(H));
    std::memcpy(out + sizeof(H), &oy, sizeof(H));
}

}  // namespace zk

using zk::fe;

#define QAP_CTX(ctx)                                        \
    do {                                                    \
        if ((ctx) == nullptr) {                             \
            zk::set_error("null zk_ctx");                   \
            return ZK_EINVAL;                               \
        }                                                   \
        cudaError_t _e = cudaSetDevice((ctx)->impl.device); \
        if (_e != cudaSuccess) {                            \
            zk::set_error(cudaGetErrorString(_e));          \
            return ZK_ECUDA;                                \
        }                                                   \
    } while (0)

extern "C" {

int zk_fr_spmv(zk_ctx* ctx, uint32_t nrows, const uint32_t* row_ptr_dev, const uint32_t* cols_dev,
               const void* coeffs_dev, const void* x_dev, void* out_dev) {
    QAP_CTX(ctx);
    if (nrows == 0) return ZK_OK;
    if (!row_ptr_dev || !cols_dev || !coeffs_dev || !x_dev || !out_dev) {
        zk::set_error("null buffer");
        return ZK_EINVAL;
    }
    zk::Ctx* c = &ctx->impl;
    ZK_LAUNCH(c, "fr_spmv", zk::fr_spmv_kernel, zk::grid_of(nrows, 256, c->num_sms), 256, 0, nrows, row_ptr_dev,
              cols_dev, static_cast<const fe*>(coeffs_dev), static_cast<const fe*>(x_dev), static_cast<fe*>(out_dev));
    ZK_TRY_CUDA(cudaGetLastError());
    return ZK_OK;
}

int zk_fr_r1cs_check(zk_ctx* ctx, const void* a, const void* b, const void* c, size_t n, uint64_t* bad) {
    QAP_CTX(ctx);
    if (bad == nullptr || (n && (!a || !b || !c))) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    *bad = 0;
    if (n == 0) return ZK_OK;
    return zk::count_bad(&ctx->impl, static_cast<const fe*>(a), static_cast<const fe*>(b),
                         static_cast<const fe*>(c), n, bad);
}

int zk_fr_r1cs_check_async(zk_ctx* ctx, const void* a, const void* b, const void* c, size_t n, void* bad_dev) {
    QAP_CTX(ctx);
    if (bad_dev == nullptr || (n && (!a || !b || !c))) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    if (n == 0) return ZK_OK;
    zk::Ctx* cc = &ctx->impl;
    ZK_LAUNCH(cc, "fr_r1cs_check", zk::fr_r1cs_check_kernel, zk::grid_of(n, 256, cc->num_sms), 256, 0,
              static_cast<const fe*>(a), static_cast<const fe*>(b), static_cast<const fe*>(c), n,
              static_cast<unsigned long long*>(bad_dev));
    ZK_TRY_CUDA(cudaGetLastError());
    return ZK_OK;
}

int zk_fr_qap_quotient(zk_ctx* ctx, void* out, const void* a, const void* b, const void* c, size_t n,
                       const uint8_t zinv[32]) {
    QAP_CTX(ctx);
    if (n == 0) return ZK_OK;
    if (!out || !a || !b || !c || !zinv) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    zk::Ctx* cx = &ctx->impl;
    ZK_LAUNCH(cx, "fr_qap_quotient", zk::fr_qap_quotient_kernel, zk::grid_of(n, 256, cx->num_sms), 256, 0,
              static_cast<fe*>(out), static_cast<const fe*>(a), static_cast<const fe*>(b),
              static_cast<const fe*>(c), n, zk::host_mont_fr(zinv));
    ZK_TRY_CUDA(cudaGetLastError());
    return ZK_OK;
}

int zk_fr_gather(zk_ctx* ctx, void* out, const void* in, const uint32_t* idx_dev, size_t n) {
    QAP_CTX(ctx);
    if (n == 0) return ZK_OK;
    if (!out || !in || !idx_dev) {
        zk::set_error("null buffer");
        return ZK_EINVAL;
    }
    zk::Ctx* c = &ctx->impl;
    ZK_LAUNCH(c, "fr_gather", zk::fr_gather_kernel, zk::grid_of(n, 256, c->num_sms), 256, 0, static_cast<fe*>(out),
              static_cast<const fe*>(in), idx_dev, n);
    ZK_TRY_CUDA(cudaGetLastError());
    return ZK_OK;
}

int zk_fr_scale(zk_ctx* ctx, void* out, const void* in, const uint8_t s[32], size_t n) {
    QAP_CTX(ctx);
    if (n == 0) return ZK_OK;
    if (!out || !in || !s) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    zk::Ctx* c = &ctx->impl;
    ZK_LAUNCH(c, "fr_scale", zk::fr_scale_kernel, zk::grid_of(n, 256, c->num_sms), 256, 0, static_cast<fe*>(out),
              static_cast<const fe*>(in), n, zk::host_mont_fr(s));
    ZK_TRY_CUDA(cudaGetLastError());
    return ZK_OK;
}

int zk_fr_powers(zk_ctx* ctx, void* out, const uint8_t base[32], size_t n) {
    QAP_CTX(ctx);
    if (n == 0) return ZK_OK;
    if (!out || !base) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    zk::Ctx* c = &ctx->impl;
    const size_t chunks = (n + zk::kPowChunk - 1) / zk::kPowChunk;
    ZK_LAUNCH(c, "fr_powers", zk::fr_powers_kernel, (unsigned)((chunks + 127) / 128), 128, 0, static_cast<fe*>(out),
              n, zk::host_mont_fr(base));
    ZK_TRY_CUDA(cudaGetLastError());
    return ZK_OK;
}

int zk_fr_div_xn_minus_1(zk_ctx* ctx, const void* a, size_t len, size_t n, void* q_out, void* r_out, size_t* qlen,
                         size_t* rlen) {
    QAP_CTX(ctx);
    if (n == 0) {
        zk::set_error("n must be positive");
        return ZK_EINVAL;
    }
    if (!qlen || !rlen || (len && !a) || !r_out) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    zk::Ctx* c = &ctx->impl;
    size_t tl = 0;
    int rc = zk::trimmed_len(c, a, len, &tl);
    if (rc != ZK_OK) return rc;
    const size_t ql = tl > n ? tl - n : 0;  // quotient length before trimming
    if (ql && !q_out) {
        zk::set_error("null quotient buffer");
        return ZK_EINVAL;
    }
    ZK_LAUNCH(c, "fr_div_xn", zk::fr_div_xn_kernel, zk::grid_of(n > ql ? n : ql, 256, c->num_sms), 256, 0,
              static_cast<const fe*>(a), tl, n, static_cast<fe*>(q_out), ql, static_cast<fe*>(r_out));
    ZK_TRY_CUDA(cudaGetLastError());
    if ((rc = zk::trimmed_len(c, q_out, ql, qlen)) != ZK_OK) return rc;
    return zk::trimmed_len(c, r_out, n, rlen);
}

int zk_host_g1_mul(const uint8_t p[64], const uint8_t k[32], uint8_t out[64]) {
    if (!p || !k || !out) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    zk::host_point_mul<zkh::F4>(p, k, out);
    return ZK_OK;
}

int zk_host_g1_add(const uint8_t p[64], const uint8_t q[64], uint8_t out[64]) {
    if (!p || !q || !out) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    zk::host_point_add<zkh::F4>(p, q, out);
    return ZK_OK;
}

int zk_host_g2_mul(const uint8_t p[128], const uint8_t k[32], uint8_t out[128]) {
    if (!p || !k || !out) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    zk::host_point_mul<zkh::F2>(p, k, out);
    return ZK_OK;
}

int zk_host_g2_add(const uint8_t p[128], const uint8_t q[128], uint8_t out[128]) {
    if (!p || !q || !out) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    zk::host_point_add<zkh::F2>(p, q, out);
    return ZK_OK;
}

}  // extern "C"
