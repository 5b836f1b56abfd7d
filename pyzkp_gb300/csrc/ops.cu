// ops.cu -- elementwise Fr/Fq kernels and fixed-base scalar multiplication.
//
// to/from Montgomery replace the per-element Python loops of _to_device /
// _from_device (runtime/kernels/cpu/kernels.py:98-172); fr_mul / fr_sub are the
// POINTWISE_MUL / POLY_SUB kernels (runtime/metal/runtime.py:204-224).
#include <cstring>
#include <vector>

#include "zk_internal.cuh"

namespace zk {

static unsigned grid_for(size_t n, int threads, int num_sms) {
    size_t blocks = (n + threads - 1) / threads;
    size_t cap = (size_t)num_sms * 16;
    if (blocks > cap) blocks = cap;
    return (unsigned)(blocks ? blocks : 1);
}

template <class F, int DIR>
__global__ void convert_kernel(fe* out, const fe* in, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        fe v = fe_ldg(in + i);
        fe_store(out + i, DIR ? fe_to_mont<F>(v) : fe_from_mont<F>(v));
    }
}

__global__ void fr_mul_kernel(fe* out, const fe* a, const fe* b, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        fe_store(out + i, fe_mul<FrP>(fe_ldg(a + i), fe_ldg(b + i)));
}

__global__ void fr_sub_kernel(fe* out, const fe* a, const fe* b, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        fe_store(out + i, fe_sub<FrP>(fe_ldg(a + i), fe_ldg(b + i)));
}

__global__ void fr_add_kernel(fe* out, const fe* a, const fe* b, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        fe_store(out + i, fe_add<FrP>(fe_ldg(a + i), fe_ldg(b + i)));
}

__global__ void last_nonzero_kernel(const fe* a, size_t n, unsigned long long* out) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        if (!fe_is_zero(fe_ldg(a + i))) atomicMax(out, (unsigned long long)(i + 1));
}

int trimmed_len(Ctx* c, const void* a, size_t n, size_t* out) {
    *out = 0;
    if (n == 0) return ZK_OK;
    ZK_CHECK_ARG(a != nullptr, "null buffer");
    unsigned long long* d = nullptr;
    int rc = scratch_alloc(c, sizeof(unsigned long long), reinterpret_cast<void**>(&d));
    if (rc != ZK_OK) return rc;
    ZK_TRY_CUDA(cudaMemsetAsync(d, 0, sizeof(unsigned long long), c->stream));
    ZK_LAUNCH(c, "last_nonzero", last_nonzero_kernel, grid_for(n, 256, c->num_sms), 256, 0,
              static_cast<const fe*>(a), n, d);
    ZK_TRY_CUDA(cudaGetLastError());
    unsigned long long h = 0;
    ZK_TRY_CUDA(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    ZK_TRY_CUDA(cudaStreamSynchronize(c->stream));
    scratch_free(c, d);
    *out = (size_t)h;
    return ZK_OK;
}

template <class F, int DIR>
int convert(Ctx* c, void* out, const void* in, size_t n) {
    if (n == 0) return ZK_OK;
    ZK_CHECK_ARG(out != nullptr && in != nullptr, "null buffer");
    ZK_LAUNCH(c, DIR ? "to_mont" : "from_mont", (convert_kernel<F, DIR>), grid_for(n, 256, c->num_sms), 256, 0,
              static_cast<fe*>(out), static_cast<const fe*>(in), n);
    ZK_TRY_CUDA(cudaGetLastError());
    return ZK_OK;
}

template int convert<FrP, 1>(Ctx*, void*, const void*, size_t);
template int convert<FrP, 0>(Ctx*, void*, const void*, size_t);
template int convert<FqP, 1>(Ctx*, void*, const void*, size_t);
template int convert<FqP, 0>(Ctx*, void*, const void*, size_t);

int fr_binary(Ctx* c, int op, void* out, const void* a, const void* b, size_t n) {
    if (n == 0) return ZK_OK;
    ZK_CHECK_ARG(out != nullptr && a != nullptr && b != nullptr, "null buffer");
    if (op == 0)
        ZK_LAUNCH(c, "fr_mul", fr_mul_kernel, grid_for(n, 256, c->num_sms), 256, 0, static_cast<fe*>(out),
                  static_cast<const fe*>(a), static_cast<const fe*>(b), n);
    else if (op == 1)
        ZK_LAUNCH(c, "fr_sub", fr_sub_kernel, grid_for(n, 256, c->num_sms), 256, 0, static_cast<fe*>(out),
                  static_cast<const fe*>(a), static_cast<const fe*>(b), n);
    else
        ZK_LAUNCH(c, "fr_add", fr_add_kernel, grid_for(n, 256, c->num_sms), 256, 0, static_cast<fe*>(out),
                  static_cast<const fe*>(a), static_cast<const fe*>(b), n);
    ZK_TRY_CUDA(cudaGetLastError());
    return ZK_OK;
}

// ---- fixed-base multiplication: out_i = [k_i] P --------------------------------------
// table[j * 256 + d] = d * 2^(8 j) * P (affine Montgomery, entry d = 0 unused).
template <class F>
__device__ fe fe_inverse(const fe& a) {
    // a^(p - 2) by left-to-right square-and-multiply over the constant exponent
    uint32_t e[8];
#pragma unroll
    for (int i = 0; i < 8; i++) e[i] = F::P(i);
    e[0] -= 2;  // p is odd and > 2: no borrow
    fe r = fe_one<F>();
    for (int limb = 7; limb >= 0; limb--) {
        for (int b = 31; b >= 0; b--) {
            r = fe_sqr<F>(r);
            if ((e[limb] >> b) & 1) r = fe_mul<F>(r, a);
        }
    }
    return r;
}

__device__ __forceinline__ fe c_inv_dev(const fe& a) { return fe_inverse<FqP>(a); }
// 1 / (a0 + a1 u) = (a0 - a1 u) / (a0^2 + a1^2)
__device__ __forceinline__ fq2 c_inv_dev(const fq2& a) {
    const fe t = fe_inverse<FqP>(c_add(c_mul(a.c0, a.c0), c_mul(a.c1, a.c1)));
    return {c_mul(a.c0, t), c_neg(c_mul(a.c1, t))};
}
__device__ __forceinline__ fe c_from_mont_dev(const fe& a) { return fe_from_mont<FqP>(a); }
__device__ __forceinline__ fq2 c_from_mont_dev(const fq2& a) {
    return {fe_from_mont<FqP>(a.c0), fe_from_mont<FqP>(a.c1)};
}

// out[i] = [k_i] P from a table of the 8-bit windows of P: table[j * 256 + d] = [d 2^(8 j)] P.
template <class C>
__global__ void fixed_base_kernel(const typename C::A* __restrict__ table, const fe* __restrict__ k, size_t n,
                                  typename C::A* __restrict__ out) {
    using T = typename C::T;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // reduce k mod r (canonical in) by a Montgomery round trip
    fe s = fe_from_mont<FrP>(fe_to_mont<FrP>(fe_ldg(k + i)));
    XyzzT<T> acc = xyzz_inf<T>();
    for (int j = 0; j < 32; j++) {
        const uint32_t d = (s.v[j >> 2] >> (8 * (j & 3))) & 0xffu;
        if (d) {
            const typename C::A p = affine_load(table + j * 256 + d);
            acc = xyzz_madd(acc, p.x, p.y);
        }
    }
    typename C::A r;
    if (xyzz_is_inf(acc)) {
        c_set_zero(r.x);
        c_set_zero(r.y);
    } else {
        const T I = c_inv_dev(c_mul(acc.ZZ, acc.ZZZ));
        const T izz = c_mul(acc.ZZZ, I);
        const T izzz = c_mul(acc.ZZ, I);
        r.x = c_from_mont_dev(c_mul(acc.X, izz));
        r.y = c_from_mont_dev(c_mul(acc.Y, izzz));
    }
    c_store(&out[i].x, r.x);
    c_store(&out[i].y, r.y);
}

template <class C>
static int fixed_base_mul_t(Ctx* c, const uint8_t* point_xy, const void* k_dev, size_t n, void* out_dev) {
    using H = typename HostOf<C>::T;
    using A = typename C::A;
    static_assert(sizeof(A) == 2 * sizeof(H), "layout");
    if (n == 0) return ZK_OK;
    ZK_CHECK_ARG(k_dev != nullptr && out_dev != nullptr, "null buffer");
    H px, py;
    std::memcpy(&px, point_xy, sizeof(H));
    std::memcpy(&py, point_xy + sizeof(H), sizeof(H));
    std::vector<A> table(32 * 256);
    std::memset(table.data(), 0, table.size() * sizeof(A));
    if (!(zkh::cis_zero(px) && zkh::cis_zero(py))) {
        zkh::XyzzT<H> base;
        base.X = zkh::cto_mont(px);
        base.Y = zkh::cto_mont(py);
        base.ZZ = zkh::cone<H>();
        base.ZZZ = zkh::cone<H>();
        std::vector<zkh::XyzzT<H>> pts(32 * 256);
        for (int j = 0; j < 32; j++) {
            pts[j * 256] = zkh::xyzz_inf<H>();
            for (int d = 1; d < 256; d++) pts[j * 256 + d] = zkh::xyzz_add(pts[j * 256 + d - 1], base);
            for (int b = 0; b < 8; b++) base = zkh::xyzz_dbl(base);
        }
        // batch normalisation: one inversion of the product of all ZZ * ZZZ
        std::vector<H> pref(pts.size());
        H run = zkh::cone<H>();
        for (size_t i = 0; i < pts.size(); i++) {
            pref[i] = run;
            if (!zkh::cis_zero(pts[i].ZZ)) run = zkh::cmul(run, zkh::cmul(pts[i].ZZ, pts[i].ZZZ));
        }
        H inv = zkh::cinv(run);
        for (size_t i = pts.size(); i-- > 0;) {
            if (zkh::cis_zero(pts[i].ZZ)) continue;
            const H zz_zzz = zkh::cmul(pts[i].ZZ, pts[i].ZZZ);
            const H I = zkh::cmul(inv, pref[i]);
            inv = zkh::cmul(inv, zz_zzz);
            const H x = zkh::cmul(pts[i].X, zkh::cmul(pts[i].ZZZ, I));
            const H y = zkh::cmul(pts[i].Y, zkh::cmul(pts[i].ZZ, I));
            std::memcpy(&table[i].x, &x, sizeof(H));
            std::memcpy(&table[i].y, &y, sizeof(H));
        }
    }
    A* dtab = nullptr;
    int rc = scratch_alloc(c, table.size() * sizeof(A), reinterpret_cast<void**>(&dtab));
    if (rc != ZK_OK) return rc;
    ZK_TRY_CUDA(cudaMemcpyAsync(dtab, table.data(), table.size() * sizeof(A), cudaMemcpyHostToDevice, c->stream));
    ZK_LAUNCH(c, sizeof(H) == 32 ? "fixed_base" : "fixed_base_g2", fixed_base_kernel<C>,
              (unsigned)((n + 127) / 128), 128, 0, dtab, static_cast<const fe*>(k_dev), n, static_cast<A*>(out_dev));
    ZK_TRY_CUDA(cudaGetLastError());
    // the host table must outlive the async copy
    ZK_TRY_CUDA(cudaStreamSynchronize(c->stream));
    scratch_free(c, dtab);
    return ZK_OK;
}

int fixed_base_mul(Ctx* c, const uint8_t point_xy[64], const void* k_dev, size_t n, void* out_dev) {
    return fixed_base_mul_t<CurveG1>(c, point_xy, k_dev, n, out_dev);
}

int fixed_base_mul_g2(Ctx* c, const uint8_t point_xy[128], const void* k_dev, size_t n, void* out_dev) {
    return fixed_base_mul_t<CurveG2>(c, point_xy, k_dev, n, out_dev);
}

}  // namespace zk

namespace zk {

// ---- IMAD throughput probes (roofline denominator) ------------------------------------
// MODE 0: carry chains shaped like one Montgomery row (mad.lo.cc / madc.hi.cc, each
//         chain serial through the carry flag);
// MODE 1: 8 independent mad.lo.u32 accumulators per thread (raw IMAD issue rate);
// MODE 2: 8 independent mad.hi.u32 accumulators per thread;
// MODE 3: 8 independent mad.wide.u32 (32x32 -> 64-bit) accumulators per thread, counted
//         as 2 IMAD each (one full-width product replaces a lo + hi pair).
template <int MODE>
__global__ void imad_probe_kernel(uint32_t iters, uint32_t seed, uint32_t* sink) {
    uint32_t a[8], x = seed ^ threadIdx.x, y = seed * 2654435761u + blockIdx.x;
#pragma unroll
    for (int i = 0; i < 8; i++) a[i] = x + i;
    for (uint32_t it = 0; it < iters; it++) {
        if constexpr (MODE == 0) {
            asm volatile(
                "mad.lo.cc.u32  %0, %8, %9, %0;\n\t"
                "madc.hi.cc.u32 %1, %8, %9, %1;\n\t"
                "madc.lo.cc.u32 %2, %8, %9, %2;\n\t"
                "madc.hi.cc.u32 %3, %8, %9, %3;\n\t"
                "madc.lo.cc.u32 %4, %8, %9, %4;\n\t"
                "madc.hi.cc.u32 %5, %8, %9, %5;\n\t"
                "madc.lo.cc.u32 %6, %8, %9, %6;\n\t"
                "madc.hi.u32    %7, %8, %9, %7;\n\t"
                : "+r"(a[0]), "+r"(a[1]), "+r"(a[2]), "+r"(a[3]), "+r"(a[4]), "+r"(a[5]), "+r"(a[6]), "+r"(a[7])
                : "r"(x), "r"(y));
            asm volatile(
                "mad.lo.cc.u32  %0, %8, %9, %0;\n\t"
                "madc.hi.cc.u32 %1, %8, %9, %1;\n\t"
                "madc.lo.cc.u32 %2, %8, %9, %2;\n\t"
                "madc.hi.cc.u32 %3, %8, %9, %3;\n\t"
                "madc.lo.cc.u32 %4, %8, %9, %4;\n\t"
                "madc.hi.cc.u32 %5, %8, %9, %5;\n\t"
                "madc.lo.cc.u32 %6, %8, %9, %6;\n\t"
                "madc.hi.u32    %7, %8, %9, %7;\n\t"
                : "+r"(a[7]), "+r"(a[6]), "+r"(a[5]), "+r"(a[4]), "+r"(a[3]), "+r"(a[2]), "+r"(a[1]), "+r"(a[0])
                : "r"(y), "r"(x));
            x += a[0];
        } else {
#pragma unroll
            for (int rep = 0; rep < 2; rep++) {
                if constexpr (MODE == 3) {
                    uint64_t w0 = a[0], w1 = a[1], w2 = a[2], w3 = a[3];
                    asm volatile(
                        "mad.wide.u32 %0, %4, %5, %0;\n\t"
                        "mad.wide.u32 %1, %4, %5, %1;\n\t"
                        "mad.wide.u32 %2, %4, %5, %2;\n\t"
                        "mad.wide.u32 %3, %4, %5, %3;\n\t"
                        "mad.wide.u32 %0, %5, %4, %0;\n\t"
                        "mad.wide.u32 %1, %5, %4, %1;\n\t"
                        "mad.wide.u32 %2, %5, %4, %2;\n\t"
                        "mad.wide.u32 %3, %5, %4, %3;\n\t"
                        : "+l"(w0), "+l"(w1), "+l"(w2), "+l"(w3)
                        : "r"(x), "r"(y));
                    a[0] = (uint32_t)w0 ^ (uint32_t)(w0 >> 32);
                    a[1] = (uint32_t)w1 ^ (uint32_t)(w1 >> 32);
                    a[2] = (uint32_t)w2 ^ (uint32_t)(w2 >> 32);
                    a[3] = (uint32_t)w3 ^ (uint32_t)(w3 >> 32);
                } else if constexpr (MODE == 1) {
                    asm volatile(
                        "mad.lo.u32 %0, %0, %8, %9;\n\t"
                        "mad.lo.u32 %1, %1, %8, %9;\n\t"
                        "mad.lo.u32 %2, %2, %8, %9;\n\t"
                        "mad.lo.u32 %3, %3, %8, %9;\n\t"
                        "mad.lo.u32 %4, %4, %8, %9;\n\t"
                        "mad.lo.u32 %5, %5, %8, %9;\n\t"
                        "mad.lo.u32 %6, %6, %8, %9;\n\t"
                        "mad.lo.u32 %7, %7, %8, %9;\n\t"
                        : "+r"(a[0]), "+r"(a[1]), "+r"(a[2]), "+r"(a[3]), "+r"(a[4]), "+r"(a[5]), "+r"(a[6]),
                          "+r"(a[7])
                        : "r"(x), "r"(y));
                } else {
                    asm volatile(
                        "mad.hi.u32 %0, %0, %8, %9;\n\t"
                        "mad.hi.u32 %1, %1, %8, %9;\n\t"
                        "mad.hi.u32 %2, %2, %8, %9;\n\t"
                        "mad.hi.u32 %3, %3, %8, %9;\n\t"
                        "mad.hi.u32 %4, %4, %8, %9;\n\t"
                        "mad.hi.u32 %5, %5, %8, %9;\n\t"
                        "mad.hi.u32 %6, %6, %8, %9;\n\t"
                        "mad.hi.u32 %7, %7, %8, %9;\n\t"
                        : "+r"(a[0]), "+r"(a[1]), "+r"(a[2]), "+r"(a[3]), "+r"(a[4]), "+r"(a[5]), "+r"(a[6]),
                          "+r"(a[7])
                        : "r"(x), "r"(y));
                }
            }
        }
    }
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) s ^= a[i];
    if (s == 0x9e3779b9u) sink[0] = s;  // keeps the chains alive
}

template <int MODE>
static int imad_probe_run(Ctx* c, uint32_t* sink, double* tera) {
    const uint32_t blocks = (uint32_t)c->num_sms * 8, threads = 256, iters = 4096;
    cudaEvent_t e0, e1;
    ZK_TRY_CUDA(cudaEventCreate(&e0));
    ZK_TRY_CUDA(cudaEventCreate(&e1));
    imad_probe_kernel<MODE><<<blocks, threads, 0, c->stream>>>(iters, 1u, sink);  // warm-up
    float best = 1e30f;
    for (int rep = 0; rep < 5; rep++) {
        ZK_TRY_CUDA(cudaEventRecord(e0, c->stream));
        imad_probe_kernel<MODE><<<blocks, threads, 0, c->stream>>>(iters, 2u + rep, sink);
        ZK_TRY_CUDA(cudaEventRecord(e1, c->stream));
        ZK_TRY_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        ZK_TRY_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) best = ms;
    }
    ZK_TRY_CUDA(cudaGetLastError());
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double ops = (double)blocks * threads * iters * 16.0 * (MODE == 3 ? 2.0 : 1.0);
    *tera = ops / (best * 1e-3) / 1e12;
    return ZK_OK;
}

int imad_probe(Ctx* c, int mode, double* tera) {
    ZK_CHECK_ARG(mode >= 0 && mode <= 3, "IMAD probe mode must be 0..3");
    uint32_t* sink = nullptr;
    int rc = scratch_alloc(c, 16, reinterpret_cast<void**>(&sink));
    if (rc != ZK_OK) return rc;
    if (mode == 0)
        rc = imad_probe_run<0>(c, sink, tera);
    else if (mode == 1)
        rc = imad_probe_run<1>(c, sink, tera);
    else if (mode == 2)
        rc = imad_probe_run<2>(c, sink, tera);
    else
        rc = imad_probe_run<3>(c, sink, tera);
    scratch_free(c, sink);
    return rc;
}

int imad_peak(Ctx* c, double* tera) {
    double best = 0.0;
    for (int mode = 0; mode < 4; mode++) {
        double t = 0.0;
        int rc = imad_probe(c, mode, &t);
        if (rc != ZK_OK) return rc;
        if (t > best) best = t;
    }
    *tera = best;
    return ZK_OK;
}

}  // namespace zk
