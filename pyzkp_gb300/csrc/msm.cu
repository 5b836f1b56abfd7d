// msm.cu -- BN254 G1 / G2 multi-scalar multiplication (Pippenger, signed digits, GLV, CSR buckets).
//
// Result semantics: the unique affine point sum_i s_i P_i, identical to
// crypto/msm/pippenger.py:10-64 and runtime/metal/msm.py:179-332 (metal_msm_g1_v2).
// The reference's Metal v2 pipeline is: signed-digit encode in Python
// (runtime/metal/msm.py:145-177), histogram / single-thread prefix sum / scatter
// into CSR (runtime/metal/ecc_source.py:437-496), one thread per bucket
// (:499-535), one thread per window reduce (:540-566), CPU Horner (msm.py:322-332).
//
// This pipeline (all on the device except the last ~W*13 point additions):
//  0. GLV (G1 and G2 bases carry phi(P) = [lambda] P behind P): every scalar is split
//     k = k1 + k2 lambda with |k1|, |k2| < 2^127 (glv_split), so the MSM runs over 2n points
//     with 128-bit scalars: W = ceil(128/c) windows instead of ceil(255/c), half the buckets.
//  1. msm_digits_kernel   scalar -> reduced scalar (zero for an infinity base), its GLV
//                         halves, and the CSR histogram of their W signed c-bit digits
//                         (|d| <= 2^(c-1)), counted with warp-aggregated atomics (__match_any_sync).
//  2. device scan         counters -> CSR row pointers (scan.cu).
//  3. msm_scatter_kernel  the digits again; entry = point index | sign << 31 in the range
//                         of its (window, |digit|) bucket (no per-entry bucket id is
//                         stored: the row pointers imply it).
//  4. msm_accumulate_*    equal-size segments of S entries per thread (load balanced
//                         even when one bucket holds 5% of all points; a segment finds
//                         its first bucket by binary search over the row pointers);
//                         buckets wholly inside a segment are final; a bucket that
//                         straddles segment boundaries leaves partial sums that one fixup
//                         thread per bucket adds (short buckets), or tree rounds (pairs,
//                         then groups of 4 units) merge, deciding "straddles" from the row
//                         pointers.
//  5. msm_bucket_blocks   per window, blocks of g buckets: sum_b b*B_b = sum_j E_j + g*WS(Y)
//                         with Y_j the block sums and E_j = -(sum of the g-1 prefix sums).
//  6. msm_targets_kernel  WS(Y) = sum_j Y_j + sum_k 2^k M_k with M_k the sum of the Y_j
//                         whose index has bit k set: plain sums, reduced by CTA trees.
//  7. host: per window S_w = T_E + g (T_Y + sum_k 2^k M_k), then Horner over windows.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <functional>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <thread>
#include <tuple>
#include <type_traits>
#include <vector>

#include "zk_internal.cuh"

namespace zk {

int device_exclusive_scan(Ctx* c, uint32_t* data, size_t n, uint32_t* total, uint32_t* scratch);
size_t scan_scratch_elems(size_t n);

static constexpr uint32_t kNone = 0xffffffffu;
#ifndef ZK_MSM_SEGMENT
#define ZK_MSM_SEGMENT 32
#endif
#ifndef ZK_MSM_BLOCKG
#define ZK_MSM_BLOCKG 8
#endif
#ifndef ZK_MSM_GROUP
#define ZK_MSM_GROUP 4  // measured at 2^20 / 2^22: merge 0.73 / 1.36 ms with 16, 0.48 / 1.02 ms with 4
#endif
static constexpr uint32_t kSegment = ZK_MSM_SEGMENT;  // entries per thread in the first accumulation round
static constexpr uint32_t kMinSegment = 8;            // ... at least, in small pipelines
static constexpr uint32_t kFirstGroup = 2;            // units merged per thread in the first merge round
static constexpr uint32_t kGroup = ZK_MSM_GROUP;      // units merged per thread in later rounds
static constexpr uint32_t kBlockG = ZK_MSM_BLOCKG;    // buckets per block in the window reduction
#ifndef ZK_MSM_BLOCKG2
// measured at 2^20 (GLV, 8 windows): level-2 pass 0.154 ms with 8, 0.068 ms with 4 (its
// threads are few and each runs a chain of g2 additions); the targets grow 0.078 -> 0.102 ms
#define ZK_MSM_BLOCKG2 4
#endif
static constexpr uint32_t kBlockG2 = ZK_MSM_BLOCKG2;  // level-1 blocks per level-2 block
// Straddling buckets over more than kFixupMax + 1 segments go to the long-bucket fixup (a
// CTA tree per bucket); small pipelines, latency-bound, send them there from kFixupMaxSmall
// + 2 segments on (a tree of log2(pieces) additions instead of a chain). Measured on GB300
// (single MSMs, 4 against 8): 2^12 0.390 -> 0.371 ms, 2^16 0.767 -> 0.753 ms, 2^14 the same;
// then 3 against 4: 2^12 0.348 -> 0.331 ms, 2^10 / 2^14 / 2^16 -0.5..-1.5% (2 is slower: the
// CTA trees of many 4-piece buckets, 2^16 0.98 ms).
static constexpr uint32_t kFixupMax = 8;
#ifndef ZK_FIXUP_MAX_SMALL
#define ZK_FIXUP_MAX_SMALL 3
#endif
static constexpr uint32_t kFixupMaxSmall = ZK_FIXUP_MAX_SMALL;
static constexpr uint32_t kSmallBucketsPerSm = 512;  // "small": fewer buckets than this per SM

struct MsmShape {
    uint32_t c;        // window bits
    uint32_t W;        // windows
    uint32_t B;        // buckets per window (|digit| in 1..B)
    uint32_t g;        // level-1 block size of the window reduction (<= B)
    uint32_t G;        // level-1 blocks per window
    uint32_t g2;       // level-2 block size (1: no second level)
    uint32_t G2;       // level-2 blocks per window (G / g2)
    uint32_t K;        // log2(G2)
    uint32_t plain;    // plain-sum targets: 2 (one level) or 3 (two levels)
    uint32_t targets;  // plain + K
    uint32_t shared;   // 1: fixed-base mode, all windows share one bucket set (window-shifted bases)
    uint32_t Wr;       // bucket sets per instance: W, or 1 in fixed-base mode
    uint32_t inst;     // MSM instances in the pipeline
    uint32_t sets;     // bucket sets to reduce: inst * Wr
    uint32_t glv;      // 1: each scalar is split k = k1 + k2 lambda (halves < 2^127, see glv_split);
                       // the phi(P) half of every instance's bases sits at bases + stride
    uint32_t seg;      // CSR entries per thread in the accumulation (kSegment, less for small pipelines)
    uint32_t fixmax;   // a straddling bucket over more than fixmax + 1 segments goes to the long-bucket fixup
};

// One MSM of a pipeline: sum_{i < n} scalars[i] * bases[i] (fixed-base mode: bases holds the
// window-shifted rows, row j at bases + j * stride). Instance k owns the global scalar
// indices [off_k, off_k + n) and the bucket sets [k Wr, (k + 1) Wr).
struct MsmInst {
    const fe* scalars;
    const void* bases;  // C::A points of the pipeline's curve
    uint32_t n;
    uint32_t stride;
};

// Block structure of the window reduction for level-1 blocks of g buckets and level-2
// blocks of g2 level-1 blocks.
static void shape_blocks(MsmShape& s, uint32_t g, uint32_t g2 = kBlockG2) {
    s.g = std::min<uint32_t>(g, s.B);
    s.G = s.B / s.g;
    s.g2 = s.G >= 2 * g2 ? g2 : 1;
    s.G2 = s.G / s.g2;
    s.K = 0;
    while ((1u << s.K) < s.G2) s.K++;
    s.plain = s.g2 > 1 ? 3 : 2;
    s.targets = s.plain + s.K;
}

static MsmShape make_shape(uint32_t c, bool glv = false) {
    MsmShape s;
    s.c = c;
    // W*c >= bits + 1 so that the top window never carries out: scalars < r < 2^254, or GLV
    // halves < 2^127
    s.W = ((glv ? 128u : 255u) + c - 1) / c;
    s.B = 1u << (c - 1);
    shape_blocks(s, kBlockG);
    s.seg = kSegment;
    s.fixmax = kFixupMax;
    s.shared = 0;
    s.Wr = s.W;
    s.inst = 1;
    s.sets = s.W;
    s.glv = glv ? 1u : 0u;
    return s;
}

uint32_t msm_auto_window(size_t n) {
    uint32_t lg = 0;
    while ((1ull << lg) < n) lg++;
    int c = (int)lg - 3;
    if (c < 4) c = 4;
    if (c > 16) c = 16;
    return (uint32_t)c;
}

// GLV: the same rule over n scalars (2n half-scalars of 128 bits), lowered while the window
// count stays the same (fewer buckets for the same entries: c = 14 -> 13, 12 stays).
// Window size of the GLV split (halves of ~127 bits). Measured on GB300 for n = 2^8 .. 2^20
// (G1, every c from about log2(n) - 6 to log2(n), uniform and witness-like scalars); the
// table holds the c with the smallest product of the two times relative to their best.
// A sparse top window (c = 9: 2 of its 9 bits used, c = 14: 2 of 14) puts a large share of
// all points into a few buckets, and so do repeated small scalars (0 and 1 in witnesses);
// the long-bucket fixup adds their pieces in trees of serial point additions (0.04 - 0.6
// ms), which the merge rounds of larger c avoid. Against the earlier rule (log2(n) - 3,
// lowered while W stays): uniform 2^8 -22%, 2^10 -19%, 2^12 -7%; witness-like 2^11 -10%,
// 2^17 -27%, 2^18 -31% (uniform +3% / +6% there). From 2^19 on c = 16 stays (uniform
// 2^19 / 2^20 best at 16, witness-like at 13 / 14).
uint32_t msm_auto_window_glv(size_t n) {
    uint32_t lg = 0;
    while ((1ull << lg) < n) lg++;
    static const uint8_t kMeasured[19] = {0, 0, 0, 0, 0, 0, 0, 0, 8, 8, 8, 9, 10, 11, 11, 13, 13, 13, 15};
    if (lg >= 8 && lg <= 18) return kMeasured[lg];
    uint32_t c = msm_auto_window(n);
    while (c > 4 && (128 + c - 2) / (c - 1) == (128 + c - 1) / c) c--;
    return c;
}

// ---- GLV scalar split -------------------------------------------------------------
// BN254 G1 has the endomorphism phi(x, y) = (beta x, y) = [lambda](x, y), with beta a cube
// root of unity in Fq and lambda one in Fr. The lattice {(a, b) : a + b lambda = 0 mod r} has
// the reduced basis v1 = (a1, -b1), v2 = (a2, b2) (extended Euclid on (r, lambda), stopped
// at the first remainder below sqrt(r); a1 b2 + a2 b1 = r). Babai rounding:
//   c1 = round(k b2 / r), c2 = round(k b1 / r),  computed as (k g + 2^255) >> 256 with
//   g = round(2^256 b / r);  k1 = k - c1 a1 - c2 a2,  k2 = c1 b1 - c2 b2,
// so k1 + k2 lambda = k (mod r) and |k1|, |k2| <= (1/2 + 2^-3.4)(a1 + a2) < 2^126.1.
// Constants as 32-bit limbs, least significant first.
__device__ __constant__ uint32_t kGlvG1[3] = {0xc7e0b3d7u, 0xd91d232eu, 0x00000002u};  // round(2^256 b2 / r)
__device__ __constant__ uint32_t kGlvG2[5] = {0x391eb18eu, 0x7a7bd9d4u, 0xa773d2cfu, 0x4ccef014u,
                                              0x00000002u};                      // round(2^256 b1 / r)
__device__ __constant__ uint32_t kGlvA1[2] = {0x94d213e3u, 0x89d32568u};         // a1 = b2
__device__ __constant__ uint32_t kGlvA2[4] = {0x1221250bu, 0x0be4e154u, 0xeeb859fdu, 0x6f4d8248u};
__device__ __constant__ uint32_t kGlvB1[4] = {0x7d4f1128u, 0x8211bbebu, 0xeeb859fcu, 0x6f4d8248u};

// (k * g + 2^255) >> 256 for k < 2^256 (8 limbs) and g of NG limbs: NG limbs.
template <int NG>
__device__ __forceinline__ void glv_round(const fe& k, const uint32_t* g, uint32_t* c) {
    uint32_t p[8 + NG];
#pragma unroll
    for (int i = 0; i < 8 + NG; i++) p[i] = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        uint64_t carry = 0;
#pragma unroll
        for (int j = 0; j < NG; j++) {
            const uint64_t t = (uint64_t)k.v[i] * g[j] + p[i + j] + carry;
            p[i + j] = (uint32_t)t;
            carry = t >> 32;
        }
        p[i + NG] = (uint32_t)carry;
    }
    uint64_t t = (uint64_t)p[7] + 0x80000000u;
#pragma unroll
    for (int i = 8; i < 8 + NG; i++) {
        t = (t >> 32) + p[i];
        c[i - 8] = (uint32_t)t;
    }
}

// acc -= a * b (mod 2^256) for a of NA limbs and b of NB limbs (sub = false: acc += a * b).
template <int NA, int NB, bool SUB>
__device__ __forceinline__ void glv_mac(uint32_t* acc, const uint32_t* a, const uint32_t* b) {
    uint32_t p[8];
#pragma unroll
    for (int i = 0; i < 8; i++) p[i] = 0;
#pragma unroll
    for (int i = 0; i < NA; i++) {
        uint64_t carry = 0;
#pragma unroll
        for (int j = 0; j < NB; j++) {
            if (i + j < 8) {
                const uint64_t t = (uint64_t)a[i] * b[j] + p[i + j] + carry;
                p[i + j] = (uint32_t)t;
                carry = t >> 32;
            }
        }
        if (i + NB < 8) p[i + NB] = (uint32_t)carry;
    }
    uint64_t t = SUB ? 1 : 0;  // acc + ~p + 1 = acc - p
#pragma unroll
    for (int i = 0; i < 8; i++) {
        t += (uint64_t)acc[i] + (SUB ? (uint32_t)~p[i] : p[i]);
        acc[i] = (uint32_t)t;
        t >>= 32;
    }
}

// |x| of a two's-complement 256-bit value with the sign in bit 255 of the result.
__device__ __forceinline__ fe glv_sign_mag(const uint32_t* x) {
    fe r;
    const uint32_t neg = x[7] >> 31;
    uint64_t t = neg;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        t += (uint64_t)(neg ? ~x[i] : x[i]);
        r.v[i] = (uint32_t)t;
        t >>= 32;
    }
    r.v[7] |= neg << 31;  // |x| < 2^127: bit 255 is free
    return r;
}

// k (canonical, < r) -> (|k1| | s1 << 255, |k2| | s2 << 255) with k = k1 + k2 lambda (mod r).
__device__ __forceinline__ void glv_split(const fe& k, fe& h0, fe& h1) {
    uint32_t c1[3], c2[5];
    glv_round<3>(k, kGlvG1, c1);
    glv_round<5>(k, kGlvG2, c2);
    uint32_t k1[8], k2[8];
#pragma unroll
    for (int i = 0; i < 8; i++) {
        k1[i] = k.v[i];
        k2[i] = 0;
    }
    glv_mac<3, 2, true>(k1, c1, kGlvA1);
    glv_mac<5, 4, true>(k1, c2, kGlvA2);
    glv_mac<3, 4, false>(k2, c1, kGlvB1);
    glv_mac<5, 2, true>(k2, c2, kGlvA1);  // b2 = a1
    h0 = glv_sign_mag(k1);
    h1 = glv_sign_mag(k2);
}

// pts[n + i] = phi(pts[i]) = (beta x_i, y_i); infinity (0, 0) stays (0, 0).
__global__ void glv_phi_kernel(affine_t* __restrict__ pts, size_t n, fe beta) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const affine_t p = affine_load(pts + i);
        fe_store(&pts[n + i].x, fe_reduce_once<FqP>(fe_mul<FqP>(p.x, beta)));  // bases stay in [0, q)
        fe_store(&pts[n + i].y, p.y);
    }
}

// G2: pts[n + i] = (beta^2 x_i, y_i) = [lambda] P_i (on the twist the same lambda goes with beta^2;
// beta^2 multiplies both Fq coordinates of x in Fq2).
__global__ void glv_phi2_kernel(affine2_t* __restrict__ pts, size_t n, fe beta2) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const affine2_t p = affine_load(pts + i);
        fe_store(&pts[n + i].x.c0, fe_reduce_once<FqP>(fe_mul<FqP>(p.x.c0, beta2)));
        fe_store(&pts[n + i].x.c1, fe_reduce_once<FqP>(fe_mul<FqP>(p.x.c1, beta2)));
        fe_store(&pts[n + i].y.c0, p.y.c0);
        fe_store(&pts[n + i].y.c1, p.y.c1);
    }
}

// beta = 0x59e26bcea0d48bacd4f263f1acdb5c4f5763473177fffffe, the cube root of unity in Fq
// with (beta x, y) = [lambda](x, y) on G1 for lambda = 0xb3c4d79d41a917585bfc41088d8daaa78b17ea66b99c90dd
// (Montgomery form; squared for G2).
static fe glv_beta_mont(bool squared) {
    const zkh::F4 canon = {{0x5763473177fffffeull, 0xd4f263f1acdb5c4full, 0x59e26bcea0d48bacull, 0}};
    zkh::F4 m = zkh::to_mont(zkh::fq(), canon);
    if (squared) m = zkh::mul(zkh::fq(), m, m);
    fe r;
    std::memcpy(r.v, m.v, 32);
    return r;
}

int glv_phi2(Ctx* c, affine2_t* pts, size_t n) {
    if (n == 0) return ZK_OK;
    static const fe beta2_m = glv_beta_mont(true);
    const unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, (size_t)c->num_sms * 16);
    ZK_LAUNCH(c, "glv_phi2", glv_phi2_kernel, blocks, 256, 0, pts, n, beta2_m);
    ZK_TRY_CUDA(cudaGetLastError());
    return ZK_OK;
}

template <class A>
__global__ void any_zero_point_kernel(const A* __restrict__ pts, size_t n, uint32_t* __restrict__ flag) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const A p = affine_load(pts + i);
        if (affine_is_zero_bits(p)) {
            atomicOr(flag, 1u);
            return;
        }
    }
}

int mark_infinity(Ctx* c, const void* pts, size_t n, bool g2, uint32_t* flag) {
    if (n == 0) return ZK_OK;
    const unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, (size_t)c->num_sms * 8);
    if (g2)
        ZK_LAUNCH(c, "any_zero_point", any_zero_point_kernel<affine2_t>, blocks, 256, 0,
                  static_cast<const affine2_t*>(pts), n, flag);
    else
        ZK_LAUNCH(c, "any_zero_point", any_zero_point_kernel<affine_t>, blocks, 256, 0,
                  static_cast<const affine_t*>(pts), n, flag);
    ZK_TRY_CUDA(cudaGetLastError());
    return ZK_OK;
}

int any_infinity(Ctx* c, const void* pts, size_t n, bool g2, bool* out) {
    *out = false;
    if (n == 0) return ZK_OK;
    uint32_t* flag = nullptr;
    int rc = scratch_alloc(c, 4, reinterpret_cast<void**>(&flag));
    if (rc != ZK_OK) return rc;
    uint32_t h = 0;
    cudaError_t e = cudaMemsetAsync(flag, 0, 4, c->stream);
    if (e == cudaSuccess) {
        rc = mark_infinity(c, pts, n, g2, flag);
        if (rc != ZK_OK) {
            scratch_free(c, flag);
            return rc;
        }
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, flag, 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    scratch_free(c, flag);
    if (e != cudaSuccess) {
        set_error(std::string("any_infinity: ") + cudaGetErrorString(e));
        return ZK_ECUDA;
    }
    *out = h != 0;
    return ZK_OK;
}

int glv_phi(Ctx* c, affine_t* pts, size_t n) {
    if (n == 0) return ZK_OK;
    static const fe beta_m = glv_beta_mont(false);
    const unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, (size_t)c->num_sms * 16);
    ZK_LAUNCH(c, "glv_phi", glv_phi_kernel, blocks, 256, 0, pts, n, beta_m);
    ZK_TRY_CUDA(cudaGetLastError());
    return ZK_OK;
}

// ---- 1. digits + histogram ----------------------------------------------------
__device__ __forceinline__ uint32_t bits_at(const fe& s, uint32_t k, uint32_t c) {
    const uint32_t limb = k >> 5, off = k & 31;
    uint64_t v = s.v[limb];
    if (limb + 1 < 8) v |= (uint64_t)s.v[limb + 1] << 32;
    // c <= 20 and off <= 31 keep off + c <= 51 bits: two limbs always suffice
    return (uint32_t)((v >> off) & ((1ull << c) - 1));
}

__device__ __forceinline__ void warp_aggregated_inc(uint32_t* counters, uint32_t key, bool active) {
#ifdef ZK_SCATTER_PLAIN
    if (active) atomicAdd(counters + key, 1u);
    return;
#endif
    const uint32_t live = __ballot_sync(0xffffffffu, active);
    if (!active) return;
    const uint32_t peers = __match_any_sync(live, key);
    const int leader = __ffs(peers) - 1;
    if ((int)(threadIdx.x & 31) == leader) atomicAdd(counters + key, (uint32_t)__popc(peers));
}

// Instance of global scalar index j: the largest k with offs[k] <= j (offs[inst] = total;
// empty instances repeat an offset and are skipped by taking the largest k).
__device__ __forceinline__ uint32_t find_inst(const uint32_t* __restrict__ offs, uint32_t ninst, uint32_t j) {
    uint32_t lo = 0, hi = ninst;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(offs + mid) <= j) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Signed digit of window w (|d| <= 2^(c-1)); `carry` runs from window to window.
// Returns mag | neg << 31, or 0 for a zero digit.
__device__ __forceinline__ uint32_t signed_digit(const fe& s, uint32_t w, const MsmShape& sh, uint32_t& carry) {
    const uint32_t v = bits_at(s, w * sh.c, sh.c) + carry;
    if (w + 1 < sh.W && v > (1u << (sh.c - 1))) {  // v in (2^(c-1), 2^c]: digit v - 2^c in [-2^(c-1)+1, 0]
        carry = 1;
        const uint32_t mag = (1u << sh.c) - v;
        return mag ? (mag | 0x80000000u) : 0u;  // v == 2^c: digit 0, only the carry moves on
    }
    carry = 0;  // v in [0, 2^(c-1)] (the top window is at most 2^(c-1), see make_shape)
    return v;
}

// Canonical scalars (reduced mod r) to `reduced` for the scatter, and the CSR histogram of
// the digits. The bases are not read here (an infinity base is skipped where the
// accumulation loads it), so the points may still be uploading while the digits run.
template <class C>
__global__ void msm_digits_kernel(const MsmInst* __restrict__ insts, const uint32_t* __restrict__ offs, uint32_t j0,
                                  uint32_t N, int scalars_mont, MsmShape sh, fe* __restrict__ reduced,
                                  uint32_t* __restrict__ counts) {
    const uint32_t j = j0 + blockIdx.x * blockDim.x + threadIdx.x;  // scalars [j0, N) in this launch
    const bool valid = j < N;
    fe s = fe_zero();
    uint32_t set0 = 0;
    if (valid) {
        const uint32_t k = find_inst(offs, sh.inst, j);
        const uint32_t i = j - __ldg(offs + k);
        s = fe_ldg(insts[k].scalars + i);
        s = scalars_mont ? fe_from_mont<FrP>(s) : fe_from_mont<FrP>(fe_to_mont<FrP>(s));
        set0 = k * sh.Wr;
        if (!sh.glv) fe_store(reduced + j, s);
    }
    if (sh.glv) {  // two half-scalars, both counted in the same window sets
        fe h[2];
        glv_split(s, h[0], h[1]);
        if (valid) {
            fe_store(reduced + 2 * (size_t)j, h[0]);
            fe_store(reduced + 2 * (size_t)j + 1, h[1]);
        }
#pragma unroll
        for (int hh = 0; hh < 2; hh++) {
            h[hh].v[7] &= 0x7fffffffu;  // drop the sign flag
            uint32_t carry = 0;
            for (uint32_t w = 0; w < sh.W; w++) {
                const uint32_t mag = signed_digit(h[hh], w, sh, carry) & 0x7fffffffu;
                warp_aggregated_inc(counts, (set0 + w) * sh.B + (mag - 1), valid && mag != 0);
            }
        }
        return;
    }
    uint32_t carry = 0;
    for (uint32_t w = 0; w < sh.W; w++) {
        const uint32_t d = signed_digit(s, w, sh, carry);
        const uint32_t mag = d & 0x7fffffffu;
        warp_aggregated_inc(counts, (set0 + (sh.shared ? 0u : w)) * sh.B + (mag - 1), valid && mag != 0);
    }
}

// ---- 3. scatter into CSR ------------------------------------------------------
// The digits again from the reduced scalars; entry = point index | sign << 31, placed in
// its bucket's CSR range (the bucket of an entry is implied by the row pointers).
__global__ void msm_scatter_kernel(const fe* __restrict__ reduced, const MsmInst* __restrict__ insts,
                                   const uint32_t* __restrict__ offs, uint32_t N, MsmShape sh,
                                   uint32_t* __restrict__ cursor, uint32_t* __restrict__ entries) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = j < N;
    uint32_t set0 = 0, i = 0, stride = 0;
    fe s = fe_zero();
    if (valid) {
        const uint32_t k = find_inst(offs, sh.inst, j);
        i = j - __ldg(offs + k);
        set0 = k * sh.Wr;
        stride = insts[k].stride;
    }
    // GLV: half h of scalar j is reduced[2j + h] (sign flag in bit 255) on point i + h * stride
    const uint32_t halves = sh.glv ? 2u : 1u;
    for (uint32_t h = 0; h < halves; h++) {
        fe s = fe_zero();
        if (valid) s = fe_load(reduced + (size_t)j * halves + h);
        const uint32_t flip = s.v[7] & 0x80000000u;  // zero unless a negative GLV half
        s.v[7] &= 0x7fffffffu;
        uint32_t carry = 0;
        for (uint32_t w = 0; w < sh.W; w++) {
            const uint32_t d = signed_digit(s, w, sh, carry);
            const bool nz = valid && d != 0;
            const uint32_t key = (set0 + (sh.shared ? 0u : w)) * sh.B + (d & 0x7fffffffu) - 1;
            // fixed-base: row w of the shifted bases; GLV: the phi(P) half for h = 1
            const uint32_t point = sh.shared ? w * stride + i : i + h * stride;
#ifdef ZK_SCATTER_PLAIN
            if (nz) entries[atomicAdd(cursor + key, 1u)] = point | ((d & 0x80000000u) ^ flip);
            continue;
#endif
            const uint32_t live = __ballot_sync(0xffffffffu, nz);
            if (nz) {
                const uint32_t peers = __match_any_sync(live, key);
                const int lane = threadIdx.x & 31;
                const int leader = __ffs(peers) - 1;
                uint32_t base = 0;
                if (lane == leader) base = atomicAdd(cursor + key, (uint32_t)__popc(peers));
                base = __shfl_sync(peers, base, leader);
                const uint32_t rank = __popc(peers & ((1u << lane) - 1));
                entries[base + rank] = point | ((d & 0x80000000u) ^ flip);
            }
        }
    }
}

// ---- 2-3 (tiled form). CSR sort without global atomics ----------------------------------
// Used when a bucket set fits shared memory (B <= kTiledMaxB). The entries of bucket set s
// (instance k = s / Wr) are enumerated in a fixed order: position set_base[s] + idx with
// idx = i * halves + h (point i, GLV half h) for window sets, idx = w * n_k + i for the one
// shared set of the fixed-base mode. Each set's positions are cut into tiles of `te`
// entries, numbered from set_tile0[s]:
//   codes     one 32-bit code per position: |d| - 1 | sign << 31, kNoCode for a zero digit
//             (digits computed once, from the canonical scalars);
//   hist      per tile, its bucket counts in shared memory -> M[tile][b] (no global atomics);
//   totals    per (set, b), the sum over the set's tiles -> row_ptr, then the exclusive scan;
//   offsets   M[tile][b] := row_ptr + the counts of the set's earlier tiles;
//   scatter   per tile, shared-memory cursors from M: entries land in tile order within each
//             bucket (the order inside a tile is that of the shared-memory atomics).
static constexpr uint32_t kNoCode = 0xffffffffu;
static constexpr uint32_t kTiledMaxB = 1u << 15;  // 128 KB of shared-memory counters
static constexpr uint32_t kTiledThreads = 1024;
static constexpr uint32_t kSortBatch = 8;  // codes loaded per thread before they are counted / placed

template <class C>
__global__ void msm_codes_kernel(const MsmInst* __restrict__ insts, const uint32_t* __restrict__ offs, uint32_t j0,
                                 uint32_t N, int scalars_mont, MsmShape sh, const uint32_t* __restrict__ set_base,
                                 uint32_t* __restrict__ codes) {
    const uint32_t j = j0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    const uint32_t k = find_inst(offs, sh.inst, j);
    const uint32_t i = j - __ldg(offs + k);
    fe s = fe_ldg(insts[k].scalars + i);
    s = scalars_mont ? fe_from_mont<FrP>(s) : fe_from_mont<FrP>(fe_to_mont<FrP>(s));
    const uint32_t set0 = k * sh.Wr;
    if (sh.glv) {
        fe h[2];
        glv_split(s, h[0], h[1]);
#pragma unroll
        for (int hh = 0; hh < 2; hh++) {
            const uint32_t flip = h[hh].v[7] & 0x80000000u;  // the half is negative
            h[hh].v[7] &= 0x7fffffffu;
            uint32_t carry = 0;
            for (uint32_t w = 0; w < sh.W; w++) {
                const uint32_t d = signed_digit(h[hh], w, sh, carry);
                const uint32_t code = d ? (((d & 0x7fffffffu) - 1) | ((d & 0x80000000u) ^ flip)) : kNoCode;
                codes[__ldg(set_base + set0 + w) + 2 * i + hh] = code;
            }
        }
        return;
    }
    const uint32_t nk = insts[k].n;
    uint32_t carry = 0;
    for (uint32_t w = 0; w < sh.W; w++) {
        const uint32_t d = signed_digit(s, w, sh, carry);
        const uint32_t code = d ? (((d & 0x7fffffffu) - 1) | (d & 0x80000000u)) : kNoCode;
        const uint32_t pos = sh.shared ? __ldg(set_base + set0) + w * nk + i : __ldg(set_base + set0 + w) + i;
        codes[pos] = code;
    }
}

// The set of tile t: the largest s with set_tile0[s] <= t.
__device__ __forceinline__ uint32_t set_of_tile(const uint32_t* __restrict__ set_tile0, uint32_t sets, uint32_t t) {
    uint32_t lo = 0, hi = sets;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(set_tile0 + mid) <= t) lo = mid;
        else hi = mid;
    }
    return lo;
}

__global__ void __launch_bounds__(kTiledThreads) msm_hist_kernel(const uint32_t* __restrict__ codes,
                                                                 const uint32_t* __restrict__ set_base,
                                                                 const uint32_t* __restrict__ set_tile0,
                                                                 uint32_t sets, uint32_t te, uint32_t B,
                                                                 uint32_t* __restrict__ M) {
    extern __shared__ uint32_t hist[];
    const uint32_t t = blockIdx.x;
    const uint32_t s = set_of_tile(set_tile0, sets, t);
    const uint32_t e0 = set_base[s] + (t - set_tile0[s]) * te;
    const uint32_t e1 = min(e0 + te, set_base[s + 1]);
    for (uint32_t b = threadIdx.x; b < B; b += blockDim.x) hist[b] = 0;
    __syncthreads();
    // kSortBatch codes in flight per thread before their counters are bumped
    for (uint32_t base = e0 + threadIdx.x; base < e1; base += blockDim.x * kSortBatch) {
        uint32_t code[kSortBatch];
#pragma unroll
        for (uint32_t q = 0; q < kSortBatch; q++) {
            const uint32_t e = base + q * blockDim.x;
            code[q] = e < e1 ? __ldg(codes + e) : kNoCode;
        }
#pragma unroll
        for (uint32_t q = 0; q < kSortBatch; q++)
            if (code[q] != kNoCode) atomicAdd(hist + (code[q] & 0x7fffffffu), 1u);
    }
    __syncthreads();
    uint32_t* out = M + (size_t)t * B;
    for (uint32_t b = threadIdx.x; b < B; b += blockDim.x) out[b] = hist[b];
}

// row_ptr[s B + b] = the count of bucket b of set s over the set's tiles.
__global__ void msm_hist_total_kernel(const uint32_t* __restrict__ M, const uint32_t* __restrict__ set_tile0,
                                      uint32_t sets, uint32_t B, uint32_t* __restrict__ row_ptr) {
    const uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= (uint64_t)sets * B) return;
    const uint32_t s = (uint32_t)(x / B), b = (uint32_t)(x % B);
    uint32_t sum = 0;
    for (uint32_t t = set_tile0[s]; t < set_tile0[s + 1]; t++) sum += M[(size_t)t * B + b];
    row_ptr[x] = sum;
}

// M[t][b] := the first position of tile t's entries of bucket b (row_ptr: scanned).
__global__ void msm_hist_offsets_kernel(uint32_t* __restrict__ M, const uint32_t* __restrict__ set_tile0,
                                        uint32_t sets, uint32_t B, const uint32_t* __restrict__ row_ptr) {
    const uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= (uint64_t)sets * B) return;
    const uint32_t s = (uint32_t)(x / B), b = (uint32_t)(x % B);
    uint32_t base = row_ptr[x];
    const uint32_t t1 = set_tile0[s + 1];
    for (uint32_t t0 = set_tile0[s]; t0 < t1; t0 += 16) {
        // 16 counts loaded before any is overwritten: the loads do not wait on the stores
        uint32_t v[16];
#pragma unroll
        for (uint32_t q = 0; q < 16; q++) v[q] = t0 + q < t1 ? M[(size_t)(t0 + q) * B + b] : 0u;
#pragma unroll
        for (uint32_t q = 0; q < 16; q++)
            if (t0 + q < t1) {
                M[(size_t)(t0 + q) * B + b] = base;
                base += v[q];
            }
    }
}

// Small pipelines: the bucket totals, their exclusive scan (row_ptr, the total at
// row_ptr[sets B]) and the per-tile cursors in one CTA, instead of four or five launches of
// a few microseconds each (the totals and cursors walk buckets strided by the CTA size, so
// the count table is read and written coalesced; the scan takes contiguous runs).
static constexpr uint32_t kMetaThreads = 1024;
// Limits of the one-CTA form (measured on GB300: 2^12 single MSM 0.374 -> 0.360 ms with it;
// at 2^14, 48 k counts, and in batches of 64 instances the one CTA ran as long as the
// launches it replaces or longer)
static constexpr uint64_t kMetaMaxBuckets = 1u << 13;  // row_ptr slots the one CTA handles
static constexpr uint64_t kMetaMaxCounts = 1u << 14;   // per-tile counts (tiles x B) it walks

__global__ void __launch_bounds__(kMetaThreads) msm_sort_meta_kernel(uint32_t* __restrict__ M,
                                                                     const uint32_t* __restrict__ set_tile0,
                                                                     uint32_t sets, uint32_t B,
                                                                     uint32_t* __restrict__ row_ptr) {
    __shared__ uint32_t part[kMetaThreads];
    const uint32_t nb = sets * B;
    // counts of bucket x over its set's tiles
    for (uint32_t x = threadIdx.x; x < nb; x += blockDim.x) {
        const uint32_t s = x / B, b = x % B;
        uint32_t tot = 0;
        for (uint32_t t = set_tile0[s]; t < set_tile0[s + 1]; t++) tot += M[(size_t)t * B + b];
        row_ptr[x] = tot;
    }
    __syncthreads();
    // exclusive scan: thread i sums the run [i per, (i + 1) per), the runs' sums are scanned
    // in shared memory, then each run is rewritten as prefixes
    const uint32_t per = (nb + blockDim.x - 1) / blockDim.x;
    const uint32_t x0 = min(nb, threadIdx.x * per), x1 = min(nb, x0 + per);
    uint32_t sum = 0;
    for (uint32_t x = x0; x < x1; x++) sum += row_ptr[x];
    part[threadIdx.x] = sum;
    __syncthreads();
    for (uint32_t off = 1; off < blockDim.x; off <<= 1) {  // inclusive Hillis-Steele scan
        const uint32_t v = threadIdx.x >= off ? part[threadIdx.x - off] : 0u;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t base = part[threadIdx.x] - sum;
    for (uint32_t x = x0; x < x1; x++) {
        const uint32_t cnt = row_ptr[x];
        row_ptr[x] = base;
        base += cnt;
    }
    if (threadIdx.x == blockDim.x - 1) row_ptr[nb] = part[blockDim.x - 1];
    __syncthreads();
    // cursors: M[t][b] := the first position of tile t's entries of bucket b
    for (uint32_t x = threadIdx.x; x < nb; x += blockDim.x) {
        const uint32_t s = x / B, b = x % B;
        uint32_t cur = row_ptr[x];
        for (uint32_t t = set_tile0[s]; t < set_tile0[s + 1]; t++) {
            const uint32_t v = M[(size_t)t * B + b];
            M[(size_t)t * B + b] = cur;
            cur += v;
        }
    }
}

__global__ void __launch_bounds__(kTiledThreads) msm_scatter_tiles_kernel(const uint32_t* __restrict__ codes,
                                                                          const uint32_t* __restrict__ set_base,
                                                                          const uint32_t* __restrict__ set_tile0,
                                                                          uint32_t te, MsmShape sh,
                                                                          const MsmInst* __restrict__ insts,
                                                                          const uint32_t* __restrict__ M,
                                                                          uint32_t* __restrict__ entries) {
    extern __shared__ uint32_t cursor[];
    const uint32_t t = blockIdx.x;
    const uint32_t s = set_of_tile(set_tile0, sh.sets, t);
    const uint32_t sb = set_base[s];
    const uint32_t e0 = sb + (t - set_tile0[s]) * te;
    const uint32_t e1 = min(e0 + te, set_base[s + 1]);
    const uint32_t* in = M + (size_t)t * sh.B;
    for (uint32_t b = threadIdx.x; b < sh.B; b += blockDim.x) cursor[b] = __ldcs(in + b);
    const uint32_t k = s / sh.Wr;
    const uint32_t nk = insts[k].n, stride = insts[k].stride;
    __syncthreads();
    for (uint32_t base = e0 + threadIdx.x; base < e1; base += blockDim.x * kSortBatch) {
        uint32_t code[kSortBatch];
#pragma unroll
        for (uint32_t q = 0; q < kSortBatch; q++) {  // the codes' last use: streamed, evict first
            const uint32_t e = base + q * blockDim.x;
            code[q] = e < e1 ? __ldcs(codes + e) : kNoCode;
        }
#pragma unroll
        for (uint32_t q = 0; q < kSortBatch; q++) {
            if (code[q] == kNoCode) continue;
            const uint32_t idx = base + q * blockDim.x - sb;
            // fixed-base: row w of the shifted bases; GLV: the phi(P) half for h = 1
            const uint32_t point = sh.shared ? (idx / nk) * stride + idx % nk
                                             : (sh.glv ? (idx >> 1) + (idx & 1) * stride : idx);
            const uint32_t pos = atomicAdd(cursor + (code[q] & 0x7fffffffu), 1u);
            entries[pos] = point | (code[q] & 0x80000000u);
        }
    }
}

// ---- 4. accumulation ------------------------------------------------------------
// Each stage below is a device body (one thread's unit, bucket or block; or one CTA's
// target / long bucket) called by its own kernel and by the persistent queue kernel
// (msm_queue_kernel). kL2: the body's point inputs were written earlier in the same launch
// (queue kernel), so they are read through L2 only.

// Emit the accumulated sum of `key` over entry range [e0, e1): final if the bucket
// lies inside the range, else into the unit's first (bucket began earlier) or last
// (bucket continues later) slot.
template <class P>
__device__ __forceinline__ void emit_piece(uint32_t key, const P& acc, uint32_t e0, uint32_t e1,
                                           const uint32_t* __restrict__ row_ptr, P* __restrict__ buckets,
                                           uint32_t* slot_keys, P* slot_pts, uint32_t unit) {
    if (row_ptr[key] < e0) {
        slot_keys[2 * unit] = key;
        xyzz_store(slot_pts + 2 * unit, acc);
    } else if (row_ptr[key + 1] > e1) {
        slot_keys[2 * unit + 1] = key;
        xyzz_store(slot_pts + 2 * unit + 1, acc);
    } else {
        xyzz_store(buckets + key, acc);
    }
}

// Bases of the instance that owns bucket `key` (sets of B buckets, Wr sets per instance).
template <class C>
__device__ __forceinline__ const typename C::A* key_bases(const MsmInst* __restrict__ insts, const MsmShape& sh,
                                                          uint32_t key) {
    return static_cast<const typename C::A*>(insts[sh.inst == 1 ? 0u : key / (sh.Wr * sh.B)].bases);
}

// The non-empty bucket holding CSR entry e: the largest k with row_ptr[k] <= e.
__device__ __forceinline__ uint32_t bucket_of(const uint32_t* __restrict__ row_ptr, uint32_t nbuckets, uint32_t e) {
    uint32_t lo = 0, hi = nbuckets;  // row_ptr[lo] <= e < row_ptr[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(row_ptr + mid) <= e) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Unit u: the CSR entries [u seg, (u + 1) seg) (M = total entries), bucket by bucket.
template <class C, bool kSkipInf>
__device__ __forceinline__ void acc_unit(const uint32_t* __restrict__ entries, uint32_t M,
                                         const uint32_t* __restrict__ row_ptr, const MsmInst* __restrict__ insts,
                                         const MsmShape& sh, uint32_t u, typename C::P* buckets, uint32_t* slot_keys,
                                         typename C::P* slot_pts, bool test_inf) {
    using P = typename C::P;
    using A = typename C::A;
    slot_keys[2 * u] = kNone;
    slot_keys[2 * u + 1] = kNone;
    const uint32_t e0 = u * sh.seg;
    if (e0 >= M) return;
    const uint32_t e1 = min(e0 + sh.seg, M);
    uint32_t cur = bucket_of(row_ptr, sh.sets * sh.B, e0);
    uint32_t end = row_ptr[cur + 1];  // > e0
    const A* bases = key_bases<C>(insts, sh, cur);
    P acc = xyzz_inf<typename C::T>();
    for (uint32_t e = e0; e < e1; e++) {
        if (e == end) {  // bucket cur ends here: emit it, move to the next non-empty bucket
            emit_piece(cur, acc, e0, e1, row_ptr, buckets, slot_keys, slot_pts, u);
            do {
                cur++;
                end = row_ptr[cur + 1];
            } while (end == e);
            bases = key_bases<C>(insts, sh, cur);
            acc = xyzz_inf<typename C::T>();
        }
        const uint32_t ent = entries[e];
        A p = affine_load(bases + (ent & 0x7fffffffu));
        if constexpr (kSkipInf)
            if (test_inf && affine_is_zero_bits(p)) continue;  // an infinity base adds nothing
        if (ent >> 31) p.y = c_neg(p.y);
        acc = xyzz_madd(acc, p.x, p.y);
    }
    emit_piece(cur, acc, e0, e1, row_ptr, buckets, slot_keys, slot_pts, u);
}

template <class C, bool kSkipInf>
__global__ void __launch_bounds__(128, C::kAccMinBlocks) msm_accumulate_kernel(const uint32_t* __restrict__ entries,
                                                             const uint32_t* __restrict__ d_total,
                                                             const uint32_t* __restrict__ row_ptr,
                                                             const MsmInst* __restrict__ insts, MsmShape sh,
                                                             uint32_t units, typename C::P* __restrict__ buckets,
                                                             uint32_t* __restrict__ slot_keys,
                                                             typename C::P* __restrict__ slot_pts,
                                                             const uint32_t* __restrict__ inf_flag) {
    const uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= units) return;
    // kSkipInf: the points may hold infinity; a flag (when given) says whether they do
    const bool test_inf = kSkipInf && (inf_flag == nullptr || *inf_flag != 0);
    acc_unit<C, kSkipInf>(entries, *d_total, row_ptr, insts, sh, u, buckets, slot_keys, slot_pts, test_inf);
}

// Round r >= 2: unit u merges the slots of units [u*group, (u+1)*group) of the previous
// round, covering entries [u * span, (u+1) * span) (span = kSegment times the product of
// the group sizes so far). The first merge round uses pairs: most straddling buckets
// cross exactly one segment boundary, so that round carries nearly all the work.
template <class C, bool kL2>
__device__ __forceinline__ void merge_unit(const uint32_t* in_keys, const typename C::P* in_pts, uint32_t in_units,
                                           uint32_t group, uint64_t M, const uint32_t* __restrict__ row_ptr,
                                           uint64_t span, uint32_t u, typename C::P* buckets, uint32_t* slot_keys,
                                           typename C::P* slot_pts) {
    slot_keys[2 * u] = kNone;
    slot_keys[2 * u + 1] = kNone;
    const uint64_t e0l = (uint64_t)u * span;
    if (e0l >= M) return;
    const uint32_t e0 = (uint32_t)e0l;
    const uint32_t e1 = (uint32_t)min(e0l + span, M);
    const uint32_t s0 = 2 * u * group;
    const uint32_t s1 = min(2 * (u + 1) * group, 2 * in_units);
    uint32_t cur = kNone;
    typename C::P acc = xyzz_inf<typename C::T>();
    for (uint32_t s = s0; s < s1; s++) {
        const uint32_t k = kL2 ? __ldcg(in_keys + s) : in_keys[s];
        if (k == kNone) continue;
        if (k != cur) {
            if (cur != kNone) emit_piece(cur, acc, e0, e1, row_ptr, buckets, slot_keys, slot_pts, u);
            cur = k;
            acc = xyzz_inf<typename C::T>();
        }
        acc = xyzz_add(acc, xyzz_get<kL2>(in_pts + s));
    }
    if (cur != kNone) emit_piece(cur, acc, e0, e1, row_ptr, buckets, slot_keys, slot_pts, u);
}

template <class C>
__global__ void __launch_bounds__(128, C::kRedMinBlocks) msm_merge_kernel(const uint32_t* __restrict__ in_keys,
                                                        const typename C::P* __restrict__ in_pts, uint32_t in_units,
                                                        uint32_t group, const uint32_t* __restrict__ d_total,
                                                        const uint32_t* __restrict__ row_ptr, uint64_t span,
                                                        uint32_t units, typename C::P* __restrict__ buckets,
                                                        uint32_t* __restrict__ slot_keys,
                                                        typename C::P* __restrict__ slot_pts) {
    const uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= units) return;
    merge_unit<C, false>(in_keys, in_pts, in_units, group, *d_total, row_ptr, span, u, buckets, slot_keys, slot_pts);
}

// Fixup instead of merge rounds (when buckets are short): a bucket k whose entries
// [row_ptr[k], row_ptr[k+1]) span units u0 < u1 left its pieces in slot 1 of unit u0 (the
// bucket continues past the segment) and in slot 0 of every unit u0 < u <= u1 (the bucket
// began before the segment). One thread per bucket adds up to sh.fixmax + 1 pieces; longer
// buckets are listed for msm_fixup_long_kernel (a CTA each).
#ifndef ZK_FIXUP_DENSITY
// measured on GB300: 2^20 plain (32 entries per bucket) fixup 0.32 vs rounds 0.48 ms; 2^20 GLV
// (64) fixup 0.27 vs rounds 0.48 ms; 2^22 GLV (256) rounds 1.0 vs fixup 6.8 ms
#define ZK_FIXUP_DENSITY 96
#endif
static constexpr uint64_t kFixupDensity = ZK_FIXUP_DENSITY;  // CSR entries per bucket up to which the fixup is used

// Buckets of at least kHugePieces pieces (a hot digit: 10% of the scalars equal to 1 put
// ~3300 pieces into one bucket at 2^20) are summed in chunks of about kChunkPieces pieces by
// many CTAs, at most kMaxChunks per bucket, the last CTA to finish one adding its chunk sums
// (one CTA for the whole bucket took 0.5 ms). Their list, count and per-bucket chunk
// counters share the long list's count block: counts[0] long buckets, counts[1] huge
// buckets, counts[2 .. 2 + hcap) chunks done per huge bucket, counts[2 + hcap ..] the huge
// buckets' keys; hcap bounds the huge buckets (units / kHugePieces + 2).
static constexpr uint32_t kHugePieces = 2048;
static constexpr uint32_t kChunkPieces = 256;
static constexpr uint32_t kMaxChunks = 64;

__host__ __device__ inline uint32_t huge_cap(uint32_t units) { return units / kHugePieces + 2; }

template <class C, bool kL2>
__device__ __forceinline__ void fixup_bucket(const uint32_t* __restrict__ row_ptr, uint32_t seg, uint32_t fixmax,
                                             const typename C::P* slot_pts, typename C::P* buckets,
                                             uint32_t* long_list, uint32_t* long_count, uint32_t hcap, uint32_t k) {
    const uint32_t b0 = row_ptr[k], b1 = row_ptr[k + 1];
    if (b1 == b0) return;
    const uint32_t u0 = b0 / seg, u1 = (b1 - 1) / seg;
    if (u0 == u1) return;  // final already (written by the accumulation)
    if (u1 - u0 >= kHugePieces) {
        long_count[2 + hcap + atomicAdd(long_count + 1, 1u)] = k;
        return;
    }
    if (u1 - u0 > fixmax) {
        long_list[atomicAdd(long_count, 1u)] = k;
        return;
    }
    typename C::P acc = xyzz_get<kL2>(slot_pts + 2 * (size_t)u0 + 1);
    for (uint32_t u = u0 + 1; u <= u1; u++) acc = xyzz_add(acc, xyzz_get<kL2>(slot_pts + 2 * (size_t)u));
    xyzz_store(buckets + k, acc);
}

template <class C>
__global__ void __launch_bounds__(128, C::kRedMinBlocks) msm_fixup_kernel(const uint32_t* __restrict__ row_ptr, uint32_t nbuckets,
                                                        uint32_t seg, uint32_t fixmax,
                                                        const typename C::P* __restrict__ slot_pts,
                                                        typename C::P* __restrict__ buckets,
                                                        uint32_t* __restrict__ long_list,
                                                        uint32_t* __restrict__ long_count, uint32_t hcap) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nbuckets) return;
    fixup_bucket<C, false>(row_ptr, seg, fixmax, slot_pts, buckets, long_list, long_count, hcap, k);
}

// The sum of the pieces of units [ua, ub] of a bucket whose first unit is u0 (its piece is
// slot 1, the others' slot 0), or of `n` consecutive points at `pts` when pts is given, by
// the CTA: strided partial sums, then a shared-memory tree over `red` (blockDim points)
// spanning the next power of two of the terms. The result is valid in thread 0.
template <class C, bool kL2>
__device__ __forceinline__ typename C::P cta_sum(const typename C::P* slot_pts, uint32_t u0, uint32_t ua, uint32_t ub,
                                                 const typename C::P* pts, uint32_t n, typename C::P* red) {
    using P = typename C::P;
    const uint32_t terms = pts != nullptr ? n : ub - ua + 1;
    uint32_t width = 1;
    while (width < terms && width < blockDim.x) width <<= 1;
    P acc = xyzz_inf<typename C::T>();
    if (threadIdx.x < width)
        for (uint32_t t = threadIdx.x; t < terms; t += width) {
            const P* src = pts != nullptr ? pts + t : slot_pts + 2 * (size_t)(ua + t) + (ua + t == u0 ? 1 : 0);
            acc = xyzz_add(acc, pts != nullptr ? xyzz_ldcg(src) : xyzz_get<kL2>(src));
        }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (uint32_t off = width / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) red[threadIdx.x] = xyzz_add(red[threadIdx.x], red[threadIdx.x + off]);
        __syncthreads();
    }
    acc = red[0];
    __syncthreads();  // red free again
    return acc;
}

// The chunks of the huge buckets (units item0, item0 + stride, ... of the CTAs: unit
// h kMaxChunks + ch is chunk ch of huge bucket h). A chunk sum goes to chunk_pts
// (h kMaxChunks + ch); the CTA whose chunk completes a bucket (counted after a fence) adds
// the bucket's chunk sums, read through L2. Nothing waits on another CTA. Not inlined: the
// long buckets' code around its call stays as it was without it (inlined, the long-bucket
// kernel ran 2^12 single MSMs 8 us slower).
template <class C, bool kL2>
__device__ __noinline__ void fixup_huge_units(const uint32_t* __restrict__ row_ptr, uint32_t seg,
                                              const typename C::P* slot_pts, typename C::P* buckets,
                                              uint32_t* long_count, uint32_t hcap, uint32_t huge,
                                              typename C::P* chunk_pts, typename C::P* red, uint32_t* s_last,
                                              uint32_t item0, uint32_t stride) {
    using P = typename C::P;
    for (uint32_t unit = item0; unit < huge * kMaxChunks; unit += stride) {
        const uint32_t h = unit / kMaxChunks, ch = unit % kMaxChunks;
        const uint32_t k = kL2 ? __ldcg(long_count + 2 + hcap + h) : long_count[2 + hcap + h];
        const uint32_t u0 = row_ptr[k] / seg, u1 = (row_ptr[k + 1] - 1) / seg;
        const uint32_t pieces = u1 - u0 + 1;
        const uint32_t nch = min(kMaxChunks, (pieces + kChunkPieces - 1) / kChunkPieces);
        if (ch >= nch) continue;  // the same for the whole CTA
        const uint32_t per = (pieces + nch - 1) / nch;
        const uint32_t ua = u0 + ch * per, ub = min(u1, ua + per - 1);
        P r = cta_sum<C, kL2>(slot_pts, u0, ua, ub, nullptr, 0, red);
        if (threadIdx.x == 0) {
            xyzz_store(chunk_pts + (size_t)h * kMaxChunks + ch, r);
            __threadfence();  // the chunk sum is visible before it is counted
            *s_last = atomicAdd(long_count + 2 + h, 1u) == nch - 1 ? 1u : 0u;
        }
        __syncthreads();
        if (*s_last) {  // every chunk of bucket k is done: add their sums
            __threadfence();
            r = cta_sum<C, kL2>(nullptr, 0, 0, 0, chunk_pts + (size_t)h * kMaxChunks, nch, red);
            if (threadIdx.x == 0) xyzz_store(buckets + k, r);
        }
        __syncthreads();  // s_last read by every thread before it is written again
    }
}

// The huge buckets' chunks, then one CTA per listed long bucket: strided partial sums, then a
// shared-memory tree over `red` (blockDim points). Long bucket i goes to CTA
// (i + huge kMaxChunks) mod stride, past the CTAs of the chunk units, so that the two kinds
// of work run side by side. (One warp per long bucket with a shuffle tree measured slower:
// 2^14 single MSM 0.127 against 0.059 ms in this kernel; the chunks in a kernel of their own
// before this one serialised the two, witness-like 2^20 0.25 against 0.14 ms.)
template <class C, bool kL2>
__device__ __forceinline__ void fixup_long_cta(const uint32_t* __restrict__ row_ptr, uint32_t seg,
                                               const typename C::P* slot_pts, typename C::P* buckets,
                                               const uint32_t* long_list, uint32_t* long_count, uint32_t hcap,
                                               typename C::P* chunk_pts, typename C::P* red, uint32_t item0,
                                               uint32_t stride) {
    using P = typename C::P;
    __shared__ uint32_t s_last;
    const uint32_t huge = kL2 ? __ldcg(long_count + 1) : long_count[1];
    if (huge != 0)
        fixup_huge_units<C, kL2>(row_ptr, seg, slot_pts, buckets, long_count, hcap, huge, chunk_pts, red, &s_last,
                                 item0, stride);
    const uint32_t count = kL2 ? __ldcg(long_count) : *long_count;
    const uint32_t shift = (uint32_t)(((uint64_t)huge * kMaxChunks) % stride);
    for (uint32_t item = (item0 + stride - shift) % stride; item < count; item += stride) {
        const uint32_t k = kL2 ? __ldcg(long_list + item) : long_list[item];
        const uint32_t u0 = row_ptr[k] / seg, u1 = (row_ptr[k + 1] - 1) / seg;
        // the tree spans the next power of two of the pieces (at most the CTA): a bucket of 16
        // segments takes 4 levels of serial additions, not log2(blockDim)
        uint32_t width = 1;
        while (width < u1 - u0 + 1 && width < blockDim.x) width <<= 1;
        P acc = xyzz_inf<typename C::T>();
        if (threadIdx.x < width)
            for (uint32_t u = u0 + threadIdx.x; u <= u1; u += width)
                acc = xyzz_add(acc, xyzz_get<kL2>(slot_pts + 2 * (size_t)u + (u == u0 ? 1 : 0)));
        red[threadIdx.x] = acc;
        __syncthreads();
        for (uint32_t off = width / 2; off > 0; off >>= 1) {
            if (threadIdx.x < off) red[threadIdx.x] = xyzz_add(red[threadIdx.x], red[threadIdx.x + off]);
            __syncthreads();
        }
        if (threadIdx.x == 0) xyzz_store(buckets + k, red[0]);
        __syncthreads();
    }
}

template <class C>
__global__ void __launch_bounds__(C::kFixupLongThreads, C::kFixupLongMinBlocks) msm_fixup_long_kernel(const uint32_t* __restrict__ row_ptr,
                                                                           uint32_t seg,
                                                                           const typename C::P* __restrict__ slot_pts,
                                                                           typename C::P* __restrict__ buckets,
                                                                           const uint32_t* __restrict__ long_list,
                                                                           uint32_t* __restrict__ long_count,
                                                                           uint32_t hcap,
                                                                           typename C::P* __restrict__ chunk_pts) {
    __shared__ typename C::P red[C::kFixupLongThreads];
    fixup_long_cta<C, false>(row_ptr, seg, slot_pts, buckets, long_list, long_count, hcap, chunk_pts, red, blockIdx.x,
                             gridDim.x);
}

// ---- 5. window reduction ----------------------------------------------------------------
// For points X_1..X_N with weights, WS(X) = sum_b b X_b. Blocks of g: X_{(j-1)g+u}, u = 1..g:
// WS(X) = sum_j E_j + g WS(Y), Y_j = block sum, E_j = -(s_1 + ... + s_{g-1}) with s_u the
// prefix sums inside the block (because sum_u u X_u = g Y_j - sum_{u<g} s_u). Applied
// twice (buckets -> Y1, E1 -> Y2, E2, F2 = block sums of E1), then WS(Y2) by plain sums:
// WS(Y2) = sum_j Y2_j + sum_k 2^k M_k, M_k = sum of Y2_j with bit k of (j - 1) set.
// Level 1: block j of window w holds buckets b = j*g + 1 .. j*g + g (stored at index b - 1).
template <class C, bool kL2>
__device__ __forceinline__ void blocks_thread(const typename C::P* buckets, const MsmShape& sh, typename C::P* Y,
                                              typename C::P* E, uint32_t t) {
    using P = typename C::P;
    const P* b = buckets + (size_t)t * sh.g;
    P s = xyzz_inf<typename C::T>();
    P e = xyzz_inf<typename C::T>();
    for (uint32_t u = 0; u < sh.g; u++) {
        s = xyzz_add(s, xyzz_get<kL2>(b + u));
        if (u + 1 < sh.g) e = xyzz_add(e, s);
    }
    xyzz_store(Y + t, s);
    xyzz_store(E + t, xyzz_neg(e));
}

template <class C>
__global__ void __launch_bounds__(128) msm_bucket_blocks_kernel(const typename C::P* __restrict__ buckets,
                                                                MsmShape sh, typename C::P* __restrict__ Y,
                                                                typename C::P* __restrict__ E) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= sh.sets * sh.G) return;
    blocks_thread<C, false>(buckets, sh, Y, E, t);
}

// Level 2 over (Y1, E1): Y2, E2 as above on Y1, and F2 = plain block sums of E1.
template <class C, bool kL2>
__device__ __forceinline__ void blocks2_thread(const typename C::P* Y1, const typename C::P* E1, const MsmShape& sh,
                                               typename C::P* Y2, typename C::P* E2, typename C::P* F2, uint32_t t) {
    using P = typename C::P;
    const size_t base = (size_t)t * sh.g2;
    P s = xyzz_inf<typename C::T>();
    P e = xyzz_inf<typename C::T>();
    P f = xyzz_inf<typename C::T>();
    for (uint32_t u = 0; u < sh.g2; u++) {
        s = xyzz_add(s, xyzz_get<kL2>(Y1 + base + u));
        if (u + 1 < sh.g2) e = xyzz_add(e, s);
        f = xyzz_add(f, xyzz_get<kL2>(E1 + base + u));
    }
    xyzz_store(Y2 + t, s);
    xyzz_store(E2 + t, xyzz_neg(e));
    xyzz_store(F2 + t, f);
}

template <class C>
__global__ void __launch_bounds__(128) msm_bucket_blocks2_kernel(const typename C::P* __restrict__ Y1,
                                                                 const typename C::P* __restrict__ E1, MsmShape sh,
                                                                 typename C::P* __restrict__ Y2,
                                                                 typename C::P* __restrict__ E2,
                                                                 typename C::P* __restrict__ F2) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= sh.sets * sh.G2) return;
    blocks2_thread<C, false>(Y1, E1, sh, Y2, E2, F2, t);
}

// ---- 6. plain sums per (window, target) ---------------------------------------------
// targets 0 .. plain-1: full sums of P0, P1 (, P2) over G2 entries per window;
// target plain + k: sum of Ylast_j over j with bit k set.
// Each target is split over `parts` CTAs (a slice of its terms each; large single bucket
// sets of the fixed-base mode have G2 up to 2^14); out[(w * targets + tg) * parts + part].
// `blk` is the CTA's index in that order; `red` holds blockDim points.
template <class C, bool kL2>
__device__ __forceinline__ void targets_cta(const typename C::P* P0, const typename C::P* P1, const typename C::P* P2,
                                            const typename C::P* Ylast, const MsmShape& sh, uint32_t parts,
                                            typename C::P* out, typename C::P* red, uint32_t blk) {
    using P = typename C::P;
    const uint32_t part = blk % parts;
    const uint32_t wt = blk / parts;
    const uint32_t w = wt / sh.targets;
    const uint32_t tg = wt % sh.targets;
    const bool bits = tg >= sh.plain;
    const P* src = bits ? Ylast : (tg == 0 ? P0 : (tg == 1 ? P1 : P2));
    src += (size_t)w * sh.G2;
    const uint32_t count = bits ? sh.G2 / 2 : sh.G2;
    const uint32_t per = (count + parts - 1) / parts;
    const uint32_t t0 = part * per, t1 = min(count, t0 + per);
    const uint32_t k = bits ? tg - sh.plain : 0;
    // the tree spans the next power of two of this slice's terms (at most the CTA)
    const uint32_t terms = t1 > t0 ? t1 - t0 : 0;
    uint32_t width = 1;
    while (width < terms && width < blockDim.x) width <<= 1;
    P acc = xyzz_inf<typename C::T>();
    if (threadIdx.x < width)
        for (uint32_t t = t0 + threadIdx.x; t < t1; t += width) {
            uint32_t j = t;
            if (bits) j = ((t >> k) << (k + 1)) | (1u << k) | (t & ((1u << k) - 1));
            acc = xyzz_add(acc, xyzz_get<kL2>(src + j));
        }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (uint32_t off = width / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) red[threadIdx.x] = xyzz_add(red[threadIdx.x], red[threadIdx.x + off]);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blk] = red[0];
}

template <class C>
__global__ void __launch_bounds__(C::kTargetThreads) msm_targets_kernel(const typename C::P* __restrict__ P0,
                                                                        const typename C::P* __restrict__ P1,
                                                                        const typename C::P* __restrict__ P2,
                                                                        const typename C::P* __restrict__ Ylast,
                                                                        MsmShape sh, uint32_t parts,
                                                                        typename C::P* __restrict__ out) {
    __shared__ typename C::P red[C::kTargetThreads];
    targets_cta<C, false>(P0, P1, P2, Ylast, sh, parts, out, red, blockIdx.x);
}

// The parts of each target summed: one CTA of kMergeThreads per (window, target).
static constexpr uint32_t kMergeThreads = 32;

template <class C, bool kL2>
__device__ __forceinline__ void targets_merge_cta(const typename C::P* in, uint32_t parts, typename C::P* out,
                                                  typename C::P* red, uint32_t blk) {
    using P = typename C::P;
    const P* src = in + (size_t)blk * parts;
    uint32_t width = 1;
    while (width < parts && width < blockDim.x) width <<= 1;
    P acc = xyzz_inf<typename C::T>();
    if (threadIdx.x < width)
        for (uint32_t t = threadIdx.x; t < parts; t += width) acc = xyzz_add(acc, xyzz_get<kL2>(src + t));
    red[threadIdx.x] = acc;
    __syncthreads();
    for (uint32_t off = width / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) red[threadIdx.x] = xyzz_add(red[threadIdx.x], red[threadIdx.x + off]);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blk] = red[0];
}

template <class C>
__global__ void __launch_bounds__(kMergeThreads) msm_targets_merge_kernel(const typename C::P* __restrict__ in,
                                                                          uint32_t parts,
                                                                          typename C::P* __restrict__ out) {
    __shared__ typename C::P red[kMergeThreads];
    targets_merge_cta<C, false>(in, parts, out, red, blockIdx.x);
}

// ---- persistent form of the post-sort stages (work queue) ----------------------------------
// All pipelines of a batch, after their sorts, in ONE launch: the queue lists (pipeline,
// stage) entries, each owning one item per CTA-sized piece of the stage -- 128 accumulation
// units (entry ranges of one instance's window sets), 128 merge units, 128 buckets of the
// fixup, a share of the long-bucket list, 128 level-1 / level-2 blocks, one (set, target,
// part) or one (set, target) merge. Entries go stage by stage (largest pipelines first within
// a stage); an item waits until its pipeline's previous stage has published all its items.
// The same ticket discipline as the NTT queue keeps it deadlock-free for any number of
// resident CTAs (the earliest unfinished item never waits), and every wait is bounded.
enum : uint32_t { kQAcc = 0, kQMerge, kQFix, kQFixLong, kQBlk1, kQBlk2, kQTgt, kQTMerge };

template <class C>
struct MsmQPipe {
    using P = typename C::P;
    const uint32_t* entries;
    const uint32_t* row_ptr;
    const uint32_t* d_total;
    const MsmInst* insts;
    const uint32_t* inf_flag;
    P* buckets;
    uint32_t* slot_keys[2];
    P* slot_pts[2];
    uint32_t* long_list;
    uint32_t* long_count;  // the count block (see fixup_bucket), hcap huge buckets at most
    P *Yb, *Eb, *Y2, *E2, *F2, *tgt_out, *tgt;
    MsmShape sh;
    uint32_t units, nbuckets, parts, skip_inf, hcap;
};

struct MsmQEntry {
    uint32_t pipe, stage, first, items;
    int32_t dep;     // entry of the pipeline's previous stage, -1 for the accumulation
    uint32_t need;   // its items
    uint32_t in_units, out_units, group, src;  // merge rounds: units in / out, group, slots read (0: a, 1: b)
    uint64_t span;
};

static constexpr uint32_t kMsmQThreads = 128;

template <class C>
__global__ void __launch_bounds__(kMsmQThreads, 2) msm_queue_kernel(const MsmQPipe<C>* __restrict__ pipes,
                                                                   const MsmQEntry* __restrict__ entries,
                                                                   uint32_t nentries, uint32_t nitems,
                                                                   uint32_t* state,
                                                                   const uint64_t* __restrict__ limit,
                                                                   uint32_t* sticky) {
    using P = typename C::P;
    __shared__ P red[kMsmQThreads];
    __shared__ MsmQEntry sE;
    __shared__ MsmQPipe<C> sQ;
    __shared__ uint32_t s_next, s_item, s_entry, s_tile, s_stop;
    volatile uint32_t* vstate = state;
    if (threadIdx.x == 0) s_next = queue_ticket(state, nitems);
    __syncthreads();
    uint32_t finished = kNone;  // warp 1, lane 0: the entry of the item this CTA just finished
    for (;;) {
        if (threadIdx.x < 32) {  // warp 0: find the next item's entry, copy it and its pipeline, wait
            const uint32_t item = s_next;
            uint32_t e = 0;
            if (threadIdx.x == 0 && item < nitems) {
                uint32_t lo = 0, hi = nentries;  // the entry holding `item`: largest e with first <= item
                while (hi - lo > 1) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (entries[mid].first <= item) lo = mid;
                    else hi = mid;
                }
                e = lo;
            }
            e = __shfl_sync(0xffffffffu, e, 0);
            if (item < nitems) {
                constexpr uint32_t kEw = sizeof(MsmQEntry) / 4, kPw = sizeof(MsmQPipe<C>) / 4;
                static_assert(sizeof(MsmQEntry) % 4 == 0 && sizeof(MsmQPipe<C>) % 4 == 0, "word copies");
                for (uint32_t w = threadIdx.x; w < kEw; w += 32)
                    reinterpret_cast<uint32_t*>(&sE)[w] = reinterpret_cast<const uint32_t*>(entries + e)[w];
                __syncwarp();
                const uint32_t pq = sE.pipe;
                for (uint32_t w = threadIdx.x; w < kPw; w += 32)
                    reinterpret_cast<uint32_t*>(&sQ)[w] = reinterpret_cast<const uint32_t*>(pipes + pq)[w];
            }
            __syncwarp();
            if (threadIdx.x == 0) {
                s_item = item;
                s_entry = e;
                s_stop = 0;
                if (item < nitems) {
                    s_tile = item - sE.first;
                    if (sE.dep >= 0) {
                        const uint32_t dep = (uint32_t)sE.dep, need = sE.need;
                        const uint64_t t0 = global_ns();
                        uint32_t ns = 32;
                        while (vstate[kQueueDone + dep] < need) {
                            // bounded: give up when the limit passes or another CTA gave up
                            if (vstate[kQueueStatus] != 0 || global_ns() - t0 > *limit) {
                                if (atomicCAS(state + kQueueStatus, 0u, e + 1u) == 0u) atomicCAS(sticky, 0u, e + 1u);
                                s_stop = 1;
                                break;
                            }
                            __nanosleep(ns);
                            if (ns < 1024) ns <<= 1;
                        }
                        __threadfence();  // acquire: the previous stage's outputs before our loads
                    }
                }
            }
        } else if (threadIdx.x == 32 && finished != kNone) {
            // warp 1 publishes the finished item while warp 0 looks up the next one
            __threadfence();  // release: the item's outputs (ordered by the barrier) before the counter
            atomicAdd(state + kQueueDone + finished, 1u);
        }
        __syncthreads();
        if (s_item >= nitems || s_stop) return;
        if (threadIdx.x == 32) finished = s_entry;
        uint32_t nxt = 0;
        if (threadIdx.x == 0) nxt = queue_ticket(state, nitems);
        const MsmQPipe<C>& q = sQ;
        const uint32_t b = s_tile;
        const uint32_t i = b * kMsmQThreads + threadIdx.x;  // the thread's unit / bucket / block
        switch (sE.stage) {
            case kQAcc:
                if (i < q.units) {
                    const bool test_inf = q.skip_inf && (q.inf_flag == nullptr || *q.inf_flag != 0);
                    acc_unit<C, true>(q.entries, *q.d_total, q.row_ptr, q.insts, q.sh, i, q.buckets, q.slot_keys[0],
                                      q.slot_pts[0], test_inf);
                }
                break;
            case kQMerge:
                if (i < sE.out_units)
                    merge_unit<C, true>(q.slot_keys[sE.src], q.slot_pts[sE.src], sE.in_units, sE.group, *q.d_total,
                                        q.row_ptr, sE.span, i, q.buckets, q.slot_keys[1 - sE.src],
                                        q.slot_pts[1 - sE.src]);
                break;
            case kQFix:
                if (i < q.nbuckets)
                    fixup_bucket<C, true>(q.row_ptr, q.sh.seg, q.sh.fixmax, q.slot_pts[0], q.buckets, q.long_list,
                                          q.long_count, q.hcap, i);
                break;
            case kQFixLong:
                fixup_long_cta<C, true>(q.row_ptr, q.sh.seg, q.slot_pts[0], q.buckets, q.long_list, q.long_count,
                                        q.hcap, q.slot_pts[1], red, b, sE.items);
                break;
            case kQBlk1:
                if (i < q.sh.sets * q.sh.G) blocks_thread<C, true>(q.buckets, q.sh, q.Yb, q.Eb, i);
                break;
            case kQBlk2:
                if (i < q.sh.sets * q.sh.G2) blocks2_thread<C, true>(q.Yb, q.Eb, q.sh, q.Y2, q.E2, q.F2, i);
                break;
            case kQTgt:
                if (q.sh.g2 > 1) targets_cta<C, true>(q.F2, q.E2, q.Y2, q.Y2, q.sh, q.parts, q.tgt_out, red, b);
                else targets_cta<C, true>(q.Eb, q.Yb, q.Yb, q.Yb, q.sh, q.parts, q.tgt_out, red, b);
                break;
            case kQTMerge:
                targets_merge_cta<C, true>(q.tgt_out, q.parts, q.tgt, red, b);
                break;
        }
        __syncthreads();  // every store of the item issued; sE, sQ and red free again
        if (threadIdx.x == 0) s_next = nxt;
    }
}

// CTAs per target: one up to 8 terms per thread; the large single bucket sets of the
// fixed-base mode (G2 up to 2^14) in slices of about 8 terms per thread, at most 64.
#ifndef ZK_TARGET_SLICE
#define ZK_TARGET_SLICE 8
#endif
template <class C>
static uint32_t target_parts(const MsmShape& sh) {
    const uint32_t slice = (uint32_t)ZK_TARGET_SLICE * (uint32_t)C::kTargetThreads;
    return std::max<uint32_t>(1, std::min<uint32_t>(64, (sh.G2 + slice - 1) / slice));
}

// ---- fixed-base precomputation ----------------------------------------------------------
// Row j of the output holds [2^(c j)] P_i in affine Montgomery form (row 0 = P_i). Per point
// the W - 1 shifted points are built by c doublings each in XYZZ, then normalised with one
// field inversion (Montgomery's trick over the point's own rows). Infinity stays (0, 0);
// no shifted point of a finite point is infinity (2^(c j) is invertible mod r).
template <class F>
__device__ fe fe_inverse_fermat(const fe& a) {
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

// Inverses of the coordinate field (the Montgomery trick's one inversion per point).
__device__ __forceinline__ fe c_inv(const fe& a) { return fe_inverse_fermat<FqP>(a); }
// (a0 + a1 u)^-1 = (a0 - a1 u) / (a0^2 + a1^2) in Fq2 = Fq[u] / (u^2 + 1)
__device__ __forceinline__ fq2 c_inv(const fq2& a) {
    const fe inv = fe_inverse_fermat<FqP>(fe_add<FqP>(fe_sqr<FqP>(a.c0), fe_sqr<FqP>(a.c1)));
    return {fe_mul<FqP>(a.c0, inv), fe_neg<FqP>(fe_mul<FqP>(a.c1, inv))};
}

template <class C>
__global__ void __launch_bounds__(128) msm_shift_bases_kernel(const typename C::A* __restrict__ bases, uint32_t n,
                                                              uint32_t c, uint32_t W, typename C::A* __restrict__ out,
                                                              typename C::P* __restrict__ tmp,
                                                              typename C::T* __restrict__ pref) {
    using A = typename C::A;
    using P = typename C::P;
    using T = typename C::T;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const A p = affine_load(bases + i);
    c_store(&out[i].x, p.x);
    c_store(&out[i].y, p.y);
    if (affine_is_inf(p)) {
        T zero;
        c_set_zero(zero);
        for (uint32_t j = 1; j < W; j++) {
            c_store(&out[(size_t)j * n + i].x, zero);
            c_store(&out[(size_t)j * n + i].y, zero);
        }
        return;
    }
    P q;
    q.X = p.x;
    q.Y = p.y;
    c_set_one(q.ZZ);
    c_set_one(q.ZZZ);
    T run;
    c_set_one(run);
    for (uint32_t j = 1; j < W; j++) {
        for (uint32_t d = 0; d < c; d++) q = xyzz_dbl(q);
        xyzz_store(tmp + (size_t)j * n + i, q);
        c_store(pref + (size_t)j * n + i, run);
        run = c_mul(run, c_mul(q.ZZ, q.ZZZ));
    }
    T inv = c_inv(run);
    for (uint32_t j = W - 1; j >= 1; j--) {
        const P t = xyzz_load(tmp + (size_t)j * n + i);
        const T zz_zzz = c_mul(t.ZZ, t.ZZZ);
        const T I = c_mul(inv, c_load(pref + (size_t)j * n + i));
        inv = c_mul(inv, zz_zzz);
        c_store(&out[(size_t)j * n + i].x, c_mul(t.X, c_mul(t.ZZZ, I)));
        c_store(&out[(size_t)j * n + i].y, c_mul(t.Y, c_mul(t.ZZ, I)));
    }
}

template <class C>
static int shift_bases_t(Ctx* c, const typename C::A* bases, size_t n, uint32_t window_bits, typename C::A** out,
                         uint32_t* windows) {
    using A = typename C::A;
    ZK_CHECK_ARG(window_bits >= 4 && window_bits <= 20, "fixed-base window_bits must be 4..20");
    ZK_CHECK_ARG(n > 0 && n < (1ull << 31), "fixed-base precomputation needs 0 < n < 2^31");
    const MsmShape sh = make_shape(window_bits);
    const uint64_t nrows = sh.W;
    ZK_CHECK_ARG(nrows * n < (1ull << 31), "fixed-base rows exceed 31-bit entry indices");
    A* rows = nullptr;
    typename C::P* tmp = nullptr;
    typename C::T* pref = nullptr;
    int rc = scratch_alloc(c, (size_t)nrows * n * sizeof(A), reinterpret_cast<void**>(&rows));
    if (rc != ZK_OK) return rc;
    if ((rc = scratch_alloc(c, (size_t)sh.W * n * sizeof(typename C::P), reinterpret_cast<void**>(&tmp))) != ZK_OK ||
        (rc = scratch_alloc(c, (size_t)sh.W * n * sizeof(typename C::T), reinterpret_cast<void**>(&pref))) != ZK_OK) {
        scratch_free(c, rows);
        scratch_free(c, tmp);
        return rc;
    }
    ZK_LAUNCH(c, "msm_shift_bases", msm_shift_bases_kernel<C>, (unsigned)((n + 127) / 128), 128, 0, bases,
              (uint32_t)n, window_bits, sh.W, rows, tmp, pref);
    ZK_TRY_CUDA(cudaGetLastError());
    scratch_free(c, tmp);
    scratch_free(c, pref);
    *out = rows;
    *windows = sh.W;
    return ZK_OK;
}

int shift_bases(Ctx* c, const affine_t* bases, size_t n, uint32_t window_bits, affine_t** out, uint32_t* windows) {
    return shift_bases_t<CurveG1>(c, bases, n, window_bits, out, windows);
}

int shift_bases_g2(Ctx* c, const affine2_t* bases, size_t n, uint32_t window_bits, affine2_t** out,
                   uint32_t* windows) {
    return shift_bases_t<CurveG2>(c, bases, n, window_bits, out, windows);
}

// ---- host ---------------------------------------------------------------------------
template <class C>
static zkh::XyzzT<typename HostOf<C>::T> to_host(const typename C::P& d) {
    static_assert(sizeof(typename C::P) == sizeof(zkh::XyzzT<typename HostOf<C>::T>), "layout");
    zkh::XyzzT<typename HostOf<C>::T> h;
    std::memcpy(&h, &d, sizeof(h));
    h.X = zkh::cnorm(h.X);  // device Fq values are lazy in [0, 2q)
    h.Y = zkh::cnorm(h.Y);
    h.ZZ = zkh::cnorm(h.ZZ);
    h.ZZZ = zkh::cnorm(h.ZZZ);
    return h;
}

template <class H>
static zkh::XyzzT<H> host_dbl_n(zkh::XyzzT<H> p, uint32_t times) {
    for (uint32_t i = 0; i < times; i++) p = zkh::xyzz_dbl(p);
    return p;
}

uint32_t msm_window_for(const Ctx* c, size_t n, bool glv) {
    uint32_t lg = 0;
    while ((1ull << lg) < n) lg++;
    if (lg < sizeof(c->tune_msm_window) && c->tune_msm_window[lg] != 0) return c->tune_msm_window[lg];
    return glv ? msm_auto_window_glv(n) : msm_auto_window(n);
}

// One pipeline: MSM instances with the same window size and mode, sharing every launch.
// Instance k's scalars are the global indices [offs[k], offs[k+1]); its bucket sets are
// [k Wr, (k + 1) Wr). All device scratch lives in one arena carved by pipe_layout.
template <class C>
struct MsmPipeT {
    using P = typename C::P;
    MsmShape sh{};
    uint64_t N = 0;            // scalars over all instances
    uint64_t max_entries = 0;  // N * W
    uint64_t nbuckets = 0;     // sets * B
    uint32_t units = 0;        // first-round accumulation units
    bool skip_inf = true;      // some instance's points may hold infinity: tested per entry
    std::vector<MsmInst> inst;
    std::vector<uint32_t> offs;     // inst + 1 prefix offsets
    std::vector<size_t> out_index;  // result slot of each instance
    MsmInst* d_inst = nullptr;
    uint32_t* d_offs = nullptr;
    uint32_t *digits = nullptr, *row_ptr = nullptr, *cursor = nullptr, *entries = nullptr, *scan_tmp = nullptr;
    uint32_t *slot_keys_a = nullptr, *slot_keys_b = nullptr;
    P *slot_pts_a = nullptr, *slot_pts_b = nullptr;
    uint32_t *long_list = nullptr, *long_count = nullptr;  // fixup mode
    P *buckets = nullptr, *Yb = nullptr, *Eb = nullptr, *Y2 = nullptr, *E2 = nullptr, *F2 = nullptr, *tgt = nullptr;
    P* tgt_parts = nullptr;  // per-part target sums before the merge (null with one part)
    // tiled CSR sort (B <= kTiledMaxB): set positions, tiles and per-tile bucket counts
    bool tiled = false;
    uint32_t te = 0, tiles = 0;
    std::vector<uint32_t> set_base_h, set_tile0_h;  // sets + 1 entries each
    uint32_t *set_base = nullptr, *set_tile0 = nullptr, *tile_hist = nullptr;
    P* h_tgt = nullptr;  // host copy of the per-set targets (sets * targets)
    uint32_t* h_total = nullptr;
    size_t host_elems() const { return (size_t)sh.sets * sh.targets; }
};

// Shape and limits of a pipeline over `jobs` (all with window c, fixed-base mode or not).
template <class C>
static int pipe_init(MsmPipeT<C>& p, uint32_t c, bool fixed, bool glv, const std::vector<MsmInst>& jobs,
                     const std::vector<size_t>& out_index, int num_sms) {
    p.sh = make_shape(c, glv);
    if (fixed) {
        p.sh.shared = 1;
        p.sh.Wr = 1;
    }
    p.sh.inst = (uint32_t)jobs.size();
    p.sh.sets = p.sh.inst * p.sh.Wr;
    p.inst = jobs;
    p.out_index = out_index;
    p.offs.assign(jobs.size() + 1, 0);
    uint64_t N = 0;
    for (size_t k = 0; k < jobs.size(); k++) {
        p.offs[k] = (uint32_t)N;
        N += jobs[k].n;
        if (fixed) ZK_CHECK_ARG((uint64_t)p.sh.W * jobs[k].stride < (1ull << 31),
                                "fixed-base rows exceed 31-bit entry indices");
        if (glv) ZK_CHECK_ARG((uint64_t)jobs[k].stride + jobs[k].n < (1ull << 31),
                              "GLV bases exceed 31-bit entry indices");
    }
    ZK_CHECK_ARG(N < (1ull << 31), "MSM batch too large: total points must be below 2^31");
    p.offs[jobs.size()] = (uint32_t)N;
    p.N = N;
    p.max_entries = N * p.sh.W * (glv ? 2 : 1);
    ZK_CHECK_ARG(p.max_entries < (1ull << 32) - kSegment, "MSM too large for 32-bit CSR offsets");
    p.nbuckets = (uint64_t)p.sh.sets * p.sh.B;
    ZK_CHECK_ARG(p.nbuckets < (1ull << 32) - 1, "MSM batch has too many buckets for 32-bit keys");
    // Small pipelines are latency-bound (each accumulation thread is a chain of seg additions,
    // each reduction thread one of g or g2): shorter segments while there are fewer than about
    // four waves of accumulation threads and buckets still span at most ~2 segments on average
    // (more pieces cost more in the fixup than the shorter chains save), smaller blocks while
    // there are fewer than two (level 1) or one (level 2) warps of block threads per SM.
    // Measured on GB300 (single MSMs): 2^12 0.67 -> 0.48 ms, 2^14 0.69 -> 0.55 ms, 2^16
    // 1.03 -> 0.88 ms, 2^18 1.89 -> 1.86 ms; 2^20 and larger unchanged.
    const uint64_t acc_threads = (uint64_t)num_sms * 2048;
    const uint64_t density = p.max_entries / std::max<uint64_t>(1, p.nbuckets);
    while (p.sh.seg > kMinSegment && p.max_entries / p.sh.seg < acc_threads && p.sh.seg / 2 >= density / 2)
        p.sh.seg /= 2;
    const uint64_t min_threads = (uint64_t)num_sms * 64;
    uint32_t g = kBlockG, g2 = kBlockG2;
    while (g > 2 && p.nbuckets / g < min_threads) g /= 2;
    while (g2 > 2 && p.nbuckets / g / g2 < min_threads / 2) g2 /= 2;
    // A small single MSM skips the level-2 blocks: the targets' trees get one level deeper,
    // but a launch and its chain of 2 g2 additions go (measured on GB300: 2^10 / 2^12 /
    // 2^14 0.327 / 0.365 / 0.490 -> 0.303 / 0.347 / 0.469 ms, 2^16 and larger the same);
    // batches keep them (64 instances of 2^10..2^14: 1.6% slower without).
    const bool small = p.nbuckets < (uint64_t)num_sms * kSmallBucketsPerSm;
    shape_blocks(p.sh, g, small && jobs.size() == 1 ? 1u : g2);
    if (small) p.sh.fixmax = kFixupMaxSmall;
    p.units = (uint32_t)((p.max_entries + p.sh.seg - 1) / p.sh.seg);
    // tiled sort when a set's counters fit shared memory: set s = k Wr + w holds n_k halves
    // entries per window (n_k W in the fixed-base mode's one set), cut into tiles of at least
    // max(8192, 2B) entries (per-tile counters: at most twice the entry count in bytes) and
    // at most 64 tiles per set
    p.tiled = p.sh.B <= kTiledMaxB;
    if (p.tiled) {
        const uint32_t halves = glv ? 2u : 1u;
        uint64_t largest = 0;
        for (const MsmInst& mi : jobs) largest = std::max<uint64_t>(largest, (uint64_t)mi.n * (fixed ? p.sh.W : halves));
        p.te = (uint32_t)std::max<uint64_t>(std::max<uint64_t>(8192u, 2ull * p.sh.B), ((largest + 63) / 64 + 1023) & ~1023ull);
        p.set_base_h.assign(p.sh.sets + 1, 0);
        p.set_tile0_h.assign(p.sh.sets + 1, 0);
        uint64_t pos = 0, tiles = 0;
        for (uint32_t k = 0; k < p.sh.inst; k++)
            for (uint32_t w = 0; w < p.sh.Wr; w++) {
                const uint64_t size = (uint64_t)jobs[k].n * (fixed ? p.sh.W : halves);
                p.set_base_h[k * p.sh.Wr + w] = (uint32_t)pos;
                p.set_tile0_h[k * p.sh.Wr + w] = (uint32_t)tiles;
                pos += size;
                tiles += (size + p.te - 1) / p.te;
            }
        ZK_CHECK_ARG(pos == p.max_entries && tiles < (1ull << 31), "MSM sort layout");
        p.set_base_h[p.sh.sets] = (uint32_t)pos;
        p.set_tile0_h[p.sh.sets] = (uint32_t)tiles;
        p.tiles = (uint32_t)tiles;
    }
    return ZK_OK;
}

// Assign the device scratch of `p` inside an arena at `base` (null: measure only);
// returns the arena bytes needed.
template <class C>
static size_t pipe_layout(MsmPipeT<C>& p, char* base) {
    using P = typename C::P;
    size_t off = 0;
    auto take = [&](size_t bytes) -> char* {
        off = (off + 255) & ~(size_t)255;
        char* r = base ? base + off : nullptr;
        off += bytes ? bytes : 16;
        return r;
    };
    const MsmShape& sh = p.sh;
    const size_t first_out = (p.units + kFirstGroup - 1) / kFirstGroup;
    p.d_inst = reinterpret_cast<MsmInst*>(take(p.inst.size() * sizeof(MsmInst)));
    p.d_offs = reinterpret_cast<uint32_t*>(take(p.offs.size() * 4));
    p.digits = reinterpret_cast<uint32_t*>(
        take(std::max<uint64_t>(p.max_entries * 4, p.N * sizeof(fe) * (sh.glv ? 2 : 1))));
    p.row_ptr = reinterpret_cast<uint32_t*>(take((p.nbuckets + 1) * 4));
    p.cursor = reinterpret_cast<uint32_t*>(take(p.nbuckets * 4));
    p.entries = reinterpret_cast<uint32_t*>(take(p.max_entries * 4));
    p.scan_tmp = reinterpret_cast<uint32_t*>(take(scan_scratch_elems(p.nbuckets) * 4));
    p.slot_keys_a = reinterpret_cast<uint32_t*>(take((size_t)2 * p.units * 4));
    p.slot_pts_a = reinterpret_cast<P*>(take((size_t)2 * p.units * sizeof(P)));
    p.slot_keys_b = reinterpret_cast<uint32_t*>(take(2 * first_out * 4));
    p.slot_pts_b = reinterpret_cast<P*>(take(2 * first_out * sizeof(P)));
    p.long_list = reinterpret_cast<uint32_t*>(take(((size_t)p.units / sh.fixmax + 2) * 4));
    // the count block: long and huge counts, the huge buckets' chunk counters and keys
    p.long_count = reinterpret_cast<uint32_t*>(take((2 + 2 * (size_t)huge_cap(p.units)) * 4));
    p.buckets = reinterpret_cast<P*>(take(p.nbuckets * sizeof(P)));
    p.Yb = reinterpret_cast<P*>(take((size_t)sh.sets * sh.G * sizeof(P)));
    p.Eb = reinterpret_cast<P*>(take((size_t)sh.sets * sh.G * sizeof(P)));
    p.Y2 = reinterpret_cast<P*>(take((size_t)sh.sets * sh.G2 * sizeof(P)));
    p.E2 = reinterpret_cast<P*>(take((size_t)sh.sets * sh.G2 * sizeof(P)));
    p.F2 = reinterpret_cast<P*>(take((size_t)sh.sets * sh.G2 * sizeof(P)));
    p.tgt = reinterpret_cast<P*>(take(p.host_elems() * sizeof(P)));
    const uint32_t parts = target_parts<C>(sh);
    p.tgt_parts = parts > 1 ? reinterpret_cast<P*>(take(p.host_elems() * parts * sizeof(P))) : nullptr;
    if (p.tiled) {
        p.set_base = reinterpret_cast<uint32_t*>(take(p.set_base_h.size() * 4));
        p.set_tile0 = reinterpret_cast<uint32_t*>(take(p.set_tile0_h.size() * 4));
        p.tile_hist = reinterpret_cast<uint32_t*>(take((size_t)p.tiles * sh.B * 4));
    }
    return off;
}

// Dynamic shared memory of the tiled sort kernels (set once per device).
static int set_sort_smem_attr(int device) {
    static std::mutex mu;
    static bool done[64] = {};
    ZK_CHECK_ARG(device >= 0 && device < 64, "device index out of range");
    std::lock_guard<std::mutex> g(mu);
    if (!done[device]) {
        ZK_TRY_CUDA(cudaFuncSetAttribute(msm_hist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTiledMaxB * 4));
        ZK_TRY_CUDA(cudaFuncSetAttribute(msm_scatter_tiles_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kTiledMaxB * 4));
        done[device] = true;
    }
    return ZK_OK;
}

// The pipeline's descriptors to the device: instances, scalar offsets, sort layout.
template <class C>
static int pipe_upload(Ctx* c, MsmPipeT<C>& p) {
    cudaStream_t st = c->stream;
    ZK_TRY_CUDA(cudaMemcpyAsync(p.d_inst, p.inst.data(), p.inst.size() * sizeof(MsmInst), cudaMemcpyHostToDevice, st));
    ZK_TRY_CUDA(cudaMemcpyAsync(p.d_offs, p.offs.data(), p.offs.size() * 4, cudaMemcpyHostToDevice, st));
    if (p.tiled) {
        ZK_TRY_CUDA(cudaMemcpyAsync(p.set_base, p.set_base_h.data(), p.set_base_h.size() * 4, cudaMemcpyHostToDevice,
                                    st));
        ZK_TRY_CUDA(cudaMemcpyAsync(p.set_tile0, p.set_tile0_h.data(), p.set_tile0_h.size() * 4,
                                    cudaMemcpyHostToDevice, st));
    }
    return ZK_OK;
}

// The CSR sort with global atomics (bucket sets larger than shared memory): digits and a
// warp-aggregated histogram, the scan, then the digits again and a scatter through cursors.
template <class C>
static int enqueue_atomic_sort(Ctx* c, MsmPipeT<C>& p, int scalars_mont) {
    cudaStream_t st = c->stream;
    const MsmShape& sh = p.sh;
    const uint32_t N = (uint32_t)p.N;
    const unsigned nblk = (unsigned)((p.N + 255) / 256);
    ZK_TRY_CUDA(cudaMemsetAsync(p.row_ptr, 0, (p.nbuckets + 1) * 4, st));
    if (!c->scalar_chunks.empty() && c->scalar_chunks.back().first == N && p.inst.size() == 1) {
        // scalars still arriving: each chunk's digits wait for its copy only
        uint32_t j0 = 0;
        for (const auto& ch : c->scalar_chunks) {
            ZK_TRY_CUDA(cudaStreamWaitEvent(st, ch.second, 0));
            ZK_LAUNCH(c, "msm_digits", msm_digits_kernel<C>, (unsigned)((ch.first - j0 + 255) / 256), 256, 0,
                      p.d_inst, p.d_offs, j0, ch.first, scalars_mont, sh, reinterpret_cast<fe*>(p.digits),
                      p.row_ptr);
            ZK_TRY_CUDA(cudaGetLastError());
            j0 = ch.first;
        }
    } else {
        // scalars still arriving on another stream, for a pipeline that does not match the
        // chunks: wait for all of them
        if (!c->scalar_chunks.empty()) ZK_TRY_CUDA(cudaStreamWaitEvent(st, c->scalar_chunks.back().second, 0));
        ZK_LAUNCH(c, "msm_digits", msm_digits_kernel<C>, nblk, 256, 0, p.d_inst, p.d_offs, 0u, N, scalars_mont, sh,
                  reinterpret_cast<fe*>(p.digits), p.row_ptr);
        ZK_TRY_CUDA(cudaGetLastError());
    }
    // row_ptr[0..nbuckets) := exclusive scan; row_ptr[nbuckets] := total
    int rc = device_exclusive_scan(c, p.row_ptr, p.nbuckets, p.row_ptr + p.nbuckets, p.scan_tmp);
    if (rc != ZK_OK) return rc;
    ZK_TRY_CUDA(cudaMemcpyAsync(p.cursor, p.row_ptr, p.nbuckets * 4, cudaMemcpyDeviceToDevice, st));
    ZK_LAUNCH(c, "msm_scatter", msm_scatter_kernel, nblk, 256, 0, reinterpret_cast<const fe*>(p.digits), p.d_inst,
              p.d_offs, N, sh, p.cursor, p.entries);
    ZK_TRY_CUDA(cudaGetLastError());
    return ZK_OK;
}

// The tiled CSR sort of a pipeline (codes, per-tile counts, totals, scan, offsets, scatter).
template <class C>
static int enqueue_tiled_sort(Ctx* c, MsmPipeT<C>& p, int scalars_mont) {
    cudaStream_t st = c->stream;
    const MsmShape& sh = p.sh;
    const uint32_t N = (uint32_t)p.N;
    int rc = set_sort_smem_attr(c->device);
    if (rc != ZK_OK) return rc;
    uint32_t* codes = p.digits;
    if (!c->scalar_chunks.empty() && c->scalar_chunks.back().first == N && p.inst.size() == 1) {
        // scalars still arriving: each chunk's codes wait for its copy only
        uint32_t j0 = 0;
        for (const auto& ch : c->scalar_chunks) {
            ZK_TRY_CUDA(cudaStreamWaitEvent(st, ch.second, 0));
            ZK_LAUNCH(c, "msm_codes", msm_codes_kernel<C>, (unsigned)((ch.first - j0 + 255) / 256), 256, 0, p.d_inst,
                      p.d_offs, j0, ch.first, scalars_mont, sh, p.set_base, codes);
            ZK_TRY_CUDA(cudaGetLastError());
            j0 = ch.first;
        }
    } else {
        if (!c->scalar_chunks.empty()) ZK_TRY_CUDA(cudaStreamWaitEvent(st, c->scalar_chunks.back().second, 0));
        ZK_LAUNCH(c, "msm_codes", msm_codes_kernel<C>, (unsigned)((p.N + 255) / 256), 256, 0, p.d_inst, p.d_offs, 0u,
                  N, scalars_mont, sh, p.set_base, codes);
        ZK_TRY_CUDA(cudaGetLastError());
    }
    const size_t smem = (size_t)sh.B * 4;
    ZK_LAUNCH(c, "msm_hist", msm_hist_kernel, p.tiles, kTiledThreads, smem, codes, p.set_base, p.set_tile0, sh.sets,
              p.te, sh.B, p.tile_hist);
    ZK_TRY_CUDA(cudaGetLastError());
    if (p.nbuckets <= kMetaMaxBuckets && (uint64_t)p.tiles * sh.B <= kMetaMaxCounts) {
        ZK_LAUNCH(c, "msm_sort_meta", msm_sort_meta_kernel, 1, kMetaThreads, 0, p.tile_hist, p.set_tile0, sh.sets,
                  sh.B, p.row_ptr);
        ZK_TRY_CUDA(cudaGetLastError());
    } else {
        const unsigned nb = (unsigned)((p.nbuckets + 255) / 256);
        ZK_LAUNCH(c, "msm_hist_total", msm_hist_total_kernel, nb, 256, 0, p.tile_hist, p.set_tile0, sh.sets, sh.B,
                  p.row_ptr);
        ZK_TRY_CUDA(cudaGetLastError());
        // row_ptr[0..nbuckets) := exclusive scan; row_ptr[nbuckets] := total
        rc = device_exclusive_scan(c, p.row_ptr, p.nbuckets, p.row_ptr + p.nbuckets, p.scan_tmp);
        if (rc != ZK_OK) return rc;
        ZK_LAUNCH(c, "msm_hist_offsets", msm_hist_offsets_kernel, nb, 256, 0, p.tile_hist, p.set_tile0, sh.sets,
                  sh.B, p.row_ptr);
        ZK_TRY_CUDA(cudaGetLastError());
    }
    ZK_LAUNCH(c, "msm_scatter_tiles", msm_scatter_tiles_kernel, p.tiles, kTiledThreads, smem, codes, p.set_base,
              p.set_tile0, p.te, sh, p.d_inst, p.tile_hist, p.entries);
    ZK_TRY_CUDA(cudaGetLastError());
    return ZK_OK;
}

// The descriptors (if `upload`), the cleared buckets and the CSR sort of a pipeline.
template <class C>
static int pipe_enqueue_sort(Ctx* c, MsmPipeT<C>& p, int scalars_mont, bool upload) {
    using P = typename C::P;
    if (upload) {
        int rc = pipe_upload(c, p);
        if (rc != ZK_OK) return rc;
    }
    ZK_TRY_CUDA(cudaMemsetAsync(p.buckets, 0, p.nbuckets * sizeof(P), c->stream));
    return p.tiled ? enqueue_tiled_sort<C>(c, p, scalars_mont) : enqueue_atomic_sort<C>(c, p, scalars_mont);
}

// The copies of the targets and the entry count to p.h_tgt / p.h_total.
template <class C>
static int pipe_enqueue_copies(Ctx* c, MsmPipeT<C>& p) {
    using P = typename C::P;
    ZK_TRY_CUDA(cudaMemcpyAsync(p.h_tgt, p.tgt, p.host_elems() * sizeof(P), cudaMemcpyDeviceToHost, c->stream));
    ZK_TRY_CUDA(cudaMemcpyAsync(p.h_total, p.row_ptr + p.nbuckets, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                c->stream));
    return ZK_OK;
}

// Accumulation, straddling pieces and window reduction of a sorted pipeline, one launch per
// stage.
template <class C>
static int pipe_enqueue_reduce(Ctx* c, MsmPipeT<C>& p) {
    using P = typename C::P;
    cudaStream_t st = c->stream;
    const MsmShape& sh = p.sh;
    // accumulation rounds (the first kernel that reads the points)
    if (c->bases_wait != nullptr) ZK_TRY_CUDA(cudaStreamWaitEvent(st, c->bases_wait, 0));
    const uint32_t* d_total = p.row_ptr + p.nbuckets;
    // point sets without infinity skip the per-entry test
    auto* accumulate = p.skip_inf ? msm_accumulate_kernel<C, true> : msm_accumulate_kernel<C, false>;
    ZK_LAUNCH(c, "msm_accumulate", accumulate, (p.units + 127) / 128, 128, 0, p.entries, d_total, p.row_ptr,
              p.d_inst, sh, p.units, p.buckets, p.slot_keys_a, p.slot_pts_a, p.skip_inf ? c->inf_flag : nullptr);
    ZK_TRY_CUDA(cudaGetLastError());
    // Partial sums of straddling buckets: short buckets (up to ~3 segments on average) by one
    // fixup pass, longer ones by merge rounds (kFixupDensity).
    if (p.max_entries <= (uint64_t)p.nbuckets * kFixupDensity) {
        const uint32_t hcap = huge_cap(p.units);
        // counts and chunk counters to zero (the keys are written before they are read)
        ZK_TRY_CUDA(cudaMemsetAsync(p.long_count, 0, (2 + (size_t)hcap) * 4, st));
        ZK_LAUNCH(c, "msm_fixup", msm_fixup_kernel<C>, (unsigned)((p.nbuckets + 127) / 128), 128, 0, p.row_ptr,
                  (uint32_t)p.nbuckets, sh.seg, sh.fixmax, p.slot_pts_a, p.buckets, p.long_list, p.long_count, hcap);
        ZK_TRY_CUDA(cudaGetLastError());
        // the chunk sums of huge buckets go to slot_pts_b (merge-round space, unused in fixup mode)
        // as many CTAs as fit at once (at least 2 per SM)
        ZK_LAUNCH(c, "msm_fixup_long", msm_fixup_long_kernel<C>,
                  (unsigned)(c->num_sms * std::max(2, C::kFixupLongMinBlocks)), C::kFixupLongThreads, 0,
                  p.row_ptr, sh.seg, p.slot_pts_a, p.buckets, p.long_list, p.long_count, hcap, p.slot_pts_b);
        ZK_TRY_CUDA(cudaGetLastError());
    } else {
        uint64_t span = sh.seg;
        uint32_t in_units = p.units;
        uint32_t *ik = p.slot_keys_a, *ok = p.slot_keys_b;
        typename C::P *ip = p.slot_pts_a, *op = p.slot_pts_b;
        uint32_t group = kFirstGroup;
        while (in_units > 1) {
            const uint32_t out_units = (in_units + group - 1) / group;
            span *= group;
            ZK_LAUNCH(c, group == kFirstGroup ? "msm_merge_pairs" : "msm_merge", msm_merge_kernel<C>, (out_units + 127) / 128,
                      128, 0, ik, ip, in_units, group, d_total, p.row_ptr, span, out_units, p.buckets, ok, op);
            ZK_TRY_CUDA(cudaGetLastError());
            std::swap(ik, ok);
            std::swap(ip, op);
            in_units = out_units;
            group = kGroup;
        }
    }

    // window reduction
    // the targets' CTAs sum G2 points each: no more threads than the power of two covering G2
    uint32_t target_threads = 32;
    while (target_threads < sh.G2 && target_threads < (uint32_t)C::kTargetThreads) target_threads <<= 1;
    const uint32_t nb1 = sh.sets * sh.G;
    ZK_LAUNCH(c, "msm_bucket_blocks", msm_bucket_blocks_kernel<C>, (nb1 + 127) / 128, 128, 0, p.buckets, sh, p.Yb, p.Eb);
    ZK_TRY_CUDA(cudaGetLastError());
    if (sh.g2 > 1) {
        const uint32_t nb2 = sh.sets * sh.G2;
        ZK_LAUNCH(c, "msm_bucket_blocks2", msm_bucket_blocks2_kernel<C>, (nb2 + 127) / 128, 128, 0, p.Yb, p.Eb, sh, p.Y2,
                  p.E2, p.F2);
        ZK_TRY_CUDA(cudaGetLastError());
    }
    const uint32_t parts = target_parts<C>(sh);
    P* tout = parts > 1 ? p.tgt_parts : p.tgt;
    if (sh.g2 > 1) {
        ZK_LAUNCH(c, "msm_targets", msm_targets_kernel<C>, sh.sets * sh.targets * parts, target_threads, 0, p.F2,
                  p.E2, p.Y2, p.Y2, sh, parts, tout);
    } else {
        ZK_LAUNCH(c, "msm_targets", msm_targets_kernel<C>, sh.sets * sh.targets * parts, target_threads, 0, p.Eb,
                  p.Yb, p.Yb, p.Yb, sh, parts, tout);
    }
    ZK_TRY_CUDA(cudaGetLastError());
    if (parts > 1) {
        ZK_LAUNCH(c, "msm_targets_merge", msm_targets_merge_kernel<C>, sh.sets * sh.targets, kMergeThreads, 0,
                  p.tgt_parts, parts, p.tgt);
        ZK_TRY_CUDA(cudaGetLastError());
    }
    return ZK_OK;
}

// Enqueue the device part of a pipeline on the context stream, ending with the copies of
// the targets and the entry count to p.h_tgt / p.h_total. Allocates nothing, so it can be
// captured into a CUDA graph (the instance descriptors are uploaded only if `upload`).
template <class C>
static int pipe_enqueue(Ctx* c, MsmPipeT<C>& p, int scalars_mont, bool upload) {
    int rc = pipe_enqueue_sort<C>(c, p, scalars_mont, upload);
    if (rc == ZK_OK) rc = pipe_enqueue_reduce<C>(c, p);
    if (rc == ZK_OK) rc = pipe_enqueue_copies<C>(c, p);
    return rc;
}

// A persistent pool of host threads for the combination step (created on first use,
// never destroyed: its threads sleep between jobs). run() executes fn(0 .. count-1) on the
// calling thread and on at most count - 1 woken workers, and returns when every task is
// done -- not when every worker has woken: a late worker finds no task left and sleeps
// again. Tasks are claimed from one atomic ticket (generation | count | next index), so a
// worker can only claim a task of the run in progress; calls are serialised.
class HostPool {
   public:
    static HostPool& get() {
        static HostPool* pool = new HostPool();
        return *pool;
    }

    void run(size_t count, const std::function<void(size_t)>& fn) {
        if (count == 1 || workers_ == 0) {  // no helper: no shared state, no lock
            for (size_t i = 0; i < count; i++) fn(i);
            return;
        }
        run_with(count, fn, [] {});
    }

    // run() in which the calling thread first executes own(): own() may take tasks itself
    // through run_one() (the same ticket, so in the same index order as the workers), e.g.
    // to consume results in order and compute whichever no worker has taken yet.
    template <class Own>
    void run_with(size_t count, const std::function<void(size_t)>& fn, Own&& own, size_t max_helpers = ~size_t(0)) {
        if (count > kMaxTasks) {
            for (size_t i = 0; i < count; i++) fn(i);
            own();
            return;
        }
        if (count == 0) {
            own();
            return;
        }
        std::lock_guard<std::mutex> serial(run_mu_);
        gen_ = (gen_ + 1) & 0xffffu;
        fn_ = &fn;
        done_.store(0, std::memory_order_relaxed);
        ticket_.store(gen_ << 48 | (uint64_t)count << 24, std::memory_order_release);
        const size_t helpers = std::min(std::min(count - 1, workers_), max_helpers);
        if (helpers > 0) {
            // the caller wakes up to kFanout workers and each woken worker up to kFanout more
            // (a wake-up is a system call of a few microseconds: a tree of them instead of a
            // row on the caller)
            const size_t first = std::min(helpers, kFanout);
            pending_.store((int64_t)(helpers - first), std::memory_order_relaxed);
            {
                std::lock_guard<std::mutex> g(mu_);
                wake_++;
            }
            for (size_t i = 0; i < first; i++) cv_.notify_one();
        }
        own();
        work();
        // the tasks still running were claimed by awake workers; the wait re-checks every
        // millisecond, so even a lost wakeup of the condition variable only costs that much
        std::unique_lock<std::mutex> g(mu_);
        while (done_.load(std::memory_order_acquire) < count)
            done_cv_.wait_for(g, std::chrono::milliseconds(1),
                              [&] { return done_.load(std::memory_order_acquire) >= count; });
    }

    // Claim and run the next task of the run in progress; false if none is left.
    bool run_one() {
        for (;;) {
            uint64_t cur = ticket_.load(std::memory_order_acquire);
            const uint64_t count = (cur >> 24) & kMaxTasks, i = cur & kMaxTasks;
            if (i >= count) return false;
            if (!ticket_.compare_exchange_weak(cur, cur + 1, std::memory_order_acq_rel)) continue;
            (*fn_)(i);
            if (done_.fetch_add(1, std::memory_order_acq_rel) + 1 == count) {
                std::lock_guard<std::mutex> g(mu_);
                done_cv_.notify_all();
            }
            return true;
        }
    }

   private:
    static constexpr size_t kMaxTasks = (1u << 24) - 1;

    HostPool() {
        const size_t hw = std::max<size_t>(1, std::thread::hardware_concurrency());
        workers_ = std::min<size_t>(hw, 16) - 1;
        for (size_t i = 0; i < workers_; i++) std::thread([this] { loop(); }).detach();
    }

    void loop() {
        uint64_t seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> g(mu_);
                cv_.wait(g, [&] { return wake_ != seen; });
                seen = wake_;
            }
            for (size_t i = 0; i < kFanout; i++)
                if (pending_.fetch_sub(1, std::memory_order_acq_rel) > 0) cv_.notify_one();
            work();
        }
    }

    // Claim and run tasks while the ticket has some left. A successful claim of task i means
    // the run that published the ticket is still waiting for task i, so fn_ is its function.
    void work() {
        while (run_one()) {
        }
    }

    size_t workers_ = 0;
    std::mutex run_mu_, mu_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(size_t)>* fn_ = nullptr;
    std::atomic<uint64_t> ticket_{0};
    std::atomic<size_t> done_{0};
    std::atomic<int64_t> pending_{0};  // wake-ups the woken workers still have to pass on
    static constexpr size_t kFanout = 2;
    uint64_t wake_ = 0;  // under mu_
    uint64_t gen_ = 0;   // under run_mu_
};

// Host: the sum S_w of window (or set) w of instance k from its targets:
//   one level   S_w = T0 + g (T1 + H)            (T0 = sum E1, T1 = sum Y1)
//   two levels  S_w = T0 + g (T1 + g2 (T2 + H))  (T0 = sum F2 = sum E1, T1 = sum E2, T2 = sum Y2)
// with H = sum_k 2^k M_k (Horner).
template <class C>
static zkh::XyzzT<typename HostOf<C>::T> window_sum(const MsmPipeT<C>& p, uint32_t k, uint32_t w) {
    using H = typename HostOf<C>::T;
    const MsmShape& sh = p.sh;
    uint32_t log_g = 0, log_g2 = 0;
    while ((1u << log_g) < sh.g) log_g++;
    while ((1u << log_g2) < sh.g2) log_g2++;
    const typename C::P* T = p.h_tgt + ((size_t)k * sh.Wr + (size_t)w) * sh.targets;
    zkh::XyzzT<H> h = zkh::xyzz_inf<H>();
    for (int b = (int)sh.K - 1; b >= 0; b--) {
        h = zkh::xyzz_dbl(h);
        h = zkh::xyzz_add(h, to_host<C>(T[sh.plain + b]));
    }
    zkh::XyzzT<H> sw = zkh::xyzz_add(h, to_host<C>(T[sh.plain - 1]));
    if (sh.plain == 3) {
        sw = host_dbl_n(sw, log_g2);
        sw = zkh::xyzz_add(sw, to_host<C>(T[1]));
    }
    sw = host_dbl_n(sw, log_g);
    return zkh::xyzz_add(sw, to_host<C>(T[0]));
}

// total = sum_w 2^(c w) S_w by Horner over the windows (one set in fixed-base mode, where
// the window shifts are already in the bases), as canonical affine bytes; get(w) yields S_w,
// asked for from the top window down.
template <class C, class Get>
static void horner_out(const MsmPipeT<C>& p, Get&& get, uint8_t* out_xy, int32_t* out_is_inf) {
    using H = typename HostOf<C>::T;
    zkh::XyzzT<H> total = zkh::xyzz_inf<H>();
    for (int w = (int)p.sh.Wr - 1; w >= 0; w--) {
        total = host_dbl_n(total, p.sh.c);
        total = zkh::xyzz_add(total, get((uint32_t)w));
    }
    H x, y;
    *out_is_inf = zkh::xyzz_to_affine_canonical(total, &x, &y) ? 1 : 0;
    std::memcpy(out_xy, &x, sizeof(H));
    std::memcpy(out_xy + sizeof(H), &y, sizeof(H));
}

#ifndef ZK_COMBINE_HELPERS
#define ZK_COMBINE_HELPERS 4
#endif
static constexpr size_t kCombineHelpers = ZK_COMBINE_HELPERS;  // pool workers of a one-instance combine

// Combine every instance of `pipes`: the window sums of all instances in parallel on the
// host pool, then each instance's Horner (in parallel across instances); a single instance
// overlaps its Horner with its window sums.
template <class C>
static void combine_all(Ctx* c, const std::vector<MsmPipeT<C>>& pipes, uint8_t* out_xy, int32_t* out_is_inf,
                        bool record = true) {
    using H = typename HostOf<C>::T;
    constexpr size_t kOut = 2 * sizeof(H);  // bytes of one affine result
    const auto t0 = std::chrono::steady_clock::now();
    struct Inst {
        uint32_t q, k;
        size_t first;  // index of its first window sum
    };
    std::vector<Inst> insts;
    std::vector<std::pair<uint32_t, uint32_t>> win;  // (instance, window)
    uint64_t entries = 0;
    for (uint32_t q = 0; q < pipes.size(); q++) {
        entries += *pipes[q].h_total;
        for (uint32_t k = 0; k < pipes[q].sh.inst; k++) {
            insts.push_back({q, k, win.size()});
            for (uint32_t w = 0; w < pipes[q].sh.Wr; w++) win.emplace_back((uint32_t)insts.size() - 1, w);
        }
    }
    std::vector<zkh::XyzzT<H>> sums(win.size());
    HostPool& pool = HostPool::get();
    if (insts.size() == 1 && win.size() > 1) {
        // One instance (the latency case): the calling thread runs the Horner from the top
        // window down while woken workers compute the lower window sums; task t is window
        // W-1-t, so tasks are claimed in the order the Horner consumes them, and the caller
        // computes any window no worker has taken yet.
        const MsmPipeT<C>& p = pipes[insts[0].q];
        const uint32_t k = insts[0].k, W = (uint32_t)win.size();
        std::unique_ptr<std::atomic<uint32_t>[]> ready(new std::atomic<uint32_t>[W]());
        const std::function<void(size_t)> task = [&](size_t t) {
            sums[t] = window_sum<C>(p, k, W - 1 - (uint32_t)t);
            ready[t].store(1, std::memory_order_release);
        };
        const size_t o = p.out_index[k];
        // a few helpers keep ahead of the Horner (a window sum costs about as much as 2-3
        // windows of its doublings)
        pool.run_with(W, task, [&] {
            horner_out<C>(p, [&](uint32_t w) -> const zkh::XyzzT<H>& {
                const uint32_t t = W - 1 - w;
                while (!ready[t].load(std::memory_order_acquire))
                    if (!pool.run_one()) std::this_thread::yield();  // a worker is on it
                return sums[t];
            }, out_xy + kOut * o, out_is_inf + o);
        }, kCombineHelpers);
    } else {
        pool.run(win.size(), [&](size_t t) {
            const Inst& in = insts[win[t].first];
            sums[t] = window_sum<C>(pipes[in.q], in.k, win[t].second);
        });
        pool.run(insts.size(), [&](size_t t) {
            const Inst& in = insts[t];
            const size_t o = pipes[in.q].out_index[in.k];
            const zkh::XyzzT<H>* sw = sums.data() + in.first;
            horner_out<C>(pipes[in.q], [sw](uint32_t w) -> const zkh::XyzzT<H>& { return sw[w]; },
                          out_xy + kOut * o, out_is_inf + o);
        });
    }
    if (!record) return;  // a worker thread of an asynchronous batch leaves the context's tables alone
    prof_host(c, "msm_host_combine",
              std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
    c->msm_entries = entries;
    if (!pipes.empty()) {
        c->msm_window_bits = pipes.back().sh.c;
        c->msm_windows = pipes.back().sh.W;
    }
}

// Group jobs into pipelines: one per (window bits, fixed-base mode, GLV), split where a
// group would exceed the 31-bit point / 32-bit entry limits.
template <class C>
static int build_pipes(Ctx* c, const MsmJob* jobs, size_t count, uint32_t window_bits,
                       std::vector<MsmPipeT<C>>* out, std::vector<size_t>* empty) {
    ZK_CHECK_ARG(window_bits == 0 || (window_bits >= 4 && window_bits <= 20), "window_bits must be 0 or 4..20");
    std::map<std::tuple<uint32_t, bool, bool>, std::vector<size_t>> groups;
    for (size_t j = 0; j < count; j++) {
        const MsmJob& b = jobs[j];
        ZK_CHECK_ARG(b.n < (1ull << 31), "MSM size must be below 2^31 points");
        if (b.n == 0) {
            empty->push_back(j);
            continue;
        }
        const bool fixed = b.shifted != nullptr && (window_bits == 0 || window_bits == b.shifted_c);
        const bool glv = !fixed && b.glv;  // fixed-base rows hold P only (plain 255-bit windows)
        const uint32_t cb = fixed ? b.shifted_c : (window_bits ? window_bits : msm_window_for(c, b.n, glv));
        groups[std::make_tuple(cb, fixed, glv)].push_back(j);
    }
    for (auto& kv : groups) {
        const uint32_t cb = std::get<0>(kv.first);
        const bool fixed = std::get<1>(kv.first);
        const bool glv = std::get<2>(kv.first);
        const uint64_t W = make_shape(cb, glv).W * (glv ? 2 : 1);  // entries per scalar
        std::vector<MsmInst> part;
        std::vector<size_t> idx;
        uint64_t N = 0;
        bool part_inf = false;
        auto flush = [&]() -> int {
            if (part.empty()) return ZK_OK;
            out->emplace_back();
            int rc = pipe_init<C>(out->back(), cb, fixed, glv, part, idx, c->num_sms);
            // the sort kernels' shared-memory limit, set here and not inside a graph capture
            if (rc == ZK_OK && out->back().tiled) rc = set_sort_smem_attr(c->device);
            out->back().skip_inf = part_inf;
            part.clear();
            idx.clear();
            N = 0;
            part_inf = false;
            return rc;
        };
        for (size_t j : kv.second) {
            const MsmJob& b = jobs[j];
            if (!part.empty() && ((N + b.n) >= (1ull << 31) || (N + b.n) * W >= (1ull << 32) - kSegment)) {
                int rc = flush();
                if (rc != ZK_OK) return rc;
            }
            MsmInst mi;
            mi.scalars = b.scalars;
            mi.bases = fixed ? b.shifted : b.bases;
            mi.n = (uint32_t)b.n;
            mi.stride = (fixed || glv) ? (uint32_t)b.stride : 0u;
            part.push_back(mi);
            idx.push_back(j);
            N += b.n;
            part_inf = part_inf || b.inf_points;
        }
        int rc = flush();
        if (rc != ZK_OK) return rc;
    }
    return ZK_OK;
}

static void set_infinity(uint8_t* out_xy, int32_t* out_is_inf, const std::vector<size_t>& which,
                         size_t out_bytes = 64) {
    for (size_t j : which) {
        std::memset(out_xy + out_bytes * j, 0, out_bytes);
        out_is_inf[j] = 1;
    }
}

// Enqueue every pipeline of a batch. With several pipelines they are spread over the
// context stream and kSideStreams side streams (largest first, each to the stream with the
// least work so far), forked from and joined back into the context stream, so that the
// latency-bound stages of small pipelines overlap the accumulation of large ones. Works
// inside a stream capture (the fork / join events make the side streams part of it).
static constexpr int kSideStreams = 3;

static int ensure_side_streams(Ctx* c) {
    while ((int)c->side_streams.size() < kSideStreams) {
        cudaStream_t st = nullptr;
        ZK_TRY_CUDA(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, c->priority));
        c->side_streams.push_back(st);
    }
    while ((int)c->side_events.size() <= kSideStreams) {
        cudaEvent_t ev = nullptr;
        ZK_TRY_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        c->side_events.push_back(ev);
    }
    return ZK_OK;
}

// ---- host side of the MSM work queue ---------------------------------------------------
// G1 only: the G2 stages together need more than 255 registers (the kernel spills ~5 KB per
// thread), so G2 batches keep one launch per stage.
template <class C>
constexpr bool kQueueForm = std::is_same<C, CurveG1>::value;

template <class C>
struct MsmQueueT {
    std::vector<MsmQPipe<C>> qp;
    std::vector<MsmQEntry> qe;
    std::vector<uint32_t> fixup_mode;  // per pipeline: 1 when its straddling pieces use the fixup
    uint32_t nitems = 0, grid = 0;
    uint64_t limit_ns = 2000000000ull;  // 2 s per wait
    size_t pipes_at = 0, entries_at = 0, limit_at = 0, state_at = 0, bytes = 0;
    char* dev = nullptr;
    uint32_t* h_status = nullptr;  // host word receiving the launch's status word
};

// The queue's entries in stage order (largest pipelines first within a stage) and its device
// layout, from the pipelines' shapes. A test limit armed on the context (zk_msm_queue_test_limit)
// makes the first waiting entry wait for one item more than its dependency has.
template <class C>
static int queue_plan(Ctx* c, const std::vector<MsmPipeT<C>>& pipes, MsmQueueT<C>& q) {
    const size_t np = pipes.size();
    std::vector<size_t> order(np);
    for (size_t k = 0; k < np; k++) order[k] = k;
    std::stable_sort(order.begin(), order.end(),
                     [&](size_t a, size_t b) { return pipes[a].max_entries > pipes[b].max_entries; });
    // each pipeline's stages as (slot, entry); slots: 0 accumulation, 1..R merge rounds, then
    // fixup, long fixup, level 1, level 2, targets, target merge
    std::vector<std::vector<std::pair<uint32_t, MsmQEntry>>> st(np);
    uint32_t rmax = 0;
    q.fixup_mode.assign(np, 0);
    const uint32_t long_items = std::max<uint32_t>(8, (uint32_t)(2 * c->num_sms / std::max<size_t>(1, np)));
    auto add = [](std::vector<std::pair<uint32_t, MsmQEntry>>& v, uint32_t slot, uint32_t stage, uint64_t items) {
        MsmQEntry e{};
        e.stage = stage;
        e.items = (uint32_t)items;
        v.push_back({slot, e});
        return &v.back().second;
    };
    for (size_t k = 0; k < np; k++) {
        const MsmPipeT<C>& p = pipes[k];
        const MsmShape& sh = p.sh;
        add(st[k], 0, kQAcc, (p.units + kMsmQThreads - 1) / kMsmQThreads);
        if (p.max_entries <= (uint64_t)p.nbuckets * kFixupDensity) {
            q.fixup_mode[k] = 1;
        } else {
            uint64_t span = sh.seg;
            uint32_t in_units = p.units, group = kFirstGroup, src = 0, r = 0;
            while (in_units > 1) {
                const uint32_t out_units = (in_units + group - 1) / group;
                span *= group;
                MsmQEntry* e = add(st[k], 1 + r, kQMerge, (out_units + kMsmQThreads - 1) / kMsmQThreads);
                e->in_units = in_units;
                e->out_units = out_units;
                e->group = group;
                e->src = src;
                e->span = span;
                src ^= 1;
                in_units = out_units;
                group = kGroup;
                r++;
            }
            rmax = std::max(rmax, r);
        }
    }
    for (size_t k = 0; k < np; k++) {
        const MsmPipeT<C>& p = pipes[k];
        const MsmShape& sh = p.sh;
        const uint32_t base = 1 + rmax;
        if (q.fixup_mode[k]) {
            add(st[k], base, kQFix, (p.nbuckets + kMsmQThreads - 1) / kMsmQThreads);
            add(st[k], base + 1, kQFixLong, long_items);
        }
        add(st[k], base + 2, kQBlk1, ((uint64_t)sh.sets * sh.G + kMsmQThreads - 1) / kMsmQThreads);
        if (sh.g2 > 1) add(st[k], base + 3, kQBlk2, ((uint64_t)sh.sets * sh.G2 + kMsmQThreads - 1) / kMsmQThreads);
        const uint32_t parts = target_parts<C>(sh);
        add(st[k], base + 4, kQTgt, (uint64_t)sh.sets * sh.targets * parts);
        if (parts > 1) add(st[k], base + 5, kQTMerge, (uint64_t)sh.sets * sh.targets);
    }
    q.qe.clear();
    q.nitems = 0;
    std::vector<int32_t> prev(np, -1);
    std::vector<size_t> pos(np, 0);
    bool armed = c->msm_queue_test_limit_ns != 0;
    auto emit = [&](size_t k) {
        MsmQEntry e = st[k][pos[k]++].second;
        e.pipe = (uint32_t)k;
        e.first = q.nitems;
        e.dep = prev[k];
        e.need = prev[k] >= 0 ? q.qe[prev[k]].items : 0;
        if (armed && e.dep >= 0) {  // the test: a wait that nothing can satisfy
            e.need += 1;
            armed = false;
        }
        prev[k] = (int32_t)q.qe.size();
        q.qe.push_back(e);
        q.nitems += e.items;
    };
    // Order: stage by stage, the largest pipelines first within a stage -- no item waits on a
    // stage that began late. (Measured on GB300: every smaller pipeline's whole chain first,
    // meant to hide its latency-bound stages behind the largest accumulation, was slower --
    // 64 instances of 2^10..2^14 5.31 against 4.59 ms -- its items wait on their own
    // previous stages.)
    for (uint32_t slot = 0; slot <= 6 + rmax; slot++)
        for (size_t k : order)
            if (pos[k] < st[k].size() && st[k][pos[k]].first == slot) emit(k);
    ZK_CHECK_ARG(q.nitems < (1u << 31), "MSM work queue too long");
    if (c->msm_queue_test_limit_ns != 0) {
        q.limit_ns = c->msm_queue_test_limit_ns;
        c->msm_queue_test_limit_ns = 0;  // one-shot
    }
    size_t off = 0;
    auto take = [&](size_t bytes) {
        off = (off + 255) & ~(size_t)255;
        const size_t r = off;
        off += bytes;
        return r;
    };
    q.pipes_at = take(np * sizeof(MsmQPipe<C>));
    q.entries_at = take(q.qe.size() * sizeof(MsmQEntry));
    q.limit_at = take(8);
    q.state_at = take((kQueueDone + q.qe.size()) * 4);
    q.bytes = (off + 255) & ~(size_t)255;
    int per_sm = 0;
    if constexpr (kQueueForm<C>)
        ZK_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, msm_queue_kernel<C>, kMsmQThreads, 0));
    q.grid = (uint32_t)std::min<uint64_t>(q.nitems, (uint64_t)std::max(1, per_sm) * c->num_sms);
    return ZK_OK;
}

// Device pointers of the laid-out pipelines into the queue, and the queue to the device at
// `dev` (not inside a capture).
template <class C>
static int queue_fill(Ctx* c, const std::vector<MsmPipeT<C>>& pipes, MsmQueueT<C>& q, char* dev) {
    q.dev = dev;
    q.qp.assign(pipes.size(), MsmQPipe<C>{});
    for (size_t k = 0; k < pipes.size(); k++) {
        const MsmPipeT<C>& p = pipes[k];
        MsmQPipe<C>& d = q.qp[k];
        d.entries = p.entries;
        d.row_ptr = p.row_ptr;
        d.d_total = p.row_ptr + p.nbuckets;
        d.insts = p.d_inst;
        d.inf_flag = p.skip_inf ? c->inf_flag : nullptr;
        d.buckets = p.buckets;
        d.slot_keys[0] = p.slot_keys_a;
        d.slot_keys[1] = p.slot_keys_b;
        d.slot_pts[0] = p.slot_pts_a;
        d.slot_pts[1] = p.slot_pts_b;
        d.long_list = p.long_list;
        d.long_count = p.long_count;
        d.hcap = huge_cap(p.units);
        d.Yb = p.Yb;
        d.Eb = p.Eb;
        d.Y2 = p.Y2;
        d.E2 = p.E2;
        d.F2 = p.F2;
        d.parts = target_parts<C>(p.sh);
        d.tgt_out = d.parts > 1 ? p.tgt_parts : p.tgt;
        d.tgt = p.tgt;
        d.sh = p.sh;
        d.units = p.units;
        d.nbuckets = (uint32_t)p.nbuckets;
        d.skip_inf = p.skip_inf ? 1u : 0u;
    }
    ZK_TRY_CUDA(cudaMemcpyAsync(dev + q.pipes_at, q.qp.data(), q.qp.size() * sizeof(MsmQPipe<C>),
                                cudaMemcpyHostToDevice, c->stream));
    ZK_TRY_CUDA(cudaMemcpyAsync(dev + q.entries_at, q.qe.data(), q.qe.size() * sizeof(MsmQEntry),
                                cudaMemcpyHostToDevice, c->stream));
    ZK_TRY_CUDA(cudaMemcpyAsync(dev + q.limit_at, &q.limit_ns, 8, cudaMemcpyHostToDevice, c->stream));
    return ZK_OK;
}

// The launch on the context stream: cleared state words, the persistent kernel, its status
// word to q.h_status (stream-ordered: read it after the stream has passed the launch).
template <class C>
static int queue_launch(Ctx* c, const std::vector<MsmPipeT<C>>& pipes, MsmQueueT<C>& q) {
    uint32_t* state = reinterpret_cast<uint32_t*>(q.dev + q.state_at);
    ZK_TRY_CUDA(cudaMemsetAsync(state, 0, (kQueueDone + q.qe.size()) * 4, c->stream));
    for (size_t k = 0; k < pipes.size(); k++)
        if (q.fixup_mode[k])
            ZK_TRY_CUDA(cudaMemsetAsync(pipes[k].long_count, 0, (2 + (size_t)huge_cap(pipes[k].units)) * 4, c->stream));
    if (c->bases_wait != nullptr) ZK_TRY_CUDA(cudaStreamWaitEvent(c->stream, c->bases_wait, 0));
    if constexpr (kQueueForm<C>) {
        ZK_LAUNCH(c, "msm_queue", msm_queue_kernel<C>, q.grid, kMsmQThreads, 0,
                  reinterpret_cast<const MsmQPipe<C>*>(q.dev + q.pipes_at),
                  reinterpret_cast<const MsmQEntry*>(q.dev + q.entries_at), (uint32_t)q.qe.size(), q.nitems, state,
                  reinterpret_cast<const uint64_t*>(q.dev + q.limit_at), state + kQueueStatus);
        ZK_TRY_CUDA(cudaGetLastError());
    }
    ZK_TRY_CUDA(cudaMemcpyAsync(q.h_status, state + kQueueStatus, 4, cudaMemcpyDeviceToHost, c->stream));
    return ZK_OK;
}

static std::string queue_message(uint32_t status) {
    return "MSM work queue: the wait of queue entry " + std::to_string(status - 1) +
           " for its pipeline's previous stage ran out; the launch stopped early";
}

// ZK_OK, or ZK_ETIMEOUT when the finished launch reported a wait that ran out.
static int queue_check(uint32_t status) {
    if (status == 0) return ZK_OK;
    set_error(queue_message(status));
    return ZK_ETIMEOUT;
}

// Enqueue every pipeline of a batch. Without a queue each pipeline runs all its stages on one
// of the context stream and the side streams; with a queue (`q`, prepared by queue_plan and
// queue_fill) the sorts run on those streams and then ONE persistent launch runs every
// pipeline's accumulation and reductions.
template <class C>
static int enqueue_all(Ctx* c, std::vector<MsmPipeT<C>>& pipes, int scalars_mont, bool upload,
                       MsmQueueT<C>* q = nullptr) {
    auto part = [&](MsmPipeT<C>& p) {
        return q ? pipe_enqueue_sort<C>(c, p, scalars_mont, upload) : pipe_enqueue<C>(c, p, scalars_mont, upload);
    };
    auto finish = [&]() {
        if (q == nullptr) return ZK_OK;
        int rc = queue_launch<C>(c, pipes, *q);
        for (size_t k = 0; rc == ZK_OK && k < pipes.size(); k++) rc = pipe_enqueue_copies<C>(c, pipes[k]);
        return rc;
    };
    if (pipes.size() == 1) {
        int rc = part(pipes[0]);
        return rc == ZK_OK ? finish() : rc;
    }
    int rc0 = ensure_side_streams(c);  // outside a capture (msm_plan_create calls it first)
    if (rc0 != ZK_OK) return rc0;
    const cudaStream_t main_stream = c->stream;
    const int nstreams = (int)std::min<size_t>(pipes.size(), kSideStreams + 1);
    ZK_TRY_CUDA(cudaEventRecord(c->side_events[0], main_stream));
    for (int k = 1; k < nstreams; k++) ZK_TRY_CUDA(cudaStreamWaitEvent(c->side_streams[k - 1], c->side_events[0], 0));
    std::vector<size_t> order(pipes.size());
    for (size_t k = 0; k < pipes.size(); k++) order[k] = k;
    std::sort(order.begin(), order.end(),
              [&](size_t a, size_t b) { return pipes[a].max_entries > pipes[b].max_entries; });
    std::vector<uint64_t> load(nstreams, 0);
    int rc = ZK_OK;
    for (size_t k : order) {
        const int s = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        load[s] += pipes[k].max_entries + 64ull * pipes[k].nbuckets;  // + fixed cost per bucket
        c->stream = s == 0 ? main_stream : c->side_streams[s - 1];
        rc = part(pipes[k]);
        c->stream = main_stream;
        if (rc != ZK_OK) break;
    }
    // join (also after a failure, so that no side stream is left outside a capture)
    for (int k = 1; k < nstreams; k++) {
        cudaEventRecord(c->side_events[k], c->side_streams[k - 1]);
        cudaStreamWaitEvent(main_stream, c->side_events[k], 0);
    }
    return rc == ZK_OK ? finish() : rc;
}

template <class C>
static int batch_run(Ctx* c, const MsmJob* jobs, size_t count, int scalars_mont, uint32_t window_bits, uint8_t* out_xy,
                     int32_t* out_is_inf) {
    std::vector<MsmPipeT<C>> pipes;
    std::vector<size_t> empty;
    int rc = build_pipes<C>(c, jobs, count, window_bits, &pipes, &empty);
    if (rc != ZK_OK) return rc;
    set_infinity(out_xy, out_is_inf, empty, 2 * sizeof(typename HostOf<C>::T));
    if (pipes.empty()) return ZK_OK;
    size_t bytes = 0, host_elems = 0;
    std::vector<size_t> at(pipes.size());
    for (size_t q = 0; q < pipes.size(); q++) {
        at[q] = bytes;
        bytes += (pipe_layout(pipes[q], nullptr) + 255) & ~(size_t)255;
        host_elems += pipes[q].host_elems();
    }
    // the work-queue form (zk_msm_batch_set_queue): its descriptors after the pipelines
    std::unique_ptr<MsmQueueT<C>> queue;
    uint32_t queue_status = 0;
    const size_t queue_at = bytes;
    if (c->msm_queue && kQueueForm<C>) {
        queue.reset(new MsmQueueT<C>());
        if ((rc = queue_plan<C>(c, pipes, *queue)) != ZK_OK) return rc;
        bytes += queue->bytes;
        queue->h_status = &queue_status;
    }
    char* arena = nullptr;
    if ((rc = scratch_alloc(c, bytes, reinterpret_cast<void**>(&arena))) != ZK_OK) return rc;
    std::vector<typename C::P> host_t(host_elems);
    std::vector<uint32_t> host_total(pipes.size());
    size_t h = 0;
    for (size_t q = 0; q < pipes.size(); q++) {
        pipe_layout(pipes[q], arena + at[q]);
        pipes[q].h_tgt = host_t.data() + h;
        pipes[q].h_total = &host_total[q];
        h += pipes[q].host_elems();
    }
    if (queue) {
        for (auto& p : pipes)
            if ((rc = pipe_upload(c, p)) != ZK_OK) break;
        if (rc == ZK_OK) rc = queue_fill<C>(c, pipes, *queue, arena + queue_at);
    }
    if (rc != ZK_OK || (rc = enqueue_all<C>(c, pipes, scalars_mont, !queue, queue.get())) != ZK_OK) {
        cudaStreamSynchronize(c->stream);
        scratch_free(c, arena);
        return rc;
    }
    scratch_free(c, arena);
    ZK_TRY_CUDA(cudaStreamSynchronize(c->stream));
    if (queue && (rc = queue_check(queue_status)) != ZK_OK) return rc;
    combine_all<C>(c, pipes, out_xy, out_is_inf);
    return ZK_OK;
}

// ---- asynchronous batches: the device part is enqueued and the call returns; a worker
// thread waits for the device, combines the windows on the host and signals completion ----
struct MsmAsync {
    cudaEvent_t done_ev = nullptr;
    Ctx* ctx = nullptr;
    void* pinned = nullptr;  // per-set targets and entry totals of every pipeline (from ctx's pool)
    size_t pinned_bytes = 0;
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv;
    bool done = false;
    int rc = ZK_OK;
    std::string error;
    virtual ~MsmAsync() {
        if (worker.joinable()) worker.join();
        if (done_ev) cudaEventDestroy(done_ev);
        if (pinned) pinned_give(ctx, pinned, pinned_bytes);
    }
    void finish(int code, const std::string& err) {
        std::lock_guard<std::mutex> g(mu);
        rc = code;
        error = err;
        done = true;
        cv.notify_all();
    }
};

template <class C>
struct MsmAsyncT : MsmAsync {
    std::vector<MsmPipeT<C>> pipes;
    std::unique_ptr<MsmQueueT<C>> queue;  // work-queue form, when the context asks for it
};

template <class C>
static int batch_submit(Ctx* c, const MsmJob* jobs, size_t count, int scalars_mont, uint32_t window_bits,
                        uint8_t* out_xy, int32_t* out_is_inf, MsmAsync** out) {
    std::unique_ptr<MsmAsyncT<C>> a(new MsmAsyncT<C>());
    std::vector<size_t> empty;
    int rc = build_pipes<C>(c, jobs, count, window_bits, &a->pipes, &empty);
    if (rc != ZK_OK) return rc;
    set_infinity(out_xy, out_is_inf, empty, 2 * sizeof(typename HostOf<C>::T));
    if (a->pipes.empty()) {
        a->done = true;
        *out = a.release();
        return ZK_OK;
    }
    std::vector<MsmPipeT<C>>& pipes = a->pipes;
    size_t bytes = 0, host_elems = 0;
    std::vector<size_t> at(pipes.size());
    for (size_t q = 0; q < pipes.size(); q++) {
        at[q] = bytes;
        bytes += (pipe_layout(pipes[q], nullptr) + 255) & ~(size_t)255;
        host_elems += pipes[q].host_elems();
    }
    const size_t queue_at = bytes;
    if (c->msm_queue && kQueueForm<C>) {
        a->queue.reset(new MsmQueueT<C>());
        if ((rc = queue_plan<C>(c, pipes, *a->queue)) != ZK_OK) return rc;
        bytes += a->queue->bytes;
    }
    // pinned host targets (then the entry totals and the queue status): the device-to-host
    // copies stay asynchronous
    const size_t host_bytes = host_elems * sizeof(typename C::P) + (pipes.size() + 1) * sizeof(uint32_t);
    a->ctx = c;
    if ((rc = pinned_take(c, host_bytes, &a->pinned, &a->pinned_bytes)) != ZK_OK) return rc;
    ZK_TRY_CUDA(cudaEventCreateWithFlags(&a->done_ev, cudaEventDisableTiming));
    char* arena = nullptr;
    if ((rc = scratch_alloc(c, bytes, reinterpret_cast<void**>(&arena))) != ZK_OK) return rc;
    auto* host_t = static_cast<typename C::P*>(a->pinned);
    auto* totals = reinterpret_cast<uint32_t*>(host_t + host_elems);
    size_t h = 0;
    for (size_t q = 0; q < pipes.size(); q++) {
        pipe_layout(pipes[q], arena + at[q]);
        pipes[q].h_tgt = host_t + h;
        pipes[q].h_total = totals + q;
        h += pipes[q].host_elems();
    }
    if (a->queue) {
        a->queue->h_status = totals + pipes.size();
        *a->queue->h_status = 0;
        for (auto& p : pipes)
            if ((rc = pipe_upload(c, p)) != ZK_OK) break;
        if (rc == ZK_OK) rc = queue_fill<C>(c, pipes, *a->queue, arena + queue_at);
    }
    if (rc != ZK_OK || (rc = enqueue_all<C>(c, pipes, scalars_mont, !a->queue, a->queue.get())) != ZK_OK) {
        cudaStreamSynchronize(c->stream);
        scratch_free(c, arena);
        return rc;
    }
    scratch_free(c, arena);  // stream-ordered: reusable only by work enqueued after this batch
    ZK_TRY_CUDA(cudaEventRecord(a->done_ev, c->stream));
    MsmAsyncT<C>* raw = a.get();
    const int device = c->device;
    raw->worker = std::thread([c, raw, device, out_xy, out_is_inf]() {
        cudaSetDevice(device);
        const cudaError_t e = cudaEventSynchronize(raw->done_ev);
        if (e != cudaSuccess) {
            raw->finish(ZK_ECUDA, std::string("asynchronous MSM batch: ") + cudaGetErrorString(e));
            return;
        }
        if (raw->queue && *raw->queue->h_status != 0) {
            raw->finish(ZK_ETIMEOUT, queue_message(*raw->queue->h_status));
            return;
        }
        combine_all<C>(c, raw->pipes, out_xy, out_is_inf, /*record=*/false);
        raw->finish(ZK_OK, "");
    });
    *out = a.release();
    return ZK_OK;
}

int msm_batch_submit(Ctx* c, const MsmJob* jobs, size_t count, int scalars_mont, uint32_t window_bits, bool g2,
                     uint8_t* out_xy, int32_t* out_is_inf, MsmAsync** out) {
    *out = nullptr;
    if (g2) return batch_submit<CurveG2>(c, jobs, count, scalars_mont, window_bits, out_xy, out_is_inf, out);
    return batch_submit<CurveG1>(c, jobs, count, scalars_mont, window_bits, out_xy, out_is_inf, out);
}

// ZK_OK once the results are written, ZK_ETIMEOUT if timeout_ms (>= 0) passed first
// (negative: wait without a limit), else the batch's error.
int msm_batch_wait(MsmAsync* a, int timeout_ms) {
    std::unique_lock<std::mutex> g(a->mu);
    if (timeout_ms < 0) {
        a->cv.wait(g, [a] { return a->done; });
    } else if (!a->cv.wait_for(g, std::chrono::milliseconds(timeout_ms), [a] { return a->done; })) {
        set_error("MSM batch still running");
        return ZK_ETIMEOUT;
    }
    if (a->rc != ZK_OK) set_error(a->error);
    return a->rc;
}

void msm_batch_release(MsmAsync* a) {
    if (a == nullptr) return;
    {
        std::unique_lock<std::mutex> g(a->mu);
        a->cv.wait(g, [a] { return a->done; });
    }
    delete a;
}

int msm_batch_run(Ctx* c, const MsmJob* jobs, size_t count, int scalars_mont, uint32_t window_bits, uint8_t* out_xy,
                  int32_t* out_is_inf) {
    return batch_run<CurveG1>(c, jobs, count, scalars_mont, window_bits, out_xy, out_is_inf);
}

int msm_g2_batch_run(Ctx* c, const MsmJob* jobs, size_t count, int scalars_mont, uint32_t window_bits,
                     uint8_t* out_xy, int32_t* out_is_inf) {
    return batch_run<CurveG2>(c, jobs, count, scalars_mont, window_bits, out_xy, out_is_inf);
}

int msm_run(Ctx* c, const affine_t* bases, const fe* scalars, size_t n, int scalars_mont, uint32_t window_bits,
            uint8_t out_xy[64], int* out_is_inf, const affine_t* shifted, uint32_t shifted_c, uint64_t stride,
            bool glv, bool inf_points) {
    MsmJob job;
    job.inf_points = inf_points;
    job.scalars = scalars;
    job.n = n;
    job.bases = bases;
    job.shifted = shifted;
    job.shifted_c = shifted_c;
    job.stride = stride;
    job.glv = glv;
    int32_t inf = 0;
    int rc = msm_batch_run(c, &job, 1, scalars_mont, window_bits, out_xy, &inf);
    *out_is_inf = inf;
    return rc;
}

// ---- batch plans: pipelines with plan-owned scalar slots and scratch, optionally replayed
// as one CUDA graph ------------------------------------------------------------------------
struct MsmPlan {
    std::vector<MsmPipeT<CurveG1>> pipes;
    std::vector<size_t> empty;
    std::vector<fe*> slots;  // device scalar slot of each job (null for empty jobs)
    size_t count = 0;
    int scalars_mont = 1;
    char* arena = nullptr;
    void* host = nullptr;  // pinned: targets and totals of every pipeline
    cudaGraphExec_t exec = nullptr;
    uint64_t kernels = 0;  // kernel launches per run
    std::unique_ptr<MsmQueueT<CurveG1>> queue;  // work-queue form
};

int msm_plan_create(Ctx* c, const MsmJob* jobs, size_t count, int scalars_mont, uint32_t window_bits, bool graph,
                    bool queue, MsmPlan** out) {
    std::unique_ptr<MsmPlan> plan(new MsmPlan());
    plan->count = count;
    plan->scalars_mont = scalars_mont;
    int rc = build_pipes<CurveG1>(c, jobs, count, window_bits, &plan->pipes, &plan->empty);
    if (rc != ZK_OK) return rc;
    if (queue && !plan->pipes.empty()) {
        plan->queue.reset(new MsmQueueT<CurveG1>());
        if ((rc = queue_plan<CurveG1>(c, plan->pipes, *plan->queue)) != ZK_OK) return rc;
    }
    // arena: scalar slots, then every pipeline's scratch
    std::vector<size_t> slot_at(count, 0);
    size_t bytes = 0;
    for (size_t j = 0; j < count; j++) {
        slot_at[j] = bytes;
        bytes += ((size_t)jobs[j].n * sizeof(fe) + 255) & ~(size_t)255;
    }
    std::vector<size_t> at(plan->pipes.size());
    size_t host_bytes = 0;
    for (size_t q = 0; q < plan->pipes.size(); q++) {
        at[q] = bytes;
        bytes += (pipe_layout(plan->pipes[q], nullptr) + 255) & ~(size_t)255;
        host_bytes += plan->pipes[q].host_elems() * sizeof(xyzz_t) + 16;
    }
    const size_t queue_at = bytes;
    if (plan->queue) {
        bytes += plan->queue->bytes;
        host_bytes += 16;  // the queue's status word
    }
    ZK_TRY_CUDA(cudaMalloc(reinterpret_cast<void**>(&plan->arena), bytes ? bytes : 16));
    cudaError_t he = cudaMallocHost(&plan->host, host_bytes ? host_bytes : 16);
    if (he != cudaSuccess) {
        cudaFree(plan->arena);
        set_error(std::string("cudaMallocHost: ") + cudaGetErrorString(he));
        return ZK_ENOMEM;
    }
    auto fail = [&](int code) {
        cudaStreamSynchronize(c->stream);
        cudaFree(plan->arena);
        cudaFreeHost(plan->host);
        return code;
    };
    plan->slots.assign(count, nullptr);
    for (size_t j = 0; j < count; j++)
        if (jobs[j].n) plan->slots[j] = reinterpret_cast<fe*>(plan->arena + slot_at[j]);
    char* hp = static_cast<char*>(plan->host);
    for (size_t q = 0; q < plan->pipes.size(); q++) {
        MsmPipeT<CurveG1>& p = plan->pipes[q];
        for (size_t k = 0; k < p.inst.size(); k++) p.inst[k].scalars = plan->slots[p.out_index[k]];
        pipe_layout(p, plan->arena + at[q]);
        p.h_tgt = reinterpret_cast<xyzz_t*>(hp);
        hp += p.host_elems() * sizeof(xyzz_t);
        p.h_total = reinterpret_cast<uint32_t*>(hp);
        hp += 16;
        const int urc = pipe_upload(c, p);
        if (urc != ZK_OK) return fail(urc);
    }
    if (plan->queue) {
        plan->queue->h_status = reinterpret_cast<uint32_t*>(hp);
        *plan->queue->h_status = 0;
        const int qrc = queue_fill<CurveG1>(c, plan->pipes, *plan->queue, plan->arena + queue_at);
        if (qrc != ZK_OK) return fail(qrc);
    }
    cudaError_t se = cudaStreamSynchronize(c->stream);
    if (se != cudaSuccess) {
        set_error(std::string("plan set-up: ") + cudaGetErrorString(se));
        return fail(ZK_ECUDA);
    }
    // kernels per run: counted from one enqueue (captured, or counted at run time)
    if (graph && !plan->pipes.empty()) {
        const bool prof_was = c->prof_on;
        const uint64_t launches_was = c->launches;
        const auto prof_was_map = c->prof;
        c->prof_on = false;
        if (int src = ensure_side_streams(c); src != ZK_OK) {
            c->prof_on = prof_was;
            return fail(src);
        }
        cudaError_t be = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
        if (be != cudaSuccess) {
            c->prof_on = prof_was;
            set_error(std::string("cudaStreamBeginCapture: ") + cudaGetErrorString(be));
            return fail(ZK_ECUDA);
        }
        int erc = ZK_OK;
        erc = enqueue_all<CurveG1>(c, plan->pipes, scalars_mont, false, plan->queue.get());
        cudaGraph_t g = nullptr;
        cudaError_t ee = cudaStreamEndCapture(c->stream, &g);
        plan->kernels = c->launches - launches_was;
        c->launches = launches_was;
        c->prof = prof_was_map;
        c->prof_on = prof_was;
        if (erc != ZK_OK || ee != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            if (erc == ZK_OK) set_error(std::string("cudaStreamEndCapture: ") + cudaGetErrorString(ee));
            return fail(erc != ZK_OK ? erc : ZK_ECUDA);
        }
        cudaError_t ie = cudaGraphInstantiate(&plan->exec, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) {
            set_error(std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ie));
            return fail(ZK_ECUDA);
        }
    }
    *out = plan.release();
    return ZK_OK;
}

int msm_plan_slot(MsmPlan* plan, size_t index, void** dev) {
    ZK_CHECK_ARG(index < plan->count, "plan instance index out of range");
    *dev = plan->slots[index];
    return ZK_OK;
}

uint64_t msm_plan_kernels(const MsmPlan* plan) { return plan->kernels; }

int msm_plan_run(Ctx* c, MsmPlan* plan, uint8_t* out_xy, int32_t* out_is_inf) {
    set_infinity(out_xy, out_is_inf, plan->empty);
    if (plan->pipes.empty()) return ZK_OK;
    if (plan->exec) {
        const int tok = prof_begin(c, "msm_plan_graph");
        ZK_TRY_CUDA(cudaGraphLaunch(plan->exec, c->stream));
        prof_end(c, tok);
        c->launches += plan->kernels - 1;  // prof_begin counted the graph launch as one
    } else {
        int rc = enqueue_all<CurveG1>(c, plan->pipes, plan->scalars_mont, false, plan->queue.get());
        if (rc != ZK_OK) {
            cudaStreamSynchronize(c->stream);
            return rc;
        }
    }
    ZK_TRY_CUDA(cudaStreamSynchronize(c->stream));
    if (plan->queue) {
        const int qrc = queue_check(*plan->queue->h_status);
        if (qrc != ZK_OK) return qrc;
    }
    combine_all<CurveG1>(c, plan->pipes, out_xy, out_is_inf);
    return ZK_OK;
}

void msm_plan_destroy(Ctx* c, MsmPlan* plan) {
    if (plan == nullptr) return;
    cudaStreamSynchronize(c->stream);
    if (plan->exec) cudaGraphExecDestroy(plan->exec);
    cudaFree(plan->arena);
    cudaFreeHost(plan->host);
    delete plan;
}

}  // namespace zk
