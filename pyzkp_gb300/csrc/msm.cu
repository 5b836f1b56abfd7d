// msm.cu -- BN254 G1 multi-scalar multiplication (Pippenger, signed digits, CSR buckets).
//
// Result semantics: the unique affine point sum_i s_i P_i, identical to
// crypto/msm/pippenger.py:10-64 and runtime/metal/msm.py:179-332 (metal_msm_g1_v2).
// The reference's Metal v2 pipeline is: signed-digit encode in Python
// (runtime/metal/msm.py:145-177), histogram / single-thread prefix sum / scatter
// into CSR (runtime/metal/ecc_source.py:437-496), one thread per bucket
// (:499-535), one thread per window reduce (:540-566), CPU Horner (msm.py:322-332).
//
// This pipeline (all on the device except the last ~W*13 point additions):
//  1. msm_digits_kernel   scalar -> W signed c-bit digits (|d| <= 2^(c-1)); CSR
//                         histogram with warp-aggregated atomics (__match_any_sync).
//  2. device scan         counters -> CSR row pointers (scan.cu).
//  3. msm_scatter_kernel  (window, |digit|) buckets: entry = point index | sign << 31.
//  4. msm_accumulate_*    equal-size segments of S entries per thread (load balanced
//                         even when one bucket holds 5% of all points); buckets wholly
//                         inside a segment are final; a bucket that straddles segment
//                         boundaries leaves partial sums that tree rounds over groups
//                         of 32 units merge, deciding "straddles" from the row pointers.
//  5. msm_bucket_blocks   per window, blocks of g buckets: sum_b b*B_b = sum_j E_j + g*WS(Y)
//                         with Y_j the block sums and E_j = -(sum of the g-1 prefix sums).
//  6. msm_targets_kernel  WS(Y) = sum_j Y_j + sum_k 2^k M_k with M_k the sum of the Y_j
//                         whose index has bit k set: plain sums, reduced by CTA trees.
//  7. host: per window S_w = T_E + g (T_Y + sum_k 2^k M_k), then Horner over windows.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <vector>

#include "zk_internal.cuh"

namespace zk {

int device_exclusive_scan(Ctx* c, uint32_t* data, size_t n, uint32_t* total);

static constexpr uint32_t kNone = 0xffffffffu;
#ifndef ZK_MSM_SEGMENT
#define ZK_MSM_SEGMENT 32
#endif
#ifndef ZK_MSM_BLOCKG
#define ZK_MSM_BLOCKG 8
#endif
static constexpr uint32_t kSegment = ZK_MSM_SEGMENT;  // entries per thread in the first accumulation round
static constexpr uint32_t kFirstGroup = 2;            // units merged per thread in the first merge round
static constexpr uint32_t kGroup = 16;                // units merged per thread in later rounds
static constexpr uint32_t kBlockG = ZK_MSM_BLOCKG;    // buckets per block in the window reduction
static constexpr int kTargetThreads = 256;

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
    uint32_t Wr;       // bucket sets to reduce: W, or 1 in fixed-base mode
    uint32_t stride;   // fixed-base mode: row stride of the shifted-bases array
};

static MsmShape make_shape(uint32_t c) {
    MsmShape s;
    s.c = c;
    s.W = (255 + c - 1) / c;  // W*c >= 255 so the top window never carries out (scalars < r < 2^254)
    s.B = 1u << (c - 1);
    s.g = std::min<uint32_t>(kBlockG, s.B);
    s.G = s.B / s.g;
    s.g2 = s.G >= 16 ? kBlockG : 1;
    s.G2 = s.G / s.g2;
    s.K = 0;
    while ((1u << s.K) < s.G2) s.K++;
    s.plain = s.g2 > 1 ? 3 : 2;
    s.targets = s.plain + s.K;
    s.shared = 0;
    s.Wr = s.W;
    s.stride = 0;
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

// ---- 1. digits + histogram ----------------------------------------------------
__device__ __forceinline__ uint32_t bits_at(const fe& s, uint32_t k, uint32_t c) {
    const uint32_t limb = k >> 5, off = k & 31;
    uint64_t v = s.v[limb];
    if (limb + 1 < 8) v |= (uint64_t)s.v[limb + 1] << 32;
    // c <= 20 and off <= 31 keep off + c <= 51 bits: two limbs always suffice
    return (uint32_t)((v >> off) & ((1ull << c) - 1));
}

__device__ __forceinline__ void warp_aggregated_inc(uint32_t* counters, uint32_t key, bool active) {
    const uint32_t live = __ballot_sync(0xffffffffu, active);
    if (!active) return;
    const uint32_t peers = __match_any_sync(live, key);
    const int leader = __ffs(peers) - 1;
    if ((int)(threadIdx.x & 31) == leader) atomicAdd(counters + key, (uint32_t)__popc(peers));
}

__global__ void msm_digits_kernel(const fe* __restrict__ scalars, const affine_t* __restrict__ bases, uint32_t n,
                                  int scalars_mont, MsmShape sh, uint32_t* __restrict__ digits,
                                  uint32_t* __restrict__ counts) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    fe s = fe_zero();
    if (valid) {
        s = fe_ldg(scalars + i);
        s = scalars_mont ? fe_from_mont<FrP>(s) : fe_from_mont<FrP>(fe_to_mont<FrP>(s));
        if (affine_is_inf(affine_load(bases + i))) s = fe_zero();
    }
    uint32_t carry = 0;
    const uint32_t half = 1u << (sh.c - 1);
    for (uint32_t w = 0; w < sh.W; w++) {
        uint32_t v = bits_at(s, w * sh.c, sh.c) + carry;
        uint32_t mag, neg;
        if (w + 1 < sh.W && v > half) {  // v in (2^(c-1), 2^c]: digit v - 2^c in [-2^(c-1)+1, 0]
            mag = (1u << sh.c) - v;
            neg = 1;
            carry = 1;
        } else {  // v in [0, 2^(c-1)] (the top window is at most 2^(c-1), see make_shape)
            mag = v;
            neg = 0;
            carry = 0;
        }
        const bool nz = valid && mag != 0;
        if (valid) digits[(size_t)w * n + i] = nz ? (mag | (neg << 31)) : 0u;
        warp_aggregated_inc(counts, (sh.shared ? 0u : w * sh.B) + (mag - 1), nz);
    }
}

// ---- 3. scatter into CSR ------------------------------------------------------
__global__ void msm_scatter_kernel(const uint32_t* __restrict__ digits, uint32_t n, MsmShape sh,
                                   uint32_t* __restrict__ cursor, uint32_t* __restrict__ entries,
                                   uint32_t* __restrict__ keys) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    for (uint32_t w = 0; w < sh.W; w++) {
        const uint32_t d = valid ? digits[(size_t)w * n + i] : 0u;
        const bool nz = d != 0;
        const uint32_t key = (sh.shared ? 0u : w * sh.B) + (d & 0x7fffffffu) - 1;
        const uint32_t point = sh.shared ? w * sh.stride + i : i;  // fixed-base: row w of the shifted bases
        const uint32_t live = __ballot_sync(0xffffffffu, nz);
        if (nz) {
            const uint32_t peers = __match_any_sync(live, key);
            const int lane = threadIdx.x & 31;
            const int leader = __ffs(peers) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(cursor + key, (uint32_t)__popc(peers));
            base = __shfl_sync(peers, base, leader);
            const uint32_t rank = __popc(peers & ((1u << lane) - 1));
            entries[base + rank] = point | (d & 0x80000000u);
            keys[base + rank] = key;
        }
    }
}

// ---- 4. accumulation ------------------------------------------------------------
// Emit the accumulated sum of `key` over entry range [e0, e1): final if the bucket
// lies inside the range, else into the unit's first (bucket began earlier) or last
// (bucket continues later) slot.
__device__ __forceinline__ void emit_piece(uint32_t key, const xyzz_t& acc, uint32_t e0, uint32_t e1,
                                           const uint32_t* __restrict__ row_ptr, xyzz_t* __restrict__ buckets,
                                           uint32_t* slot_keys, xyzz_t* slot_pts, uint32_t unit) {
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

__global__ void __launch_bounds__(128) msm_accumulate_kernel(const uint32_t* __restrict__ entries,
                                                             const uint32_t* __restrict__ keys,
                                                             const uint32_t* __restrict__ d_total,
                                                             const uint32_t* __restrict__ row_ptr,
                                                             const affine_t* __restrict__ bases, uint32_t units,
                                                             xyzz_t* __restrict__ buckets,
                                                             uint32_t* __restrict__ slot_keys,
                                                             xyzz_t* __restrict__ slot_pts) {
    const uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= units) return;
    slot_keys[2 * u] = kNone;
    slot_keys[2 * u + 1] = kNone;
    const uint32_t M = *d_total;
    const uint32_t e0 = u * kSegment;
    if (e0 >= M) return;
    const uint32_t e1 = min(e0 + kSegment, M);
    uint32_t cur = keys[e0];
    xyzz_t acc = xyzz_inf();
    for (uint32_t e = e0; e < e1; e++) {
        const uint32_t k = keys[e];
        if (k != cur) {
            emit_piece(cur, acc, e0, e1, row_ptr, buckets, slot_keys, slot_pts, u);
            cur = k;
            acc = xyzz_inf();
        }
        const uint32_t ent = entries[e];
        affine_t p = affine_load(bases + (ent & 0x7fffffffu));
        if (ent >> 31) p.y = fe_neg<FqP>(p.y);
        acc = xyzz_madd(acc, p.x, p.y);
    }
    emit_piece(cur, acc, e0, e1, row_ptr, buckets, slot_keys, slot_pts, u);
}

// Round r >= 2: unit u merges the slots of units [u*group, (u+1)*group) of the previous
// round, covering entries [u * span, (u+1) * span) (span = kSegment times the product of
// the group sizes so far). The first merge round uses pairs: most straddling buckets
// cross exactly one segment boundary, so that round carries nearly all the work.
__global__ void __launch_bounds__(128) msm_merge_kernel(const uint32_t* __restrict__ in_keys,
                                                        const xyzz_t* __restrict__ in_pts, uint32_t in_units,
                                                        uint32_t group, const uint32_t* __restrict__ d_total,
                                                        const uint32_t* __restrict__ row_ptr, uint64_t span,
                                                        uint32_t units, xyzz_t* __restrict__ buckets,
                                                        uint32_t* __restrict__ slot_keys,
                                                        xyzz_t* __restrict__ slot_pts) {
    const uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= units) return;
    slot_keys[2 * u] = kNone;
    slot_keys[2 * u + 1] = kNone;
    const uint64_t M = *d_total;
    const uint64_t e0l = (uint64_t)u * span;
    if (e0l >= M) return;
    const uint32_t e0 = (uint32_t)e0l;
    const uint32_t e1 = (uint32_t)min(e0l + span, M);
    const uint32_t s0 = 2 * u * group;
    const uint32_t s1 = min(2 * (u + 1) * group, 2 * in_units);
    uint32_t cur = kNone;
    xyzz_t acc = xyzz_inf();
    for (uint32_t s = s0; s < s1; s++) {
        const uint32_t k = in_keys[s];
        if (k == kNone) continue;
        if (k != cur) {
            if (cur != kNone) emit_piece(cur, acc, e0, e1, row_ptr, buckets, slot_keys, slot_pts, u);
            cur = k;
            acc = xyzz_inf();
        }
        acc = xyzz_add(acc, xyzz_load(in_pts + s));
    }
    if (cur != kNone) emit_piece(cur, acc, e0, e1, row_ptr, buckets, slot_keys, slot_pts, u);
}

// ---- 5. window reduction ----------------------------------------------------------------
// For points X_1..X_N with weights, WS(X) = sum_b b X_b. Blocks of g: X_{(j-1)g+u}, u = 1..g:
// WS(X) = sum_j E_j + g WS(Y), Y_j = block sum, E_j = -(s_1 + ... + s_{g-1}) with s_u the
// prefix sums inside the block (because sum_u u X_u = g Y_j - sum_{u<g} s_u). Applied
// twice (buckets -> Y1, E1 -> Y2, E2, F2 = block sums of E1), then WS(Y2) by plain sums:
// WS(Y2) = sum_j Y2_j + sum_k 2^k M_k, M_k = sum of Y2_j with bit k of (j - 1) set.
// Level 1: block j of window w holds buckets b = j*g + 1 .. j*g + g (stored at index b - 1).
__global__ void __launch_bounds__(128) msm_bucket_blocks_kernel(const xyzz_t* __restrict__ buckets, MsmShape sh,
                                                                xyzz_t* __restrict__ Y, xyzz_t* __restrict__ E) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= sh.Wr * sh.G) return;
    const xyzz_t* b = buckets + (size_t)t * sh.g;
    xyzz_t s = xyzz_inf();
    xyzz_t e = xyzz_inf();
    for (uint32_t u = 0; u < sh.g; u++) {
        s = xyzz_add(s, xyzz_load(b + u));
        if (u + 1 < sh.g) e = xyzz_add(e, s);
    }
    xyzz_store(Y + t, s);
    xyzz_store(E + t, xyzz_neg(e));
}

// Level 2 over (Y1, E1): Y2, E2 as above on Y1, and F2 = plain block sums of E1.
__global__ void __launch_bounds__(128) msm_bucket_blocks2_kernel(const xyzz_t* __restrict__ Y1,
                                                                 const xyzz_t* __restrict__ E1, MsmShape sh,
                                                                 xyzz_t* __restrict__ Y2, xyzz_t* __restrict__ E2,
                                                                 xyzz_t* __restrict__ F2) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= sh.Wr * sh.G2) return;
    const size_t base = (size_t)t * sh.g2;
    xyzz_t s = xyzz_inf();
    xyzz_t e = xyzz_inf();
    xyzz_t f = xyzz_inf();
    for (uint32_t u = 0; u < sh.g2; u++) {
        s = xyzz_add(s, xyzz_load(Y1 + base + u));
        if (u + 1 < sh.g2) e = xyzz_add(e, s);
        f = xyzz_add(f, xyzz_load(E1 + base + u));
    }
    xyzz_store(Y2 + t, s);
    xyzz_store(E2 + t, xyzz_neg(e));
    xyzz_store(F2 + t, f);
}

// ---- 6. plain sums per (window, target) ---------------------------------------------
// targets 0 .. plain-1: full sums of P0, P1 (, P2) over G2 entries per window;
// target plain + k: sum of Ylast_j over j with bit k set.
__global__ void __launch_bounds__(kTargetThreads) msm_targets_kernel(const xyzz_t* __restrict__ P0,
                                                                     const xyzz_t* __restrict__ P1,
                                                                     const xyzz_t* __restrict__ P2,
                                                                     const xyzz_t* __restrict__ Ylast, MsmShape sh,
                                                                     xyzz_t* __restrict__ out) {
    __shared__ xyzz_t red[kTargetThreads];
    const uint32_t w = blockIdx.x / sh.targets;
    const uint32_t tg = blockIdx.x % sh.targets;
    const bool bits = tg >= sh.plain;
    const xyzz_t* src = bits ? Ylast : (tg == 0 ? P0 : (tg == 1 ? P1 : P2));
    src += (size_t)w * sh.G2;
    const uint32_t count = bits ? sh.G2 / 2 : sh.G2;
    const uint32_t k = bits ? tg - sh.plain : 0;
    xyzz_t acc = xyzz_inf();
    for (uint32_t t = threadIdx.x; t < count; t += blockDim.x) {
        uint32_t j = t;
        if (bits) j = ((t >> k) << (k + 1)) | (1u << k) | (t & ((1u << k) - 1));
        acc = xyzz_add(acc, xyzz_load(src + j));
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (uint32_t off = blockDim.x / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) red[threadIdx.x] = xyzz_add(red[threadIdx.x], red[threadIdx.x + off]);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = red[0];
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

__global__ void __launch_bounds__(128) msm_shift_bases_kernel(const affine_t* __restrict__ bases, uint32_t n,
                                                              uint32_t c, uint32_t W, affine_t* __restrict__ out,
                                                              xyzz_t* __restrict__ tmp, fe* __restrict__ pref) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const affine_t p = affine_load(bases + i);
    fe_store(&out[i].x, p.x);
    fe_store(&out[i].y, p.y);
    if (affine_is_inf(p)) {
        for (uint32_t j = 1; j < W; j++) {
            fe_store(&out[(size_t)j * n + i].x, fe_zero());
            fe_store(&out[(size_t)j * n + i].y, fe_zero());
        }
        return;
    }
    xyzz_t q;
    q.X = p.x;
    q.Y = p.y;
    q.ZZ = fe_one<FqP>();
    q.ZZZ = fe_one<FqP>();
    fe run = fe_one<FqP>();
    for (uint32_t j = 1; j < W; j++) {
        for (uint32_t d = 0; d < c; d++) q = xyzz_dbl(q);
        xyzz_store(tmp + (size_t)j * n + i, q);
        fe_store(pref + (size_t)j * n + i, run);
        run = fe_mul<FqP>(run, fe_mul<FqP>(q.ZZ, q.ZZZ));
    }
    fe inv = fe_inverse_fermat<FqP>(run);
    for (uint32_t j = W - 1; j >= 1; j--) {
        const xyzz_t t = xyzz_load(tmp + (size_t)j * n + i);
        const fe zz_zzz = fe_mul<FqP>(t.ZZ, t.ZZZ);
        const fe I = fe_mul<FqP>(inv, fe_load(pref + (size_t)j * n + i));
        inv = fe_mul<FqP>(inv, zz_zzz);
        fe_store(&out[(size_t)j * n + i].x, fe_mul<FqP>(t.X, fe_mul<FqP>(t.ZZZ, I)));
        fe_store(&out[(size_t)j * n + i].y, fe_mul<FqP>(t.Y, fe_mul<FqP>(t.ZZ, I)));
    }
}

int shift_bases(Ctx* c, const affine_t* bases, size_t n, uint32_t window_bits, affine_t** out, uint32_t* windows) {
    ZK_CHECK_ARG(window_bits >= 4 && window_bits <= 20, "fixed-base window_bits must be 4..20");
    ZK_CHECK_ARG(n > 0 && n < (1ull << 31), "fixed-base precomputation needs 0 < n < 2^31");
    const MsmShape sh = make_shape(window_bits);
    ZK_CHECK_ARG((uint64_t)sh.W * n < (1ull << 31), "fixed-base rows exceed 31-bit entry indices");
    affine_t* rows = nullptr;
    xyzz_t* tmp = nullptr;
    fe* pref = nullptr;
    int rc = scratch_alloc(c, (size_t)sh.W * n * sizeof(affine_t), reinterpret_cast<void**>(&rows));
    if (rc != ZK_OK) return rc;
    if ((rc = scratch_alloc(c, (size_t)sh.W * n * sizeof(xyzz_t), reinterpret_cast<void**>(&tmp))) != ZK_OK ||
        (rc = scratch_alloc(c, (size_t)sh.W * n * sizeof(fe), reinterpret_cast<void**>(&pref))) != ZK_OK) {
        scratch_free(c, rows);
        scratch_free(c, tmp);
        return rc;
    }
    ZK_LAUNCH(c, "msm_shift_bases", msm_shift_bases_kernel, (unsigned)((n + 127) / 128), 128, 0, bases, (uint32_t)n,
              window_bits, sh.W, rows, tmp, pref);
    ZK_TRY_CUDA(cudaGetLastError());
    scratch_free(c, tmp);
    scratch_free(c, pref);
    *out = rows;
    *windows = sh.W;
    return ZK_OK;
}

// ---- host ---------------------------------------------------------------------------
static zkh::Xyzz to_host(const xyzz_t& d) {
    zkh::Xyzz h;
    std::memcpy(h.X.v, d.X.v, 32);
    std::memcpy(h.Y.v, d.Y.v, 32);
    std::memcpy(h.ZZ.v, d.ZZ.v, 32);
    std::memcpy(h.ZZZ.v, d.ZZZ.v, 32);
    return h;
}

static zkh::Xyzz host_dbl_n(zkh::Xyzz p, uint32_t times) {
    for (uint32_t i = 0; i < times; i++) p = zkh::xyzz_dbl(p);
    return p;
}

int msm_run(Ctx* c, const affine_t* bases, const fe* scalars, size_t n, int scalars_mont, uint32_t window_bits,
            uint8_t out_xy[64], int* out_is_inf, const affine_t* shifted, uint32_t shifted_c, uint64_t stride) {
    ZK_CHECK_ARG(n < (1ull << 31), "MSM size must be below 2^31 points");
    ZK_CHECK_ARG(window_bits == 0 || (window_bits >= 4 && window_bits <= 20), "window_bits must be 0 or 4..20");
    if (n == 0) {
        std::memset(out_xy, 0, 64);
        *out_is_inf = 1;
        return ZK_OK;
    }
    // fixed-base mode: the bases carry window-shifted rows [2^(c j)] P_i (zk_bases_precompute)
    const bool fixed = shifted != nullptr && (window_bits == 0 || window_bits == shifted_c);
    const uint32_t cbits = fixed ? shifted_c : (window_bits ? window_bits : msm_auto_window(n));
    MsmShape sh = make_shape(cbits);
    if (fixed) {
        sh.shared = 1;
        sh.Wr = 1;
        sh.stride = (uint32_t)stride;
        ZK_CHECK_ARG((uint64_t)sh.W * stride < (1ull << 31), "fixed-base rows exceed 31-bit entry indices");
    }
    const affine_t* acc_bases = fixed ? shifted : bases;
    const uint64_t nbuckets = (uint64_t)sh.Wr * sh.B;
    const uint64_t max_entries = (uint64_t)n * sh.W;
    ZK_CHECK_ARG(max_entries < (1ull << 32) - kSegment, "MSM too large for 32-bit CSR offsets");

    // scratch layout
    uint32_t *digits = nullptr, *row_ptr = nullptr, *cursor = nullptr, *entries = nullptr, *keys = nullptr;
    xyzz_t *buckets = nullptr, *Yb = nullptr, *Eb = nullptr, *Y2 = nullptr, *E2 = nullptr, *F2 = nullptr,
           *tgt = nullptr;
    std::vector<void*> allocs;
    auto alloc = [&](size_t bytes, void** p) -> int {
        int rc = scratch_alloc(c, bytes, p);
        if (rc == ZK_OK) allocs.push_back(*p);
        return rc;
    };
    auto release = [&]() {
        for (void* p : allocs) scratch_free(c, p);
        allocs.clear();
    };
    int rc;
    if ((rc = alloc(max_entries * 4, (void**)&digits)) != ZK_OK ||
        (rc = alloc((nbuckets + 1) * 4, (void**)&row_ptr)) != ZK_OK ||
        (rc = alloc(nbuckets * 4, (void**)&cursor)) != ZK_OK ||
        (rc = alloc(max_entries * 4, (void**)&entries)) != ZK_OK ||
        (rc = alloc(max_entries * 4, (void**)&keys)) != ZK_OK ||
        (rc = alloc(nbuckets * sizeof(xyzz_t), (void**)&buckets)) != ZK_OK ||
        (rc = alloc((size_t)sh.Wr * sh.G * sizeof(xyzz_t), (void**)&Yb)) != ZK_OK ||
        (rc = alloc((size_t)sh.Wr * sh.G * sizeof(xyzz_t), (void**)&Eb)) != ZK_OK ||
        (rc = alloc((size_t)sh.Wr * sh.G2 * sizeof(xyzz_t), (void**)&Y2)) != ZK_OK ||
        (rc = alloc((size_t)sh.Wr * sh.G2 * sizeof(xyzz_t), (void**)&E2)) != ZK_OK ||
        (rc = alloc((size_t)sh.Wr * sh.G2 * sizeof(xyzz_t), (void**)&F2)) != ZK_OK ||
        (rc = alloc((size_t)sh.Wr * sh.targets * sizeof(xyzz_t), (void**)&tgt)) != ZK_OK) {
        release();
        return rc;
    }
    cudaStream_t st = c->stream;
    ZK_TRY_CUDA(cudaMemsetAsync(row_ptr, 0, (nbuckets + 1) * 4, st));
    ZK_TRY_CUDA(cudaMemsetAsync(buckets, 0, nbuckets * sizeof(xyzz_t), st));

    const uint32_t nn = (uint32_t)n;
    ZK_LAUNCH(c, "msm_digits", msm_digits_kernel, (nn + 255) / 256, 256, 0, scalars, bases, nn, scalars_mont, sh, digits,
              row_ptr);
    ZK_TRY_CUDA(cudaGetLastError());
    // row_ptr[0..nbuckets) := exclusive scan; row_ptr[nbuckets] := total
    if ((rc = device_exclusive_scan(c, row_ptr, nbuckets, row_ptr + nbuckets)) != ZK_OK) {
        release();
        return rc;
    }
    ZK_TRY_CUDA(cudaMemcpyAsync(cursor, row_ptr, nbuckets * 4, cudaMemcpyDeviceToDevice, st));
    ZK_LAUNCH(c, "msm_scatter", msm_scatter_kernel, (nn + 255) / 256, 256, 0, digits, nn, sh, cursor, entries, keys);
    ZK_TRY_CUDA(cudaGetLastError());

    // accumulation rounds
    const uint32_t* d_total = row_ptr + nbuckets;
    uint32_t units = (uint32_t)((max_entries + kSegment - 1) / kSegment);
    uint32_t *slot_keys_a = nullptr, *slot_keys_b = nullptr;
    xyzz_t *slot_pts_a = nullptr, *slot_pts_b = nullptr;
    if ((rc = alloc((size_t)2 * units * 4, (void**)&slot_keys_a)) != ZK_OK ||
        (rc = alloc((size_t)2 * units * sizeof(xyzz_t), (void**)&slot_pts_a)) != ZK_OK ||
        (rc = alloc((size_t)2 * ((units + kFirstGroup - 1) / kFirstGroup) * 4, (void**)&slot_keys_b)) != ZK_OK ||
        (rc = alloc((size_t)2 * ((units + kFirstGroup - 1) / kFirstGroup) * sizeof(xyzz_t), (void**)&slot_pts_b)) !=
            ZK_OK) {
        release();
        return rc;
    }
    ZK_LAUNCH(c, "msm_accumulate", msm_accumulate_kernel, (units + 127) / 128, 128, 0, entries, keys, d_total, row_ptr,
              acc_bases, units, buckets, slot_keys_a, slot_pts_a);
    ZK_TRY_CUDA(cudaGetLastError());
    uint64_t span = kSegment;
    uint32_t in_units = units;
    uint32_t *ik = slot_keys_a, *ok = slot_keys_b;
    xyzz_t *ip = slot_pts_a, *op = slot_pts_b;
    uint32_t group = kFirstGroup;
    while (in_units > 1) {
        const uint32_t out_units = (in_units + group - 1) / group;
        span *= group;
        ZK_LAUNCH(c, group == kFirstGroup ? "msm_merge_pairs" : "msm_merge", msm_merge_kernel, (out_units + 127) / 128,
                  128, 0, ik, ip, in_units, group, d_total, row_ptr, span, out_units, buckets, ok, op);
        ZK_TRY_CUDA(cudaGetLastError());
        std::swap(ik, ok);
        std::swap(ip, op);
        in_units = out_units;
        group = kGroup;
    }

    // window reduction
    const uint32_t nblk = sh.Wr * sh.G;
    ZK_LAUNCH(c, "msm_bucket_blocks", msm_bucket_blocks_kernel, (nblk + 127) / 128, 128, 0, buckets, sh, Yb, Eb);
    ZK_TRY_CUDA(cudaGetLastError());
    if (sh.g2 > 1) {
        const uint32_t nblk2 = sh.Wr * sh.G2;
        ZK_LAUNCH(c, "msm_bucket_blocks2", msm_bucket_blocks2_kernel, (nblk2 + 127) / 128, 128, 0, Yb, Eb, sh, Y2, E2,
                  F2);
        ZK_TRY_CUDA(cudaGetLastError());
        ZK_LAUNCH(c, "msm_targets", msm_targets_kernel, sh.Wr * sh.targets, kTargetThreads, 0, F2, E2, Y2, Y2, sh, tgt);
    } else {
        ZK_LAUNCH(c, "msm_targets", msm_targets_kernel, sh.Wr * sh.targets, kTargetThreads, 0, Eb, Yb, Yb, Yb, sh, tgt);
    }
    ZK_TRY_CUDA(cudaGetLastError());
    std::vector<xyzz_t> host_t((size_t)sh.Wr * sh.targets);
    uint32_t total_entries = 0;
    ZK_TRY_CUDA(cudaMemcpyAsync(host_t.data(), tgt, host_t.size() * sizeof(xyzz_t), cudaMemcpyDeviceToHost, st));
    ZK_TRY_CUDA(cudaMemcpyAsync(&total_entries, d_total, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    ZK_TRY_CUDA(cudaStreamSynchronize(st));
    release();
    c->msm_entries = total_entries;
    c->msm_window_bits = sh.c;
    c->msm_windows = sh.W;

    // host: one level   S_w = T0 + g (T1 + H)            (T0 = sum E1, T1 = sum Y1)
    //       two levels  S_w = T0 + g (T1 + g2 (T2 + H))  (T0 = sum F2 = sum E1, T1 = sum E2, T2 = sum Y2)
    // with H = sum_k 2^k M_k (Horner); then total = sum_w 2^(c w) S_w (Horner over windows).
    const auto t_host0 = std::chrono::steady_clock::now();
    uint32_t log_g = 0, log_g2 = 0;
    while ((1u << log_g) < sh.g) log_g++;
    while ((1u << log_g2) < sh.g2) log_g2++;
    zkh::Xyzz total = zkh::xyzz_inf();
    for (int w = (int)sh.Wr - 1; w >= 0; w--) {
        const xyzz_t* T = host_t.data() + (size_t)w * sh.targets;
        zkh::Xyzz h = zkh::xyzz_inf();
        for (int k = (int)sh.K - 1; k >= 0; k--) {
            h = zkh::xyzz_dbl(h);
            h = zkh::xyzz_add(h, to_host(T[sh.plain + k]));
        }
        zkh::Xyzz sw = zkh::xyzz_add(h, to_host(T[sh.plain - 1]));
        if (sh.plain == 3) {
            sw = host_dbl_n(sw, log_g2);
            sw = zkh::xyzz_add(sw, to_host(T[1]));
        }
        sw = host_dbl_n(sw, log_g);
        sw = zkh::xyzz_add(sw, to_host(T[0]));
        total = host_dbl_n(total, sh.c);
        total = zkh::xyzz_add(total, sw);
    }
    prof_host(c, "msm_host_combine",
              std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_host0).count());
    zkh::F4 x, y;
    *out_is_inf = zkh::xyzz_to_affine_canonical(total, &x, &y) ? 1 : 0;
    std::memcpy(out_xy, x.v, 32);
    std::memcpy(out_xy + 32, y.v, 32);
    return ZK_OK;
}

}  // namespace zk
