// ntt.cu -- Fr NTT / iNTT / coset NTT for sm_103a.
//
// Semantics: crypto/poly/ntt.py:103-146 (the transforms behind the ROOTS_* and
// COSET_* ops, runtime/kernels/cpu/kernels.py:175-250). Natural order in and out.
//
// Algorithm: radix-2^k Stockham autosort passes. With n = R_1 R_2 ... R_P and
// L = R_1 ... R_{p-1} before pass p, pass p computes, for every column
// c = j L + k (j < n/(R L), k < L) and m, q < R:
//     y_m = in[c + m n/R] * w_{RL}^(m k),   z_q = sum_m y_m w_R^(m q),
//     out[j R L + k + q L] = z_q,
// where w_N = omega^(n/N). Radix 2 with n/2 threads per pass is the reference's
// Metal v2 (runtime/metal/runtime.py:336-362); here one CTA runs a whole radix-R
// column group in shared memory (R up to 2^11) so a 2^22 transform makes two HBM
// round trips instead of 22. Inside the CTA the R-point DFT is a decimation-in-
// frequency sequence of radix-2 stages in place in shared memory, read back in
// bit-reversed order. Coset scaling (shift^g) is applied while loading the first
// pass and the inverse scale (n^-1 shift^-i) while storing the last pass.
//
// Shared memory holds each 32-byte element as two 16-byte planes (low/high limbs)
// so that eight consecutive elements cover all 32 banks; element positions are
// XOR-swizzled so the bit-reversed read-back does not hit one bank group.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>

#include "zk_internal.cuh"

namespace zk {

static constexpr int kNttThreads = 256;
#ifndef ZK_NTT_MINB
// resident CTAs per SM the single-transform pass kernel is compiled for: 2 (up to 128
// registers) against 3 (85: the radix-4 steps then spill ~80 bytes) measured on GB300 with
// radix-4 steps: 2^20 0.282 / 0.292 ms, 2^22 1.222 / 1.234 ms, 2^12 0.022 / 0.023 ms
#define ZK_NTT_MINB 2
#endif
#ifndef ZK_NTT_BATCH_MINB
// ... and the batch and queue kernels: their many small tiles (256-element tiles of 128
// active threads) want the third CTA per SM (64 coset NTTs of 2^10..2^20: 2.87 ms at 3,
// 3.00 ms at 2)
#define ZK_NTT_BATCH_MINB 3
#endif
static constexpr int kMaxLogR = 11;       // 2048 elements * 32 B = 64 KB of shared memory
static constexpr int kTileLogElems = 11;  // largest tile: R * T = 2048 elements per CTA
// Default tile: 2^8 elements per CTA, or one radix-R column when R is larger. Measured on
// GB300 (forward NTT, L2 flushed): 2^12 74 -> 22 us, 2^16 91 -> 34 us, 2^20 333 -> 298 us
// against 2^11-element tiles; tiles of 2^6..2^8 are within 5% of one another at every size.
static constexpr int kDefaultTileLog = 8;

struct NttPassParams {
    const fe* in;
    fe* out;
    const fe* radix_tw;  // w_R^i, i < R/2
    const fe* tw_lo;
    const fe* tw_hi;
    const fe* pre_lo;
    const fe* pre_hi;
    const fe* post_lo;
    const fe* post_hi;
    uint32_t in_len;  // valid input elements (first pass), <= n
    uint32_t log_n;
    uint32_t log_r;
    uint32_t log_t;
    uint32_t log_l;
    uint32_t s_bits;
    uint32_t last;  // 1 on the last pass: outputs reduced to [0, r)
    uint32_t reduce_in;  // 1 on the first pass of a transform of canonical values: inputs of any
                         // 256 bits brought into [0, 2r) as they are loaded
};

// Butterflies, twiddles and scales run on lazy Fr values in [0, 2r) (FrLazyP); inputs are
// canonical, intermediate passes store lazy values, the last pass stores canonical ones.
using FrN = FrLazyP;

__device__ __forceinline__ fe lookup2(const fe* lo, const fe* hi, uint32_t e, uint32_t s_bits) {
    if (s_bits == kNttFullTable) return fe_ldg(lo + e);
    fe a = fe_ldg(lo + (e & ((1u << s_bits) - 1)));
    uint32_t h = e >> s_bits;
    if (h == 0) return a;
    return fe_mul<FrN>(a, fe_ldg(hi + h));
}

__device__ __forceinline__ uint32_t swz(uint32_t pos, uint32_t log_r) {
    return log_r >= 6 ? (pos ^ ((pos >> (log_r - 3)) & 7u)) : pos;
}

__device__ __forceinline__ fe smem_get(const uint4* s_lo, const uint4* s_hi, uint32_t i) {
    uint4 a = s_lo[i], b = s_hi[i];
    fe r;
    r.v[0] = a.x;
    r.v[1] = a.y;
    r.v[2] = a.z;
    r.v[3] = a.w;
    r.v[4] = b.x;
    r.v[5] = b.y;
    r.v[6] = b.z;
    r.v[7] = b.w;
    return r;
}

__device__ __forceinline__ void smem_put(uint4* s_lo, uint4* s_hi, uint32_t i, const fe& v) {
    s_lo[i] = make_uint4(v.v[0], v.v[1], v.v[2], v.v[3]);
    s_hi[i] = make_uint4(v.v[4], v.v[5], v.v[6], v.v[7]);
}

// One CTA's tile `tile` of one pass (shared by the single-transform, the batch and the
// queue kernel). l2_in: the pass input was written earlier in the same launch (a runtime
// flag rather than a template argument: one copy of the body in the queue kernel).
__device__ __forceinline__ void ntt_pass_body(const NttPassParams& P, uint32_t tile, uint4* smem,
                                              bool l2_in = false) {
    const uint32_t log_r = P.log_r, log_t = P.log_t;
    const uint32_t R = 1u << log_r, T = 1u << log_t, E = R << log_t;
    uint4* s_lo = smem;
    uint4* s_hi = smem + E;
    const uint32_t c0 = tile << log_t;
    const uint32_t stride_log = P.log_n - log_r;
    const uint32_t l_mask = (1u << P.log_l) - 1;
    const uint32_t tw_shift = P.log_n - log_r - P.log_l;

    // ---- load (+ coset scale on the first pass, + inter-pass twiddle) ----
    for (uint32_t idx = threadIdx.x; idx < E; idx += blockDim.x) {
        const uint32_t m = idx >> log_t, t = idx & (T - 1);
        const uint32_t col = c0 + t;
        const uint32_t g = col + (m << stride_log);
        fe v = g < P.in_len ? (l2_in ? fe_ldcg(P.in + g) : fe_ldg(P.in + g)) : fe_zero();
        if (P.reduce_in) v = fe_reduce_2p<FrN>(fe_reduce_4p<FrN>(v));
        if (P.pre_lo != nullptr && g < P.in_len) v = fe_mul<FrN>(v, lookup2(P.pre_lo, P.pre_hi, g, P.s_bits));
        if (P.log_l != 0) {
            const uint32_t e = (m * (col & l_mask)) << tw_shift;
            if (e != 0) v = fe_mul<FrN>(v, lookup2(P.tw_lo, P.tw_hi, e, P.s_bits));
        }
        smem_put(s_lo, s_hi, (swz(m, log_r) << log_t) + t, v);
    }
    __syncthreads();

    // ---- R-point DFT per column: DIF stages in shared memory ----
    // Pairs of radix-2 stages (st, st + 1) run as one radix-4 step: for j < h/2 (h = the
    // half-size of stage st) the elements i0, i0 + h/2, i0 + h, i0 + 3h/2 of a block of 2h
    // are closed under both stages, so one thread loads four, applies the four butterflies
    // (the same products as two radix-2 stages) and stores four: half the shared-memory
    // round trips, index computations and barriers. An odd stage count ends radix-2.
    uint32_t st0 = 0;
#ifndef ZK_NTT_RADIX2
    // only while every thread has a radix-4 step: small tiles (E / 4 < blockDim) keep the
    // radix-2 stages and all their threads busy (2^16 in 2^8-element tiles: 0.047 ms with
    // radix-4 steps, 0.035 ms with radix-2)
    for (; st0 + 1 < log_r && (E >> 2) >= blockDim.x; st0 += 2) {
        const uint32_t log_h = log_r - st0 - 1;  // stage st0 pairs (x, x + h)
        const uint32_t h = 1u << log_h, hq = h >> 1;
        for (uint32_t qi = threadIdx.x; qi < (E >> 2); qi += blockDim.x) {
            const uint32_t t = qi & (T - 1), b = qi >> log_t;
            const uint32_t j = b & (hq - 1);
            const uint32_t i0 = ((b >> (log_h - 1)) << (log_h + 1)) + j;
            const uint32_t a0 = (swz(i0, log_r) << log_t) + t;
            const uint32_t a1 = (swz(i0 + hq, log_r) << log_t) + t;
            const uint32_t a2 = (swz(i0 + h, log_r) << log_t) + t;
            const uint32_t a3 = (swz(i0 + h + hq, log_r) << log_t) + t;
            const fe x0 = smem_get(s_lo, s_hi, a0), x1 = smem_get(s_lo, s_hi, a1);
            const fe x2 = smem_get(s_lo, s_hi, a2), x3 = smem_get(s_lo, s_hi, a3);
            // stage st0: (x0, x2) with twiddle index j, (x1, x3) with j + h/2
            const fe p0 = fe_add<FrN>(x0, x2);
            fe p2 = fe_sub<FrN>(x0, x2);
            if (j != 0) p2 = fe_mul<FrN>(p2, fe_ldg(P.radix_tw + (j << st0)));
            const fe p1 = fe_add<FrN>(x1, x3);
            const fe p3 = fe_mul<FrN>(fe_sub<FrN>(x1, x3), fe_ldg(P.radix_tw + ((j + hq) << st0)));
            // stage st0 + 1: (p0, p1) and (p2, p3), twiddle index j
            fe q1 = fe_sub<FrN>(p0, p1), q3 = fe_sub<FrN>(p2, p3);
            if (j != 0) {
                const fe w = fe_ldg(P.radix_tw + (j << (st0 + 1)));
                q1 = fe_mul<FrN>(q1, w);
                q3 = fe_mul<FrN>(q3, w);
            }
            smem_put(s_lo, s_hi, a0, fe_add<FrN>(p0, p1));
            smem_put(s_lo, s_hi, a1, q1);
            smem_put(s_lo, s_hi, a2, fe_add<FrN>(p2, p3));
            smem_put(s_lo, s_hi, a3, q3);
        }
        __syncthreads();
    }
#endif
    for (uint32_t st = st0; st < log_r; st++) {
        const uint32_t log_h = log_r - st - 1;
        const uint32_t h = 1u << log_h;
        for (uint32_t bi = threadIdx.x; bi < (E >> 1); bi += blockDim.x) {
            const uint32_t t = bi & (T - 1), b = bi >> log_t;
            const uint32_t j = b & (h - 1);
            const uint32_t i0 = ((b >> log_h) << (log_h + 1)) + j;
            const uint32_t a0 = (swz(i0, log_r) << log_t) + t;
            const uint32_t a1 = (swz(i0 + h, log_r) << log_t) + t;
            fe u = smem_get(s_lo, s_hi, a0);
            fe v = smem_get(s_lo, s_hi, a1);
            fe sum = fe_add<FrN>(u, v);
            fe diff = fe_sub<FrN>(u, v);
            if (j != 0) diff = fe_mul<FrN>(diff, fe_ldg(P.radix_tw + (j << st)));
            smem_put(s_lo, s_hi, a0, sum);
            smem_put(s_lo, s_hi, a1, diff);
        }
        __syncthreads();
    }

    // ---- store z_q (at bit-reversed position), + final scale on the last pass ----
    for (uint32_t idx = threadIdx.x; idx < E; idx += blockDim.x) {
        uint32_t q, t;
        if (P.log_l == 0) {  // output of the tile is one contiguous block: walk q fastest
            q = idx & (R - 1);
            t = idx >> log_r;
        } else {  // runs of T consecutive columns: walk t fastest
            q = idx >> log_t;
            t = idx & (T - 1);
        }
        const uint32_t col = c0 + t;
        const uint32_t pos = log_r ? (__brev(q) >> (32 - log_r)) : 0;
        fe val = smem_get(s_lo, s_hi, (swz(pos, log_r) << log_t) + t);
        const uint32_t o = ((col >> P.log_l) << (log_r + P.log_l)) + (col & l_mask) + (q << P.log_l);
        if (P.post_lo != nullptr) {
            fe s = P.post_hi != nullptr ? lookup2(P.post_lo, P.post_hi, o, P.s_bits) : fe_ldg(P.post_lo);
            val = fe_mul<FrN>(val, s);
        }
        if (P.last) val = fe_reduce_once<FrP>(val);
        fe_store(P.out + o, val);
    }
}

__global__ void __launch_bounds__(kNttThreads, ZK_NTT_MINB) ntt_pass_kernel(NttPassParams P) {
    extern __shared__ uint4 smem[];
    ntt_pass_body(P, blockIdx.x, smem);
}

// Batch: one launch runs the same pass level of many transforms. CTA b runs tile
// b - first_tile[i] of item i, the largest i with first_tile[i] <= b; the item's
// parameters are staged in shared memory once per CTA.
__global__ void __launch_bounds__(kNttThreads, ZK_NTT_BATCH_MINB) ntt_pass_batch_kernel(const NttPassParams* __restrict__ items,
                                                                       const uint32_t* __restrict__ first_tile,
                                                                       uint32_t nitems) {
    extern __shared__ uint4 smem[];
    __shared__ NttPassParams sP;
    __shared__ uint32_t s_tile;
    if (threadIdx.x == 0) {
        uint32_t lo = 0, hi = nitems;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (first_tile[mid] <= blockIdx.x) lo = mid;
            else hi = mid;
        }
        sP = items[lo];
        s_tile = blockIdx.x - first_tile[lo];
    }
    __syncthreads();
    ntt_pass_body(sP, s_tile, smem);
}

// ---- persistent launch from a device work queue --------------------------------------------
// The queue is the list of (transform, pass) entries in queue order; entry e owns the items
// [first, first + tiles), one per tile of that pass. Every CTA of one launch takes items from
// a ticket counter until the queue is empty. An item of pass p > 0 waits until `need` tiles of
// the transform's pass p - 1 (entry `dep`) have finished: entries are ordered pass level by
// pass level (the largest transforms first within a level), so every item waited on was
// taken earlier by a running CTA, whose own dependencies were taken earlier still -- the
// earliest unfinished item never waits, and the launch cannot deadlock whatever the number
// of resident CTAs. A transform's pass p + 1 starts as soon as its own pass p is done, while
// other transforms are still in pass p (no launch boundary between levels).
struct NttQueueEntry {
    NttPassParams P;
    uint32_t first;  // first item of the entry in queue order
    uint32_t tiles;  // items (CTAs of the pass)
    int32_t dep;     // entry of the transform's previous pass, -1 for a first pass
    uint32_t need;   // finished items of `dep` to wait for (its tiles)
};


// Entries whose first items are cached in shared memory for the item lookup (more entries:
// the lookup reads the global table).
static constexpr uint32_t kQueueSmemEntries = 1024;
static constexpr uint32_t kNone32 = 0xffffffffu;


__global__ void __launch_bounds__(kNttThreads, ZK_NTT_BATCH_MINB) ntt_queue_kernel(const NttQueueEntry* __restrict__ entries,
                                                                  uint32_t nentries, uint32_t nitems,
                                                                  uint32_t* state,
                                                                  const uint64_t* __restrict__ limit,
                                                                  uint32_t* sticky) {
    extern __shared__ uint4 smem[];
    __shared__ NttQueueEntry sE;
    __shared__ uint32_t s_first[kQueueSmemEntries];
    __shared__ uint32_t s_next, s_item, s_entry, s_tile, s_stop;
    volatile uint32_t* vstate = state;
    const bool cached = nentries <= kQueueSmemEntries;
    if (cached)
        for (uint32_t e = threadIdx.x; e < nentries; e += blockDim.x) s_first[e] = entries[e].first;
    if (threadIdx.x == 0) s_next = queue_ticket(state, nitems);
    __syncthreads();
    uint32_t finished = kNone32;  // warp 1, lane 0: the entry of the tile this CTA just finished
    for (;;) {
        if (threadIdx.x < 32) {  // warp 0: find the next item's entry, copy it, wait for its dependency
            const uint32_t item = s_next;
            uint32_t e = 0;
            if (threadIdx.x == 0 && item < nitems) {
                uint32_t lo = 0, hi = nentries;  // the entry holding `item`: largest e with first <= item
                while (hi - lo > 1) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if ((cached ? s_first[mid] : entries[mid].first) <= item) lo = mid;
                    else hi = mid;
                }
                e = lo;
            }
            e = __shfl_sync(0xffffffffu, e, 0);
            constexpr uint32_t kWords = sizeof(NttQueueEntry) / 4;
            static_assert(kWords <= 32 && sizeof(NttQueueEntry) % 4 == 0, "queue entry copy by one warp");
            if (item < nitems && threadIdx.x < kWords)
                reinterpret_cast<uint32_t*>(&sE)[threadIdx.x] =
                    reinterpret_cast<const uint32_t*>(entries + e)[threadIdx.x];
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
                        __threadfence();  // acquire: the previous pass's outputs before our loads
                    }
                }
            }
        } else if (threadIdx.x == 32 && finished != kNone32) {
            // warp 1 publishes the finished tile while warp 0 looks up the next item
            __threadfence();  // release: the tile's outputs (ordered by the barrier) before the counter
            atomicAdd(state + kQueueDone + finished, 1u);
        }
        __syncthreads();
        if (s_item >= nitems || s_stop) return;
        if (threadIdx.x == 32) finished = s_entry;
        // the next item's ticket now: its latency hides behind this tile. The item is taken
        // only after this one's dependency is met, which keeps the earliest unfinished item
        // always runnable.
        uint32_t nxt = 0;
        if (threadIdx.x == 0) nxt = queue_ticket(state, nitems);
        ntt_pass_body(sE.P, s_tile, smem, sE.dep >= 0);
        __syncthreads();  // every store of the tile issued; sE and s_tile free again
        if (threadIdx.x == 0) s_next = nxt;
    }
}

// full[e] = lo[e mod 2^s] hi[e >> s] for e < n: a two-level table flattened into one
// (canonical Montgomery values), so that a pass reads each factor with one load.
__global__ void ntt_expand_table_kernel(fe* __restrict__ full, const fe* __restrict__ lo, const fe* __restrict__ hi,
                                        uint32_t s_bits, uint32_t n) {
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        fe a = fe_ldg(lo + (e & ((1u << s_bits) - 1)));
        const uint32_t h = e >> s_bits;
        if (h != 0) a = fe_mul<FrP>(a, fe_ldg(hi + h));
        fe_store(full + e, a);
    }
}

// ------------------------------------------------------------------------------
// host side: plans and launches
// ------------------------------------------------------------------------------
// Plans up to 2^kFullTableMaxLog keep full tables (n * 32 bytes per table, at most three
// per plan) while the context holds less than kFullTableBudget bytes of them; larger or
// later plans keep the two-level split (a second load and a product per factor).
static constexpr uint32_t kFullTableMaxLog = 22;
static constexpr size_t kFullTableBudget = (size_t)8 << 30;
static zkh::F4 load_canon(const uint8_t b[32]) {
    zkh::F4 r;
    std::memcpy(r.v, b, 32);
    return r;
}

static int upload_table(Ctx* c, NttPlan* plan, const std::vector<zkh::F4>& v, fe** out) {
    void* p = nullptr;
    ZK_TRY_CUDA(cudaMalloc(&p, v.size() * 32));
    plan->allocations.push_back(p);
    ZK_TRY_CUDA(cudaMemcpyAsync(p, v.data(), v.size() * 32, cudaMemcpyHostToDevice, c->stream));
    *out = static_cast<fe*>(p);
    return ZK_OK;
}

// powers base^i for i < count (Montgomery)
static std::vector<zkh::F4> powers(const zkh::F4& base, size_t count) {
    const zkh::Field& F = zkh::fr();
    std::vector<zkh::F4> v(count);
    zkh::F4 cur = zkh::one(F);
    for (size_t i = 0; i < count; i++) {
        v[i] = cur;
        cur = zkh::mul(F, cur, base);
    }
    return v;
}

// Radix bits per pass: the tuned split for log_n when one is set (bits summing to log_n,
// each 1..11), else the fewest passes of at most 11 bits, as equal as possible.
static void split_passes(uint32_t log_n, NttPlan* plan, const uint8_t* tuned = nullptr) {
    if (log_n == 0) {
        plan->npass = 0;
        return;
    }
    if (tuned != nullptr && tuned[0] != 0) {
        int np = 0;
        for (int p = 0; p < 4 && tuned[p] != 0; p++) plan->pass_log_r[np++] = tuned[p];
        plan->npass = np;
        return;
    }
    int np = (int)((log_n + kMaxLogR - 1) / kMaxLogR);
    if (np < 1) np = 1;
    uint32_t base = log_n / np, extra = log_n % np;
    plan->npass = np;
    for (int p = 0; p < np; p++) plan->pass_log_r[p] = base + ((uint32_t)p < extra ? 1u : 0u);
}

static int build_plan(Ctx* c, int mode, uint32_t log_n, const zkh::F4& omega_m, const zkh::F4& shift_m,
                      NttPlan** out) {
    const zkh::Field& F = zkh::fr();
    NttPlan* plan = new NttPlan();
    plan->log_n = log_n;
    split_passes(log_n, plan, c->tune_ntt_split[log_n]);
    const bool inverse = (mode == ZK_NTT_COEFFS_FROM_EVALS || mode == ZK_NTT_COSET_COEFFS_FROM_EVALS);
    const zkh::F4 w = inverse ? zkh::inv(F, omega_m) : omega_m;
    const uint64_t n = 1ull << log_n;
    plan->s_bits = (log_n + 1) / 2;
    const uint64_t lo_count = 1ull << plan->s_bits;
    const uint64_t hi_count = (n >> plan->s_bits) + 1;
    int rc;
    // two-level twiddle table: w^i and w^(i 2^s)
    {
        std::vector<zkh::F4> lo = powers(w, lo_count);
        zkh::F4 ws = zkh::pow_u64(F, w, lo_count);
        std::vector<zkh::F4> hi = powers(ws, hi_count);
        if ((rc = upload_table(c, plan, lo, &plan->tw_lo)) != ZK_OK) return rc;
        if ((rc = upload_table(c, plan, hi, &plan->tw_hi)) != ZK_OK) return rc;
    }
    for (int p = 0; p < plan->npass; p++) {
        const uint32_t lr = plan->pass_log_r[p];
        const zkh::F4 wr = zkh::pow_u64(F, w, n >> lr);
        std::vector<zkh::F4> t = powers(wr, std::max<uint64_t>(1, (1ull << lr) / 2));
        if ((rc = upload_table(c, plan, t, &plan->radix_tw[p])) != ZK_OK) return rc;
    }
    if (mode == ZK_NTT_COSET_EVALS_FROM_COEFFS) {
        std::vector<zkh::F4> lo = powers(shift_m, lo_count);
        zkh::F4 ss = zkh::pow_u64(F, shift_m, lo_count);
        std::vector<zkh::F4> hi = powers(ss, hi_count);
        if ((rc = upload_table(c, plan, lo, &plan->pre_lo)) != ZK_OK) return rc;
        if ((rc = upload_table(c, plan, hi, &plan->pre_hi)) != ZK_OK) return rc;
    }
    if (inverse) {
        zkh::F4 nn = {{n, 0, 0, 0}};
        zkh::F4 ninv = zkh::inv(F, zkh::to_mont(F, nn));
        if (mode == ZK_NTT_COEFFS_FROM_EVALS) {
            std::vector<zkh::F4> one(1, ninv);
            if ((rc = upload_table(c, plan, one, &plan->post_lo)) != ZK_OK) return rc;
        } else {
            // coefficient i is scaled by n^-1 shift^-i; a zero shift scales every i > 0 by 0
            zkh::F4 is = zkh::is_zero(shift_m) ? shift_m : zkh::inv(F, shift_m);
            std::vector<zkh::F4> lo = powers(is, lo_count);
            for (auto& x : lo) x = zkh::mul(F, x, ninv);
            zkh::F4 iss = zkh::pow_u64(F, is, lo_count);
            std::vector<zkh::F4> hi = powers(iss, hi_count);
            if ((rc = upload_table(c, plan, lo, &plan->post_lo)) != ZK_OK) return rc;
            if ((rc = upload_table(c, plan, hi, &plan->post_hi)) != ZK_OK) return rc;
        }
    }
    const size_t table_bytes = (size_t)n * 32;
    const int tables = 1 + (plan->pre_hi != nullptr) + (plan->post_hi != nullptr);
    if (log_n <= kFullTableMaxLog && c->ntt_full_table_bytes + tables * table_bytes <= kFullTableBudget) {
        fe** lo_of[3] = {&plan->tw_lo, &plan->pre_lo, &plan->post_lo};
        fe** hi_of[3] = {&plan->tw_hi, &plan->pre_hi, &plan->post_hi};
        for (int t = 0; t < 3; t++) {
            if (*hi_of[t] == nullptr) continue;  // absent, or a constant factor (post_lo[0])
            void* p = nullptr;
            ZK_TRY_CUDA(cudaMalloc(&p, table_bytes));
            plan->allocations.push_back(p);
            c->ntt_full_table_bytes += table_bytes;
            const unsigned blocks = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)c->num_sms * 8);
            ZK_LAUNCH(c, "ntt_table", ntt_expand_table_kernel, blocks, 256, 0, static_cast<fe*>(p), *lo_of[t],
                      *hi_of[t], plan->s_bits, (uint32_t)n);
            ZK_TRY_CUDA(cudaGetLastError());
            *lo_of[t] = static_cast<fe*>(p);
            *hi_of[t] = static_cast<fe*>(p);  // non-null: a table, not a constant
        }
        plan->s_bits = kNttFullTable;
    }
    *out = plan;
    return ZK_OK;
}

static int get_plan(Ctx* c, int mode, uint32_t log_n, const uint8_t omega[32], const uint8_t shift[32],
                    NttPlan** out) {
    std::string key(reinterpret_cast<const char*>(omega), 32);
    key.append(reinterpret_cast<const char*>(shift), 32);
    key.push_back((char)mode);
    key.push_back((char)log_n);
    key.append(reinterpret_cast<const char*>(c->tune_ntt_split[log_n]), 4);
    auto it = c->ntt_plans.find(key);
    if (it != c->ntt_plans.end()) {
        *out = it->second;
        return ZK_OK;
    }
    const zkh::Field& F = zkh::fr();
    zkh::F4 om = zkh::to_mont(F, load_canon(omega));
    zkh::F4 sh = zkh::to_mont(F, load_canon(shift));
    // omega must have order exactly n: omega^(n/2) == -1 (and omega^n == 1 for n == 1 is vacuous)
    if (log_n >= 1) {
        zkh::F4 h = zkh::pow_u64(F, om, 1ull << (log_n - 1));
        zkh::F4 m1 = zkh::neg(F, zkh::one(F));
        if (!zkh::eq(h, m1)) {
            set_error("omega is not a primitive n-th root of unity (omega^(n/2) != -1)");
            return ZK_EINVAL;
        }
    }
    NttPlan* plan = nullptr;
    int rc = build_plan(c, mode, log_n, om, sh, &plan);
    if (rc != ZK_OK) return rc;
    c->ntt_plans[key] = plan;
    *out = plan;
    return ZK_OK;
}

// Dynamic shared memory of the pass kernels (set once per device).
static int set_smem_attr(int device) {
    static std::mutex mu;
    static bool done[64] = {};
    ZK_CHECK_ARG(device >= 0 && device < 64, "device index out of range");
    std::lock_guard<std::mutex> g(mu);
    if (!done[device]) {
        ZK_TRY_CUDA(cudaFuncSetAttribute(ntt_pass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (2 << kTileLogElems) * 16));
        ZK_TRY_CUDA(cudaFuncSetAttribute(ntt_pass_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (2 << kTileLogElems) * 16));
        ZK_TRY_CUDA(cudaFuncSetAttribute(ntt_queue_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (2 << kTileLogElems) * 16));
        done[device] = true;
    }
    return ZK_OK;
}

// Columns per CTA of a radix-2^lr pass of a 2^log_n transform: fill a tile of up to
// 2^tile_log elements, but not beyond the number of columns. ZK_NTT_TILE_LOG (5..11)
// overrides kDefaultTileLog (read once per process).
static uint32_t pass_log_t(uint32_t log_n, uint32_t lr) {
    static const int tile_log = [] {
        const char* e = std::getenv("ZK_NTT_TILE_LOG");
        const int v = e ? std::atoi(e) : 0;
        return (v >= 5 && v <= kTileLogElems) ? v : kDefaultTileLog;
    }();
    uint32_t lt = tile_log > (int)lr ? tile_log - lr : 0;
    if (lt > log_n - lr) lt = log_n - lr;
    return lt;
}

// One launch of one pass.
struct PassLaunch {
    NttPassParams P;
    uint32_t blocks, threads, smem;
};

// Scratch elements a transform needs for its intermediate passes.
static size_t pass_scratch_elems(const NttPlan* plan, const fe* out, const fe* in) {
    const size_t n = (size_t)1 << plan->log_n;
    if (plan->npass <= 1) return 0;
    if (plan->npass == 2 || in != out) return n;
    return 2 * n;  // in place with 3+ passes: two scratch buffers, `out` only for the last pass
}

// The passes of one transform: pass p reads the previous pass's output. Intermediate
// passes go to scratch (and, out of place with 3+ passes, alternate with `out` so that
// one scratch buffer suffices); the last pass writes `out`.
static void make_passes(const NttPlan* plan, fe* out, const fe* in, uint32_t valid, fe* scratch,
                        std::vector<PassLaunch>* launches, bool canon_io = false) {
    const uint32_t log_n = plan->log_n;
    const uint64_t n = 1ull << log_n;
    launches->clear();
    NttPassParams P{};
    P.tw_lo = plan->tw_lo;
    P.tw_hi = plan->tw_hi;
    P.s_bits = plan->s_bits;
    if (log_n == 0) {  // n == 1: the transform is the identity up to the scale factors
        P.in = in;
        P.out = out;
        P.radix_tw = plan->tw_lo;
        P.pre_lo = plan->pre_lo;
        P.pre_hi = plan->pre_hi;
        P.post_lo = plan->post_lo;
        P.post_hi = plan->post_hi;
        P.in_len = valid;
        P.last = 1;
        P.reduce_in = canon_io ? 1u : 0u;
        launches->push_back({P, 1, 32, 2 * 16});
        return;
    }
    const bool two_scratch = plan->npass >= 3 && in == out;
    uint32_t log_l = 0;
    const fe* src = in;
    for (int p = 0; p < plan->npass; p++) {
        const uint32_t lr = plan->pass_log_r[p];
        const uint32_t lt = pass_log_t(log_n, lr);
        const int remaining = plan->npass - 1 - p;
        fe* dst;
        if (remaining == 0) dst = out;
        else if (two_scratch) dst = scratch + (size_t)(p & 1) * n;
        else dst = (remaining % 2 == 0) ? out : scratch;
        P.in = src;
        P.out = dst;
        P.radix_tw = plan->radix_tw[p];
        P.pre_lo = p == 0 ? plan->pre_lo : nullptr;
        P.pre_hi = p == 0 ? plan->pre_hi : nullptr;
        P.post_lo = remaining == 0 ? plan->post_lo : nullptr;
        P.post_hi = remaining == 0 ? plan->post_hi : nullptr;
        P.in_len = p == 0 ? valid : (uint32_t)n;
        P.log_n = log_n;
        P.log_r = lr;
        P.log_t = lt;
        P.log_l = log_l;
        P.last = remaining == 0 ? 1u : 0u;
        P.reduce_in = canon_io && p == 0 ? 1u : 0u;
        const uint32_t elems = 1u << (lr + lt);
        const uint32_t threads = elems / 2 < (uint32_t)kNttThreads ? (elems / 2 < 32 ? 32 : elems / 2) : kNttThreads;
        launches->push_back({P, (uint32_t)(n >> (lr + lt)), threads, elems * 32});
        src = dst;
        log_l += lr;
    }
}

static int check_job(int mode, const fe* out, const fe* in, size_t in_len, uint32_t log_n) {
    ZK_CHECK_ARG(mode >= 0 && mode <= 3, "invalid NTT mode");
    ZK_CHECK_ARG(log_n <= 28, "domain too large for BN254 root of unity (log2 n > 28)");
    const uint64_t n = 1ull << log_n;
    const bool inverse = (mode == ZK_NTT_COEFFS_FROM_EVALS || mode == ZK_NTT_COSET_COEFFS_FROM_EVALS);
    ZK_CHECK_ARG(!inverse || in_len == n, "inverse transforms need len(evals) == n (a power of two)");
    ZK_CHECK_ARG(out != nullptr && (in != nullptr || in_len == 0), "null buffer");
    return ZK_OK;
}

// canon_io: `in` holds canonical values and `out` receives canonical ones, with no
// Montgomery conversion: the transform is linear and every constant it multiplies by is a
// Montgomery form, so running it on x (read as the Montgomery form of x / R) yields the
// Montgomery form of NTT(x) / R, which is NTT(x) itself.
int ntt_run(Ctx* c, int mode, fe* out, const fe* in, size_t in_len, uint32_t log_n, const uint8_t omega[32],
            const uint8_t shift[32], bool canon_io) {
    int rc = check_job(mode, out, in, in_len, log_n);
    if (rc != ZK_OK) return rc;
    const uint64_t n = 1ull << log_n;
    NttPlan* plan = nullptr;
    {
        std::lock_guard<std::mutex> g(c->mu);
        if ((rc = get_plan(c, mode, log_n, omega, shift, &plan)) != ZK_OK) return rc;
    }
    if ((rc = set_smem_attr(c->device)) != ZK_OK) return rc;
    const uint32_t valid = (uint32_t)(in_len < n ? in_len : n);
    fe* scratch = nullptr;
    const size_t se = pass_scratch_elems(plan, out, in);
    if (se && (rc = scratch_alloc(c, se * 32, reinterpret_cast<void**>(&scratch))) != ZK_OK) return rc;
    std::vector<PassLaunch> launches;
    make_passes(plan, out, in, valid, scratch, &launches, canon_io);
    for (const PassLaunch& L : launches) {
        ZK_LAUNCH(c, "ntt_pass", ntt_pass_kernel, L.blocks, L.threads, L.smem, L.P);
        ZK_TRY_CUDA(cudaGetLastError());
    }
    if (scratch) scratch_free(c, scratch);
    return ZK_OK;
}

// ---- batches: one launch per pass level over every transform of the batch ----------------
struct NttBatch {
    std::vector<std::vector<PassLaunch>> jobs;  // passes of each transform
    std::vector<size_t> scratch_at;             // element offset of each job's scratch
    size_t scratch_elems = 0;
    // per level: items and their first tiles, uploaded to `desc`
    std::vector<std::vector<NttPassParams>> items;
    std::vector<std::vector<uint32_t>> first;
    std::vector<uint32_t> blocks, threads, smem;
    size_t desc_bytes = 0;
    std::vector<size_t> items_at, first_at;  // byte offsets inside desc
    char* desc = nullptr;
    fe* scratch = nullptr;
    // queue form (one persistent launch): entries in queue order, then the wait limit (ns)
    // and the state words (ticket, status, finished items per entry), all inside desc
    bool queue = false;
    std::vector<NttQueueEntry> qentries;
    uint32_t qitems = 0, qsmem = 32, qgrid = 0;
    size_t queue_at = 0, limit_at = 0, state_at = 0;
    uint64_t limit_ns = 2000000000ull;
};

static int batch_prepare(Ctx* c, const NttJob* jobs, size_t count, NttBatch* b) {
    b->jobs.assign(count, {});
    b->scratch_at.assign(count, 0);
    std::vector<NttPlan*> plans(count, nullptr);
    for (size_t j = 0; j < count; j++) {
        const NttJob& J = jobs[j];
        int rc = check_job(J.mode, J.out, J.in, J.in_len, J.log_n);
        if (rc != ZK_OK) return rc;
        ZK_CHECK_ARG(J.omega != nullptr, "null omega");
        std::lock_guard<std::mutex> g(c->mu);
        static const uint8_t one[32] = {1};
        if ((rc = get_plan(c, J.mode, J.log_n, J.omega, J.shift ? J.shift : one, &plans[j])) != ZK_OK) return rc;
        b->scratch_at[j] = b->scratch_elems;
        b->scratch_elems += pass_scratch_elems(plans[j], J.out, J.in);
    }
    size_t levels = 0;
    for (size_t j = 0; j < count; j++) levels = std::max<size_t>(levels, std::max(plans[j]->npass, 1));
    b->items.assign(levels, {});
    b->first.assign(levels, {});
    b->blocks.assign(levels, 0);
    b->threads.assign(levels, 32);
    b->smem.assign(levels, 32);
    return ZK_OK;
}

// Pass parameters once the scratch address is known, grouped by level, and the
// descriptor layout (items then first tiles, per level).
static int batch_layout(const NttJob* jobs, size_t count, NttBatch* b, Ctx* c) {
    for (auto& v : b->items) v.clear();
    for (auto& v : b->first) v.clear();
    std::fill(b->blocks.begin(), b->blocks.end(), 0);
    for (size_t j = 0; j < count; j++) {
        const NttJob& J = jobs[j];
        NttPlan* plan = nullptr;
        {
            std::lock_guard<std::mutex> g(c->mu);
            static const uint8_t one[32] = {1};
            int rc = get_plan(c, J.mode, J.log_n, J.omega, J.shift ? J.shift : one, &plan);
            if (rc != ZK_OK) return rc;
        }
        const uint64_t n = 1ull << J.log_n;
        const uint32_t valid = (uint32_t)(J.in_len < n ? J.in_len : n);
        make_passes(plan, J.out, J.in, valid, b->scratch ? b->scratch + b->scratch_at[j] : nullptr, &b->jobs[j]);
        for (size_t L = 0; L < b->jobs[j].size(); L++) {
            const PassLaunch& pl = b->jobs[j][L];
            b->first[L].push_back(b->blocks[L]);
            b->items[L].push_back(pl.P);
            b->blocks[L] += pl.blocks;
            b->threads[L] = std::max(b->threads[L], pl.threads);
            b->smem[L] = std::max(b->smem[L], pl.smem);
        }
    }
    size_t off = 0;
    b->items_at.assign(b->items.size(), 0);
    b->first_at.assign(b->items.size(), 0);
    for (size_t L = 0; L < b->items.size(); L++) {
        off = (off + 255) & ~(size_t)255;
        b->items_at[L] = off;
        off += b->items[L].size() * sizeof(NttPassParams);
        off = (off + 255) & ~(size_t)255;
        b->first_at[L] = off;
        off += b->first[L].size() * 4;
    }
    if (b->queue) {
        // every CTA that can be resident at once, and no more CTAs than items
        b->qsmem = 32;
        uint64_t items = 0;
        for (size_t j = 0; j < count; j++)
            for (const PassLaunch& pl : b->jobs[j]) {
                b->qsmem = std::max(b->qsmem, pl.smem);
                items += pl.blocks;
            }
        int per_sm = 0;
        ZK_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ntt_queue_kernel, kNttThreads, b->qsmem));
        b->qgrid = (uint32_t)std::min<uint64_t>(items, (uint64_t)std::max(1, per_sm) * c->num_sms);
        // Queue order: pass level by pass level, the largest transforms first within a level,
        // so that the first items of the next level belong to the transforms whose previous
        // pass began earliest; every entry follows the entry it waits for. (Measured on
        // GB300: queueing a transform's next pass two waves after its previous one, to read
        // its intermediate from L2, was slower: 64 mixed transforms 3.11 against 2.98 ms,
        // 64 small ones 0.165 against 0.12 ms -- its items wait on unfinished passes.)
        std::vector<size_t> order(count);
        for (size_t j = 0; j < count; j++) order[j] = j;
        std::stable_sort(order.begin(), order.end(),
                         [&](size_t a, size_t z) { return jobs[a].log_n > jobs[z].log_n; });
        std::vector<int32_t> prev(count, -1);
        b->qentries.clear();
        b->qitems = 0;
        for (size_t L = 0; L < b->items.size(); L++) {
            for (size_t j : order) {
                if (L >= b->jobs[j].size()) continue;
                const PassLaunch& pl = b->jobs[j][L];
                NttQueueEntry e{};
                e.P = pl.P;
                e.first = b->qitems;
                e.tiles = pl.blocks;
                e.dep = prev[j];
                e.need = L ? b->jobs[j][L - 1].blocks : 0u;
                prev[j] = (int32_t)b->qentries.size();
                b->qentries.push_back(e);
                b->qitems += pl.blocks;
            }
        }
        off = (off + 255) & ~(size_t)255;
        b->queue_at = off;
        off += b->qentries.size() * sizeof(NttQueueEntry);
        off = (off + 255) & ~(size_t)255;
        b->limit_at = off;
        off += 8;
        b->state_at = off;
        off += (kQueueDone + b->qentries.size()) * 4;
    }
    b->desc_bytes = off ? off : 16;
    return ZK_OK;
}

static int batch_upload(Ctx* c, NttBatch* b) {
    for (size_t L = 0; L < b->items.size(); L++) {
        ZK_TRY_CUDA(cudaMemcpyAsync(b->desc + b->items_at[L], b->items[L].data(),
                                    b->items[L].size() * sizeof(NttPassParams), cudaMemcpyHostToDevice, c->stream));
        ZK_TRY_CUDA(cudaMemcpyAsync(b->desc + b->first_at[L], b->first[L].data(), b->first[L].size() * 4,
                                    cudaMemcpyHostToDevice, c->stream));
    }
    if (b->queue) {
        ZK_TRY_CUDA(cudaMemcpyAsync(b->desc + b->queue_at, b->qentries.data(),
                                    b->qentries.size() * sizeof(NttQueueEntry), cudaMemcpyHostToDevice, c->stream));
        ZK_TRY_CUDA(cudaMemcpyAsync(b->desc + b->limit_at, &b->limit_ns, 8, cudaMemcpyHostToDevice, c->stream));
    }
    return ZK_OK;
}

static int batch_enqueue(Ctx* c, const NttBatch* b) {
    if (b->queue) {
        if (b->qitems == 0) return ZK_OK;
        uint32_t* state = reinterpret_cast<uint32_t*>(b->desc + b->state_at);
        ZK_TRY_CUDA(cudaMemsetAsync(state, 0, (kQueueDone + b->qentries.size()) * 4, c->stream));
        ZK_LAUNCH(c, "ntt_queue", ntt_queue_kernel, b->qgrid, kNttThreads, b->qsmem,
                  reinterpret_cast<const NttQueueEntry*>(b->desc + b->queue_at), (uint32_t)b->qentries.size(),
                  b->qitems, state, reinterpret_cast<const uint64_t*>(b->desc + b->limit_at), c->ntt_queue_err);
        ZK_TRY_CUDA(cudaGetLastError());
        return ZK_OK;
    }
    for (size_t L = 0; L < b->items.size(); L++) {
        if (b->blocks[L] == 0) continue;
        ZK_LAUNCH(c, "ntt_pass_batch", ntt_pass_batch_kernel, b->blocks[L], b->threads[L], b->smem[L],
                  reinterpret_cast<const NttPassParams*>(b->desc + b->items_at[L]),
                  reinterpret_cast<const uint32_t*>(b->desc + b->first_at[L]), (uint32_t)b->items[L].size());
        ZK_TRY_CUDA(cudaGetLastError());
    }
    return ZK_OK;
}

// The context's work-queue error word (allocated once, before any capture can need it).
static int ensure_queue_word(Ctx* c) {
    std::lock_guard<std::mutex> g(c->mu);
    if (c->ntt_queue_err == nullptr) {
        ZK_TRY_CUDA(cudaMalloc(reinterpret_cast<void**>(&c->ntt_queue_err), 4));
        ZK_TRY_CUDA(cudaMemsetAsync(c->ntt_queue_err, 0, 4, c->stream));
    }
    return ZK_OK;
}

int ntt_queue_status(Ctx* c) {
    if (c->ntt_queue_err == nullptr) return ZK_OK;
    ZK_TRY_CUDA(cudaStreamSynchronize(c->stream));
    uint32_t v = 0;
    ZK_TRY_CUDA(cudaMemcpy(&v, c->ntt_queue_err, 4, cudaMemcpyDeviceToHost));
    if (v == 0) return ZK_OK;
    ZK_TRY_CUDA(cudaMemset(c->ntt_queue_err, 0, 4));
    set_error("NTT work queue: the wait of queue entry " + std::to_string(v - 1) +
              " for its previous pass ran out; that launch stopped early and its outputs are incomplete");
    return ZK_ETIMEOUT;
}

int ntt_batch_run(Ctx* c, const NttJob* jobs, size_t count) {
    if (count == 0) return ZK_OK;
    NttBatch b;
    b.queue = c->ntt_queue;
    int rc = batch_prepare(c, jobs, count, &b);
    if (rc != ZK_OK) return rc;
    if ((rc = set_smem_attr(c->device)) != ZK_OK) return rc;
    if (b.queue && (rc = ensure_queue_word(c)) != ZK_OK) return rc;
    if ((rc = batch_layout(jobs, count, &b, c)) != ZK_OK) return rc;  // sizes only
    char* arena = nullptr;
    const size_t scratch_bytes = ((b.scratch_elems * 32) + 255) & ~(size_t)255;
    if ((rc = scratch_alloc(c, scratch_bytes + b.desc_bytes, reinterpret_cast<void**>(&arena))) != ZK_OK) return rc;
    b.scratch = reinterpret_cast<fe*>(arena);
    b.desc = arena + scratch_bytes;
    if ((rc = batch_layout(jobs, count, &b, c)) == ZK_OK && (rc = batch_upload(c, &b)) == ZK_OK)
        rc = batch_enqueue(c, &b);
    scratch_free(c, arena);
    return rc;
}

struct NttBatchPlan {
    NttBatch b;
    char* arena = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t kernels = 0;
};

int ntt_plan_create(Ctx* c, const NttJob* jobs, size_t count, bool graph, bool queue, NttBatchPlan** out) {
    std::unique_ptr<NttBatchPlan> plan(new NttBatchPlan());
    NttBatch& b = plan->b;
    b.queue = queue;
    int rc = batch_prepare(c, jobs, count, &b);
    if (rc != ZK_OK) return rc;
    if ((rc = set_smem_attr(c->device)) != ZK_OK) return rc;
    if (queue && (rc = ensure_queue_word(c)) != ZK_OK) return rc;
    if ((rc = batch_layout(jobs, count, &b, c)) != ZK_OK) return rc;
    const size_t scratch_bytes = ((b.scratch_elems * 32) + 255) & ~(size_t)255;
    ZK_TRY_CUDA(cudaMalloc(reinterpret_cast<void**>(&plan->arena), scratch_bytes + b.desc_bytes));
    b.scratch = reinterpret_cast<fe*>(plan->arena);
    b.desc = plan->arena + scratch_bytes;
    auto fail = [&](int code) {
        cudaStreamSynchronize(c->stream);
        cudaFree(plan->arena);
        return code;
    };
    if ((rc = batch_layout(jobs, count, &b, c)) != ZK_OK || (rc = batch_upload(c, &b)) != ZK_OK) return fail(rc);
    cudaError_t se = cudaStreamSynchronize(c->stream);
    if (se != cudaSuccess) {
        set_error(std::string("NTT plan set-up: ") + cudaGetErrorString(se));
        return fail(ZK_ECUDA);
    }
    if (graph && count) {
        const bool prof_was = c->prof_on;
        const uint64_t launches_was = c->launches;
        const auto prof_was_map = c->prof;
        c->prof_on = false;
        cudaError_t be = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
        if (be != cudaSuccess) {
            c->prof_on = prof_was;
            set_error(std::string("cudaStreamBeginCapture: ") + cudaGetErrorString(be));
            return fail(ZK_ECUDA);
        }
        const int erc = batch_enqueue(c, &b);
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

int ntt_plan_run(Ctx* c, NttBatchPlan* plan) {
    if (plan->exec) {
        const int tok = prof_begin(c, "ntt_plan_graph");
        ZK_TRY_CUDA(cudaGraphLaunch(plan->exec, c->stream));
        prof_end(c, tok);
        c->launches += plan->kernels - 1;  // prof_begin counted the graph launch as one
        return ZK_OK;
    }
    return batch_enqueue(c, &plan->b);
}

uint64_t ntt_plan_kernels(const NttBatchPlan* plan) { return plan->kernels; }

int ntt_queue_selftest(Ctx* c, uint64_t limit_ns, uint32_t* entry_out) {
    // one 2^12 transform (two passes, or three under a tuned split) on zeroed buffers: the
    // second pass's items wait for one first-pass tile more than the queue holds, so their
    // waits run out (and a third pass's, waiting on the second, too)
    const uint32_t log_n = 12;
    static const uint8_t one[32] = {1};
    uint8_t omega[32];
    {
        // omega = 5^((r - 1) / 2^12): a primitive 2^12-th root of unity (5 generates Fr^*)
        const zkh::Field& F = zkh::fr();
        uint64_t e[4];
        std::memcpy(e, F.p, 32);
        e[0] -= 1;  // r - 1 (r is odd)
        for (uint32_t i = 0; i < log_n; i++)
            for (int k = 0; k < 4; k++) e[k] = (e[k] >> 1) | (k < 3 ? e[k + 1] << 63 : 0);
        const zkh::F4 om = zkh::pow(F, zkh::to_mont(F, zkh::F4{{5, 0, 0, 0}}), e);
        const zkh::F4 canon = zkh::from_mont(F, om);
        std::memcpy(omega, canon.v, 32);
    }
    fe* buf = nullptr;
    const size_t n = (size_t)1 << log_n;
    ZK_TRY_CUDA(cudaMalloc(reinterpret_cast<void**>(&buf), n * 32 * 2));
    auto done = [&](int rc) {
        cudaStreamSynchronize(c->stream);
        cudaFree(buf);
        return rc;
    };
    if (cudaMemsetAsync(buf, 0, n * 32 * 2, c->stream) != cudaSuccess) return done(ZK_ECUDA);
    NttJob J;
    J.mode = ZK_NTT_EVALS_FROM_COEFFS;
    J.out = buf + n;
    J.in = buf;
    J.in_len = n;
    J.log_n = log_n;
    J.omega = omega;
    J.shift = one;
    NttBatchPlan* plan = nullptr;
    int rc = ntt_plan_create(c, &J, 1, false, true, &plan);
    if (rc != ZK_OK) return done(rc);
    NttBatch& b = plan->b;
    rc = ZK_EINVAL;
    if (b.qentries.size() >= 2 && b.qentries[1].dep == 0) {
        b.qentries[1].need = b.qentries[0].tiles + 1;  // one tile more than pass 1 has
        b.limit_ns = limit_ns;
        rc = batch_upload(c, &b);
        if (rc == ZK_OK) rc = batch_enqueue(c, &b);
    } else {
        set_error("NTT queue self-test: unexpected plan shape");
    }
    uint32_t st = 0;
    if (rc == ZK_OK) {
        cudaError_t e = cudaMemcpyAsync(&st, b.desc + b.state_at + 4 * kQueueStatus, 4, cudaMemcpyDeviceToHost,
                                        c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) {
            set_error(std::string("NTT queue self-test: ") + cudaGetErrorString(e));
            rc = ZK_ECUDA;
        }
    }
    ntt_plan_destroy(c, plan);
    if (rc != ZK_OK) return done(rc);
    *entry_out = st;
    // the sticky context record is the self-test's own: clear it
    cudaMemsetAsync(c->ntt_queue_err, 0, 4, c->stream);
    return done(st == 0 ? ZK_OK : ZK_ETIMEOUT);
}

void ntt_plan_destroy(Ctx* c, NttBatchPlan* plan) {
    if (plan == nullptr) return;
    cudaStreamSynchronize(c->stream);
    if (plan->exec) cudaGraphExecDestroy(plan->exec);
    cudaFree(plan->arena);
    delete plan;
}

}  // namespace zk

// ==============================================================================
// Allocation-free NTT entry point (zk_ntt_noalloc).
//
// Some callers cannot allocate device memory when they transform: a serving process
// that reserved the whole device up front for its own pool, code that must not pay
// cudaMalloc's implicit device synchronisation on a latency-critical path, or a
// library embedded in a host whose allocator owns the GPU. zk_ntt_noalloc runs the
// same passes as zk_ntt but takes its scratch -- the intermediate pass buffer and the
// twiddle / scale tables, which zk_ntt allocates and caches -- from one file-scope
// static device array of fixed size. Limits and rules:
//   * n <= 2^16 (kNoAllocMaxLogN); larger sizes are rejected with ZK_EINVAL;
//   * the array is shared by every call on a device and keeps the last call's
//     contents; nothing in it has to start at zero (each call rebuilds its tables on
//     the device and its first pass writes every element the second pass reads), but
//     calls that overlap on the GPU (different streams, or different contexts of one
//     device) race on it and must be serialised by the caller;
//   * the tables are computed on the device by a kernel that receives their generators
//     by value (no host buffer is read by the GPU, so nothing on the host outlives the
//     call);
//   * the first call on each device does the set-up (cudaGetSymbolAddress of the
//     array, the kernel's shared-memory attribute), so that first call should come
//     before any stream capture;
//   * no cudaMalloc, cudaFree or other allocating routine is called.
// ==============================================================================
namespace zk {

static constexpr uint32_t kNoAllocMaxLogN = 16;
static constexpr size_t kNoAllocDataElems = (size_t)1 << kNoAllocMaxLogN;
// tables for log_n <= 16: two-level twiddles (<= 256 + 257), radix tables (<= 1024),
// first-pass scale (<= 513), last-pass scale (<= 513): at most 2563 elements
static constexpr size_t kNoAllocTableElems = 4096;

static __device__ __align__(256) fe g_ntt_noalloc_scratch[kNoAllocDataElems + kNoAllocTableElems];

static constexpr int kNoAllocMaxDevices = 64;
static std::mutex g_noalloc_mu;
static fe* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// Once per device, with that device current: device address of the static array.
static int noalloc_setup(int device, fe** out) {
    ZK_CHECK_ARG(device >= 0 && device < kNoAllocMaxDevices, "device index out of range for zk_ntt_noalloc");
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    if (g_noalloc_ptr[device] == nullptr) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_ntt_noalloc_scratch);
        if (e != cudaSuccess) {
            set_error(std::string("cudaGetSymbolAddress(g_ntt_noalloc_scratch): ") + cudaGetErrorString(e));
            return ZK_ECUDA;
        }
        int rc = set_smem_attr(device);
        if (rc != ZK_OK) return rc;
        g_noalloc_ptr[device] = static_cast<fe*>(p);
    }
    *out = g_noalloc_ptr[device];
    return ZK_OK;
}

// The tables as segments: table[off + i] = start * base^i for i < count (Montgomery),
// built on the device from these values, which the launch carries by value.
static constexpr int kNoAllocMaxSegs = 10;
struct NoAllocTableSpec {
    uint32_t nseg;
    uint32_t off[kNoAllocMaxSegs];
    uint32_t count[kNoAllocMaxSegs];
    fe start[kNoAllocMaxSegs];
    fe base[kNoAllocMaxSegs];
};

__global__ void ntt_noalloc_tables_kernel(fe* __restrict__ tables, NoAllocTableSpec S) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t s = 0; s < S.nseg; s++) {
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < S.count[s]; i += stride) {
            fe acc = S.start[s];
            fe b = S.base[s];
            for (uint32_t e = i; e != 0; e >>= 1) {  // square-and-multiply, exponent i < 2^10
                if (e & 1) acc = fe_mul<FrP>(acc, b);
                if (e > 1) b = fe_mul<FrP>(b, b);
            }
            fe_store(tables + S.off[s] + i, acc);
        }
    }
}

static fe to_fe(const zkh::F4& x) {
    fe r;
    std::memcpy(r.v, x.v, 32);
    return r;
}

// Appends the segment start * base^i, i < count, at *pos; false when the spec is full.
static bool add_segment(NoAllocTableSpec* S, size_t* pos, const zkh::F4& base, size_t count,
                        const zkh::F4* start = nullptr) {
    if (S->nseg >= (uint32_t)kNoAllocMaxSegs) return false;
    const uint32_t k = S->nseg++;
    S->off[k] = (uint32_t)*pos;
    S->count[k] = (uint32_t)count;
    S->start[k] = to_fe(start ? *start : zkh::one(zkh::fr()));
    S->base[k] = to_fe(base);
    *pos += count;
    return true;
}

static int ntt_run_noalloc(Ctx* c, int mode, fe* out, const fe* in, size_t in_len, uint32_t log_n,
                           const uint8_t omega[32], const uint8_t shift[32]) {
    ZK_CHECK_ARG(mode >= 0 && mode <= 3, "invalid NTT mode");
    ZK_CHECK_ARG(log_n <= kNoAllocMaxLogN, "zk_ntt_noalloc supports n <= 2^16 (its static scratch size)");
    const uint64_t n = 1ull << log_n;
    const bool inverse = (mode == ZK_NTT_COEFFS_FROM_EVALS || mode == ZK_NTT_COSET_COEFFS_FROM_EVALS);
    ZK_CHECK_ARG(!inverse || in_len == n, "inverse transforms need len(evals) == n (a power of two)");
    ZK_CHECK_ARG(out != nullptr && (in != nullptr || in_len == 0), "null buffer");
    fe* base = nullptr;
    int rc = noalloc_setup(c->device, &base);
    if (rc != ZK_OK) return rc;
    fe* data = base;
    fe* tables = base + kNoAllocDataElems;

    const zkh::Field& F = zkh::fr();
    const zkh::F4 om = zkh::to_mont(F, load_canon(omega));
    const zkh::F4 sh = zkh::to_mont(F, load_canon(shift));
    if (log_n >= 1) {
        zkh::F4 h = zkh::pow_u64(F, om, 1ull << (log_n - 1));
        if (!zkh::eq(h, zkh::neg(F, zkh::one(F)))) {
            set_error("omega is not a primitive n-th root of unity (omega^(n/2) != -1)");
            return ZK_EINVAL;
        }
    }
    NttPlan plan;  // shape only: every table pointer below points into the static array
    plan.log_n = log_n;
    split_passes(log_n, &plan);
    plan.s_bits = (log_n + 1) / 2;
    const uint64_t lo_count = 1ull << plan.s_bits;
    const uint64_t hi_count = (n >> plan.s_bits) + 1;
    const zkh::F4 w = inverse ? zkh::inv(F, om) : om;

    NoAllocTableSpec spec{};
    bool ok = true;
    size_t pos = 0;
    const size_t off_lo = pos;
    ok = ok && add_segment(&spec, &pos, w, lo_count);
    const size_t off_hi = pos;
    ok = ok && add_segment(&spec, &pos, zkh::pow_u64(F, w, lo_count), hi_count);
    size_t off_radix[4] = {0, 0, 0, 0};
    for (int p = 0; p < plan.npass; p++) {
        off_radix[p] = pos;
        const uint32_t lr = plan.pass_log_r[p];
        ok = ok && add_segment(&spec, &pos, zkh::pow_u64(F, w, n >> lr), std::max<uint64_t>(1, (1ull << lr) / 2));
    }
    size_t off_pre_lo = 0, off_pre_hi = 0, off_post_lo = 0, off_post_hi = 0;
    bool has_pre = false, has_post = false, post_const = false;
    if (mode == ZK_NTT_COSET_EVALS_FROM_COEFFS) {
        has_pre = true;
        off_pre_lo = pos;
        ok = ok && add_segment(&spec, &pos, sh, lo_count);
        off_pre_hi = pos;
        ok = ok && add_segment(&spec, &pos, zkh::pow_u64(F, sh, lo_count), hi_count);
    }
    if (inverse) {
        has_post = true;
        zkh::F4 nn = {{n, 0, 0, 0}};
        zkh::F4 ninv = zkh::inv(F, zkh::to_mont(F, nn));
        off_post_lo = pos;
        if (mode == ZK_NTT_COEFFS_FROM_EVALS) {
            post_const = true;
            ok = ok && add_segment(&spec, &pos, zkh::one(F), 1, &ninv);
        } else {
            zkh::F4 is = zkh::is_zero(sh) ? sh : zkh::inv(F, sh);
            ok = ok && add_segment(&spec, &pos, is, lo_count, &ninv);
            off_post_hi = pos;
            ok = ok && add_segment(&spec, &pos, zkh::pow_u64(F, is, lo_count), hi_count);
        }
    }
    if (!ok || pos > kNoAllocTableElems) {
        set_error("zk_ntt_noalloc: table layout exceeds the static scratch");
        return ZK_EINVAL;
    }
    ZK_LAUNCH(c, "ntt_noalloc_tables", ntt_noalloc_tables_kernel, 8, 256, 0, tables, spec);
    ZK_TRY_CUDA(cudaGetLastError());

    const uint32_t valid = (uint32_t)(in_len < n ? in_len : n);
    NttPassParams P{};
    P.tw_lo = tables + off_lo;
    P.tw_hi = tables + off_hi;
    P.s_bits = plan.s_bits;
    if (log_n == 0) {
        P.in = in;
        P.out = out;
        P.radix_tw = tables + off_lo;
        P.pre_lo = has_pre ? tables + off_pre_lo : nullptr;
        P.pre_hi = has_pre ? tables + off_pre_hi : nullptr;
        P.post_lo = has_post ? tables + off_post_lo : nullptr;
        P.post_hi = (has_post && !post_const) ? tables + off_post_hi : nullptr;
        P.in_len = valid;
        P.last = 1;
        ZK_LAUNCH(c, "ntt_pass", ntt_pass_kernel, 1, 32, 2 * 16, P);
        ZK_TRY_CUDA(cudaGetLastError());
        return ZK_OK;
    }
    uint32_t log_l = 0;
    const fe* src = in;
    for (int p = 0; p < plan.npass; p++) {
        const uint32_t lr = plan.pass_log_r[p];
        const uint32_t lt = pass_log_t(log_n, lr);
        const int remaining = plan.npass - 1 - p;
        fe* dst = (remaining % 2 == 0) ? out : data;
        P.in = src;
        P.out = dst;
        P.radix_tw = tables + off_radix[p];
        P.pre_lo = (p == 0 && has_pre) ? tables + off_pre_lo : nullptr;
        P.pre_hi = (p == 0 && has_pre) ? tables + off_pre_hi : nullptr;
        const bool last = p == plan.npass - 1;
        P.post_lo = (last && has_post) ? tables + off_post_lo : nullptr;
        P.post_hi = (last && has_post && !post_const) ? tables + off_post_hi : nullptr;
        P.in_len = p == 0 ? valid : (uint32_t)n;
        P.log_n = log_n;
        P.log_r = lr;
        P.log_t = lt;
        P.log_l = log_l;
        P.last = last ? 1u : 0u;
        const uint32_t elems = 1u << (lr + lt);
        const uint32_t threads = elems / 2 < (uint32_t)kNttThreads ? (elems / 2 < 32 ? 32 : elems / 2) : kNttThreads;
        const uint32_t blocks = (uint32_t)(n >> (lr + lt));
        ZK_LAUNCH(c, "ntt_pass", ntt_pass_kernel, blocks, threads, (size_t)elems * 32, P);
        ZK_TRY_CUDA(cudaGetLastError());
        src = dst;
        log_l += lr;
    }
    return ZK_OK;
}

}  // namespace zk

extern "C" int zk_ntt_noalloc(zk_ctx* ctx, int mode, void* out_dev, const void* in_dev, size_t in_len, uint32_t log_n,
                              const uint8_t omega[32], const uint8_t shift[32]) {
    if (ctx == nullptr || omega == nullptr) {
        zk::set_error("null zk_ctx or omega");
        return ZK_EINVAL;
    }
    cudaError_t e = cudaSetDevice(ctx->impl.device);
    if (e != cudaSuccess) {
        zk::set_error(cudaGetErrorString(e));
        return ZK_ECUDA;
    }
    static const uint8_t one[32] = {1};
    return zk::ntt_run_noalloc(&ctx->impl, mode, static_cast<zk::fe*>(out_dev), static_cast<const zk::fe*>(in_dev),
                               in_len, log_n, omega, shift ? shift : one);
}
