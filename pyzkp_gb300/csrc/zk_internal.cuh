// zk_internal.cuh -- shared declarations of the zkgpu library (not part of the public ABI).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/zkgpu.h"
#include "curve.cuh"
#include "field.cuh"
#include "host_field.hpp"

namespace zk {

void set_error(const std::string& msg);

// Host coordinate type of each curve (the same bytes as the device type).
template <class C>
struct HostOf;
template <>
struct HostOf<CurveG1> {
    using T = zkh::F4;
};
template <>
struct HostOf<CurveG2> {
    using T = zkh::F2;
};

#define ZK_TRY_CUDA(call)                                                                     \
    do {                                                                                      \
        cudaError_t _e = (call);                                                              \
        if (_e != cudaSuccess) {                                                              \
            ::zk::set_error(std::string(#call) + ": " + cudaGetErrorString(_e));              \
            return _e == cudaErrorMemoryAllocation ? ZK_ENOMEM : ZK_ECUDA;                    \
        }                                                                                     \
    } while (0)

#define ZK_CHECK_ARG(cond, msg)      \
    do {                             \
        if (!(cond)) {               \
            ::zk::set_error(msg);    \
            return ZK_EINVAL;        \
        }                            \
    } while (0)

// NttPlan::s_bits value of a plan whose twiddle and scale tables hold every power (one
// load per factor) instead of the two-level lo/hi split (a load pair and a product).
static constexpr uint32_t kNttFullTable = 31;

// Device tables of one NTT configuration (transform size, root, coset shift, direction).
struct NttPlan {
    uint32_t log_n = 0;
    int npass = 0;
    uint32_t pass_log_r[4] = {0, 0, 0, 0};
    fe* radix_tw[4] = {nullptr, nullptr, nullptr, nullptr};  // omega_R^i, i < R/2, per pass
    uint32_t s_bits = 0;  // split of two-level tables; kNttFullTable: tw/pre/post_lo are full tables
    fe* tw_lo = nullptr;                                       // omega^i, i < 2^s
    fe* tw_hi = nullptr;                                       // omega^(i 2^s), i < n / 2^s
    fe* pre_lo = nullptr;                                      // first-pass input scale (coset forward)
    fe* pre_hi = nullptr;
    fe* post_lo = nullptr;  // last-pass output scale (inverse: n^-1 [shift^-i])
    fe* post_hi = nullptr;  // null: post_lo[0] is a constant factor
    std::vector<void*> allocations;
};

// Per-kernel accounting (zk_prof_*): launches are always counted; with profiling on,
// each launch is bracketed by events on the context stream and resolved lazily.
struct ProfEntry {
    uint64_t launches = 0;
    double total_ms = 0.0;
};

struct ProfPending {
    std::string name;
    cudaEvent_t start, stop;
};

struct Ctx {
    int device = 0;
    int num_sms = 0;
    int priority = 0;  // CUDA stream priority of the context stream and its side / copy streams
    // the stream ZK_LAUNCH and the copies use: the context stream, pointed at a side or
    // copy stream for the span of one enqueue (a batch pipeline, an upload) and then restored
    cudaStream_t stream = nullptr;
    std::mutex mu;
    std::map<std::string, NttPlan*> ntt_plans;
    size_t ntt_full_table_bytes = 0;  // device bytes held by full (one-load) NTT tables
    // zk_ntt_batch as one persistent launch from a device work queue (zk_ntt_batch_set_queue),
    // and the device word where such launches record a wait that ran out (zk_ntt_queue_status)
    bool ntt_queue = false;
    uint32_t* ntt_queue_err = nullptr;
    // MSM batches as sorts + one persistent launch of every pipeline's later stages
    // (zk_msm_batch_set_queue); a one-shot test limit for the next queue's waits
    // (zk_msm_queue_test_limit: its first waiting entry then waits for an item too many)
    bool msm_queue = false;
    uint64_t msm_queue_test_limit_ns = 0;
    uint64_t launches = 0;
    bool prof_on = false;
    std::map<std::string, ProfEntry> prof;
    std::vector<ProfPending> prof_pending;
    std::vector<cudaEvent_t> event_pool;
    cudaEvent_t timer_start = nullptr, timer_stop = nullptr;
    // zk_msm_g1_host: a second stream uploads and converts the bases while the scalars'
    // digits are sorted; MSM pipelines wait on `bases_wait` (when set) before reading points.
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t copy_go = nullptr, copy_done = nullptr;
    cudaEvent_t bases_wait = nullptr;
    // ... and the scalars arrive in chunks on that stream: (end index, event recorded after
    // its copy); a single-instance pipeline of that size runs its digits chunk by chunk
    std::vector<std::pair<uint32_t, cudaEvent_t>> scalar_chunks;
    cudaEvent_t chunk_ev[4] = {nullptr, nullptr, nullptr, nullptr};
    // ... and a device word set there when some uploaded point is infinity: while `inf_flag`
    // is set, accumulations that test for infinity do so only if the word is non-zero
    uint32_t* inf_flag_dev = nullptr;
    const uint32_t* inf_flag = nullptr;
    // zk_msm_g1_host_submit: two device staging buffers used in turn, so that one call's
    // uploads overlap the previous call's MSM; free_ev (main stream) releases a buffer
    struct HostStage {
        void* dev = nullptr;
        size_t bytes = 0;
        cudaEvent_t free_ev = nullptr;
        bool used = false;
    };
    HostStage host_stage[2];
    int host_stage_next = 0;
    // zk_ntt_host_submit: the same for host-buffer NTTs (input copy on copy_stream, the
    // transform on the context stream, the output copy on d2h_stream); h2d_ev / comp_ev
    // order the three, free_ev releases the buffer after its output copy. Three buffers: a
    // buffer is held by its input copy, transform and output copy in turn, so with two the
    // next input copy waited for an output copy and a stream of calls ran below the
    // transform's rate.
    struct NttStage {
        void* dev = nullptr;
        size_t bytes = 0;
        cudaEvent_t free_ev = nullptr, h2d_ev = nullptr, comp_ev = nullptr;
        bool used = false;
    };
    static constexpr int kNttStages = 3;
    NttStage ntt_stage[kNttStages];
    int ntt_stage_next = 0;
    cudaStream_t d2h_stream = nullptr;
    // MSM batches spread their pipelines over the context stream and these (fork / join
    // events); created on first use
    std::vector<cudaStream_t> side_streams;
    std::vector<cudaEvent_t> side_events;  // fork, then one join event per side stream
    uint64_t msm_entries = 0;
    uint32_t msm_window_bits = 0, msm_windows = 0;
    // tuning tables (zk_tune_*, zk_autotune_*): 0 means the built-in rule
    uint8_t tune_msm_window[32] = {};    // MSM window bits by ceil(log2 n)
    uint8_t tune_ntt_split[29][4] = {};  // NTT radix bits per pass by log2 n
    // page-locked result buffers of asynchronous MSM batches, kept for reuse: allocating
    // and freeing page-locked memory per batch can wait for the whole device
    std::mutex pinned_mu;
    std::multimap<size_t, void*> pinned_free;  // size -> block
};

// A page-locked block of at least `bytes` from the context's free list (else a new one of
// exactly `bytes`; *got = its size); pinned_give returns it. Both are thread-safe.
int pinned_take(Ctx* c, size_t bytes, void** p, size_t* got);
void pinned_give(Ctx* c, void* p, size_t bytes);

int prof_begin(Ctx* c, const char* name);
void prof_end(Ctx* c, int token);
int prof_resolve(Ctx* c);
// Host-side work inside a library call, recorded in the same table when profiling is on
// (not counted as a kernel launch).
void prof_host(Ctx* c, const char* name, double ms);

// Work queues of the persistent kernels (ntt_queue_kernel, msm_queue_kernel): state words,
// zeroed before each launch -- the ticket, the status, then one finished-item counter per
// queue entry. Status 0: every item ran; otherwise 1 + the entry whose wait ran out.
static constexpr uint32_t kQueueTicket = 0, kQueueStatus = 1, kQueueDone = 2;

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// The next item of a queue (nitems once a wait has run out somewhere: the launch winds down).
__device__ __forceinline__ uint32_t queue_ticket(uint32_t* state, uint32_t nitems) {
    volatile uint32_t* vstate = state;
    return vstate[kQueueStatus] != 0 ? nitems : atomicAdd(state + kQueueTicket, 1u);
}

// Launch `kernel` on the context stream with launch accounting.
#define ZK_LAUNCH(ctxp, name, kernel, grid, block, smem, ...)                 \
    do {                                                                      \
        int _tok = ::zk::prof_begin((ctxp), (name));                          \
        kernel<<<(grid), (block), (smem), (ctxp)->stream>>>(__VA_ARGS__);     \
        ::zk::prof_end((ctxp), _tok);                                         \
    } while (0)

// Stream-ordered scratch allocation on the context stream (pooled by the driver).
int scratch_alloc(Ctx* c, size_t bytes, void** p);
void scratch_free(Ctx* c, void* p);

// kernels implemented in the .cu files
int ntt_run(Ctx* c, int mode, fe* out, const fe* in, size_t in_len, uint32_t log_n, const uint8_t omega[32],
            const uint8_t shift[32], bool canon_io = false);
int msm_run(Ctx* c, const affine_t* bases, const fe* scalars, size_t n, int scalars_mont, uint32_t window_bits,
            uint8_t out_xy[64], int* out_is_inf, const affine_t* shifted = nullptr, uint32_t shifted_c = 0,
            uint64_t stride = 0, bool glv = false, bool inf_points = true);
// Whether any of the n stored points (affine_t, or affine2_t when g2) is infinity (all zero);
// synchronises the context stream.
int any_infinity(Ctx* c, const void* pts, size_t n, bool g2, bool* out);
// The same on the context stream without waiting: ORs 1 into *flag if a point is infinity.
int mark_infinity(Ctx* c, const void* pts, size_t n, bool g2, uint32_t* flag);
// G1 bases with the GLV half: pts[n + i] = phi(pts[i]) = (beta x_i, y_i) for i < n.
int glv_phi(Ctx* c, affine_t* pts, size_t n);
// G2 bases with the GLV half: pts[n + i] = (beta^2 x_i, y_i) = [lambda] P_i.
int glv_phi2(Ctx* c, affine2_t* pts, size_t n);

// One MSM of a batch: sum_{i < n} scalars[i] * bases[i]; `shifted` (optional) holds the
// window-shifted rows [2^(c j)] bases[i] with row stride `stride` for fixed-base mode.
struct MsmJob {
    const fe* scalars = nullptr;
    uint64_t n = 0;
    const void* bases = nullptr;  // affine_t (G1) or affine2_t (G2) points
    const void* shifted = nullptr;  // affine_t (G1) or affine2_t (G2) rows
    uint32_t shifted_c = 0;
    uint64_t stride = 0;  // points in the base set: row stride of `shifted`, offset of the GLV half
    bool glv = false;     // G1 bases whose phi(P) half sits at bases + stride (GLV split scalars)
    bool inf_points = true;  // the points may hold infinity (all zero): the accumulation tests each
};
struct MsmPlan;
uint32_t msm_auto_window(size_t n);
uint32_t msm_auto_window_glv(size_t n);
uint32_t msm_window_for(const Ctx* c, size_t n, bool glv = false);
int msm_batch_run(Ctx* c, const MsmJob* jobs, size_t count, int scalars_mont, uint32_t window_bits, uint8_t* out_xy,
                  int32_t* out_is_inf);
// G2: out_xy holds 128 bytes per instance (x.c0, x.c1, y.c0, y.c1); no fixed-base mode
int msm_g2_batch_run(Ctx* c, const MsmJob* jobs, size_t count, int scalars_mont, uint32_t window_bits,
                     uint8_t* out_xy, int32_t* out_is_inf);
struct MsmAsync;
int msm_batch_submit(Ctx* c, const MsmJob* jobs, size_t count, int scalars_mont, uint32_t window_bits, bool g2,
                     uint8_t* out_xy, int32_t* out_is_inf, MsmAsync** out);
int msm_batch_wait(MsmAsync* a, int timeout_ms);
void msm_batch_release(MsmAsync* a);
int msm_plan_create(Ctx* c, const MsmJob* jobs, size_t count, int scalars_mont, uint32_t window_bits, bool graph,
                    bool queue, MsmPlan** out);
int msm_plan_slot(MsmPlan* plan, size_t index, void** dev);
uint64_t msm_plan_kernels(const MsmPlan* plan);
int msm_plan_run(Ctx* c, MsmPlan* plan, uint8_t* out_xy, int32_t* out_is_inf);
void msm_plan_destroy(Ctx* c, MsmPlan* plan);
int shift_bases(Ctx* c, const affine_t* bases, size_t n, uint32_t window_bits, affine_t** out, uint32_t* windows);
int shift_bases_g2(Ctx* c, const affine2_t* bases, size_t n, uint32_t window_bits, affine2_t** out,
                   uint32_t* windows);

// One transform of an NTT batch (the arguments of ntt_run).
struct NttJob {
    int mode = 0;
    fe* out = nullptr;
    const fe* in = nullptr;
    size_t in_len = 0;
    uint32_t log_n = 0;
    const uint8_t* omega = nullptr;
    const uint8_t* shift = nullptr;  // null: 1
};
struct NttBatchPlan;
int ntt_batch_run(Ctx* c, const NttJob* jobs, size_t count);
int ntt_plan_create(Ctx* c, const NttJob* jobs, size_t count, bool graph, bool queue, NttBatchPlan** out);
// ZK_OK, or ZK_ETIMEOUT when a work-queue launch since the last call gave up waiting
// (synchronises the context stream; clears the record)
int ntt_queue_status(Ctx* c);
// A work-queue launch whose second pass waits for one more first-pass tile than exist, with
// the given wait limit: returns its status (ZK_ETIMEOUT expected), for tests of the limit.
int ntt_queue_selftest(Ctx* c, uint64_t limit_ns, uint32_t* entry_out);
int ntt_plan_run(Ctx* c, NttBatchPlan* plan);
uint64_t ntt_plan_kernels(const NttBatchPlan* plan);
void ntt_plan_destroy(Ctx* c, NttBatchPlan* plan);

}  // namespace zk

struct zk_ctx {
    zk::Ctx impl;
};

struct zk_fence {
    int device = 0;
    cudaEvent_t ev = nullptr;
};

struct zk_bases {
    zk_ctx* ctx;
    // G1: 2n Montgomery affine points, (0, 0) = infinity: P_0..P_{n-1}, then their GLV images
    // phi(P_i) = (beta x_i, y_i) (null for G2 bases)
    zk::affine_t* dev;
    size_t n;
    zk::affine2_t* dev2 = nullptr;  // G2: 2n Montgomery affine points over Fq2, then their GLV images
                                    // (beta^2 x, y) (null for G1 bases)
    zk::affine_t* shifted = nullptr;  // fixed-base rows [2^(c j)] P_i, j < shifted_windows, row stride n
    zk::affine2_t* shifted2 = nullptr;  // the same rows of G2 bases
    uint32_t shifted_c = 0;
    uint32_t shifted_windows = 0;
    bool has_inf = true;  // some point is infinity (found on the device when the set is created)
};

struct zk_batch {
    zk::MsmAsync* impl;
};

struct zk_msm_plan {
    zk_ctx* ctx;
    zk::MsmPlan* impl;
};

struct zk_ntt_plan {
    zk_ctx* ctx;
    zk::NttBatchPlan* impl;
};
