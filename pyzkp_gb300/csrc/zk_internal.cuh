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

// Device tables of one NTT configuration (transform size, root, coset shift, direction).
struct NttPlan {
    uint32_t log_n = 0;
    int npass = 0;
    uint32_t pass_log_r[4] = {0, 0, 0, 0};
    fe* radix_tw[4] = {nullptr, nullptr, nullptr, nullptr};  // omega_R^i, i < R/2, per pass
    uint32_t s_bits = 0;                                       // split of two-level tables
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
    cudaStream_t stream = nullptr;
    std::mutex mu;
    std::map<std::string, NttPlan*> ntt_plans;
    uint64_t launches = 0;
    bool prof_on = false;
    std::map<std::string, ProfEntry> prof;
    std::vector<ProfPending> prof_pending;
    std::vector<cudaEvent_t> event_pool;
    cudaEvent_t timer_start = nullptr, timer_stop = nullptr;
    uint64_t msm_entries = 0;
    uint32_t msm_window_bits = 0, msm_windows = 0;
};

int prof_begin(Ctx* c, const char* name);
void prof_end(Ctx* c, int token);
int prof_resolve(Ctx* c);
// Host-side work inside a library call, recorded in the same table when profiling is on
// (not counted as a kernel launch).
void prof_host(Ctx* c, const char* name, double ms);

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
            const uint8_t shift[32]);
int msm_run(Ctx* c, const affine_t* bases, const fe* scalars, size_t n, int scalars_mont, uint32_t window_bits,
            uint8_t out_xy[64], int* out_is_inf, const affine_t* shifted = nullptr, uint32_t shifted_c = 0,
            uint64_t stride = 0);
int shift_bases(Ctx* c, const affine_t* bases, size_t n, uint32_t window_bits, affine_t** out, uint32_t* windows);

}  // namespace zk

struct zk_ctx {
    zk::Ctx impl;
};

struct zk_bases {
    zk_ctx* ctx;
    zk::affine_t* dev;  // Montgomery affine, (0, 0) = infinity
    size_t n;
    zk::affine_t* shifted = nullptr;  // fixed-base rows [2^(c j)] P_i, j < shifted_windows, row stride n
    uint32_t shifted_c = 0;
    uint32_t shifted_windows = 0;
};
