// capi.cu -- extern "C" entry points declared in include/zkgpu.h.
#include <chrono>
#include <cstring>
#include <iterator>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "zk_internal.cuh"

namespace zk {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

int scratch_alloc(Ctx* c, size_t bytes, void** p) {
    *p = nullptr;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMallocAsync(p, bytes, c->stream);
    if (e != cudaSuccess) {
        set_error(std::string("cudaMallocAsync(") + std::to_string(bytes) + "): " + cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? ZK_ENOMEM : ZK_ECUDA;
    }
    return ZK_OK;
}

void scratch_free(Ctx* c, void* p) {
    if (p) cudaFreeAsync(p, c->stream);
}

int pinned_take(Ctx* c, size_t bytes, void** p, size_t* got) {
    {
        std::lock_guard<std::mutex> g(c->pinned_mu);
        auto it = c->pinned_free.lower_bound(bytes);
        // reuse a block of up to 4x the size asked for; a larger one stays for larger asks
        if (it != c->pinned_free.end() && it->first <= 4 * bytes + 4096) {
            *p = it->second;
            *got = it->first;
            c->pinned_free.erase(it);
            return ZK_OK;
        }
    }
    ZK_TRY_CUDA(cudaMallocHost(p, bytes ? bytes : 16));
    *got = bytes ? bytes : 16;
    return ZK_OK;
}

void pinned_give(Ctx* c, void* p, size_t bytes) {
    if (p == nullptr) return;
    std::lock_guard<std::mutex> g(c->pinned_mu);
    c->pinned_free.emplace(bytes, p);
}

static cudaEvent_t take_event(Ctx* c) {
    if (!c->event_pool.empty()) {
        cudaEvent_t e = c->event_pool.back();
        c->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

int prof_begin(Ctx* c, const char* name) {
    c->launches++;
    if (!c->prof_on) {
        c->prof[name].launches++;
        return -1;
    }
    ProfPending p;
    p.name = name;
    p.start = take_event(c);
    p.stop = take_event(c);
    cudaEventRecord(p.start, c->stream);
    c->prof_pending.push_back(p);
    return (int)c->prof_pending.size() - 1;
}

void prof_host(Ctx* c, const char* name, double ms) {
    if (!c->prof_on) return;
    ProfEntry& e = c->prof[name];
    e.launches++;
    e.total_ms += ms;
}

void prof_end(Ctx* c, int token) {
    if (token < 0) return;
    cudaEventRecord(c->prof_pending[token].stop, c->stream);
}

int prof_resolve(Ctx* c) {
    if (c->prof_pending.empty()) return ZK_OK;
    ZK_TRY_CUDA(cudaStreamSynchronize(c->stream));
    for (auto& p : c->prof_pending) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p.start, p.stop);
        ProfEntry& e = c->prof[p.name];
        e.launches++;
        e.total_ms += ms;
        c->event_pool.push_back(p.start);
        c->event_pool.push_back(p.stop);
    }
    c->prof_pending.clear();
    return ZK_OK;
}

template <class F, int DIR>
int convert(Ctx* c, void* out, const void* in, size_t n);
int fr_binary(Ctx* c, int op, void* out, const void* a, const void* b, size_t n);
int fixed_base_mul(Ctx* c, const uint8_t point_xy[64], const void* k_dev, size_t n, void* out_dev);
int fixed_base_mul_g2(Ctx* c, const uint8_t point_xy[128], const void* k_dev, size_t n, void* out_dev);
int imad_peak(Ctx* c, double* tera);
int imad_probe(Ctx* c, int mode, double* tera);
int trimmed_len(Ctx* c, const void* a, size_t n, size_t* out);

}  // namespace zk

using zk::Ctx;

#define CTX_OR_FAIL(ctx)                         \
    do {                                         \
        if ((ctx) == nullptr) {                  \
            zk::set_error("null zk_ctx");        \
            return ZK_EINVAL;                    \
        }                                        \
        cudaError_t _e = cudaSetDevice((ctx)->impl.device); \
        if (_e != cudaSuccess) {                 \
            zk::set_error(cudaGetErrorString(_e)); \
            return ZK_ECUDA;                     \
        }                                        \
    } while (0)

extern "C" {

const char* zk_last_error(void) { return zk::g_last_error.c_str(); }

int zk_version(void) { return 1; }

int zk_ctx_create_prio(int device, int priority, zk_ctx** out) {
    if (out == nullptr) {
        zk::set_error("null output pointer");
        return ZK_EINVAL;
    }
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        zk::set_error(std::string("no CUDA device available: ") + (e != cudaSuccess ? cudaGetErrorString(e) : "0"));
        return ZK_ENODEV;
    }
    if (device < 0 || device >= count) {
        zk::set_error("device index out of range");
        return ZK_EINVAL;
    }
    ZK_TRY_CUDA(cudaSetDevice(device));
    int least = 0, greatest = 0;
    ZK_TRY_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    // clamp into the device's range (greatest is the most urgent, numerically smallest)
    if (priority > least) priority = least;
    if (priority < greatest) priority = greatest;
    std::unique_ptr<zk_ctx> c(new zk_ctx());
    c->impl.device = device;
    c->impl.priority = priority;
    ZK_TRY_CUDA(cudaDeviceGetAttribute(&c->impl.num_sms, cudaDevAttrMultiProcessorCount, device));
    ZK_TRY_CUDA(cudaStreamCreateWithPriority(&c->impl.stream, cudaStreamNonBlocking, priority));
    // keep freed stream-ordered allocations cached in the device pool
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t threshold = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
    }
    *out = c.release();
    return ZK_OK;
}

int zk_ctx_create(int device, zk_ctx** out) { return zk_ctx_create_prio(device, 0, out); }

int zk_stream_priority_range(int* least, int* greatest) {
    if (least == nullptr || greatest == nullptr) {
        zk::set_error("null output pointer");
        return ZK_EINVAL;
    }
    ZK_TRY_CUDA(cudaDeviceGetStreamPriorityRange(least, greatest));
    return ZK_OK;
}

int zk_ctx_destroy(zk_ctx* ctx) {
    if (ctx == nullptr) return ZK_OK;
    cudaSetDevice(ctx->impl.device);
    cudaStreamSynchronize(ctx->impl.stream);
    zk::prof_resolve(&ctx->impl);
    for (cudaEvent_t e : ctx->impl.event_pool) cudaEventDestroy(e);
    if (ctx->impl.timer_start) cudaEventDestroy(ctx->impl.timer_start);
    if (ctx->impl.timer_stop) cudaEventDestroy(ctx->impl.timer_stop);
    for (auto& kv : ctx->impl.ntt_plans) {
        for (void* p : kv.second->allocations) cudaFree(p);
        delete kv.second;
    }
    if (ctx->impl.copy_stream) {
        cudaStreamSynchronize(ctx->impl.copy_stream);
        cudaStreamDestroy(ctx->impl.copy_stream);
    }
    for (cudaStream_t st : ctx->impl.side_streams) {
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
    }
    for (cudaEvent_t ev : ctx->impl.side_events) cudaEventDestroy(ev);
    if (ctx->impl.copy_go) cudaEventDestroy(ctx->impl.copy_go);
    if (ctx->impl.copy_done) cudaEventDestroy(ctx->impl.copy_done);
    for (cudaEvent_t ev : ctx->impl.chunk_ev)
        if (ev) cudaEventDestroy(ev);
    if (ctx->impl.inf_flag_dev) cudaFree(ctx->impl.inf_flag_dev);
    for (auto& st : ctx->impl.host_stage) {
        if (st.dev) cudaFree(st.dev);
        if (st.free_ev) cudaEventDestroy(st.free_ev);
    }
    if (ctx->impl.d2h_stream) {
        cudaStreamSynchronize(ctx->impl.d2h_stream);
        cudaStreamDestroy(ctx->impl.d2h_stream);
    }
    for (auto& st : ctx->impl.ntt_stage) {
        if (st.dev) cudaFree(st.dev);
        for (cudaEvent_t ev : {st.free_ev, st.h2d_ev, st.comp_ev})
            if (ev) cudaEventDestroy(ev);
    }
    if (ctx->impl.ntt_queue_err) cudaFree(ctx->impl.ntt_queue_err);
    for (auto& kv : ctx->impl.pinned_free) cudaFreeHost(kv.second);
    cudaStreamDestroy(ctx->impl.stream);
    delete ctx;
    return ZK_OK;
}

int zk_ctx_sync(zk_ctx* ctx) {
    CTX_OR_FAIL(ctx);
    ZK_TRY_CUDA(cudaStreamSynchronize(ctx->impl.stream));
    return ZK_OK;
}

int zk_ctx_stream(zk_ctx* ctx, void** stream_out) {
    CTX_OR_FAIL(ctx);
    *stream_out = reinterpret_cast<void*>(ctx->impl.stream);
    return ZK_OK;
}

int zk_ctx_num_sms(zk_ctx* ctx, int* out) {
    CTX_OR_FAIL(ctx);
    *out = ctx->impl.num_sms;
    return ZK_OK;
}

int zk_d2d(zk_ctx* ctx, void* dst_dev, const void* src_dev, size_t bytes) {
    CTX_OR_FAIL(ctx);
    if (bytes == 0) return ZK_OK;
    ZK_TRY_CUDA(cudaMemcpyAsync(dst_dev, src_dev, bytes, cudaMemcpyDeviceToDevice, ctx->impl.stream));
    return ZK_OK;
}

int zk_fr_trimmed_len(zk_ctx* ctx, const void* a, size_t n, size_t* out) {
    CTX_OR_FAIL(ctx);
    if (out == nullptr) {
        zk::set_error("null output pointer");
        return ZK_EINVAL;
    }
    return zk::trimmed_len(&ctx->impl, a, n, out);
}

int zk_memset(zk_ctx* ctx, void* dptr, int value, size_t bytes) {
    CTX_OR_FAIL(ctx);
    if (bytes == 0) return ZK_OK;
    ZK_TRY_CUDA(cudaMemsetAsync(dptr, value, bytes, ctx->impl.stream));
    return ZK_OK;
}

int zk_launch_count(zk_ctx* ctx, uint64_t* out) {
    CTX_OR_FAIL(ctx);
    *out = ctx->impl.launches;
    return ZK_OK;
}

int zk_prof_enable(zk_ctx* ctx, int on) {
    CTX_OR_FAIL(ctx);
    int rc = zk::prof_resolve(&ctx->impl);
    ctx->impl.prof_on = on != 0;
    return rc;
}

int zk_prof_reset(zk_ctx* ctx) {
    CTX_OR_FAIL(ctx);
    int rc = zk::prof_resolve(&ctx->impl);
    ctx->impl.prof.clear();
    return rc;
}

int zk_prof_count(zk_ctx* ctx, int* nkernels) {
    CTX_OR_FAIL(ctx);
    int rc = zk::prof_resolve(&ctx->impl);
    *nkernels = (int)ctx->impl.prof.size();
    return rc;
}

int zk_prof_get(zk_ctx* ctx, int idx, char* name_buf, size_t name_len, uint64_t* launches, double* total_ms) {
    CTX_OR_FAIL(ctx);
    int rc = zk::prof_resolve(&ctx->impl);
    if (rc != ZK_OK) return rc;
    if (idx < 0 || idx >= (int)ctx->impl.prof.size() || name_buf == nullptr || name_len == 0) {
        zk::set_error("profile index out of range");
        return ZK_EINVAL;
    }
    auto it = ctx->impl.prof.begin();
    std::advance(it, idx);
    std::strncpy(name_buf, it->first.c_str(), name_len - 1);
    name_buf[name_len - 1] = 0;
    *launches = it->second.launches;
    *total_ms = it->second.total_ms;
    return ZK_OK;
}

int zk_timer_start(zk_ctx* ctx) {
    CTX_OR_FAIL(ctx);
    zk::Ctx* c = &ctx->impl;
    if (!c->timer_start) ZK_TRY_CUDA(cudaEventCreate(&c->timer_start));
    if (!c->timer_stop) ZK_TRY_CUDA(cudaEventCreate(&c->timer_stop));
    ZK_TRY_CUDA(cudaEventRecord(c->timer_start, c->stream));
    return ZK_OK;
}

int zk_timer_stop(zk_ctx* ctx, double* ms) {
    CTX_OR_FAIL(ctx);
    zk::Ctx* c = &ctx->impl;
    if (!c->timer_start || !c->timer_stop) {
        zk::set_error("zk_timer_stop without zk_timer_start");
        return ZK_EINVAL;
    }
    ZK_TRY_CUDA(cudaEventRecord(c->timer_stop, c->stream));
    ZK_TRY_CUDA(cudaEventSynchronize(c->timer_stop));
    float f = 0.f;
    ZK_TRY_CUDA(cudaEventElapsedTime(&f, c->timer_start, c->timer_stop));
    *ms = f;
    return ZK_OK;
}

int zk_msm_last_stats(zk_ctx* ctx, uint64_t* entries, uint32_t* window_bits, uint32_t* windows) {
    CTX_OR_FAIL(ctx);
    *entries = ctx->impl.msm_entries;
    *window_bits = ctx->impl.msm_window_bits;
    *windows = ctx->impl.msm_windows;
    return ZK_OK;
}

int zk_imad_peak(zk_ctx* ctx, double* tera_imad_per_s) {
    CTX_OR_FAIL(ctx);
    return zk::imad_peak(&ctx->impl, tera_imad_per_s);
}

int zk_imad_probe(zk_ctx* ctx, int mode, double* tera_imad_per_s) {
    CTX_OR_FAIL(ctx);
    return zk::imad_probe(&ctx->impl, mode, tera_imad_per_s);
}

int zk_alloc(zk_ctx* ctx, size_t bytes, void** dptr) {
    CTX_OR_FAIL(ctx);
    if (dptr == nullptr) {
        zk::set_error("null output pointer");
        return ZK_EINVAL;
    }
    return zk::scratch_alloc(&ctx->impl, bytes, dptr);
}

int zk_free(zk_ctx* ctx, void* dptr) {
    CTX_OR_FAIL(ctx);
    zk::scratch_free(&ctx->impl, dptr);
    return ZK_OK;
}

int zk_h2d(zk_ctx* ctx, void* dst_dev, const void* src_host, size_t bytes) {
    CTX_OR_FAIL(ctx);
    if (bytes == 0) return ZK_OK;
    ZK_TRY_CUDA(cudaMemcpyAsync(dst_dev, src_host, bytes, cudaMemcpyHostToDevice, ctx->impl.stream));
    ZK_TRY_CUDA(cudaStreamSynchronize(ctx->impl.stream));
    return ZK_OK;
}

int zk_d2h(zk_ctx* ctx, void* dst_host, const void* src_dev, size_t bytes) {
    CTX_OR_FAIL(ctx);
    if (bytes == 0) return ZK_OK;
    ZK_TRY_CUDA(cudaMemcpyAsync(dst_host, src_dev, bytes, cudaMemcpyDeviceToHost, ctx->impl.stream));
    ZK_TRY_CUDA(cudaStreamSynchronize(ctx->impl.stream));
    return ZK_OK;
}

int zk_h2d_async(zk_ctx* ctx, void* dst_dev, const void* src_host, size_t bytes) {
    CTX_OR_FAIL(ctx);
    if (bytes == 0) return ZK_OK;
    if (dst_dev == nullptr || src_host == nullptr) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    ZK_TRY_CUDA(cudaMemcpyAsync(dst_dev, src_host, bytes, cudaMemcpyHostToDevice, ctx->impl.stream));
    return ZK_OK;
}

int zk_d2h_async(zk_ctx* ctx, void* dst_host, const void* src_dev, size_t bytes) {
    CTX_OR_FAIL(ctx);
    if (bytes == 0) return ZK_OK;
    if (dst_host == nullptr || src_dev == nullptr) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    ZK_TRY_CUDA(cudaMemcpyAsync(dst_host, src_dev, bytes, cudaMemcpyDeviceToHost, ctx->impl.stream));
    return ZK_OK;
}

int zk_fence_record(zk_ctx* ctx, zk_fence** out) {
    CTX_OR_FAIL(ctx);
    if (out == nullptr) {
        zk::set_error("null output pointer");
        return ZK_EINVAL;
    }
    *out = nullptr;
    std::unique_ptr<zk_fence> f(new zk_fence());
    f->device = ctx->impl.device;
    ZK_TRY_CUDA(cudaEventCreateWithFlags(&f->ev, cudaEventDisableTiming));
    cudaError_t e = cudaEventRecord(f->ev, ctx->impl.stream);
    if (e != cudaSuccess) {
        cudaEventDestroy(f->ev);
        zk::set_error(std::string("cudaEventRecord: ") + cudaGetErrorString(e));
        return ZK_ECUDA;
    }
    *out = f.release();
    return ZK_OK;
}

int zk_fence_wait(zk_fence* f, int timeout_ms) {
    if (f == nullptr) {
        zk::set_error("null zk_fence");
        return ZK_EINVAL;
    }
    cudaSetDevice(f->device);
    if (timeout_ms < 0) {
        ZK_TRY_CUDA(cudaEventSynchronize(f->ev));
        return ZK_OK;
    }
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms);
    for (;;) {
        const cudaError_t e = cudaEventQuery(f->ev);
        if (e == cudaSuccess) return ZK_OK;
        if (e != cudaErrorNotReady) {
            zk::set_error(std::string("zk_fence_wait: ") + cudaGetErrorString(e));
            return ZK_ECUDA;
        }
        if (std::chrono::steady_clock::now() >= deadline) {
            zk::set_error("zk_fence_wait: the fence has not passed yet");
            return ZK_ETIMEOUT;
        }
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

int zk_fence_destroy(zk_fence* f) {
    if (f == nullptr) return ZK_OK;
    cudaSetDevice(f->device);
    cudaEventDestroy(f->ev);
    delete f;
    return ZK_OK;
}

int zk_host_alloc(size_t bytes, void** out) {
    ZK_TRY_CUDA(cudaMallocHost(out, bytes ? bytes : 16));
    return ZK_OK;
}

int zk_host_free(void* p) {
    if (p) ZK_TRY_CUDA(cudaFreeHost(p));
    return ZK_OK;
}

int zk_fr_to_mont(zk_ctx* ctx, void* out, const void* in, size_t n) {
    CTX_OR_FAIL(ctx);
    return zk::convert<zk::FrP, 1>(&ctx->impl, out, in, n);
}

int zk_fr_from_mont(zk_ctx* ctx, void* out, const void* in, size_t n) {
    CTX_OR_FAIL(ctx);
    return zk::convert<zk::FrP, 0>(&ctx->impl, out, in, n);
}

int zk_fq_to_mont(zk_ctx* ctx, void* out, const void* in, size_t n) {
    CTX_OR_FAIL(ctx);
    return zk::convert<zk::FqP, 1>(&ctx->impl, out, in, n);
}

int zk_fq_from_mont(zk_ctx* ctx, void* out, const void* in, size_t n) {
    CTX_OR_FAIL(ctx);
    return zk::convert<zk::FqP, 0>(&ctx->impl, out, in, n);
}

int zk_fr_mul(zk_ctx* ctx, void* out, const void* a, const void* b, size_t n) {
    CTX_OR_FAIL(ctx);
    return zk::fr_binary(&ctx->impl, 0, out, a, b, n);
}

int zk_fr_sub(zk_ctx* ctx, void* out, const void* a, const void* b, size_t n) {
    CTX_OR_FAIL(ctx);
    return zk::fr_binary(&ctx->impl, 1, out, a, b, n);
}

int zk_fr_add(zk_ctx* ctx, void* out, const void* a, const void* b, size_t n) {
    CTX_OR_FAIL(ctx);
    return zk::fr_binary(&ctx->impl, 2, out, a, b, n);
}

int zk_ntt(zk_ctx* ctx, int mode, void* out_dev, const void* in_dev, size_t in_len, uint32_t log_n,
           const uint8_t omega[32], const uint8_t shift[32]) {
    CTX_OR_FAIL(ctx);
    static const uint8_t one[32] = {1};
    if (omega == nullptr) {
        zk::set_error("null omega");
        return ZK_EINVAL;
    }
    return zk::ntt_run(&ctx->impl, mode, static_cast<zk::fe*>(out_dev), static_cast<const zk::fe*>(in_dev), in_len,
                       log_n, omega, shift ? shift : one);
}

static int bases_from_dev_canonical(zk_ctx* ctx, const void* xy_dev, size_t n, zk_bases** out) {
    zk_bases* b = new zk_bases();
    b->ctx = ctx;
    b->n = n;
    b->dev = nullptr;
    int rc = zk::scratch_alloc(&ctx->impl, 2 * n * sizeof(zk::affine_t), reinterpret_cast<void**>(&b->dev));
    if (rc != ZK_OK) {
        delete b;
        return rc;
    }
    // (x, y) canonical -> Montgomery, as 2n base-field elements; (0, 0) stays (0, 0); then
    // the GLV images phi(P_i) behind them
    rc = zk::convert<zk::FqP, 1>(&ctx->impl, b->dev, xy_dev, 2 * n);
    if (rc == ZK_OK) rc = zk::glv_phi(&ctx->impl, b->dev, n);
    if (rc == ZK_OK) rc = zk::any_infinity(&ctx->impl, b->dev, n, false, &b->has_inf);
    if (rc != ZK_OK) {
        zk::scratch_free(&ctx->impl, b->dev);
        delete b;
        return rc;
    }
    *out = b;
    return ZK_OK;
}

int zk_bases_create(zk_ctx* ctx, const void* xy_canonical_host, size_t n, zk_bases** out) {
    CTX_OR_FAIL(ctx);
    if (out == nullptr || (n && xy_canonical_host == nullptr)) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    void* tmp = nullptr;
    int rc = zk::scratch_alloc(&ctx->impl, n * 64, &tmp);
    if (rc != ZK_OK) return rc;
    if (n) ZK_TRY_CUDA(cudaMemcpyAsync(tmp, xy_canonical_host, n * 64, cudaMemcpyHostToDevice, ctx->impl.stream));
    rc = bases_from_dev_canonical(ctx, tmp, n, out);
    zk::scratch_free(&ctx->impl, tmp);
    if (rc == ZK_OK) ZK_TRY_CUDA(cudaStreamSynchronize(ctx->impl.stream));
    return rc;
}

int zk_bases_create_dev(zk_ctx* ctx, const void* xy_canonical_dev, size_t n, zk_bases** out) {
    CTX_OR_FAIL(ctx);
    if (out == nullptr || (n && xy_canonical_dev == nullptr)) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    int rc = bases_from_dev_canonical(ctx, xy_canonical_dev, n, out);
    if (rc == ZK_OK) ZK_TRY_CUDA(cudaStreamSynchronize(ctx->impl.stream));
    return rc;
}

int zk_bases_precompute(zk_ctx* ctx, zk_bases* b, uint32_t window_bits) {
    CTX_OR_FAIL(ctx);
    if (b == nullptr || (b->dev == nullptr && b->dev2 == nullptr)) {
        zk::set_error("zk_bases_precompute needs a bases handle");
        return ZK_EINVAL;
    }
    if ((b->shifted || b->shifted2) && b->shifted_c == window_bits) return ZK_OK;
    uint32_t windows = 0;
    int rc = ZK_OK;
    if (b->dev2) {  // G2 bases
        zk::affine2_t* rows = nullptr;
        if ((rc = zk::shift_bases_g2(&ctx->impl, b->dev2, b->n, window_bits, &rows, &windows)) != ZK_OK) return rc;
        if (b->shifted2) zk::scratch_free(&ctx->impl, b->shifted2);
        b->shifted2 = rows;
    } else {
        zk::affine_t* rows = nullptr;
        // rows of P only: rows of phi(P) as well (GLV halves over one shared bucket set) measured
        // slower in the steady state (2^20: 234 vs 251 Mpts/s at the best window of each), their
        // short top windows crowding a few buckets
        if ((rc = zk::shift_bases(&ctx->impl, b->dev, b->n, window_bits, &rows, &windows)) != ZK_OK) return rc;
        if (b->shifted) zk::scratch_free(&ctx->impl, b->shifted);
        b->shifted = rows;
    }
    b->shifted_c = window_bits;
    b->shifted_windows = windows;
    ZK_TRY_CUDA(cudaStreamSynchronize(ctx->impl.stream));
    return ZK_OK;
}

int zk_bases_destroy(zk_bases* b) {
    if (b == nullptr) return ZK_OK;
    cudaSetDevice(b->ctx->impl.device);
    if (b->shifted) zk::scratch_free(&b->ctx->impl, b->shifted);
    if (b->shifted2) zk::scratch_free(&b->ctx->impl, b->shifted2);
    if (b->dev) zk::scratch_free(&b->ctx->impl, b->dev);
    if (b->dev2) zk::scratch_free(&b->ctx->impl, b->dev2);
    delete b;
    return ZK_OK;
}

int zk_bases_count(const zk_bases* b, size_t* n) {
    if (b == nullptr || n == nullptr) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    *n = b->n;
    return ZK_OK;
}

int zk_msm_g1(zk_ctx* ctx, const zk_bases* bases, size_t offset, const void* scalars_dev, size_t n, int scalars_mont,
              uint32_t window_bits, uint8_t out_xy[64], int* out_is_inf) {
    CTX_OR_FAIL(ctx);
    if (bases == nullptr || out_xy == nullptr || out_is_inf == nullptr || (n && scalars_dev == nullptr)) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    if (bases->dev == nullptr) {
        zk::set_error("zk_msm_g1 needs G1 bases (this handle holds G2 points)");
        return ZK_EINVAL;
    }
    if (offset > bases->n || n > bases->n - offset) {
        zk::set_error("scalars length exceeds points length");
        return ZK_EINVAL;
    }
    return zk::msm_run(&ctx->impl, bases->dev + offset, static_cast<const zk::fe*>(scalars_dev), n, scalars_mont,
                       window_bits, out_xy, out_is_inf, bases->shifted ? bases->shifted + offset : nullptr,
                       bases->shifted_c, bases->n, /*glv=*/true, bases->has_inf);
}

// The lazily created resources of the host-buffer MSMs, each under its own check: a failure
// part way leaves the rest to be created by the next call.
static int host_msm_resources(Ctx* c) {
    if (c->copy_stream == nullptr)
        ZK_TRY_CUDA(cudaStreamCreateWithPriority(&c->copy_stream, cudaStreamNonBlocking, c->priority));
    if (c->copy_go == nullptr) ZK_TRY_CUDA(cudaEventCreateWithFlags(&c->copy_go, cudaEventDisableTiming));
    if (c->copy_done == nullptr) ZK_TRY_CUDA(cudaEventCreateWithFlags(&c->copy_done, cudaEventDisableTiming));
    for (cudaEvent_t& ev : c->chunk_ev)
        if (ev == nullptr) ZK_TRY_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    return ZK_OK;
}

// On the copy stream (after `wait`, an event on the main stream that orders the reuse of the
// device buffers): the scalars first, alone on the link, in chunks whose digits the main
// stream sorts as each arrives (one chunk below 2^18 scalars); then the points, converted
// there too, with the infinity flag (only the accumulation, after the sort, waits for those:
// copy_done). Sets c->scalar_chunks; returns the first CUDA error.
static cudaError_t host_msm_upload(Ctx* c, cudaEvent_t wait, const void* xy_canonical_host,
                                   const void* scalars_host, size_t n, void* bases, void* scalars,
                                   uint32_t* inf_flag, int* rc) {
    const size_t nchunks = n >= ((size_t)1 << 18) ? 4 : 1;
    c->scalar_chunks.clear();
    cudaError_t e = wait ? cudaStreamWaitEvent(c->copy_stream, wait, 0) : cudaSuccess;
    for (size_t q = 0, j0 = 0; q < nchunks && e == cudaSuccess; q++) {
        const size_t j1 = q + 1 == nchunks ? n : std::min(n, ((q + 1) * n / nchunks + 255) & ~(size_t)255);
        e = cudaMemcpyAsync(static_cast<uint8_t*>(scalars) + j0 * 32, static_cast<const uint8_t*>(scalars_host) + j0 * 32,
                            (j1 - j0) * 32, cudaMemcpyHostToDevice, c->copy_stream);
        if (e == cudaSuccess) e = cudaEventRecord(c->chunk_ev[q], c->copy_stream);
        c->scalar_chunks.emplace_back((uint32_t)j1, c->chunk_ev[q]);
        j0 = j1;
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(bases, xy_canonical_host, n * 64, cudaMemcpyHostToDevice, c->copy_stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(inf_flag, 0, 4, c->copy_stream);
    if (e == cudaSuccess) {
        // on the copy stream: mark infinity points, then convert and add the GLV images
        const cudaStream_t main_stream = c->stream;
        c->stream = c->copy_stream;
        *rc = zk::mark_infinity(c, bases, n, false, inf_flag);
        if (*rc == ZK_OK) *rc = zk::convert<zk::FqP, 1>(c, bases, bases, 2 * n);
        if (*rc == ZK_OK) *rc = zk::glv_phi(c, static_cast<zk::affine_t*>(bases), n);
        c->stream = main_stream;
        e = cudaEventRecord(c->copy_done, c->copy_stream);
    }
    return e;
}

int zk_msm_g1_host(zk_ctx* ctx, const void* xy_canonical_host, const void* scalars_host, size_t n, int scalars_mont,
                   uint32_t window_bits, uint8_t out_xy[64], int* out_is_inf) {
    CTX_OR_FAIL(ctx);
    if (out_xy == nullptr || out_is_inf == nullptr || (n && (xy_canonical_host == nullptr || scalars_host == nullptr))) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    if (n == 0) {
        std::memset(out_xy, 0, 64);
        *out_is_inf = 1;
        return ZK_OK;
    }
    Ctx* c = &ctx->impl;
    int rc = host_msm_resources(c);
    if (rc != ZK_OK) return rc;
    if (c->inf_flag_dev == nullptr) ZK_TRY_CUDA(cudaMalloc(reinterpret_cast<void**>(&c->inf_flag_dev), 4));
    void* bases = nullptr;
    void* scalars = nullptr;
    if ((rc = zk::scratch_alloc(c, 2 * n * sizeof(zk::affine_t), &bases)) != ZK_OK) return rc;
    if ((rc = zk::scratch_alloc(c, n * 32, &scalars)) != ZK_OK) {
        zk::scratch_free(c, bases);
        return rc;
    }
    // the copies wait for the main stream's earlier work (the scratch may have served it)
    const cudaStream_t main_stream = c->stream;
    cudaError_t e = cudaEventRecord(c->copy_go, main_stream);
    if (e == cudaSuccess)
        e = host_msm_upload(c, c->copy_go, xy_canonical_host, scalars_host, n, bases, scalars, c->inf_flag_dev, &rc);
    // main stream: digits and sort; the accumulation waits for copy_done (and with it for
    // the infinity flag)
    if (e == cudaSuccess && rc == ZK_OK) {
        c->bases_wait = c->copy_done;
        c->inf_flag = c->inf_flag_dev;
        rc = zk::msm_run(c, static_cast<const zk::affine_t*>(bases), static_cast<const zk::fe*>(scalars), n,
                         scalars_mont, window_bits, out_xy, out_is_inf, nullptr, 0, n, /*glv=*/true);
        c->inf_flag = nullptr;
        c->bases_wait = nullptr;
    }
    c->scalar_chunks.clear();
    // the frees are ordered on the main stream: after the copy stream is done with `bases`
    cudaStreamWaitEvent(main_stream, c->copy_done, 0);
    zk::scratch_free(c, scalars);
    zk::scratch_free(c, bases);
    if (e != cudaSuccess) {
        zk::set_error(std::string("zk_msm_g1_host: ") + cudaGetErrorString(e));
        cudaStreamSynchronize(main_stream);
        return ZK_ECUDA;
    }
    return rc;
}

int zk_msm_g1_host_submit(zk_ctx* ctx, const void* xy_canonical_host, const void* scalars_host, size_t n,
                          int scalars_mont, uint32_t window_bits, uint8_t* out_xy, int32_t* out_is_inf,
                          zk_batch** out) {
    CTX_OR_FAIL(ctx);
    if (out == nullptr || out_xy == nullptr || out_is_inf == nullptr ||
        (n && (xy_canonical_host == nullptr || scalars_host == nullptr))) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    *out = nullptr;
    Ctx* c = &ctx->impl;
    zk::MsmJob job;
    job.n = n;
    job.stride = n;
    job.glv = true;
    zk::MsmAsync* impl = nullptr;
    if (n == 0) {  // nothing to upload: a finished batch holding the identity
        int rc = zk::msm_batch_submit(c, &job, 1, scalars_mont, window_bits, false, out_xy, out_is_inf, &impl);
        if (rc != ZK_OK) return rc;
        *out = new zk_batch{impl};
        return ZK_OK;
    }
    int rc = host_msm_resources(c);
    if (rc != ZK_OK) return rc;
    // one of two staging buffers (points with their GLV images, scalars, infinity flag); its
    // previous user (two calls back) released it with free_ev on the main stream
    Ctx::HostStage& slot = c->host_stage[c->host_stage_next];
    const size_t scal_at = 2 * n * sizeof(zk::affine_t), flag_at = scal_at + ((n * 32 + 255) & ~(size_t)255);
    const size_t need = flag_at + 256;
    if (slot.free_ev == nullptr) ZK_TRY_CUDA(cudaEventCreateWithFlags(&slot.free_ev, cudaEventDisableTiming));
    if (slot.bytes < need) {
        if (slot.dev != nullptr) {
            ZK_TRY_CUDA(cudaEventSynchronize(slot.free_ev));
            cudaFree(slot.dev);
            slot.dev = nullptr;
            slot.bytes = 0;
        }
        void* p = nullptr;
        if (cudaMalloc(&p, need) != cudaSuccess) {
            cudaGetLastError();
            zk::set_error("zk_msm_g1_host_submit: device memory exhausted for the staging buffer");
            return ZK_ENOMEM;
        }
        slot.dev = p;
        slot.bytes = need;
        slot.used = false;
    }
    c->host_stage_next ^= 1;
    char* base = static_cast<char*>(slot.dev);
    uint32_t* flag = reinterpret_cast<uint32_t*>(base + flag_at);
    cudaError_t e = host_msm_upload(c, slot.used ? slot.free_ev : nullptr, xy_canonical_host, scalars_host, n, base,
                                    base + scal_at, flag, &rc);
    if (e == cudaSuccess && rc == ZK_OK) {
        job.bases = reinterpret_cast<const zk::affine_t*>(base);
        job.scalars = reinterpret_cast<const zk::fe*>(base + scal_at);
        c->bases_wait = c->copy_done;
        c->inf_flag = flag;
        rc = zk::msm_batch_submit(c, &job, 1, scalars_mont, window_bits, false, out_xy, out_is_inf, &impl);
        c->inf_flag = nullptr;
        c->bases_wait = nullptr;
    }
    c->scalar_chunks.clear();
    // the buffer is free again once the main stream has passed this MSM (and the copy stream
    // its uploads, which the MSM waited for)
    cudaStreamWaitEvent(c->stream, c->copy_done, 0);
    cudaEventRecord(slot.free_ev, c->stream);
    slot.used = true;
    if (e != cudaSuccess) {
        zk::set_error(std::string("zk_msm_g1_host_submit: ") + cudaGetErrorString(e));
        cudaStreamSynchronize(c->stream);
        if (impl) zk::msm_batch_release(impl);
        return ZK_ECUDA;
    }
    if (rc != ZK_OK) return rc;
    *out = new zk_batch{impl};
    return ZK_OK;
}

int zk_g1_fixed_base_mul(zk_ctx* ctx, const uint8_t point_xy[64], const void* k_dev, size_t n, void* out_xy_dev) {
    CTX_OR_FAIL(ctx);
    if (point_xy == nullptr) {
        zk::set_error("null point");
        return ZK_EINVAL;
    }
    return zk::fixed_base_mul(&ctx->impl, point_xy, k_dev, n, out_xy_dev);
}

// ---- batched MSM ------------------------------------------------------------------------
static int make_jobs(size_t count, const zk_bases* const* bases, const uint64_t* offsets,
                     const void* const* scalars_dev, const uint64_t* sizes, std::vector<zk::MsmJob>* jobs,
                     bool g2 = false) {
    if (count && (bases == nullptr || sizes == nullptr)) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    jobs->resize(count);
    for (size_t k = 0; k < count; k++) {
        const zk_bases* b = bases[k];
        const uint64_t off = offsets ? offsets[k] : 0;
        if (b == nullptr) {
            zk::set_error("null bases handle in batch");
            return ZK_EINVAL;
        }
        if ((g2 ? (const void*)b->dev2 : (const void*)b->dev) == nullptr) {
            zk::set_error(g2 ? "G2 MSM needs G2 bases" : "G1 MSM needs G1 bases");
            return ZK_EINVAL;
        }
        if (off > b->n || sizes[k] > b->n - off) {
            zk::set_error("scalars length exceeds points length");
            return ZK_EINVAL;
        }
        zk::MsmJob& j = (*jobs)[k];
        j.scalars = scalars_dev ? static_cast<const zk::fe*>(scalars_dev[k]) : nullptr;
        if (scalars_dev && sizes[k] && j.scalars == nullptr) {
            zk::set_error("null scalars in batch");
            return ZK_EINVAL;
        }
        j.n = sizes[k];
        if (g2) {
            j.bases = b->dev2 + off;
            j.shifted = b->shifted2 ? b->shifted2 + off : nullptr;
            j.glv = true;
        } else {
            j.bases = b->dev + off;
            j.shifted = b->shifted ? b->shifted + off : nullptr;
            j.glv = true;
        }
        j.shifted_c = b->shifted_c;
        j.stride = b->n;
        j.inf_points = b->has_inf;
    }
    return ZK_OK;
}

int zk_msm_g1_batch(zk_ctx* ctx, size_t count, const zk_bases* const* bases, const uint64_t* offsets,
                    const void* const* scalars_dev, const uint64_t* sizes, int scalars_mont, uint32_t window_bits,
                    uint8_t* out_xy, int32_t* out_is_inf) {
    CTX_OR_FAIL(ctx);
    if (count && (scalars_dev == nullptr || out_xy == nullptr || out_is_inf == nullptr)) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    std::vector<zk::MsmJob> jobs;
    int rc = make_jobs(count, bases, offsets, scalars_dev, sizes, &jobs);
    if (rc != ZK_OK) return rc;
    return zk::msm_batch_run(&ctx->impl, jobs.data(), count, scalars_mont, window_bits, out_xy, out_is_inf);
}

static int batch_submit_common(zk_ctx* ctx, bool g2, size_t count, const zk_bases* const* bases,
                               const uint64_t* offsets, const void* const* scalars_dev, const uint64_t* sizes,
                               int scalars_mont, uint32_t window_bits, uint8_t* out_xy, int32_t* out_is_inf,
                               zk_batch** out) {
    CTX_OR_FAIL(ctx);
    if (out == nullptr || (count && (scalars_dev == nullptr || out_xy == nullptr || out_is_inf == nullptr))) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    *out = nullptr;
    std::vector<zk::MsmJob> jobs;
    int rc = make_jobs(count, bases, offsets, scalars_dev, sizes, &jobs, g2);
    if (rc != ZK_OK) return rc;
    zk::MsmAsync* a = nullptr;
    rc = zk::msm_batch_submit(&ctx->impl, jobs.data(), count, scalars_mont, window_bits, g2, out_xy, out_is_inf, &a);
    if (rc != ZK_OK) return rc;
    *out = new zk_batch{a};
    return ZK_OK;
}

int zk_msm_g1_batch_submit(zk_ctx* ctx, size_t count, const zk_bases* const* bases, const uint64_t* offsets,
                           const void* const* scalars_dev, const uint64_t* sizes, int scalars_mont,
                           uint32_t window_bits, uint8_t* out_xy, int32_t* out_is_inf, zk_batch** out) {
    return batch_submit_common(ctx, false, count, bases, offsets, scalars_dev, sizes, scalars_mont, window_bits,
                               out_xy, out_is_inf, out);
}

int zk_msm_g2_batch_submit(zk_ctx* ctx, size_t count, const zk_bases* const* bases, const uint64_t* offsets,
                           const void* const* scalars_dev, const uint64_t* sizes, int scalars_mont,
                           uint32_t window_bits, uint8_t* out_xy, int32_t* out_is_inf, zk_batch** out) {
    return batch_submit_common(ctx, true, count, bases, offsets, scalars_dev, sizes, scalars_mont, window_bits,
                               out_xy, out_is_inf, out);
}

int zk_batch_wait(zk_batch* batch, int timeout_ms) {
    if (batch == nullptr) {
        zk::set_error("null zk_batch");
        return ZK_EINVAL;
    }
    return zk::msm_batch_wait(batch->impl, timeout_ms);
}

int zk_batch_destroy(zk_batch* batch) {
    if (batch == nullptr) return ZK_OK;
    zk::msm_batch_release(batch->impl);
    delete batch;
    return ZK_OK;
}

int zk_msm_plan_create(zk_ctx* ctx, size_t count, const zk_bases* const* bases, const uint64_t* offsets,
                       const uint64_t* sizes, int scalars_mont, uint32_t window_bits, int use_graph,
                       zk_msm_plan** out) {
    CTX_OR_FAIL(ctx);
    if (out == nullptr) {
        zk::set_error("null output pointer");
        return ZK_EINVAL;
    }
    *out = nullptr;
    std::vector<zk::MsmJob> jobs;
    int rc = make_jobs(count, bases, offsets, nullptr, sizes, &jobs);
    if (rc != ZK_OK) return rc;
    if (use_graph & ~(ZK_MSM_PLAN_GRAPH | ZK_MSM_PLAN_QUEUE)) {
        zk::set_error("unknown MSM plan flags");
        return ZK_EINVAL;
    }
    zk::MsmPlan* impl = nullptr;
    rc = zk::msm_plan_create(&ctx->impl, jobs.data(), count, scalars_mont, window_bits,
                             (use_graph & ZK_MSM_PLAN_GRAPH) != 0, (use_graph & ZK_MSM_PLAN_QUEUE) != 0, &impl);
    if (rc != ZK_OK) return rc;
    *out = new zk_msm_plan{ctx, impl};
    return ZK_OK;
}

int zk_msm_batch_set_queue(zk_ctx* ctx, int on) {
    CTX_OR_FAIL(ctx);
    ctx->impl.msm_queue = on != 0;
    return ZK_OK;
}

int zk_msm_queue_test_limit(zk_ctx* ctx, uint64_t limit_us) {
    CTX_OR_FAIL(ctx);
    if (limit_us == 0 || limit_us > 10000000ull) {
        zk::set_error("zk_msm_queue_test_limit: limit_us must be in [1, 10^7]");
        return ZK_EINVAL;
    }
    ctx->impl.msm_queue_test_limit_ns = limit_us * 1000ull;
    return ZK_OK;
}

int zk_msm_plan_scalars(zk_msm_plan* plan, size_t index, void** scalars_dev) {
    if (plan == nullptr || scalars_dev == nullptr) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    return zk::msm_plan_slot(plan->impl, index, scalars_dev);
}

int zk_msm_plan_run(zk_msm_plan* plan, uint8_t* out_xy, int32_t* out_is_inf) {
    if (plan == nullptr || out_xy == nullptr || out_is_inf == nullptr) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    CTX_OR_FAIL(plan->ctx);
    return zk::msm_plan_run(&plan->ctx->impl, plan->impl, out_xy, out_is_inf);
}

int zk_msm_plan_launches(zk_msm_plan* plan, uint64_t* kernels) {
    if (plan == nullptr || kernels == nullptr) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    *kernels = zk::msm_plan_kernels(plan->impl);
    return ZK_OK;
}

int zk_msm_plan_destroy(zk_msm_plan* plan) {
    if (plan == nullptr) return ZK_OK;
    cudaSetDevice(plan->ctx->impl.device);
    zk::msm_plan_destroy(&plan->ctx->impl, plan->impl);
    delete plan;
    return ZK_OK;
}

// ---- G2 -------------------------------------------------------------------------------------
int zk_g2_fixed_base_mul(zk_ctx* ctx, const uint8_t point_xy[128], const void* k_dev, size_t n, void* out_xy_dev) {
    CTX_OR_FAIL(ctx);
    if (point_xy == nullptr) {
        zk::set_error("null point");
        return ZK_EINVAL;
    }
    return zk::fixed_base_mul_g2(&ctx->impl, point_xy, k_dev, n, out_xy_dev);
}

static int bases_g2_create(zk_ctx* ctx, const void* xy_canonical, size_t n, cudaMemcpyKind kind, zk_bases** out) {
    CTX_OR_FAIL(ctx);
    if (out == nullptr || (n && xy_canonical == nullptr)) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    zk_bases* b = new zk_bases();
    b->ctx = ctx;
    b->n = n;
    b->dev = nullptr;
    int rc = zk::scratch_alloc(&ctx->impl, 2 * n * sizeof(zk::affine2_t), reinterpret_cast<void**>(&b->dev2));
    if (rc != ZK_OK) {
        delete b;
        return rc;
    }
    if (n) {
        cudaError_t e = cudaMemcpyAsync(b->dev2, xy_canonical, n * sizeof(zk::affine2_t), kind, ctx->impl.stream);
        // (x.c0, x.c1, y.c0, y.c1) canonical -> Montgomery, as 4n base-field elements in place
        if (e == cudaSuccess) {
            rc = zk::convert<zk::FqP, 1>(&ctx->impl, b->dev2, b->dev2, 4 * n);
            if (rc == ZK_OK) rc = zk::glv_phi2(&ctx->impl, b->dev2, n);  // the GLV images behind them
            if (rc == ZK_OK) rc = zk::any_infinity(&ctx->impl, b->dev2, n, true, &b->has_inf);
        } else {
            zk::set_error(std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e));
            rc = ZK_ECUDA;
        }
        if (rc == ZK_OK && (e = cudaStreamSynchronize(ctx->impl.stream)) != cudaSuccess) {
            zk::set_error(std::string("cudaStreamSynchronize: ") + cudaGetErrorString(e));
            rc = ZK_ECUDA;
        }
    }
    if (rc != ZK_OK) {
        zk::scratch_free(&ctx->impl, b->dev2);
        delete b;
        return rc;
    }
    *out = b;
    return ZK_OK;
}

int zk_bases_g2_create(zk_ctx* ctx, const void* xy_canonical_host, size_t n, zk_bases** out) {
    return bases_g2_create(ctx, xy_canonical_host, n, cudaMemcpyHostToDevice, out);
}

int zk_bases_g2_create_dev(zk_ctx* ctx, const void* xy_canonical_dev, size_t n, zk_bases** out) {
    return bases_g2_create(ctx, xy_canonical_dev, n, cudaMemcpyDeviceToDevice, out);
}

int zk_msm_g2(zk_ctx* ctx, const zk_bases* bases, size_t offset, const void* scalars_dev, size_t n, int scalars_mont,
              uint32_t window_bits, uint8_t out_xy[128], int* out_is_inf) {
    CTX_OR_FAIL(ctx);
    if (bases == nullptr || out_xy == nullptr || out_is_inf == nullptr) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    const uint64_t off = offset, size = n;
    std::vector<zk::MsmJob> jobs;
    int rc = make_jobs(1, &bases, &off, &scalars_dev, &size, &jobs, true);
    if (rc != ZK_OK) return rc;
    int32_t inf = 0;
    rc = zk::msm_g2_batch_run(&ctx->impl, jobs.data(), 1, scalars_mont, window_bits, out_xy, &inf);
    *out_is_inf = inf;
    return rc;
}

int zk_msm_g2_batch(zk_ctx* ctx, size_t count, const zk_bases* const* bases, const uint64_t* offsets,
                    const void* const* scalars_dev, const uint64_t* sizes, int scalars_mont, uint32_t window_bits,
                    uint8_t* out_xy, int32_t* out_is_inf) {
    CTX_OR_FAIL(ctx);
    if (count && (scalars_dev == nullptr || out_xy == nullptr || out_is_inf == nullptr)) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    std::vector<zk::MsmJob> jobs;
    int rc = make_jobs(count, bases, offsets, scalars_dev, sizes, &jobs, true);
    if (rc != ZK_OK) return rc;
    return zk::msm_g2_batch_run(&ctx->impl, jobs.data(), count, scalars_mont, window_bits, out_xy, out_is_inf);
}

// ---- batched NTT ------------------------------------------------------------------------
static int make_ntt_jobs(size_t count, const int* modes, void* const* outs, const void* const* ins,
                         const uint64_t* in_lens, const uint32_t* log_ns, const uint8_t* omegas,
                         const uint8_t* shifts, std::vector<zk::NttJob>* jobs) {
    if (count && (modes == nullptr || outs == nullptr || ins == nullptr || in_lens == nullptr || log_ns == nullptr ||
                  omegas == nullptr)) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    jobs->resize(count);
    for (size_t k = 0; k < count; k++) {
        zk::NttJob& j = (*jobs)[k];
        j.mode = modes[k];
        j.out = static_cast<zk::fe*>(outs[k]);
        j.in = static_cast<const zk::fe*>(ins[k]);
        j.in_len = in_lens[k];
        j.log_n = log_ns[k];
        j.omega = omegas + 32 * k;
        j.shift = shifts ? shifts + 32 * k : nullptr;
    }
    return ZK_OK;
}

int zk_ntt_batch(zk_ctx* ctx, size_t count, const int* modes, void* const* outs, const void* const* ins,
                 const uint64_t* in_lens, const uint32_t* log_ns, const uint8_t* omegas, const uint8_t* shifts) {
    CTX_OR_FAIL(ctx);
    std::vector<zk::NttJob> jobs;
    int rc = make_ntt_jobs(count, modes, outs, ins, in_lens, log_ns, omegas, shifts, &jobs);
    if (rc != ZK_OK) return rc;
    return zk::ntt_batch_run(&ctx->impl, jobs.data(), count);
}

int zk_ntt_plan_create(zk_ctx* ctx, size_t count, const int* modes, void* const* outs, const void* const* ins,
                       const uint64_t* in_lens, const uint32_t* log_ns, const uint8_t* omegas, const uint8_t* shifts,
                       int use_graph, zk_ntt_plan** out) {
    CTX_OR_FAIL(ctx);
    if (out == nullptr) {
        zk::set_error("null output pointer");
        return ZK_EINVAL;
    }
    *out = nullptr;
    std::vector<zk::NttJob> jobs;
    int rc = make_ntt_jobs(count, modes, outs, ins, in_lens, log_ns, omegas, shifts, &jobs);
    if (rc != ZK_OK) return rc;
    if (use_graph & ~(ZK_NTT_PLAN_GRAPH | ZK_NTT_PLAN_QUEUE)) {
        zk::set_error("unknown NTT plan flags");
        return ZK_EINVAL;
    }
    zk::NttBatchPlan* impl = nullptr;
    rc = zk::ntt_plan_create(&ctx->impl, jobs.data(), count, (use_graph & ZK_NTT_PLAN_GRAPH) != 0,
                             (use_graph & ZK_NTT_PLAN_QUEUE) != 0, &impl);
    if (rc != ZK_OK) return rc;
    *out = new zk_ntt_plan{ctx, impl};
    return ZK_OK;
}

int zk_ntt_host_submit(zk_ctx* ctx, int mode, void* out_host, const void* in_host, size_t in_len, uint32_t log_n,
                       const uint8_t omega[32], const uint8_t shift[32], zk_fence** done) {
    CTX_OR_FAIL(ctx);
    if (done == nullptr || out_host == nullptr || omega == nullptr || (in_len && in_host == nullptr)) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    *done = nullptr;
    if (log_n > 28) {
        zk::set_error("domain too large for BN254 root of unity (log2 n > 28)");
        return ZK_EINVAL;
    }
    Ctx* c = &ctx->impl;
    const size_t n = (size_t)1 << log_n, valid = in_len < n ? in_len : n;
    const bool inverse = (mode == ZK_NTT_COEFFS_FROM_EVALS || mode == ZK_NTT_COSET_COEFFS_FROM_EVALS);
    if (mode < 0 || mode > 3 || (inverse && in_len != n)) {
        zk::set_error(mode < 0 || mode > 3 ? "invalid NTT mode" : "inverse transforms need len(evals) == n (a power of two)");
        return ZK_EINVAL;
    }
    if (c->copy_stream == nullptr)
        ZK_TRY_CUDA(cudaStreamCreateWithPriority(&c->copy_stream, cudaStreamNonBlocking, c->priority));
    if (c->d2h_stream == nullptr)
        ZK_TRY_CUDA(cudaStreamCreateWithPriority(&c->d2h_stream, cudaStreamNonBlocking, c->priority));
    Ctx::NttStage& slot = c->ntt_stage[c->ntt_stage_next];
    for (cudaEvent_t* ev : {&slot.free_ev, &slot.h2d_ev, &slot.comp_ev})
        if (*ev == nullptr) ZK_TRY_CUDA(cudaEventCreateWithFlags(ev, cudaEventDisableTiming));
    const size_t need = n * 32;
    if (slot.bytes < need) {
        if (slot.dev != nullptr) {
            ZK_TRY_CUDA(cudaEventSynchronize(slot.free_ev));
            cudaFree(slot.dev);
            slot.dev = nullptr;
            slot.bytes = 0;
        }
        void* p = nullptr;
        if (cudaMalloc(&p, need) != cudaSuccess) {
            cudaGetLastError();
            zk::set_error("zk_ntt_host_submit: device memory exhausted for the staging buffer");
            return ZK_ENOMEM;
        }
        slot.dev = p;
        slot.bytes = need;
        slot.used = false;
    }
    c->ntt_stage_next = (c->ntt_stage_next + 1) % Ctx::kNttStages;
    std::unique_ptr<zk_fence> f(new zk_fence());
    f->device = c->device;
    ZK_TRY_CUDA(cudaEventCreateWithFlags(&f->ev, cudaEventDisableTiming));
    auto* buf = static_cast<zk::fe*>(slot.dev);
    // input copy (after the buffer's previous output copy), transform in place on the
    // canonical values (no Montgomery conversion: ntt_run's canon_io), output copy
    cudaError_t e = slot.used ? cudaStreamWaitEvent(c->copy_stream, slot.free_ev, 0) : cudaSuccess;
    if (e == cudaSuccess && valid)
        e = cudaMemcpyAsync(buf, in_host, valid * 32, cudaMemcpyHostToDevice, c->copy_stream);
    if (e == cudaSuccess) e = cudaEventRecord(slot.h2d_ev, c->copy_stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, slot.h2d_ev, 0);
    int rc = ZK_OK;
    if (e == cudaSuccess) {
        static const uint8_t one[32] = {1};
        rc = zk::ntt_run(c, mode, buf, buf, valid, log_n, omega, shift ? shift : one, /*canon_io=*/true);
        e = cudaEventRecord(slot.comp_ev, c->stream);
    }
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->d2h_stream, slot.comp_ev, 0);
    if (e == cudaSuccess && rc == ZK_OK)
        e = cudaMemcpyAsync(out_host, buf, n * 32, cudaMemcpyDeviceToHost, c->d2h_stream);
    if (e == cudaSuccess) e = cudaEventRecord(slot.free_ev, c->d2h_stream);
    if (e == cudaSuccess) e = cudaEventRecord(f->ev, c->d2h_stream);
    slot.used = true;
    if (e != cudaSuccess) {
        zk::set_error(std::string("zk_ntt_host_submit: ") + cudaGetErrorString(e));
        cudaEventDestroy(f->ev);
        return ZK_ECUDA;
    }
    if (rc != ZK_OK) {
        cudaEventDestroy(f->ev);
        return rc;
    }
    *done = f.release();
    return ZK_OK;
}

int zk_ntt_batch_set_queue(zk_ctx* ctx, int on) {
    CTX_OR_FAIL(ctx);
    ctx->impl.ntt_queue = on != 0;
    return ZK_OK;
}

int zk_ntt_queue_status(zk_ctx* ctx) {
    CTX_OR_FAIL(ctx);
    return zk::ntt_queue_status(&ctx->impl);
}

int zk_ntt_queue_selftest(zk_ctx* ctx, uint64_t limit_us, uint32_t* entry_out) {
    CTX_OR_FAIL(ctx);
    if (entry_out == nullptr || limit_us == 0 || limit_us > 10000000ull) {
        zk::set_error("zk_ntt_queue_selftest: limit_us must be in [1, 10^7] and entry_out non-null");
        return ZK_EINVAL;
    }
    return zk::ntt_queue_selftest(&ctx->impl, limit_us * 1000ull, entry_out);
}

int zk_ntt_plan_run(zk_ntt_plan* plan) {
    if (plan == nullptr) {
        zk::set_error("null plan");
        return ZK_EINVAL;
    }
    CTX_OR_FAIL(plan->ctx);
    return zk::ntt_plan_run(&plan->ctx->impl, plan->impl);
}

int zk_ntt_plan_launches(zk_ntt_plan* plan, uint64_t* kernels) {
    if (plan == nullptr || kernels == nullptr) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    *kernels = zk::ntt_plan_kernels(plan->impl);
    return ZK_OK;
}

int zk_ntt_plan_destroy(zk_ntt_plan* plan) {
    if (plan == nullptr) return ZK_OK;
    cudaSetDevice(plan->ctx->impl.device);
    zk::ntt_plan_destroy(&plan->ctx->impl, plan->impl);
    delete plan;
    return ZK_OK;
}

}  // extern "C"
