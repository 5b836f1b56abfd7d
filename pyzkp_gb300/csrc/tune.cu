// tune.cu -- tuning tables of a context: MSM window bits by size and NTT radix split by
// size, set directly, measured on the device (zk_autotune_msm / zk_autotune_ntt), and
// saved to / loaded from a small JSON file:
//   {"msm_window": {"20": 17, ...}, "ntt_split": {"20": [10, 10], ...}}
// The reference picks its window by a fixed rule (max(4, min(16, bitlen(n) - 2)),
// runtime/kernels/cpu/kernels.py:553-571) and has no NTT radix choice; the results of a
// tuned run are identical, only the time changes.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <functional>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "zk_internal.cuh"

namespace zk {

// A tuned choice replaces the built-in one only when it is faster by this fraction: the
// candidates are timed alone, one call each, and a smaller gain is within run-to-run noise
// (and may not carry over to batched use).
static constexpr double kTuneMargin = 0.03;

static uint32_t ceil_log2(size_t n) {
    uint32_t lg = 0;
    while ((1ull << lg) < n) lg++;
    return lg;
}

static int check_split(uint32_t log_n, uint32_t npass, const uint32_t* bits) {
    ZK_CHECK_ARG(log_n <= 28, "log_n must be <= 28");
    if (npass == 0) return ZK_OK;
    ZK_CHECK_ARG(npass <= 4 && bits != nullptr, "an NTT split has 1..4 passes");
    uint32_t sum = 0;
    for (uint32_t p = 0; p < npass; p++) {
        ZK_CHECK_ARG(bits[p] >= 1 && bits[p] <= 11, "NTT pass radix bits must be 1..11");
        sum += bits[p];
    }
    ZK_CHECK_ARG(sum == log_n, "NTT pass radix bits must sum to log_n");
    return ZK_OK;
}

static int set_split(Ctx* c, uint32_t log_n, uint32_t npass, const uint32_t* bits) {
    int rc = check_split(log_n, npass, bits);
    if (rc != ZK_OK) return rc;
    std::lock_guard<std::mutex> g(c->mu);
    for (int p = 0; p < 4; p++) c->tune_ntt_split[log_n][p] = (uint8_t)((uint32_t)p < npass ? bits[p] : 0);
    return ZK_OK;
}

static void get_split(const Ctx* c, uint32_t log_n, uint32_t* npass, uint32_t bits[4]) {
    const uint8_t* t = c->tune_ntt_split[log_n];
    if (t[0] != 0) {
        uint32_t np = 0;
        for (int p = 0; p < 4 && t[p]; p++) bits[np++] = t[p];
        *npass = np;
        return;
    }
    // the built-in split (fewest passes of <= 11 bits, as equal as possible)
    if (log_n == 0) {
        *npass = 0;
        return;
    }
    const uint32_t np = (log_n + 10) / 11;
    for (uint32_t p = 0; p < np; p++) bits[p] = log_n / np + (p < log_n % np ? 1u : 0u);
    *npass = np;
}

// ---- minimal JSON for the tuning file -----------------------------------------------------
struct JsonIn {
    const std::string& s;
    size_t i = 0;
    bool ok = true;
    void ws() {
        while (i < s.size() && (s[i] == ' ' || s[i] == '\n' || s[i] == '\r' || s[i] == '\t')) i++;
    }
    bool eat(char ch) {
        ws();
        if (i < s.size() && s[i] == ch) {
            i++;
            return true;
        }
        return false;
    }
    std::string str() {
        ws();
        std::string r;
        if (!eat('"')) {
            ok = false;
            return r;
        }
        while (i < s.size() && s[i] != '"') r.push_back(s[i++]);
        if (!eat('"')) ok = false;
        return r;
    }
    long num() {
        ws();
        size_t j = i;
        while (j < s.size() && (s[j] == '-' || (s[j] >= '0' && s[j] <= '9'))) j++;
        if (j == i) {
            ok = false;
            return 0;
        }
        long v = std::stol(s.substr(i, j - i));
        i = j;
        return v;
    }
};

static std::string tune_json(const Ctx* c) {
    std::string out = "{\n  \"msm_window\": {";
    bool first = true;
    for (uint32_t lg = 0; lg < sizeof(c->tune_msm_window); lg++) {
        if (!c->tune_msm_window[lg]) continue;
        out += (first ? "" : ", ") + std::string("\"") + std::to_string(lg) + "\": " +
               std::to_string(c->tune_msm_window[lg]);
        first = false;
    }
    out += "},\n  \"ntt_split\": {";
    first = true;
    for (uint32_t lg = 0; lg <= 28; lg++) {
        const uint8_t* t = c->tune_ntt_split[lg];
        if (!t[0]) continue;
        out += (first ? "" : ", ") + std::string("\"") + std::to_string(lg) + "\": [";
        for (int p = 0; p < 4 && t[p]; p++) out += (p ? ", " : "") + std::to_string(t[p]);
        out += "]";
        first = false;
    }
    out += "}\n}\n";
    return out;
}

static int parse_tune(Ctx* c, const std::string& text) {
    uint8_t msm[32] = {};
    uint8_t split[29][4] = {};
    JsonIn in{text};
    if (!in.eat('{')) {
        set_error("tuning file: expected a JSON object");
        return ZK_EINVAL;
    }
    bool more = !in.eat('}');
    while (more && in.ok) {
        const std::string section = in.str();
        if (!in.eat(':') || !in.eat('{')) {
            set_error("tuning file: expected an object for " + section);
            return ZK_EINVAL;
        }
        bool inner = !in.eat('}');
        while (inner && in.ok) {
            const long lg = std::stol("0" + in.str());
            if (!in.eat(':')) in.ok = false;
            if (section == "msm_window") {
                const long v = in.num();
                if (lg < 0 || lg >= 32 || v < 4 || v > 20) {
                    set_error("tuning file: msm_window entries need 0 <= log_n < 32 and 4..20 bits");
                    return ZK_EINVAL;
                }
                msm[lg] = (uint8_t)v;
            } else if (section == "ntt_split") {
                uint32_t bits[4] = {0, 0, 0, 0}, np = 0;
                if (!in.eat('[')) in.ok = false;
                bool elems = in.ok && !in.eat(']');
                while (elems && in.ok) {
                    const long v = in.num();
                    if (np >= 4 || v < 1 || v > 11) {
                        set_error("tuning file: ntt_split entries need 1..4 passes of 1..11 bits");
                        return ZK_EINVAL;
                    }
                    bits[np++] = (uint32_t)v;
                    elems = in.eat(',');
                    if (!elems && !in.eat(']')) in.ok = false;
                }
                if (lg < 0 || lg > 28 || check_split((uint32_t)lg, np, bits) != ZK_OK) {
                    set_error("tuning file: invalid ntt_split for log_n " + std::to_string(lg));
                    return ZK_EINVAL;
                }
                for (int p = 0; p < 4; p++) split[lg][p] = (uint8_t)bits[p];
            } else {
                set_error("tuning file: unknown section " + section);
                return ZK_EINVAL;
            }
            inner = in.eat(',');
            if (!inner && !in.eat('}')) in.ok = false;
        }
        more = in.eat(',');
        if (!more && !in.eat('}')) in.ok = false;
    }
    if (!in.ok) {
        set_error("tuning file: malformed JSON");
        return ZK_EINVAL;
    }
    std::lock_guard<std::mutex> g(c->mu);
    std::memcpy(c->tune_msm_window, msm, sizeof(msm));
    std::memcpy(c->tune_ntt_split, split, sizeof(split));
    return ZK_OK;
}

// ---- measurement -----------------------------------------------------------------------
// Wall time of one synchronous MSM call (device work plus the host combine), best of reps.
static int time_msm(Ctx* c, const zk_bases* b, const fe* scalars, size_t n, uint32_t cbits, int reps, double* ms) {
    uint8_t xy[64];
    int inf = 0;
    double best = 1e30;
    for (int r = 0; r < reps + 1; r++) {
        const auto t0 = std::chrono::steady_clock::now();
        int rc = msm_run(c, b->dev, scalars, n, 1, cbits, xy, &inf, nullptr, 0, b->n, /*glv=*/true, b->has_inf);
        if (rc != ZK_OK) return rc;
        const double t = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (r > 0 && t < best) best = t;  // the first call warms the pool and caches
    }
    *ms = best;
    return ZK_OK;
}

static int time_ntt(Ctx* c, fe* data, uint32_t log_n, int reps, double* ms) {
    // omega_n = ROOT_2_28^(2^(28 - log_n)), the reference's root (crypto/poly/ntt.py:8,13-24)
    const zkh::Field& F = zkh::fr();
    static const uint64_t kRoot28[4] = {0x9bd61b6e725b19f0ull, 0x402d111e41112ed4ull, 0x00e0a7eb8ef62abcull,
                                        0x2a3c09f0a58a7e85ull};
    zkh::F4 root;
    std::memcpy(root.v, kRoot28, 32);
    zkh::F4 w = zkh::pow_u64(F, zkh::to_mont(F, root), 1ull << (28 - log_n));
    zkh::F4 wc = zkh::from_mont(F, w);
    uint8_t omega[32], one[32] = {1};
    std::memcpy(omega, wc.v, 32);
    cudaEvent_t e0, e1;
    ZK_TRY_CUDA(cudaEventCreate(&e0));
    ZK_TRY_CUDA(cudaEventCreate(&e1));
    double best = 1e30;
    int rc = ZK_OK;
    for (int r = 0; r < reps + 1 && rc == ZK_OK; r++) {
        cudaEventRecord(e0, c->stream);
        rc = ntt_run(c, ZK_NTT_EVALS_FROM_COEFFS, data, data, (size_t)1 << log_n, log_n, omega, one);
        cudaEventRecord(e1, c->stream);
        if (rc == ZK_OK && cudaEventSynchronize(e1) == cudaSuccess) {
            float t = 0.f;
            cudaEventElapsedTime(&t, e0, e1);
            if (r > 0 && t < best) best = t;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = best;
    return rc;
}

}  // namespace zk

using zk::Ctx;

#define TUNE_CTX(ctx)                                      \
    do {                                                   \
        if ((ctx) == nullptr) {                            \
            zk::set_error("null zk_ctx");                  \
            return ZK_EINVAL;                              \
        }                                                  \
        cudaError_t _e = cudaSetDevice((ctx)->impl.device); \
        if (_e != cudaSuccess) {                           \
            zk::set_error(cudaGetErrorString(_e));         \
            return ZK_ECUDA;                               \
        }                                                  \
    } while (0)

extern "C" {

int zk_tune_set_msm_window(zk_ctx* ctx, uint32_t log_n, uint32_t window_bits) {
    TUNE_CTX(ctx);
    if (log_n >= 32 || (window_bits != 0 && (window_bits < 4 || window_bits > 20))) {
        zk::set_error("zk_tune_set_msm_window: log_n < 32 and window_bits 0 or 4..20");
        return ZK_EINVAL;
    }
    ctx->impl.tune_msm_window[log_n] = (uint8_t)window_bits;
    return ZK_OK;
}

int zk_tune_get_msm_window(zk_ctx* ctx, uint64_t n, uint32_t* window_bits) {
    TUNE_CTX(ctx);
    if (window_bits == nullptr) {
        zk::set_error("null pointer");
        return ZK_EINVAL;
    }
    *window_bits = zk::msm_window_for(&ctx->impl, n, /*glv=*/true);  // the window of a G1 MSM
    return ZK_OK;
}

int zk_tune_set_ntt_split(zk_ctx* ctx, uint32_t log_n, uint32_t npass, const uint32_t* bits) {
    TUNE_CTX(ctx);
    return zk::set_split(&ctx->impl, log_n, npass, bits);
}

int zk_tune_get_ntt_split(zk_ctx* ctx, uint32_t log_n, uint32_t* npass, uint32_t bits[4]) {
    TUNE_CTX(ctx);
    if (log_n > 28 || npass == nullptr || bits == nullptr) {
        zk::set_error("zk_tune_get_ntt_split: log_n <= 28 and non-null outputs");
        return ZK_EINVAL;
    }
    bits[0] = bits[1] = bits[2] = bits[3] = 0;
    zk::get_split(&ctx->impl, log_n, npass, bits);
    return ZK_OK;
}

int zk_autotune_save(zk_ctx* ctx, const char* path) {
    TUNE_CTX(ctx);
    if (path == nullptr) {
        zk::set_error("null path");
        return ZK_EINVAL;
    }
    const std::string text = zk::tune_json(&ctx->impl);
    FILE* f = std::fopen(path, "wb");
    if (f == nullptr) {
        zk::set_error(std::string("cannot write ") + path);
        return ZK_EINVAL;
    }
    const size_t w = std::fwrite(text.data(), 1, text.size(), f);
    std::fclose(f);
    if (w != text.size()) {
        zk::set_error(std::string("short write to ") + path);
        return ZK_EINVAL;
    }
    return ZK_OK;
}

int zk_autotune_load(zk_ctx* ctx, const char* path) {
    TUNE_CTX(ctx);
    if (path == nullptr) {
        zk::set_error("null path");
        return ZK_EINVAL;
    }
    FILE* f = std::fopen(path, "rb");
    if (f == nullptr) {
        zk::set_error(std::string("cannot read ") + path);
        return ZK_EINVAL;
    }
    std::string text;
    char buf[4096];
    size_t r;
    while ((r = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, r);
    std::fclose(f);
    try {
        return zk::parse_tune(&ctx->impl, text);
    } catch (const std::exception&) {  // a number std::stol rejects
        zk::set_error("tuning file: malformed number");
        return ZK_EINVAL;
    }
}

// Time windows c in [rule - 2, rule + 2] for MSMs of 2^log_n points over the first 2^log_n
// bases and scalars (Montgomery, device), keep the fastest in the table.
int zk_autotune_msm(zk_ctx* ctx, const zk_bases* bases, const void* scalars_dev, uint32_t log_n, int reps,
                    uint32_t* best_window, double* best_ms) {
    TUNE_CTX(ctx);
    if (bases == nullptr || scalars_dev == nullptr || log_n >= 31 || ((size_t)1 << log_n) > bases->n) {
        zk::set_error("zk_autotune_msm: needs 2^log_n bases and scalars");
        return ZK_EINVAL;
    }
    const size_t n = (size_t)1 << log_n;
    const uint32_t rule = zk::msm_auto_window_glv(n);
    // the built-in window is timed first and kept unless another beats it by kTuneMargin
    double rule_ms = 0;
    int rc0 = zk::time_msm(&ctx->impl, bases, static_cast<const zk::fe*>(scalars_dev), n, rule, reps < 1 ? 1 : reps,
                           &rule_ms);
    if (rc0 != ZK_OK) return rc0;
    uint32_t best_c = rule;
    double best = rule_ms;
    for (int d = -2; d <= 2; d++) {
        const int cb = (int)rule + d;
        if (d == 0 || cb < 4 || cb > 20) continue;
        double ms = 0;
        int rc = zk::time_msm(&ctx->impl, bases, static_cast<const zk::fe*>(scalars_dev), n, (uint32_t)cb,
                              reps < 1 ? 1 : reps, &ms);
        if (rc != ZK_OK) return rc;
        if (ms < best && ms < rule_ms * (1.0 - zk::kTuneMargin)) {
            best = ms;
            best_c = (uint32_t)cb;
        }
    }
    // 0 = the built-in rule (so a later change of the rule is not masked by a stored copy)
    ctx->impl.tune_msm_window[zk::ceil_log2(n)] = best_c == rule ? 0 : (uint8_t)best_c;
    if (best_window) *best_window = best_c;
    if (best_ms) *best_ms = best;
    return ZK_OK;
}

// Time NTT splits of 2^log_n (the fewest passes and one more, parts within 2 bits of each
// other) as in-place forward transforms of data_dev (2^log_n elements, contents are
// overwritten), keep the fastest in the table.
int zk_autotune_ntt(zk_ctx* ctx, void* data_dev, uint32_t log_n, int reps, uint32_t* npass, uint32_t bits[4],
                    double* best_ms) {
    TUNE_CTX(ctx);
    if (data_dev == nullptr || log_n < 1 || log_n > 28) {
        zk::set_error("zk_autotune_ntt: needs 1 <= log_n <= 28 and a buffer of 2^log_n elements");
        return ZK_EINVAL;
    }
    zk::Ctx* c = &ctx->impl;
    // Splits with the fewest passes only: a split with one pass more (e.g. 6 + 6 + 6 bits at
    // 2^18) could win alone by a few percent with its smaller tiles, but in a batch, where
    // other transforms fill the GPU anyway, it only adds a pass level and a round trip
    // through HBM (64 coset NTTs of 2^10..2^20 on GB300: tuned 2.96 against 2.87 ms).
    const uint32_t min_np = (log_n + 10) / 11;
    std::vector<std::vector<uint32_t>> cands;
    for (uint32_t np = min_np; np <= min_np; np++) {
        if (np > log_n) break;
        // all compositions of log_n into np parts of 1..11 bits, max - min <= 2
        std::vector<uint32_t> part(np, 1);
        std::function<void(uint32_t, uint32_t)> rec = [&](uint32_t k, uint32_t left) {
            if (k + 1 == np) {
                if (left < 1 || left > 11) return;
                part[k] = left;
                const auto mm = std::minmax_element(part.begin(), part.end());
                if (*mm.second - *mm.first <= 2) cands.push_back(part);
                return;
            }
            for (uint32_t v = 1; v <= 11 && v < left; v++) {
                part[k] = v;
                rec(k + 1, left - v);
            }
        };
        rec(0, log_n);
    }
    uint8_t saved[4];
    std::memcpy(saved, c->tune_ntt_split[log_n], 4);
    // the built-in split is timed first and kept unless a candidate beats it by kTuneMargin
    {
        std::lock_guard<std::mutex> g(c->mu);
        std::memset(c->tune_ntt_split[log_n], 0, 4);
    }
    double rule_ms = 0;
    int rc0 = zk::time_ntt(c, static_cast<zk::fe*>(data_dev), log_n, reps < 1 ? 1 : reps, &rule_ms);
    if (rc0 != ZK_OK) {
        std::memcpy(c->tune_ntt_split[log_n], saved, 4);
        return rc0;
    }
    uint32_t rule_np = 0, rule_bits[4] = {0, 0, 0, 0};
    zk::get_split(c, log_n, &rule_np, rule_bits);
    double best = rule_ms;
    std::vector<uint32_t> best_split;  // empty: the built-in split
    for (const auto& cand : cands) {
        if (cand.size() == rule_np && std::equal(cand.begin(), cand.end(), rule_bits)) continue;
        int rc = zk::set_split(c, log_n, (uint32_t)cand.size(), cand.data());
        double ms = 0;
        if (rc == ZK_OK) rc = zk::time_ntt(c, static_cast<zk::fe*>(data_dev), log_n, reps < 1 ? 1 : reps, &ms);
        if (rc != ZK_OK) {
            std::memcpy(c->tune_ntt_split[log_n], saved, 4);
            return rc;
        }
        if (ms < best && ms < rule_ms * (1.0 - zk::kTuneMargin)) {
            best = ms;
            best_split = cand;
        }
    }
    if (best_split.empty()) {
        std::lock_guard<std::mutex> g(c->mu);
        std::memset(c->tune_ntt_split[log_n], 0, 4);
    } else {
        zk::set_split(c, log_n, (uint32_t)best_split.size(), best_split.data());
    }
    if (npass && bits) zk::get_split(c, log_n, npass, bits);
    if (best_ms) *best_ms = best;
    return ZK_OK;
}

}  // extern "C"
