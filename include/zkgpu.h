/*
 * zkgpu.h -- C ABI of the GB300 (sm_103a) prover hot path for pyZKP:
 * BN254 G1 multi-scalar multiplication and the Fr NTT / iNTT / coset NTT.
 *
 * Drop-in boundary. The reference (fzybravery/pyZKP) reaches its GPU path through
 * KernelFns registered under (OpType, Device.METAL, Backend.METAL)
 * (runtime/kernels/metal/kernels.py:12-20) and called by Executor._run_node
 * (runtime/executor.py:185-197). Those KernelFns are rebuilt in Python
 * (pyzkp_gb300/plugin.py) on top of the entry points below, bound with ctypes
 * (pyzkp_gb300/_native.py). Every entry point is plain C: pointers, sizes and
 * integer status codes; no C++ exceptions cross the boundary.
 *
 * Data layout (identical bytes to the reference's "fr_mont_u64x4" buffers,
 * runtime/metal/buffer.py:7-15 and runtime/kernels/cpu/kernels.py:135-141):
 *   - a field element is 32 bytes, little endian, 8 x uint32 (= 4 x uint64) limbs;
 *     "Montgomery" means the value a * 2^256 mod p, "canonical" the value itself;
 *   - an affine G1 point is 64 bytes: x then y (Fq); (0, 0) denotes infinity.
 * Device pointers are CUDA device addresses on the context's device.
 * All functions return ZK_OK (0) or an error code; zk_last_error() describes the
 * last failure of the calling thread.
 */
#ifndef ZKGPU_H
#define ZKGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ZK_OK 0
#define ZK_EINVAL 1 /* bad argument; the Python layer raises ValueError like the reference */
#define ZK_ECUDA 2  /* CUDA runtime failure; RuntimeError */
#define ZK_ENOMEM 3 /* device memory exhausted; MemoryError */
#define ZK_ENODEV 4 /* no usable CUDA device; RuntimeError (runtime/context.py:33-34) */
#define ZK_ETIMEOUT 5 /* zk_batch_wait: the batch is still running when the time limit passed */

typedef struct zk_ctx zk_ctx;
typedef struct zk_bases zk_bases;
typedef struct zk_batch zk_batch; /* an asynchronous MSM batch (zk_batch_wait / zk_batch_destroy) */
typedef struct zk_fence zk_fence; /* a point on a stream (zk_fence_wait / zk_fence_destroy) */

/* Message of the last failure on this thread ("" if none). */
const char *zk_last_error(void);

/* ABI version of this library. */
int zk_version(void);

/*
 * Context: one device, one CUDA stream, cached NTT tables.
 * Replaces MetalRuntime.create_default / MetalContext.create_default
 * (runtime/metal/runtime.py:493-629, runtime/context.py:42-47).
 */
int zk_ctx_create(int device, zk_ctx **out);
/* The same with a CUDA stream priority for the context's streams (lower = more urgent;
 * clamped into zk_stream_priority_range). A serving loop gives its short requests a more
 * urgent context, so that their kernels are scheduled ahead of a long batch's. No
 * counterpart in the reference (its Metal command queue has no priorities). */
int zk_ctx_create_prio(int device, int priority, zk_ctx **out);
int zk_stream_priority_range(int *least, int *greatest);
int zk_ctx_destroy(zk_ctx *ctx);
/* Block until all work queued on the context stream has finished. */
int zk_ctx_sync(zk_ctx *ctx);
/* The context's cudaStream_t, for callers that enqueue their own work. */
int zk_ctx_stream(zk_ctx *ctx, void **stream_out);
/* Number of SMs of the context's device. */
int zk_ctx_num_sms(zk_ctx *ctx, int *out);

/*
 * Kernel accounting, for measurement (no counterpart in the reference, whose
 * Trace only times whole ops, runtime/trace.py:49-101). Every kernel the library
 * launches is counted; with profiling enabled each launch is also bracketed by
 * CUDA events on the context stream and its device time accumulated per kernel.
 */
int zk_launch_count(zk_ctx *ctx, uint64_t *out);
int zk_prof_enable(zk_ctx *ctx, int on);
int zk_prof_reset(zk_ctx *ctx);
int zk_prof_count(zk_ctx *ctx, int *nkernels);
int zk_prof_get(zk_ctx *ctx, int idx, char *name_buf, size_t name_len, uint64_t *launches, double *total_ms);
/* Device time between zk_timer_start and zk_timer_stop, from CUDA events recorded on
 * the context stream (stop synchronises; host work inside synchronous calls counts). */
int zk_timer_start(zk_ctx *ctx);
int zk_timer_stop(zk_ctx *ctx, double *ms);
/* Shape of the last zk_msm_g1 call: CSR entries (non-zero signed digits), window bits, windows. */
int zk_msm_last_stats(zk_ctx *ctx, uint64_t *entries, uint32_t *window_bits, uint32_t *windows);
/* Measured throughput of the 32-bit integer multiply-add pipe, in 10^12 IMAD instructions
 * per second: probe mode 0 = carry chains shaped like a Montgomery row (mad.lo.cc /
 * madc.hi.cc), 1 = independent mad.lo.u32, 2 = independent mad.hi.u32; zk_imad_peak is
 * the largest of the three (the roofline denominator of the IMAD-bound kernels). */
int zk_imad_probe(zk_ctx *ctx, int mode, double *tera_imad_per_s);
int zk_imad_peak(zk_ctx *ctx, double *tera_imad_per_s);

/*
 * Device memory (stream-ordered pool of the context). Replaces
 * MemoryPool.alloc_metal / release_metal (runtime/memory.py:56-91).
 */
int zk_alloc(zk_ctx *ctx, size_t bytes, void **dptr);
int zk_free(zk_ctx *ctx, void *dptr);
/* Copies on the context stream; both block until the copy is complete. */
int zk_h2d(zk_ctx *ctx, void *dst_dev, const void *src_host, size_t bytes);
int zk_d2h(zk_ctx *ctx, void *dst_host, const void *src_dev, size_t bytes);
/* The same copies without waiting: they return once enqueued on the context stream. The
 * host buffer must stay valid -- and, for zk_d2h_async, unread -- until the stream has
 * passed the copy (a fence, zk_ctx_sync or a blocking call); page-locked memory
 * (zk_host_alloc) lets the copy overlap other work. */
int zk_h2d_async(zk_ctx *ctx, void *dst_dev, const void *src_host, size_t bytes);
int zk_d2h_async(zk_ctx *ctx, void *dst_host, const void *src_dev, size_t bytes);
/* Fence: a point on the context stream after everything enqueued so far.
 * zk_fence_wait returns ZK_OK once the device has passed it, ZK_ETIMEOUT if timeout_ms
 * (>= 0; 0 = just ask) passes first; a negative timeout waits without a limit. No
 * counterpart in the reference (its Metal ops wait for completion inside every op). */
int zk_fence_record(zk_ctx *ctx, zk_fence **out);
int zk_fence_wait(zk_fence *f, int timeout_ms);
int zk_fence_destroy(zk_fence *f);
/* Device-to-device copy on the context stream (asynchronous). */
int zk_d2d(zk_ctx *ctx, void *dst_dev, const void *src_dev, size_t bytes);
/* Fill bytes of device memory (asynchronous on the context stream). */
int zk_memset(zk_ctx *ctx, void *dptr, int value, size_t bytes);
/* Page-locked host memory for fast copies. */
int zk_host_alloc(size_t bytes, void **out);
int zk_host_free(void *p);

/*
 * Fr vectors of n elements (device pointers, in-place allowed).
 * zk_fr_to_mont / zk_fr_from_mont replace the Montgomery packing loops of
 * _to_device / _from_device (runtime/kernels/cpu/kernels.py:98-172); to_mont
 * reduces any 256-bit input modulo r first (int(x) % FR_MODULUS).
 */
int zk_fr_to_mont(zk_ctx *ctx, void *out, const void *in, size_t n);
int zk_fr_from_mont(zk_ctx *ctx, void *out, const void *in, size_t n);
/* Same for Fq (base-field coordinates, e.g. affine points as 2n elements). */
int zk_fq_to_mont(zk_ctx *ctx, void *out, const void *in, size_t n);
int zk_fq_from_mont(zk_ctx *ctx, void *out, const void *in, size_t n);
/* out[i] = a[i] * b[i] (Montgomery in, Montgomery out): POINTWISE_MUL,
 * runtime/kernels/metal/kernels.py:175-222 / runtime/metal/runtime.py:204-213. */
int zk_fr_mul(zk_ctx *ctx, void *out, const void *a, const void *b, size_t n);
/* out[i] = a[i] - b[i]: POLY_SUB on equal lengths, runtime/kernels/metal/kernels.py:122-167. */
int zk_fr_sub(zk_ctx *ctx, void *out, const void *a, const void *b, size_t n);
/* out[i] = a[i] + b[i] (the Groth16 setup's query exponents). */
int zk_fr_add(zk_ctx *ctx, void *out, const void *a, const void *b, size_t n);
/* *out = 1 + index of the last non-zero element of a[0..n) (0 if all are zero): the
 * trailing-zero trim of crypto/poly/cpu_ref.py:_trim used by poly_sub (:18-25). Blocks. */
int zk_fr_trimmed_len(zk_ctx *ctx, const void *a, size_t n, size_t *out);

/*
 * NTT family over Fr, natural order in and out, Montgomery in and out.
 * Semantics of crypto/poly/ntt.py:103-146 and of the op KernelFns
 * runtime/kernels/cpu/kernels.py:175-250 (which the Metal versions at
 * runtime/kernels/metal/kernels.py:225-381,418-827 replace):
 *   ZK_NTT_EVALS_FROM_COEFFS        evals[i] = sum_j a_j omega^(ij); the input of
 *                                   in_len elements is zero-padded or truncated to n
 *   ZK_NTT_COEFFS_FROM_EVALS        inverse; requires in_len == n
 *   ZK_NTT_COSET_EVALS_FROM_COEFFS  a_j scaled by shift^j first (j < min(in_len, n))
 *   ZK_NTT_COSET_COEFFS_FROM_EVALS  inverse, then coefficient i scaled by shift^-i
 *                                   (by 0 for i > 0 when shift == 0, as ntt.py:136-146)
 * omega and shift are 32-byte canonical little-endian values. omega must be a
 * primitive n-th root of unity (omega^(n/2) == -1 for n >= 2), else ZK_EINVAL.
 * n = 2^log_n, log_n <= 28 (2-adicity of r, crypto/poly/ntt.py:9,21-22).
 * out holds n elements; it may be the same buffer as in (in place) but must not
 * overlap it otherwise.
 */
#define ZK_NTT_EVALS_FROM_COEFFS 0
#define ZK_NTT_COEFFS_FROM_EVALS 1
#define ZK_NTT_COSET_EVALS_FROM_COEFFS 2
#define ZK_NTT_COSET_COEFFS_FROM_EVALS 3
int zk_ntt(zk_ctx *ctx, int mode, void *out_dev, const void *in_dev, size_t in_len, uint32_t log_n,
           const uint8_t omega[32], const uint8_t shift[32]);

/*
 * The same transform between HOST buffers of canonical elements, asynchronous: in_host
 * holds in_len canonical elements (32 bytes each), out_host receives n canonical elements.
 * The shape of the reference's NTT ops, which take and return Python lists
 * (runtime/kernels/cpu/kernels.py:175-250). Returns once the work is enqueued, with a fence
 * (zk_fence_wait, then zk_fence_destroy) that passes when out_host is written; the host
 * buffers must stay valid (and in_host unchanged) until then -- pinned memory keeps the
 * copies asynchronous. The input copy, the transform (run on the canonical values
 * directly: it is linear and its constants are Montgomery forms, so no conversion pass is
 * needed; inputs of any 256 bits are reduced mod r) and the output copy run on three
 * streams, and the context uses three device staging buffers in turn, so a stream of calls
 * overlaps one call's output copy, the next call's input copy and a transform (the host
 * link carries both directions at once). shift may be NULL (1). Errors as zk_ntt. No
 * reference counterpart for the asynchrony.
 */
int zk_ntt_host_submit(zk_ctx *ctx, int mode, void *out_host, const void *in_host, size_t in_len, uint32_t log_n,
                       const uint8_t omega[32], const uint8_t shift[32], zk_fence **done);

/*
 * Batched NTTs: transform k is zk_ntt(modes[k], outs[k], ins[k], in_lens[k], log_ns[k],
 * omegas + 32k, shifts + 32k) (shifts may be NULL: all 1), with the same semantics and
 * errors. All transforms of the batch run their first pass in one launch, their second
 * pass in the next, and so on (at most three launches up to n = 2^28), each CTA looking
 * up its transform and tile in a prefix table. Asynchronous on the context stream like
 * zk_ntt. No reference counterpart (the reference runs one op at a time).
 */
int zk_ntt_batch(zk_ctx *ctx, size_t count, const int *modes, void *const *outs, const void *const *ins,
                 const uint64_t *in_lens, const uint32_t *log_ns, const uint8_t *omegas, const uint8_t *shifts);

/*
 * Work-queue form of a batch (north_star's "(instance, pass, tile) items"; no reference
 * counterpart, the reference runs one op at a time): every pass of every transform in ONE
 * persistent launch. Items are (transform, pass, tile), queued pass level by pass level
 * with the largest transforms first; each CTA takes the next item from a device ticket,
 * and an item of pass p > 0 waits (on the device) until its own transform's pass p - 1 has
 * finished, so a transform's next pass starts while other transforms are still in the
 * previous one. Every wait is bounded (2 s): a wait that runs out stops that launch early,
 * and zk_ntt_queue_status reports it.
 *   zk_ntt_batch_set_queue  on != 0: zk_ntt_batch on this context uses the queue form
 *                           (default off: one launch per pass level).
 *   zk_ntt_queue_status     synchronises the context stream; ZK_OK, or ZK_ETIMEOUT if a
 *                           work-queue launch of this context gave up since the last call
 *                           (its outputs are then incomplete).
 *   zk_ntt_queue_selftest   for tests of the bound: one work-queue launch of a 2^12
 *                           transform whose second pass waits for a first-pass tile that
 *                           does not exist, with a wait limit of limit_us (1..10^7 us);
 *                           returns ZK_ETIMEOUT with *entry_out = 1 + the queue entry whose
 *                           wait ran out first (the second pass, or a third one waiting on
 *                           it), the context staying usable; else ZK_OK or an error.
 */
int zk_ntt_batch_set_queue(zk_ctx *ctx, int on);
int zk_ntt_queue_status(zk_ctx *ctx);
int zk_ntt_queue_selftest(zk_ctx *ctx, uint64_t limit_us, uint32_t *entry_out);

/*
 * NTT batch plan: the descriptors and scratch of a zk_ntt_batch with fixed buffers,
 * prepared once. flags (the use_graph argument): ZK_NTT_PLAN_GRAPH (1) makes a run one
 * CUDA graph launch; ZK_NTT_PLAN_QUEUE (2) runs the batch in its work-queue form (one
 * persistent launch, see zk_ntt_batch_set_queue). zk_ntt_plan_run is asynchronous on the
 * context stream; the buffers must outlive the plan.
 */
#define ZK_NTT_PLAN_GRAPH 1
#define ZK_NTT_PLAN_QUEUE 2
typedef struct zk_ntt_plan zk_ntt_plan;
int zk_ntt_plan_create(zk_ctx *ctx, size_t count, const int *modes, void *const *outs, const void *const *ins,
                       const uint64_t *in_lens, const uint32_t *log_ns, const uint8_t *omegas, const uint8_t *shifts,
                       int use_graph, zk_ntt_plan **out);
int zk_ntt_plan_run(zk_ntt_plan *plan);
int zk_ntt_plan_launches(zk_ntt_plan *plan, uint64_t *kernels);
int zk_ntt_plan_destroy(zk_ntt_plan *plan);

/*
 * Groth16 prover vectors (protocols/groth16/prove.py:80-126, r1cs.py:84-92,
 * qap.py:53-101). Fr vectors are Montgomery device arrays; all asynchronous on the
 * context stream except zk_fr_r1cs_check and zk_fr_div_xn_minus_1, which block.
 *   zk_fr_spmv          out[i] = sum_{j in row i} coeffs[j] * x[cols[j]]: a CSR matrix
 *                       (row_ptr nrows + 1, cols, coeffs Montgomery) times x -- the
 *                       R1CS rows A w, B w, C w of eval_r1cs_vectors.
 *   zk_fr_r1cs_check    *bad = #{i : a[i] b[i] != c[i]}: zero iff A B - C vanishes on the
 *                       domain, i.e. the remainder of qap.py:94-95 is empty.
 *   zk_fr_r1cs_check_async  the same count added to the uint64 at bad_dev (device memory,
 *                       zeroed by the caller) without waiting: a serving loop reads it
 *                       with the request's other results and fails only that request.
 *   zk_fr_qap_quotient  out[i] = (a[i] b[i] - c[i]) * zinv (zinv canonical): on the coset
 *                       shift * <omega>, zinv = (shift^n - 1)^-1 divides by X^n - 1.
 *   zk_fr_gather        out[i] = in[idx[i]] (idx uint32 device).
 *   zk_fr_scale         out[i] = in[i] * s (s canonical).
 *   zk_fr_powers        out[i] = base^i (base canonical).
 *   zk_fr_div_xn_minus_1  DIV_XN_MINUS_1 (crypto/poly/fast.py:8-37 through
 *                       runtime/kernels/cpu/kernels.py:312-323): quotient and remainder
 *                       of a[0..len) by X^n - 1, trailing zeros trimmed (*qlen, *rlen).
 *                       q_out holds max(len - n, 0) elements, r_out n elements.
 */
int zk_fr_spmv(zk_ctx *ctx, uint32_t nrows, const uint32_t *row_ptr_dev, const uint32_t *cols_dev,
               const void *coeffs_dev, const void *x_dev, void *out_dev);
int zk_fr_r1cs_check(zk_ctx *ctx, const void *a, const void *b, const void *c, size_t n, uint64_t *bad);
int zk_fr_r1cs_check_async(zk_ctx *ctx, const void *a, const void *b, const void *c, size_t n, void *bad_dev);
int zk_fr_qap_quotient(zk_ctx *ctx, void *out, const void *a, const void *b, const void *c, size_t n,
                       const uint8_t zinv[32]);
int zk_fr_gather(zk_ctx *ctx, void *out, const void *in, const uint32_t *idx_dev, size_t n);
int zk_fr_scale(zk_ctx *ctx, void *out, const void *in, const uint8_t s[32], size_t n);
int zk_fr_powers(zk_ctx *ctx, void *out, const uint8_t base[32], size_t n);
int zk_fr_div_xn_minus_1(zk_ctx *ctx, const void *a, size_t len, size_t n, void *q_out, void *r_out, size_t *qlen,
                         size_t *rlen);

/*
 * PLONK quotient step (protocols/plonk/prove.py:395-420).
 *   zk_fr_batch_inv          BATCH_INV (crypto/field/batch.py:8-38 through
 *                            runtime/kernels/cpu/kernels.py:_batch_inv): out[i] = in[i]^-1,
 *                            0 for a zero input; out may equal in. Asynchronous.
 *   zk_plonk_quotient_evals  PLONK_T_QUOTIENT_EVALS (runtime/kernels/cpu/kernels.py:
 *                            _plonk_t_quotient_evals): from 15 extended-coset evaluation
 *                            vectors of length m (a, b, c, z, pi, ql, qr, qm, qo, qc, s1, s2,
 *                            s3, z(omega x), L1; Montgomery) and the op's attrs (canonical:
 *                            omega_m, shift, shift_n, alpha, beta, gamma, k1, k2; n), writes
 *                            num (gate + alpha perm + alpha^2 (z - 1) L1) and
 *                            zh = shift_n (omega_m^n)^i - 1. Asynchronous.
 */
int zk_fr_batch_inv(zk_ctx *ctx, void *out, const void *in, size_t n);
int zk_plonk_quotient_evals(zk_ctx *ctx, const void *const *inputs, size_t m, uint64_t n, const uint8_t omega_m[32],
                            const uint8_t shift[32], const uint8_t shift_n[32], const uint8_t alpha[32],
                            const uint8_t beta[32], const uint8_t gamma[32], const uint8_t k1[32],
                            const uint8_t k2[32], void *num_out, void *zh_out);

/*
 * Host (CPU) point arithmetic for proof assembly, affine canonical in and out as above:
 * g1_mul / g2_mul (crypto/ecc/bn254.py g1_mul / g2_mul; k reduced mod r) and g1_add /
 * g2_add. No context, no device.
 */
int zk_host_g1_mul(const uint8_t p[64], const uint8_t k[32], uint8_t out[64]);
int zk_host_g1_add(const uint8_t p[64], const uint8_t q[64], uint8_t out[64]);
int zk_host_g2_mul(const uint8_t p[128], const uint8_t k[32], uint8_t out[128]);
int zk_host_g2_add(const uint8_t p[128], const uint8_t q[128], uint8_t out[128]);

/*
 * Tuning tables of a context (0 = the built-in rule). MSM: window bits for MSMs whose
 * ceil(log2 n) is log_n (the reference's fixed rule is max(4, min(16, bitlen(n) - 2)),
 * runtime/kernels/cpu/kernels.py:553-571; this library's default is a measured table per
 * size). NTT: radix bits of each pass for 2^log_n (1..4 passes of 1..11 bits summing
 * to log_n; default: the fewest passes, as equal as possible). zk_tune_get_* report the
 * effective choice. zk_autotune_msm / zk_autotune_ntt time the built-in choice and the
 * candidates on the device and keep a candidate only if it beats the built-in choice by
 * more than 3% (else the entry stays 0; best_ms: the kept choice's time); zk_autotune_save / _load write and read the
 * tables as JSON ({"msm_window": {"20": 17}, "ntt_split": {"20": [10, 10]}}). Tuning
 * changes timings only, never results. No reference counterpart.
 */
int zk_tune_set_msm_window(zk_ctx *ctx, uint32_t log_n, uint32_t window_bits);
int zk_tune_get_msm_window(zk_ctx *ctx, uint64_t n, uint32_t *window_bits);
int zk_tune_set_ntt_split(zk_ctx *ctx, uint32_t log_n, uint32_t npass, const uint32_t *bits);
int zk_tune_get_ntt_split(zk_ctx *ctx, uint32_t log_n, uint32_t *npass, uint32_t bits[4]);
int zk_autotune_msm(zk_ctx *ctx, const zk_bases *bases, const void *scalars_dev, uint32_t log_n, int reps,
                    uint32_t *best_window, double *best_ms);
int zk_autotune_ntt(zk_ctx *ctx, void *data_dev, uint32_t log_n, int reps, uint32_t *npass, uint32_t bits[4],
                    double *best_ms);
int zk_autotune_save(zk_ctx *ctx, const char *path);
int zk_autotune_load(zk_ctx *ctx, const char *path);

/*
 * zk_ntt without any device allocation. No counterpart in the reference: it is for
 * callers that cannot allocate device memory while they transform (a process whose
 * memory budget was reserved up front by its own pool, or a latency-critical path
 * that must avoid cudaMalloc's implicit synchronisation). Same arguments and results
 * as zk_ntt; the intermediate buffer and the twiddle / scale tables live in one
 * static device array of the library (2 MiB + 128 KiB per device that loads it,
 * held until exit), so n <= 2^16 (log_n <= 16, larger sizes give ZK_EINVAL). Every
 * call on a device shares that array: calls that overlap on the GPU race and must be
 * serialised by the caller. Each call rebuilds its tables on the device from values its
 * kernel launch carries, so the GPU reads no host memory of the library. The first call
 * on each device sets up the array's device address; make that first call before any
 * stream capture.
 */
int zk_ntt_noalloc(zk_ctx *ctx, int mode, void *out_dev, const void *in_dev, size_t in_len, uint32_t log_n,
                   const uint8_t omega[32], const uint8_t shift[32]);

/*
 * Resident G1 bases (affine, converted to Montgomery once on the device).
 * Replaces the per-call packing of _pack_g1_point (runtime/metal/msm.py:13-34,
 * 79-85, 200-204). Input: n affine canonical points, 64 bytes each, (0,0) = infinity,
 * from host memory (zk_bases_create) or device memory (zk_bases_create_dev).
 */
int zk_bases_create(zk_ctx *ctx, const void *xy_canonical_host, size_t n, zk_bases **out);
int zk_bases_create_dev(zk_ctx *ctx, const void *xy_canonical_dev, size_t n, zk_bases **out);
int zk_bases_destroy(zk_bases *b);
/*
 * Fixed-base precomputation for a base set used by many MSMs (the reference's
 * fixed_base_precompute / msm_fixed_base, crypto/msm/pippenger.py:217-295, and the
 * fixed_base attrs of runtime/kernels/cpu/kernels.py:560-569). Instead of the
 * reference's per-point table d*P_i (d < 2^w; 17 GB at n = 2^20, w = 8) the library
 * stores the window-shifted rows [2^(c j)] P_i for j < ceil(255/c) (W*n*64 bytes); every
 * later zk_msm_g1 on these bases (with window_bits 0 or c) then sums all windows in one
 * bucket set: no per-window bucket reduction and no doubling chain. Same result.
 */
/* G2 handles (zk_bases_g2_create) take the same call: rows of G2 points, 128 bytes each. */
int zk_bases_precompute(zk_ctx *ctx, zk_bases *b, uint32_t window_bits);
int zk_bases_count(const zk_bases *b, size_t *n);

/*
 * G1 MSM: sum_i scalars[i] * bases[offset + i] for i < n, returned as an affine
 * canonical point (out_xy = x || y, 64 bytes; *out_is_inf = 1 and (0,0) for infinity).
 * The result is the unique affine point, identical to crypto/msm/pippenger.py:10-64
 * (through the op semantics of runtime/kernels/cpu/kernels.py:553-571) and to the
 * Metal path metal_msm_g1 / metal_msm_g1_v2 (runtime/metal/msm.py:65-332).
 * scalars_dev: n device elements, Montgomery (scalars_mont = 1, the TO_DEVICE form)
 * or canonical 256-bit values (scalars_mont = 0; reduced mod r first).
 * window_bits: 0 = automatic, else 4..20 (signed digits, 2^(c-1) buckets per window).
 */
int zk_msm_g1(zk_ctx *ctx, const zk_bases *bases, size_t offset, const void *scalars_dev, size_t n,
              int scalars_mont, uint32_t window_bits, uint8_t out_xy[64], int *out_is_inf);
/*
 * G1 MSM from host memory in one call: the shape of metal_msm_g1 (runtime/metal/msm.py:65-143),
 * which packs and uploads the points on every call (_msm_g1, runtime/kernels/metal/kernels.py:84-120).
 * xy_canonical_host: n affine canonical points (64 bytes each, (0,0) = infinity);
 * scalars_host: n elements as for zk_msm_g1 (scalars_mont selects the form). On a second
 * stream the scalars go up first (in chunks whose digits are computed as each arrives),
 * then the points, converted there while the digits are sorted; the bucket accumulation
 * waits for them. Pinned host memory (zk_host_alloc) makes the copies asynchronous. Same
 * result as zk_bases_create + zk_h2d + zk_msm_g1.
 */
int zk_msm_g1_host(zk_ctx *ctx, const void *xy_canonical_host, const void *scalars_host, size_t n,
                   int scalars_mont, uint32_t window_bits, uint8_t out_xy[64], int *out_is_inf);

/*
 * The same, asynchronous (a stream of host-buffer MSMs, as a serving loop issues them):
 * returns once the work is enqueued, with a batch handle to pass to zk_batch_wait and then
 * zk_batch_destroy;
 * out_xy / out_is_inf are written when the batch completes, and the host buffers must stay
 * valid (and unchanged) until then -- pinned memory keeps the copies asynchronous. The
 * context keeps two device staging buffers and uses them in turn, so a call's uploads run
 * while the previous call's MSM computes (the host link is otherwise idle then); a call
 * waits for the MSM two calls back to release its buffer. Same result as zk_msm_g1_host. No
 * reference counterpart (the reference's Metal MSM blocks per call).
 */
int zk_msm_g1_host_submit(zk_ctx *ctx, const void *xy_canonical_host, const void *scalars_host, size_t n,
                          int scalars_mont, uint32_t window_bits, uint8_t *out_xy, int32_t *out_is_inf,
                          zk_batch **out);

/*
 * Batched G1 MSM: out[k] = sum_i scalars[k][i] * bases[k][offsets[k] + i] for i < sizes[k],
 * k < count. Replaces the per-instance loops of MSM_G1_BATCH and KZG_BATCH_COMMIT
 * (_msm_g1_batch / _kzg_batch_commit, runtime/kernels/cpu/kernels.py:441-496, which call
 * msm_pippenger_batch, crypto/msm/pippenger.py:124-214, on the prefix points[:len(s)];
 * Metal: runtime/kernels/metal/kernels.py:22-82). Instances with the same window size
 * share one pipeline (one launch per stage for all of them); instances of size 0 give
 * infinity. bases[k] may repeat one handle; offsets may be NULL (all 0). Results as in
 * zk_msm_g1: out_xy holds count * 64 bytes, out_is_inf count flags. window_bits: 0 =
 * tuned or automatic per instance, else 4..20 for all.
 */
int zk_msm_g1_batch(zk_ctx *ctx, size_t count, const zk_bases *const *bases, const uint64_t *offsets,
                    const void *const *scalars_dev, const uint64_t *sizes, int scalars_mont, uint32_t window_bits,
                    uint8_t *out_xy, int32_t *out_is_inf);

/*
 * G2 (the sextic twist over Fq2 = Fq[u]/(u^2 + 1)): MSM_G2, computed by the reference on
 * the CPU only (_msm_g2 / _msm_g2_impl, runtime/kernels/cpu/kernels.py:338-348,574-582;
 * Groth16's b_query_g2 * w, protocols/groth16/prove.py:76-77). Bases are affine canonical
 * (x.c0, x.c1, y.c0, y.c1), 128 bytes each, element c0 + c1 u as py_ecc's FQ2([c0, c1]);
 * all-zero is infinity. The handle is freed by zk_bases_destroy and is accepted only by
 * the G2 calls. Results are 128 bytes in the same layout (all zero and *out_is_inf = 1 for
 * infinity). Same pipeline as G1 with Fq2 coordinates; no fixed-base mode.
 */
int zk_bases_g2_create(zk_ctx *ctx, const void *xy_canonical_host, size_t n, zk_bases **out);
int zk_bases_g2_create_dev(zk_ctx *ctx, const void *xy_canonical_dev, size_t n, zk_bases **out);
/* out[i] = [k_i] P on G2 (P host canonical, 128 bytes; k and out as zk_g1_fixed_base_mul). */
int zk_g2_fixed_base_mul(zk_ctx *ctx, const uint8_t point_xy[128], const void *k_dev, size_t n, void *out_xy_dev);
int zk_msm_g2(zk_ctx *ctx, const zk_bases *bases, size_t offset, const void *scalars_dev, size_t n,
              int scalars_mont, uint32_t window_bits, uint8_t out_xy[128], int *out_is_inf);
int zk_msm_g2_batch(zk_ctx *ctx, size_t count, const zk_bases *const *bases, const uint64_t *offsets,
                    const void *const *scalars_dev, const uint64_t *sizes, int scalars_mont, uint32_t window_bits,
                    uint8_t *out_xy, int32_t *out_is_inf);

/*
 * Asynchronous batches (the batch_submit / batch_wait pair of the serving layer, which
 * calls the library from its own loop thread while the reference's KernelFns are
 * synchronous: runtime/executor.py:167-218). zk_msm_g1_batch_submit / zk_msm_g2_batch_submit
 * take the arguments of zk_msm_g1_batch / zk_msm_g2_batch, enqueue the device work on the
 * context stream and return; a library thread combines the windows on the host when the
 * device is done. zk_batch_wait returns ZK_OK once out_xy / out_is_inf are written,
 * ZK_ETIMEOUT if timeout_ms (>= 0; negative waits without a limit) passed first (call it
 * again), or the batch's error. Scalars, bases and the output arrays must stay valid until
 * then; zk_batch_destroy waits for the batch and frees it, and every batch of a context
 * must be destroyed before the context. Work enqueued on the context after a submit runs
 * after that batch's device part (one stream).
 */
int zk_msm_g1_batch_submit(zk_ctx *ctx, size_t count, const zk_bases *const *bases, const uint64_t *offsets,
                           const void *const *scalars_dev, const uint64_t *sizes, int scalars_mont,
                           uint32_t window_bits, uint8_t *out_xy, int32_t *out_is_inf, zk_batch **out);
int zk_msm_g2_batch_submit(zk_ctx *ctx, size_t count, const zk_bases *const *bases, const uint64_t *offsets,
                           const void *const *scalars_dev, const uint64_t *sizes, int scalars_mont,
                           uint32_t window_bits, uint8_t *out_xy, int32_t *out_is_inf, zk_batch **out);
int zk_batch_wait(zk_batch *batch, int timeout_ms);
int zk_batch_destroy(zk_batch *batch);

/*
 * Work-queue form of MSM batches (north_star's "(instance, window, bucket-range) items";
 * no reference counterpart): after each pipeline's CSR sort, ONE persistent launch runs
 * every pipeline's later stages -- the accumulation over (instance set, window, bucket
 * range) units, the straddling-piece fixup or merge rounds, the two levels of the window
 * reduction and the per-window target sums -- as items of a device queue, each waiting
 * (bounded, 2 s) until its pipeline's previous stage has published all its items.
 *   zk_msm_batch_set_queue   on != 0: zk_msm_g1_batch / zk_msm_g2_batch and their
 *                            asynchronous forms on this context use it (default off).
 *   zk_msm_queue_test_limit  for tests of the bound: the next work-queue launch of this
 *                            context gets a wait limit of limit_us (1..10^7 us) and its first
 *                            waiting item waits for one item more than exist, so the launch
 *                            stops early and that call returns ZK_ETIMEOUT (the context stays
 *                            usable; the setting is used once).
 */
int zk_msm_batch_set_queue(zk_ctx *ctx, int on);
int zk_msm_queue_test_limit(zk_ctx *ctx, uint64_t limit_us);

/*
 * Batch plan: a zk_msm_g1_batch with fixed shapes, prepared once and run many times
 * (serving, repeated commitments). The plan owns one scalar slot per instance
 * (zk_msm_plan_scalars: device address of sizes[k] elements, filled by the caller by
 * zk_h2d or by a kernel such as zk_ntt writing into it), all scratch and pinned result
 * buffers, so a run allocates nothing. flags (the use_graph argument): ZK_MSM_PLAN_GRAPH
 * (1) captures the device work of a run once as a CUDA graph, each run then one graph
 * launch; ZK_MSM_PLAN_QUEUE (2) runs the plan in the work-queue form above (a run whose
 * queue gave up returns ZK_ETIMEOUT). The bases handles must outlive the plan. No
 * reference counterpart (the reference rebuilds its batch per call).
 */
#define ZK_MSM_PLAN_GRAPH 1
#define ZK_MSM_PLAN_QUEUE 2
typedef struct zk_msm_plan zk_msm_plan;
int zk_msm_plan_create(zk_ctx *ctx, size_t count, const zk_bases *const *bases, const uint64_t *offsets,
                       const uint64_t *sizes, int scalars_mont, uint32_t window_bits, int use_graph,
                       zk_msm_plan **out);
int zk_msm_plan_scalars(zk_msm_plan *plan, size_t index, void **scalars_dev);
int zk_msm_plan_run(zk_msm_plan *plan, uint8_t *out_xy, int32_t *out_is_inf);
/* Kernel launches one run makes (the nodes of its graph). */
int zk_msm_plan_launches(zk_msm_plan *plan, uint64_t *kernels);
int zk_msm_plan_destroy(zk_msm_plan *plan);

/*
 * out[i] = [k_i] P for one affine point P (host, canonical) and n scalars k_i
 * (device, canonical); out is device memory of n affine canonical points.
 * Used for synthetic bases [k_i]G and for key generation from known exponents.
 */
int zk_g1_fixed_base_mul(zk_ctx *ctx, const uint8_t point_xy[64], const void *k_dev, size_t n, void *out_xy_dev);

#ifdef __cplusplus
}
#endif

#endif /* ZKGPU_H */
