"""Benchmark of the BN254 prover hot path on GB300: G1 MSM (Mpts/s) and Fr NTT (Melem/s) at 2^20.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

A step of the headline (``value``) is one G1 MSM over n = 2^20 points: bases are
[k_i]G with k_i uniform in [1, r), resident on the device in Montgomery form;
scalars uniform in [0, r), resident in Montgomery form (the TO_DEVICE layout).
L2 is flushed (a 256 MB memset) before every timed step; each step is timed with
CUDA events on the library's stream and includes the host-side final window
combination of the MSM. ``e2e`` is the same MSM through the C ABI from pinned host
buffers: per step the affine bases (64 B/point) and the canonical scalars
(32 B/point) are copied host->device, converted and summed, and the affine result
(64 B) returns to the host. The Fr NTT at 2^20 (forward, omega = omega_for_size(n))
is measured the same way in ``ntt``; a 2^22 forward NTT is reported in ``ntt_2_22``.

Multi-GPU: one process per GPU (torchrun); the MSM does not need a collective, so
ranks run independent replicas of the step and ``value`` sums their throughput
over the slowest rank's time ("replicas only").

``--impl reference`` times the reference's algorithms restated in C (oracle/,
crypto/msm/pippenger.py:10-64 with the window rule of
runtime/kernels/cpu/kernels.py:559, and crypto/poly/ntt.py:42-100) on all host
cores, on the same workload.
"""

from __future__ import annotations

import argparse
import hashlib
import json
import os
import statistics
import subprocess
import sys
from typing import Optional
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "G1 MSM Mpts/s & Fr NTT Melem/s @2^20; proofs/s + p50/p99 vs plain (bit-exact)"
LOG_N = 20
FLUSH_BYTES = 256 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--log-n", type=int, default=LOG_N)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--only", default="all", choices=["all", "msm", "ntt", "batch", "serve", "plonk", "g2"],
                    help="msm / ntt: only that kernel family, no e2e (short commands for profiling)")
    return ap.parse_args()


# ------------------------------------------------------------------------------ ranks
class Ranks:
    def __init__(self, gpus: int) -> None:
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.dist = None
        if self.world > 1:
            import torch.distributed as dist

            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self) -> None:
        if self.dist is not None:
            self.dist.barrier()

    def max(self, v: float) -> float:
        if self.dist is None:
            return v
        import torch

        t = torch.tensor([v], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self) -> None:
        if self.dist is not None:
            self.dist.destroy_process_group()


# ------------------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int) -> None:
        self.device = device
        self.proc = None
        self.path = None

    def start(self) -> None:
        fd, self.path = tempfile.mkstemp(prefix="clocks_", suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, val in zip(names, parts[5:9]):
                    if val.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------------------ inputs
def make_inputs(ctx, log_n: int):
    from pyzkp_gb300 import synth

    n = 1 << log_n
    seed = synth.seed_for(2, log_n)
    k = synth.base_dlogs(seed, n)
    s = synth.fr_uniform(seed, n)
    dk = ctx.to_device(k)
    bases_xy = ctx.alloc(n * 64)
    ctx.g1_fixed_base_mul((1, 2), dk, n, bases_xy)
    host_xy = bases_xy.download().view("<u8").reshape(n, 8)
    return n, seed, k, s, bases_xy, host_xy


def ntt_omega(n: int) -> int:
    from pyzkp_gb300 import synth

    root = 19103219067921713944291392827692070036145651957329286315305642004821462161904  # 2^28-th root
    return pow(root, 1 << (28 - (n.bit_length() - 1)), synth.FR_MODULUS)


# ------------------------------------------------------------------------------ GPU arm
def run_gpu(args, ranks: Ranks) -> dict:
    from pyzkp_gb300 import _native as N
    from pyzkp_gb300 import synth

    ctx = N.Context(ranks.local)
    L = N.load()
    if args.only == "batch":
        flush = ctx.alloc(FLUSH_BYTES)
        return {"batch": run_gpu_batch(ctx, args, flush)}
    if args.only == "serve":
        return {"groth16_serve": run_gpu_serve(ctx, args)}
    if args.only == "plonk":
        return {"plonk_quotient_2_20": run_gpu_plonk(ctx, args, ctx.alloc(FLUSH_BYTES))}
    if args.only == "g2":
        return {"msm_g2": run_gpu_g2(ctx, args, ctx.alloc(FLUSH_BYTES))}
    if args.only == "ntt":
        flush = ctx.alloc(FLUSH_BYTES)
        peaks = load_peaks()
        return run_gpu_ntt(ctx, args, ranks, args.log_n, flush, imad_peak(ctx)[1], peaks.get("hbm_gbs") or 6800.0,
                           brief=True)
    log_n = args.log_n
    n, seed, k, s, bases_xy, host_xy = make_inputs(ctx, log_n)
    bases = ctx.bases_from_device(bases_xy, n)
    ds = ctx.to_device(s)
    ctx.fr_to_mont(ds, ds, n)
    flush = ctx.alloc(FLUSH_BYTES)
    imad_probes, imad_tops = imad_peak(ctx)

    def msm_step():
        return ctx.msm_g1(bases, ds, n)

    # clocks are sampled from the warm-up to the end of the last timed GPU section
    sampler = ClockSampler(ranks.local)
    sampler.start()
    for _ in range(args.warmup):
        res = msm_step()

    launches0 = ctx.launch_count()
    ranks.barrier()
    ctx.sync()
    times = []
    for _ in range(args.steps):
        ctx.memset(flush, 1)
        ctx.timer_start()
        msm_step()
        times.append(ctx.timer_stop())
    ctx.sync()
    ranks.barrier()
    launches = ctx.launch_count() - launches0
    total_ms = ranks.max(sum(times))
    mpts = n * args.steps * ranks.world / (total_ms * 1e-3) / 1e6
    stats = ctx.msm_last_stats()

    # per-kernel device times (profiling pass, same workload)
    ctx.prof_reset()
    ctx.prof_enable(True)
    prof_steps = 3
    for _ in range(prof_steps):
        ctx.memset(flush, 1)
        msm_step()
    ctx.prof_enable(False)
    table = ctx.prof_table()
    ctx.prof_reset()
    acc_launches, acc_ms = table.get("msm_accumulate", (1, 0.0))
    acc_ms_launch = acc_ms / max(1, acc_launches)
    entries = stats["entries"]
    # algorithmic work of one accumulate launch: one XYZZ mixed addition (8M + 2S = 10 Fq
    # multiplications) per CSR entry; a Montgomery multiplication with 8 limbs is 2*8^2 + 8 = 136
    # 32x32->64 multiply-accumulates, i.e. 272 IMAD (lo + hi) instructions.
    acc_imad = entries * 10 * 272
    acc_tops = acc_imad / (acc_ms_launch * 1e-3) / 1e12
    # algorithmic bytes: per entry the 4-byte CSR entry + the 64-byte affine base
    acc_bytes = entries * 68
    peaks = load_peaks()
    hbm_peak = peaks.get("hbm_gbs") or 6800.0
    roofline = {
        "kernel": "msm_accumulate",
        "bound": "imad",
        "achieved": round(acc_tops, 3),
        "peak": round(imad_tops, 3),
        "unit": "T IMAD/s",
        "frac": round(acc_tops / imad_tops, 4),
        "peak_source": ("measured in this run (no IMAD figure in MEASURED_PEAKS.json): the fastest rate of "
                        "32x32->64 multiply-accumulates, as lo+hi pairs (harmonic mean of the mad.lo and mad.hi "
                        "probes) or as mad.wide, counted as 2 IMAD each like the algorithmic work"),
        "imad_probes_T_per_s": imad_probes,
        "peak_model": imad_model(ctx, acc_tops),
        "launch_ms": round(acc_ms_launch, 4),
        "share_of_step": round(acc_ms / max(1e-9, sum(v[1] for v in table.values())), 4),
        "traffic": traffic_of("msm_accumulate", log_n),
        "traffic_unit": "DRAM bytes per launch (ncu capture of this benchmark)",
        "hbm": {"achieved": round(acc_bytes / (acc_ms_launch * 1e-3) / 1e9, 1), "peak": hbm_peak,
                "unit": "GB/s", "frac": round(acc_bytes / (acc_ms_launch * 1e-3) / 1e9 / hbm_peak, 4),
                "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks.get("hbm_gbs") else "fallback 6800"},
        "algorithmic_work": f"{entries} CSR entries x 10 Fq mults x 272 IMAD; {entries} x 68 B",
        "whole_msm_model": msm_model(n, total_ms / args.steps, imad_tops),
        "sort_kernels": sort_kernels(table, prof_steps, n, entries, hbm_peak),
    }
    kernels = {name: {"launches": la // prof_steps, "ms_per_step": round(ms / prof_steps, 4)}
               for name, (la, ms) in sorted(table.items())}

    if args.only == "msm":
        return {"metric": METRIC, "value": round(mpts, 3), "unit": "Mpts/s", "kernels": kernels,
                "msm_result": [hex(res[0]), hex(res[1])] if res else None,
                "roofline": roofline, "gpu_launches": launches, "clocks": sampler.stop()}

    # e2e through the C ABI from pinned host memory
    pin_xy = ctx.pinned(n * 64)
    pin_xy.array[:] = host_xy.view(np.uint8).reshape(-1)
    pin_s = ctx.pinned(n * 32)
    pin_s.array[:] = s.view(np.uint8).reshape(-1)
    d_s = ctx.alloc(n * 32)
    import ctypes

    out = (ctypes.c_uint8 * 64)()
    inf = ctypes.c_int()

    def e2e_step():  # one call: points and scalars from pinned host memory -> host point
        N.check(L.zk_msm_g1_host(ctx.handle, pin_xy.ptr, pin_s.ptr, n, 0, 0, out, ctypes.byref(inf)),
                "zk_msm_g1_host")

    def e2e_step_separate():  # the same through three calls (bases handle, scalar copy, MSM)
        h = ctypes.c_void_p()
        N.check(L.zk_bases_create(ctx.handle, pin_xy.ptr, n, ctypes.byref(h)), "zk_bases_create")
        N.check(L.zk_h2d(ctx.handle, d_s.ptr, pin_s.ptr, n * 32), "zk_h2d")
        N.check(L.zk_msm_g1(ctx.handle, h, 0, d_s.ptr, n, 0, 0, out, ctypes.byref(inf)), "zk_msm_g1")
        L.zk_bases_destroy(h)

    def timed_e2e(step):
        for _ in range(args.warmup):
            step()
        ok = (int.from_bytes(bytes(out)[:32], "little"), int.from_bytes(bytes(out)[32:], "little")) == res
        ranks.barrier()
        times = []
        for _ in range(args.steps):
            ctx.memset(flush, 1)
            ctx.timer_start()
            step()
            times.append(ctx.timer_stop())
        return n * args.steps * ranks.world / (ranks.max(sum(times)) * 1e-3) / 1e6, ok

    e2e_mpts, e2e_ok = timed_e2e(e2e_step)
    e2e_sep_mpts, e2e_sep_ok = timed_e2e(e2e_step_separate)

    def timed_e2e_stream():
        # a stream of host-buffer MSMs through zk_msm_g1_host_submit: step k + 1's uploads
        # run while step k computes; every step uploads its points and scalars and reads its
        # result back; wall clock from the first submit to the last result
        for _ in range(args.warmup):
            b = ctx.msm_g1_host_submit(pin_xy, pin_s, n)
            b.wait()
            b.destroy()
        ranks.barrier()
        ctx.memset(flush, 1)
        ctx.sync()
        ok = True
        t0 = time.perf_counter()
        pend = []
        for _ in range(args.steps):
            pend.append(ctx.msm_g1_host_submit(pin_xy, pin_s, n))
            if len(pend) > 1:
                b = pend.pop(0)
                ok = ok and b.wait() == [res]
                b.destroy()
        for b in pend:
            ok = ok and b.wait() == [res]
            b.destroy()
        t = ranks.max(time.perf_counter() - t0)
        return n * args.steps * ranks.world / t / 1e6, ok

    e2e_stream_mpts, e2e_stream_ok = timed_e2e_stream()

    ntt = run_gpu_ntt(ctx, args, ranks, 20, flush, imad_tops, hbm_peak)
    ntt22 = run_gpu_ntt(ctx, args, ranks, 22, flush, imad_tops, hbm_peak, brief=True)
    clocks = sampler.stop()
    msm_4096 = run_gpu_msm_4096(ctx, args, flush) if ranks.world == 1 else None
    g2 = run_gpu_g2(ctx, args, flush) if ranks.world == 1 else None
    sweep = run_gpu_msm_sweep(ctx, args, flush) if ranks.world == 1 else None
    fixed = run_gpu_fixed_base(ctx, args, flush) if ranks.world == 1 else None
    fixed_sweep = ({f"2^{lg}": run_gpu_fixed_base(ctx, args, flush, log_n=lg) for lg in range(16, 23)}
                   if ranks.world == 1 else None)
    ntt_sweep = run_gpu_ntt_sweep(ctx, args, flush) if ranks.world == 1 else None
    batch = run_gpu_batch(ctx, args, flush) if ranks.world == 1 else None
    serve_res = run_gpu_serve(ctx, args) if ranks.world == 1 else None
    plonk = run_gpu_plonk(ctx, args, flush) if ranks.world == 1 else None

    result = {
        "metric": METRIC,
        "value": round(mpts, 3),
        "unit": "Mpts/s",
        "n_gpus": ranks.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(total_ms / args.steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u32 limbs (exact BN254 Fq/Fr Montgomery arithmetic)",
        "data": "synthetic: seeded PCG64 scalars uniform in [0,r); bases [k_i]G, k_i uniform in [1,r)",
        "config": {"workload": f"G1 MSM n=2^{log_n} (uniform scalars) + Fr NTT n=2^20", "n": n, "seed": seed,
                   "window_bits": stats["window_bits"], "l2": "flushed (256 MB memset) before every timed step"},
        "config_detail": {"bases": "resident (uploaded once, GLV images built on the device)",
                          "windows": stats["windows"], "csr_entries": entries, "ntt_sizes": [20, 22],
                          "parallelism": f"replicas x{ranks.world}"},
        "msm_result": [hex(res[0]), hex(res[1])] if res else None,
        "e2e": {"value": round(e2e_stream_mpts, 3), "unit": "Mpts/s", "h2d_bytes_per_step": n * 96,
                "d2h_bytes_per_step": 64 + 4, "result_ok": e2e_stream_ok,
                "path": "zk_msm_g1_host_submit per step (pinned host affine points and canonical scalars "
                        "uploaded every step; the host point read back every step) as a stream: step k+1's "
                        "uploads run while step k computes; wall clock from the first submit to the last result",
                "one_call": {"value": round(e2e_mpts, 3), "result_ok": e2e_ok,
                             "path": "zk_msm_g1_host, one synchronous call per step (points uploaded on a "
                                     "second stream while the digits are sorted), device-event timed"},
                "separate_calls": {"value": round(e2e_sep_mpts, 3), "result_ok": e2e_sep_ok,
                                   "path": "zk_bases_create + zk_h2d + zk_msm_g1"}},
        "gpu_launches": launches,
        "gpu_launches_per_step": launches // max(1, args.steps),
        "kernels": kernels,
        "roofline": roofline,
        "ntt": ntt,
        "ntt_2_22": ntt22,
        "msm_2_12": msm_4096,
        "msm_g2": g2,
        "msm_sweep": sweep,
        "msm_fixed_base_2_20": fixed,
        "msm_fixed_base_sweep": fixed_sweep,
        "ntt_sweep": ntt_sweep,
        "batch_64": batch,
        "groth16_serve": serve_res,
        "plonk_quotient_2_20": plonk,
        "clocks": clocks,
    }
    return result


def run_gpu_ntt(ctx, args, ranks, log_n, flush, imad_tops, hbm_peak, brief=False) -> dict:
    from pyzkp_gb300 import _native as N
    from pyzkp_gb300 import synth

    n = 1 << log_n
    v = synth.fr_uniform(synth.seed_for(1, log_n), n)
    om = ntt_omega(n)
    din = ctx.to_device(v)
    ctx.fr_to_mont(din, din, n)
    dout = ctx.alloc(n * 32)
    for _ in range(args.warmup):
        ctx.ntt(N.NTT_EVALS_FROM_COEFFS, dout, din, n, log_n, om)
    ranks.barrier()
    times = []
    for _ in range(args.steps):
        ctx.memset(flush, 1)
        ctx.timer_start()
        ctx.ntt(N.NTT_EVALS_FROM_COEFFS, dout, din, n, log_n, om)
        times.append(ctx.timer_stop())
    total = ranks.max(sum(times))
    melem = n * args.steps * ranks.world / (total * 1e-3) / 1e6
    out = {"metric": f"Fr NTT Melem/s @2^{log_n} (forward)", "value": round(melem, 2), "unit": "Melem/s",
           "ms_per_step": round(total / args.steps, 4)}
    # per-pass device time
    ctx.prof_reset()
    ctx.prof_enable(True)
    for _ in range(3):
        ctx.memset(flush, 1)
        ctx.ntt(N.NTT_EVALS_FROM_COEFFS, dout, din, n, log_n, om)
    ctx.prof_enable(False)
    la, ms = ctx.prof_table().get("ntt_pass", (1, 0.0))
    ctx.prof_reset()
    passes = la // 3
    pass_ms = ms / max(1, la)
    # per pass: every element read once and written once (64 B); radix-2 work of log2(R) stages,
    # (n/2) log2(R) butterflies of one Montgomery multiplication (136 wide MACs = 272 IMAD)
    log_r = log_n / max(1, passes)
    pass_bytes = 64 * n
    pass_imad = (n / 2) * log_r * 272
    gbs = pass_bytes / (pass_ms * 1e-3) / 1e9
    tops = pass_imad / (pass_ms * 1e-3) / 1e12
    out["roofline"] = {"kernel": "ntt_pass", "bound": "imad", "achieved": round(tops, 3), "peak": round(imad_tops, 3),
                       "unit": "T IMAD/s", "frac": round(tops / imad_tops, 4), "passes": passes,
                       "launch_ms": round(pass_ms, 4), "traffic": traffic_of("ntt_pass", log_n),
                       "hbm": {"achieved": round(gbs, 1), "peak": hbm_peak, "unit": "GB/s",
                               "frac": round(gbs / hbm_peak, 4), "per": "pass (64 B/element each pass)"},
                       "hbm_transform": {"achieved": round(64 * n / (passes * pass_ms * 1e-3) / 1e9, 1),
                                         "peak": hbm_peak, "unit": "GB/s",
                                         "frac": round(64 * n / (passes * pass_ms * 1e-3) / 1e9 / hbm_peak, 4),
                                         "per": "transform (64 B/element in and out once, over all passes)"},
                       "algorithmic_work": "per pass 64 B/element; (n/2) log2(R) butterflies x 272 IMAD"}
    if not brief:
        # e2e: canonical host input -> device, to Montgomery, NTT, back to canonical, device -> host
        pin_in = ctx.pinned(n * 32)
        pin_in.array[:] = v.view(np.uint8).reshape(-1)
        pin_out = ctx.pinned(n * 32)
        L = N.load()

        def e2e():
            N.check(L.zk_h2d(ctx.handle, din.ptr, pin_in.ptr, n * 32))
            ctx.fr_to_mont(din, din, n)
            ctx.ntt(N.NTT_EVALS_FROM_COEFFS, dout, din, n, log_n, om)
            ctx.fr_from_mont(dout, dout, n)
            N.check(L.zk_d2h(ctx.handle, pin_out.ptr, dout.ptr, n * 32))

        for _ in range(args.warmup):
            e2e()
        ts = []
        for _ in range(args.steps):
            ctx.memset(flush, 1)
            ctx.timer_start()
            e2e()
            ts.append(ctx.timer_stop())
        tot = ranks.max(sum(ts))
        one_call = n * args.steps * ranks.world / (tot * 1e-3) / 1e6
        # a stream of host-buffer transforms (zk_ntt_host_submit): each step copies its input
        # up and its output back; one step's output copy, the next step's input copy and a
        # transform run at once. Three host buffer pairs in turn (the context's three staging
        # buffers), at most three calls in flight; wall clock.
        pins = [(pin_in, pin_out)] + [(ctx.pinned(n * 32), ctx.pinned(n * 32)) for _ in range(2)]
        for pi, _ in pins[1:]:
            pi.array[:] = pin_in.array
        ref = None
        for _ in range(args.warmup):
            f = ctx.ntt_host_submit(N.NTT_EVALS_FROM_COEFFS, pin_out, pin_in, n, log_n, om)
            f.wait()
            f.destroy()
            ref = bytes(pin_out.array[:64])
        ranks.barrier()
        ctx.memset(flush, 1)
        ctx.sync()
        ok = True
        t0 = time.perf_counter()
        pend = []
        for k in range(args.steps):
            pi, po = pins[k % len(pins)]
            pend.append((ctx.ntt_host_submit(N.NTT_EVALS_FROM_COEFFS, po, pi, n, log_n, om), po))
            if len(pend) >= len(pins):
                f, po_done = pend.pop(0)
                f.wait()
                f.destroy()
                ok = ok and bytes(po_done.array[:64]) == ref
        for f, po_done in pend:
            f.wait()
            f.destroy()
            ok = ok and bytes(po_done.array[:64]) == ref
        stream_t = ranks.max(time.perf_counter() - t0)
        # the same call one at a time (submit, then wait for its fence), wall clock
        ctx.memset(flush, 1)
        ctx.sync()
        sync_ok = True
        t0 = time.perf_counter()
        for _ in range(args.steps):
            f = ctx.ntt_host_submit(N.NTT_EVALS_FROM_COEFFS, pin_out, pin_in, n, log_n, om)
            f.wait()
            f.destroy()
            sync_ok = sync_ok and bytes(pin_out.array[:64]) == ref
        sync_t = ranks.max(time.perf_counter() - t0)
        out["e2e"] = {"value": round(n * args.steps * ranks.world / stream_t / 1e6, 2), "unit": "Melem/s",
                      "h2d_bytes_per_step": n * 32, "d2h_bytes_per_step": n * 32, "result_ok": ok,
                      "path": "zk_ntt_host_submit per step (canonical pinned input up, canonical output back "
                              "every step) as a stream of up to three calls in flight: output copy, next input "
                              "copy and transform at once; wall clock",
                      "one_call": {"value": round(n * args.steps * ranks.world / sync_t / 1e6, 2), "result_ok": sync_ok,
                                   "path": "zk_ntt_host_submit + zk_fence_wait per step, one call at a time, "
                                           "wall clock"},
                      "separate_calls": {"value": round(one_call, 2),
                                         "path": "zk_h2d + zk_fr_to_mont + zk_ntt + zk_fr_from_mont + zk_d2h per "
                                                 "step, device-event timed"}}
    return out


def run_gpu_ntt_sweep(ctx, args, flush, sizes=(12, 16, 20, 22)) -> dict:
    """The four transforms (ROOTS_/COSET_ EVALS/COEFFS, shift 5) at 2^12..2^22,
    device-resident Montgomery data, L2 flushed before each step (median of the steps)."""
    from pyzkp_gb300 import _native as N
    from pyzkp_gb300 import synth

    modes = (("evals_from_coeffs", N.NTT_EVALS_FROM_COEFFS, 1), ("coeffs_from_evals", N.NTT_COEFFS_FROM_EVALS, 1),
             ("coset_evals_from_coeffs", N.NTT_COSET_EVALS_FROM_COEFFS, 5),
             ("coset_coeffs_from_evals", N.NTT_COSET_COEFFS_FROM_EVALS, 5))
    out = {}
    steps = max(3, min(args.steps, 10))
    for log_n in sizes:
        n = 1 << log_n
        om = ntt_omega(n)
        din = ctx.to_device(synth.fr_uniform(synth.seed_for(1, log_n), n))
        ctx.fr_to_mont(din, din, n)
        dout = ctx.alloc(n * 32)
        row = {}
        for name, mode, shift in modes:
            for _ in range(2):
                ctx.ntt(mode, dout, din, n, log_n, om, shift)
            ts = []
            for _ in range(steps):
                ctx.memset(flush, 1)
                ctx.timer_start()
                ctx.ntt(mode, dout, din, n, log_n, om, shift)
                ts.append(ctx.timer_stop())
            ms = statistics.median(ts)
            row[name] = {"Melem_s": round(n / (ms * 1e-3) / 1e6, 1), "ms": round(ms, 4)}
        out[f"2^{log_n}"] = row
    return out


# DRAM traffic per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the dominant
# kernels, from one ncu capture of this benchmark on a GB300 with the current build:
#   ncu --set full --clock-control none -k regex:<kernel> -s <skip> -c 1 -o <report>
#       python bench.py --only <msm|ntt> [--log-n 22] --steps 2 --warmup 3 --no-cpu-baseline
# keyed by (kernel, log2 n); the NTT figure is the mean of the two passes of a 2^22 transform
# (first 134.3 + 81.8 MB, second, with the twiddle-table gathers, 290.2 + 101.4 MB).
NCU_TRAFFIC_BYTES = {("msm_accumulate", 20): 1351.736e6 + 110.563e6,
                     ("ntt_pass", 22): (134.305e6 + 81.835e6 + 290.209e6 + 101.394e6) / 2}


def traffic_of(kernel: str, log_n: int):
    """DRAM bytes of one launch from the ncu capture, or None for a workload not captured."""
    t = NCU_TRAFFIC_BYTES.get((kernel, log_n))
    return None if t is None else int(t)


def sort_kernels(table: dict, steps: int, n: int, entries: int, hbm_peak: float) -> dict:
    """HBM view of the CSR sort (the memory-bound stages): algorithmic bytes per launch over
    the live kernel time. Tiled sort: msm_codes reads the 32-byte scalars and writes one
    4-byte code per (point, window); msm_hist reads the codes; msm_scatter_tiles reads them
    again and writes one 4-byte entry each (its per-tile counters are not counted). Atomic
    sort (bucket sets over 2^15): msm_digits reads the scalars and writes the two 32-byte
    GLV halves; msm_scatter reads the halves and writes the entries. `stage`: every sort
    kernel together (scan and per-tile counter passes, or their one-CTA form, included) against the stage's own
    minimum, the scalars in and the entries out."""
    out = {}
    for name, nbytes in (("msm_codes", n * 32 + entries * 4), ("msm_hist", entries * 4),
                         ("msm_scatter_tiles", entries * 8), ("msm_digits", n * (32 + 64)),
                         ("msm_scatter", n * 64 + entries * 4)):
        la, ms = table.get(name, (0, 0.0))
        if not la:
            continue
        t = ms / la
        gbs = nbytes / (t * 1e-3) / 1e9
        out[name] = {"ms": round(t, 4), "bytes": nbytes, "GB_s": round(gbs, 1), "frac": round(gbs / hbm_peak, 4)}
    names = ("msm_codes", "msm_hist", "msm_hist_total", "msm_hist_offsets", "msm_sort_meta", "msm_scatter_tiles",
             "msm_digits", "msm_scatter", "scan_tiles", "scan_add")
    t = sum(table[k][1] / steps for k in names if k in table and table[k][0])
    if t > 0:
        nbytes = n * 32 + entries * 4
        gbs = nbytes / (t * 1e-3) / 1e9
        out["stage"] = {"ms": round(t, 4), "bytes": nbytes, "GB_s": round(gbs, 1), "frac": round(gbs / hbm_peak, 4),
                        "kernels": [k for k in names if k in table and table[k][0]]}
    return out


def msm_model(n: int, ms: float, imad_tops: float) -> dict:
    """Implementation-independent work of a whole G1 MSM of n points: with the window c* that
    minimises the model (not the implementation's window), W = ceil(255/c*),
    M = [n W 10 (mixed XYZZ additions) + 2 W 2^(c*-1) 14 (bucket running sums) + W c* 10
    (doublings)] Fq multiplications of 136 wide MACs (272 IMAD) each."""
    def fq_mults(c):
        W = -(-255 // c)
        return n * W * 10 + 2 * W * (1 << (c - 1)) * 14 + W * c * 10
    c_star = min(range(4, 25), key=fq_mults)
    m = fq_mults(c_star)
    tops = m * 272 / (ms * 1e-3) / 1e12
    return {"c_star": c_star, "fq_mults": m, "wide_macs": m * 136, "achieved_T_IMAD_s": round(tops, 3),
            "frac": round(tops / imad_tops, 4), "ms": round(ms, 4)}


def imad_model(ctx, achieved_tops: float) -> dict:
    """The denominator checked without the probe: SMs x SM clock x the nominal 64 32-bit
    integer multiply-adds per clock per SM (the CUDA throughput table for compute capability
    10.x). The probe's mad.wide rate counted as 2 IMAD per wide product exceeds it (about 82
    per clock per SM), so the probe's peak is the stricter denominator and the one used."""
    sms = ctx.num_sms()
    mhz = None
    try:
        import subprocess

        out = subprocess.run(["nvidia-smi", "--query-gpu=clocks.max.sm", "--format=csv,noheader,nounits", "-i", "0"],
                             capture_output=True, text=True, timeout=10).stdout.strip().splitlines()
        mhz = float(out[0]) if out else None
    except Exception:  # noqa: BLE001 -- no nvidia-smi: the model is left out
        mhz = None
    if not mhz:
        return {"note": "SM clock unavailable"}
    nominal = sms * mhz * 1e6 * 64 / 1e12
    return {"sms": sms, "sm_max_mhz": mhz, "imad_per_clock_per_sm": 64, "T_IMAD_s": round(nominal, 2),
            "frac_of_nominal": round(achieved_tops / nominal, 4)}


def imad_peak(ctx):
    """Probe the integer pipe; return (probes, peak) in 10^12 IMAD/s (a wide MAC = 2 IMAD)."""
    pr = {"carry_chain": ctx.imad_probe(0), "mad_lo": ctx.imad_probe(1), "mad_hi": ctx.imad_probe(2),
          "mad_wide_as_2": ctx.imad_probe(3)}
    pair = 1.0 / (1.0 / pr["mad_lo"] + 1.0 / pr["mad_hi"])  # wide MACs/s as lo + hi
    wide = pr["mad_wide_as_2"] / 2.0  # wide MACs/s as mad.wide
    peak = 2.0 * max(pair, wide)
    return {k: round(v, 3) for k, v in pr.items()}, peak


def run_gpu_msm_sweep(ctx, args, flush, sizes=(16, 17, 18, 19, 20, 21, 22)) -> dict:
    """MSM size sweep 2^16..2^22 under uniform and witness-like scalars (resident inputs)."""
    from pyzkp_gb300 import synth

    out = {}
    steps = max(3, min(args.steps, 10))
    for log_n in sizes:
        n = 1 << log_n
        seed = synth.seed_for(2, log_n)
        dk = ctx.to_device(synth.base_dlogs(seed, n))
        xy = ctx.alloc(n * 64)
        ctx.g1_fixed_base_mul((1, 2), dk, n, xy)
        bases = ctx.bases_from_device(xy, n)
        del dk, xy
        row = {}
        for kind, gen in (("uniform", synth.fr_uniform), ("witness_like", synth.fr_witness_like)):
            ds = ctx.to_device(gen(seed, n))
            ctx.fr_to_mont(ds, ds, n)
            for _ in range(2):
                ctx.msm_g1(bases, ds, n)
            ts = []
            for _ in range(steps):
                ctx.memset(flush, 1)
                ctx.timer_start()
                ctx.msm_g1(bases, ds, n)
                ts.append(ctx.timer_stop())
            row[kind] = {"Mpts_s": round(n / (statistics.median(ts) * 1e-3) / 1e6, 2),
                         "ms": round(statistics.median(ts), 4)}
        out[f"2^{log_n}"] = row
        bases.free()
    return out


def run_gpu_msm_4096(ctx, args, flush, steps: int = 50) -> dict:
    """The 4096-point G1 MSM the reference runs on CPU (bases [k_i]G, uniform scalars, seed
    family 0): device time with resident inputs, and end to end through zk_msm_g1_host from
    pinned host memory. The result goes to the CPU baseline leg for the known-answer check."""
    from pyzkp_gb300 import synth

    log_n = 12
    n = 1 << log_n
    seed = synth.seed_for(0, log_n)
    k, s = synth.base_dlogs(seed, n), synth.fr_uniform(seed, n)
    dk = ctx.to_device(k)
    xy = ctx.alloc(n * 64)
    ctx.g1_fixed_base_mul((1, 2), dk, n, xy)
    bases = ctx.bases_from_device(xy, n)
    pin_xy = ctx.pinned(n * 64)
    pin_xy.array[:] = xy.download().view(np.uint8).reshape(-1)
    pin_s = ctx.pinned(n * 32)
    pin_s.array[:] = s.view(np.uint8).reshape(-1)
    ds = ctx.to_device(s)
    ctx.fr_to_mont(ds, ds, n)

    def timed(step):
        for _ in range(max(3, args.warmup)):
            r = step()
        ts = []
        for _ in range(steps):
            ctx.memset(flush, 1)
            ctx.timer_start()
            step()
            ts.append(ctx.timer_stop())
        return statistics.median(ts), r

    ms, res = timed(lambda: ctx.msm_g1(bases, ds, n))
    e2e_ms, res_host = timed(lambda: ctx.msm_g1_host(pin_xy, pin_s, n))
    bases.free()
    return {"n": n, "seed": seed, "ms": round(ms, 4), "Mpts_s": round(n / (ms * 1e-3) / 1e6, 2),
            "e2e": {"ms": round(e2e_ms, 4), "Mpts_s": round(n / (e2e_ms * 1e-3) / 1e6, 2),
                    "h2d_bytes_per_step": n * 96, "d2h_bytes_per_step": 64 + 4,
                    "path": "zk_msm_g1_host(pinned host affine points, pinned canonical scalars)"},
            "steps": steps, "device_equals_host_call": res == res_host,
            "msm_result": [hex(res[0]), hex(res[1])] if res else None,
            "l2": "flushed (256 MB memset) before every timed step"}


def run_gpu_g2(ctx, args, flush, sizes=(16, 18, 20)) -> dict:
    """G2 MSMs (the group of the Groth16 B query): bases [k_i]G2 from the device fixed-base
    multiplication, uniform scalars, GLV split, L2 flushed before each timed call. The result
    of the largest size goes to the CPU baseline leg for the known-answer check."""
    from pyzkp_gb300 import synth
    from pyzkp_gb300.groth16 import G2_GEN

    out = {}
    steps = max(3, min(args.steps, 10))
    for lg in sizes:
        n = 1 << lg
        seed = synth.seed_for(6, lg)
        dk = ctx.to_device(synth.base_dlogs(seed, n))
        xy = ctx.alloc(n * 128)
        ctx.g2_fixed_base_mul(G2_GEN, dk, n, xy)
        bases = ctx.bases_g2_from_device(xy, n)
        del dk, xy
        ds = ctx.to_device(synth.fr_uniform(seed, n))
        ctx.fr_to_mont(ds, ds, n)
        for _ in range(2):
            res = ctx.msm_g2(bases, ds, n)
        ts = []
        for _ in range(steps):
            ctx.memset(flush, 1)
            ctx.timer_start()
            ctx.msm_g2(bases, ds, n)
            ts.append(ctx.timer_stop())
        ms = statistics.median(ts)
        row = {"n": n, "seed": seed, "ms": round(ms, 3), "Mpts_s": round(n / (ms * 1e-3) / 1e6, 2),
               "window_bits": ctx.msm_last_stats()["window_bits"]}
        if lg == max(sizes):
            row["msm_result"] = None if res is None else [hex(v) for v in (res[0][0], res[0][1], res[1][0], res[1][1])]
        out[f"2^{lg}"] = row
        bases.free()
    return out


def run_gpu_fixed_base(ctx, args, flush, log_n: int = 20, calls: int = 16) -> dict:
    """One base set reused across 16 MSMs (fixed-base rows computed on the first call)."""
    from pyzkp_gb300 import plugin, synth

    n = 1 << log_n
    seed = synth.seed_for(2, log_n) + 7
    dk = ctx.to_device(synth.base_dlogs(seed, n))
    xy = ctx.alloc(n * 64)
    ctx.g1_fixed_base_mul((1, 2), dk, n, xy)
    bases = ctx.bases_from_device(xy, n)
    c = plugin.fixed_base_window(n)
    scal = [ctx.to_device(synth.fr_uniform(seed + i, n)) for i in range(calls)]
    for d in scal:
        ctx.fr_to_mont(d, d, n)
    ctx.memset(flush, 1)
    ctx.timer_start()
    ctx.bases_precompute(bases, c)
    ctx.msm_g1(bases, scal[0], n)
    first = ctx.timer_stop()
    ts = []
    for i in range(1, calls):
        ctx.memset(flush, 1)
        ctx.timer_start()
        ctx.msm_g1(bases, scal[i], n)
        ts.append(ctx.timer_stop())
    steady = statistics.median(ts)
    return {"n": n, "calls": calls, "window_bits": c, "first_call_ms": round(first, 3),
            "steady_ms": round(steady, 4), "steady_Mpts_s": round(n / (steady * 1e-3) / 1e6, 2),
            "note": "first call includes the window-shifted base rows (zk_bases_precompute)"}


def run_gpu_batch(ctx, args, flush, count: int = 64, lo: int = 10, hi: int = 20) -> dict:
    """64 MSMs + 64 NTTs with sizes 2^U, U ~ Uniform[lo, hi] (MSM n = round(2^U), NTT n =
    2^round(U)): plain per-instance calls against the batched engine (direct, then as a
    CUDA-graph plan, then with autotuned windows / radix splits). Results must agree bit
    for bit with the per-instance calls."""
    from pyzkp_gb300 import _native as N
    from pyzkp_gb300 import synth

    seed = synth.seed_for(3, hi)
    rng = np.random.default_rng(seed)
    msm_sizes = [int(round(2 ** u)) for u in rng.uniform(lo, hi, size=count)]
    ntt_logs = [int(round(u)) for u in rng.uniform(lo, hi, size=count)]
    nmax = 1 << hi
    dk = ctx.to_device(synth.base_dlogs(seed, nmax))
    xy = ctx.alloc(nmax * 64)
    ctx.g1_fixed_base_mul((1, 2), dk, nmax, xy)
    bases = ctx.bases_from_device(xy, nmax)
    del dk, xy
    total = sum(msm_sizes)
    flat = ctx.to_device(synth.fr_uniform(seed + 1, total))
    ctx.fr_to_mont(flat, flat, total)
    ptrs, off = [], 0
    for m in msm_sizes:
        ptrs.append(flat.ptr + 32 * off)
        off += m
    reps = max(3, min(args.steps, 5))

    def timed(fn):
        fn()  # warm-up: pools, tables, plans
        ts = []
        for _ in range(reps):
            ctx.memset(flush, 1)
            ctx.timer_start()
            fn()
            ts.append(ctx.timer_stop())
        return statistics.median(ts)

    def plain_msm():
        return [ctx.msm_g1(bases, N.DeviceArray(ctx, m * 32, ptr=p, owned=False), m)
                for m, p in zip(msm_sizes, ptrs)]

    ref = plain_msm()
    out = {"instances": count, "msm_sizes_log2_range": [lo, hi], "msm_points": total,
           "ntt_sizes": {f"2^{k}": ntt_logs.count(k) for k in sorted(set(ntt_logs))}}
    t_plain = timed(plain_msm)
    got = ctx.msm_g1_batch(bases, ptrs, msm_sizes)
    t_batch = timed(lambda: ctx.msm_g1_batch(bases, ptrs, msm_sizes))
    plan = ctx.msm_plan(bases, msm_sizes, use_graph=True)
    for j, m in enumerate(msm_sizes):
        ctx.d2d(plan.slot(j), N.DeviceArray(ctx, m * 32, ptr=ptrs[j], owned=False), m * 32)
    got_plan = plan.run()
    t_plan = timed(plan.run)
    plan_launches = plan.launches()
    plan.free()
    # the work-queue form: the sorts, then every pipeline's later stages in one launch
    qplan = ctx.msm_plan(bases, msm_sizes, use_graph=True, queue=True)
    for j, m in enumerate(msm_sizes):
        ctx.d2d(qplan.slot(j), N.DeviceArray(ctx, m * 32, ptr=ptrs[j], owned=False), m * 32)
    got_queue = qplan.run()
    t_queue = timed(qplan.run)
    queue_launches = qplan.launches()
    qplan.free()
    # small instances only (2^10..2^14), where launch latency weighs most
    small_sizes = [int(round(2 ** u)) for u in rng.uniform(lo, 14, size=count)]
    small = {"points": sum(small_sizes)}
    small_src = ctx.to_device(synth.fr_uniform(seed + 2, max(small_sizes)))
    ctx.fr_to_mont(small_src, small_src, max(small_sizes))
    small_ref = None
    for name, q in (("plan_graph", False), ("plan_graph_queue", True)):
        sp = ctx.msm_plan(bases, small_sizes, use_graph=True, queue=q)
        for j, m in enumerate(small_sizes):
            ctx.d2d(sp.slot(j), small_src, m * 32)
        r = sp.run()
        small[name + "_ms"] = round(timed(sp.run), 4)
        small[name + "_kernels"] = sp.launches()
        small_ref = small_ref or r
        small["bit_exact"] = small.get("bit_exact", True) and r == small_ref
        sp.free()
    # autotuned windows for every size class of the batch (best of c in rule +- 2)
    t0 = time.perf_counter()
    tuned = {}
    for lg in sorted(set(max(1, m - 1).bit_length() for m in msm_sizes)):
        lg = min(lg, hi)
        c, _ = ctx.autotune_msm(bases, flat, lg, reps=1)
        tuned[lg] = c
    tune_s = time.perf_counter() - t0
    plan = ctx.msm_plan(bases, msm_sizes, use_graph=True)
    for j, m in enumerate(msm_sizes):
        ctx.d2d(plan.slot(j), N.DeviceArray(ctx, m * 32, ptr=ptrs[j], owned=False), m * 32)
    got_tuned = plan.run()
    t_tuned = timed(plan.run)
    plan.free()
    out["msm"] = {
        "plain_ms": round(t_plain, 3), "batch_ms": round(t_batch, 3), "plan_graph_ms": round(t_plan, 3),
        "plan_graph_tuned_ms": round(t_tuned, 3), "plan_graph_queue_ms": round(t_queue, 3),
        "plain_Mpts_s": round(total / (t_plain * 1e-3) / 1e6, 2),
        "batch_Mpts_s": round(total / (t_batch * 1e-3) / 1e6, 2),
        "plan_graph_Mpts_s": round(total / (t_plan * 1e-3) / 1e6, 2),
        "plan_graph_tuned_Mpts_s": round(total / (t_tuned * 1e-3) / 1e6, 2),
        "plan_graph_queue_Mpts_s": round(total / (t_queue * 1e-3) / 1e6, 2),
        "graph_kernels": plan_launches, "queue_graph_kernels": queue_launches,
        "tuned_windows": {f"2^{k}": v for k, v in tuned.items()},
        "autotune_s": round(tune_s, 2),
        "bit_exact_vs_plain": got == ref and got_plan == ref and got_tuned == ref and got_queue == ref,
        "small_2_10_to_2_14": small,
    }
    for lg in tuned:
        ctx.tune_set_msm_window(lg, 0)
    del flat

    # NTTs: coset forward (shift 5) of uniform inputs, out of place
    bufs = []
    for j, lg in enumerate(ntt_logs):
        n = 1 << lg
        a = ctx.to_device(synth.fr_uniform(seed + 100 + j, n))
        ctx.fr_to_mont(a, a, n)
        bufs.append((a, ctx.alloc(n * 32)))
    jobs = [(2, o, a, 1 << lg, lg, ntt_omega(1 << lg), 5) for (a, o), lg in zip(bufs, ntt_logs)]
    elems = sum(1 << lg for lg in ntt_logs)

    def plain_ntt():
        for (mode, o, a, ln, lg, om, sh) in jobs:
            ctx.ntt(mode, o, a, ln, lg, om, sh)

    def snapshot():
        ctx.sync()
        return [hashlib.sha256(o.download((1 << lg) * 32).tobytes()).hexdigest() for (_, o, _, _, lg, _, _) in jobs]

    plain_ntt()
    ref_n = snapshot()
    t_nplain = timed(plain_ntt)
    t_nbatch = timed(lambda: ctx.ntt_batch(jobs))
    ok_batch = snapshot() == ref_n
    nplan = ctx.ntt_plan(jobs, use_graph=True)
    t_nplan = timed(nplan.run)
    ok_plan = snapshot() == ref_n
    nplan_launches = nplan.launches()
    nplan.free()
    # the work-queue form: every pass of every transform in one persistent launch
    nplan = ctx.ntt_plan(jobs, use_graph=True, queue=True)
    t_nqueue = timed(nplan.run)
    ctx.ntt_queue_status()
    ok_queue = snapshot() == ref_n
    nqueue_launches = nplan.launches()
    nplan.free()
    # small transforms only (2^10..2^14), where launch latency weighs most
    small_logs = [int(round(u)) for u in rng.uniform(lo, 14, size=count)]
    small_bufs = []
    for j, lg in enumerate(small_logs):
        a = ctx.to_device(synth.fr_uniform(seed + 300 + j, 1 << lg))
        ctx.fr_to_mont(a, a, 1 << lg)
        small_bufs.append((a, ctx.alloc((1 << lg) * 32)))
    small_jobs = [(2, o, a, 1 << lg, lg, ntt_omega(1 << lg), 5) for (a, o), lg in zip(small_bufs, small_logs)]
    small = {"elements": sum(1 << lg for lg in small_logs)}
    small_ref = None
    for name, q in (("plan_graph", False), ("plan_graph_queue", True)):
        sp = ctx.ntt_plan(small_jobs, use_graph=True, queue=q)
        small[name + "_ms"] = round(timed(sp.run), 4)
        ctx.ntt_queue_status()
        ctx.sync()
        h = [hashlib.sha256(o.download((1 << lg) * 32).tobytes()).hexdigest()
             for (_, o, _, _, lg, _, _) in small_jobs]
        small_ref = small_ref or h
        small["bit_exact"] = small.get("bit_exact", True) and h == small_ref
        sp.free()
    del small_bufs, small_jobs
    t0 = time.perf_counter()
    splits = {}
    scratch = ctx.alloc((1 << hi) * 32)
    for lg in sorted(set(ntt_logs)):
        splits[lg], _ = ctx.autotune_ntt(scratch, lg, reps=3)
    del scratch
    ntune_s = time.perf_counter() - t0
    nplan = ctx.ntt_plan(jobs, use_graph=True)
    t_ntuned = timed(nplan.run)
    ok_tuned = snapshot() == ref_n
    nplan.free()
    for lg in splits:
        ctx.tune_set_ntt_split(lg, [])
    out["ntt"] = {
        "mode": "coset forward, shift 5", "elements": elems,
        "plain_ms": round(t_nplain, 3), "batch_ms": round(t_nbatch, 3), "plan_graph_ms": round(t_nplan, 3),
        "plan_graph_tuned_ms": round(t_ntuned, 3), "plan_graph_queue_ms": round(t_nqueue, 3),
        "plain_Melem_s": round(elems / (t_nplain * 1e-3) / 1e6, 1),
        "batch_Melem_s": round(elems / (t_nbatch * 1e-3) / 1e6, 1),
        "plan_graph_Melem_s": round(elems / (t_nplan * 1e-3) / 1e6, 1),
        "plan_graph_tuned_Melem_s": round(elems / (t_ntuned * 1e-3) / 1e6, 1),
        "plan_graph_queue_Melem_s": round(elems / (t_nqueue * 1e-3) / 1e6, 1),
        "graph_kernels": nplan_launches, "queue_graph_kernels": nqueue_launches,
        "tuned_splits": {f"2^{k}": v for k, v in splits.items()},
        "autotune_s": round(ntune_s, 2), "bit_exact_vs_plain": ok_batch and ok_plan and ok_tuned and ok_queue,
        "small_2_10_to_2_14": small,
    }
    bases.free()
    return out


def run_gpu_plonk(ctx, args, flush, log_n: int = 20) -> dict:
    """The PLONK quotient step of protocols/plonk/prove.py:319-420 at n = 2^log_n, extended
    domain m = 4n: 15 coset NTTs of the n-coefficient polynomials to m evaluations (z also at
    shift * omega_n), PLONK_T_QUOTIENT_EVALS, BATCH_INV of Z_H, POINTWISE_MUL and the coset
    iNTT of t -- as device calls, inputs resident, L2 flushed before each step. The 15
    evaluation vectors, the numerators and Z_H are gathered at 16 indices into the private
    key ``_samples``; the CPU baseline leg checks them (``cpu_check_plonk``) and drops the key."""
    from pyzkp_gb300 import _native as N
    from pyzkp_gb300 import synth

    R = synth.FR_MODULUS
    n, m, lg_m = 1 << log_n, 4 << log_n, log_n + 2
    om_m, om_n = ntt_omega(m), ntt_omega(n)
    seed = synth.seed_for(5, log_n)
    shift = 7 + seed % 1000
    alpha, beta, gamma, k1, k2 = (synth.limbs_to_ints(synth.fr_uniform(seed + j, 1))[0] for j in range(5))
    coeffs = []
    for j in range(15):
        d = ctx.to_device(synth.fr_uniform(seed + 10 + j, n))
        ctx.fr_to_mont(d, d, n)
        coeffs.append(d)
    ext = [ctx.alloc(m * 32) for _ in range(15)]
    num, zh, inv, t = (ctx.alloc(m * 32) for _ in range(4))
    jobs = [(N.NTT_COSET_EVALS_FROM_COEFFS, ext[j], coeffs[j], n, lg_m, om_m, shift * om_n % R if j == 13 else shift)
            for j in range(15)]
    shift_n = pow(shift, n, R)

    def step():
        ctx.ntt_batch(jobs)
        ctx.plonk_quotient_evals(ext, m, n, om_m, shift, shift_n, alpha, beta, gamma, k1, k2, num, zh)
        ctx.fr_batch_inv(inv, zh, m)
        ctx.fr_mul(t, num, inv, m)
        ctx.ntt(N.NTT_COSET_COEFFS_FROM_EVALS, t, t, m, lg_m, om_m, shift)

    for _ in range(2):
        step()
    steps = max(3, min(args.steps, 10))
    ts = []
    for _ in range(steps):
        ctx.memset(flush, 1)
        ctx.timer_start()
        step()
        ts.append(ctx.timer_stop())
    ms = statistics.median(ts)
    # sampled check: the 15 evaluation vectors and num / zh at 16 indices, back to canonical
    ctx.ntt_batch(jobs)
    ctx.plonk_quotient_evals(ext, m, n, om_m, shift, shift_n, alpha, beta, gamma, k1, k2, num, zh)
    idx = np.array([0, 1, m - 1] + [int(x) for x in np.random.default_rng(seed).integers(0, m, 13)], dtype=np.uint32)
    didx = ctx.to_device(idx)
    got = []
    for src in ext + [num, zh]:
        g = ctx.alloc(idx.size * 32)
        ctx.fr_gather(g, src, didx, idx.size)
        ctx.fr_from_mont(g, g, idx.size)
        got.append(synth.limbs_to_ints(g.download().view("<u8").reshape(-1, 4)))
    samples = {"idx": [int(i) for i in idx], "got": got, "n": n, "om_m": om_m, "shift": shift,
               "shift_n": shift_n, "params": (alpha, beta, gamma, k1, k2)}
    return {"n": n, "m": m, "ms": round(ms, 3), "Melem_s_extended": round(m / (ms * 1e-3) / 1e6, 1),
            "steps": steps, "sampled_check_ok": None, "_samples": samples,
            "work": "15 coset NTTs n -> 4n (one batched call), quotient evals, batch inverse, product, coset iNTT"}


_SERVE_VERIFY_JOBS: list = []


def run_gpu_serve(ctx, args, requests: int = 200, grid=tuple(x / 2 for x in range(20, 37))) -> dict:
    """Groth16 proof serving: Poisson arrivals, request sizes m = round(2^U), U ~ Uniform[10, 18],
    snapped to resident circuits at U on a 0.5 grid (a circuit needs its own proving key);
    synthetic diagonal R1CS (x_i y_i = z_i), keys from a fast own setup. Continuous batching
    (three slot contexts, the first at the most urgent stream priority for small requests)
    against batch-at-a-time and the plain one-at-a-time prover on the same traces; the proofs
    of every mode must agree bit for bit, and every continuous-mode proof is verified with the
    reference's verification equation by the CPU leg (off the timed path)."""
    from pyzkp_gb300 import groth16 as G
    from pyzkp_gb300 import serve

    t0 = time.perf_counter()
    keys, wits, sizes, pubs = {}, {}, {}, {}
    for i, u in enumerate(grid):
        m = int(round(2 ** u))
        keys[i] = G.setup(ctx, G.diagonal_r1cs(m), G.Trapdoors.seeded(0x5E7 + i))
        wits[i], pubs[i] = G.diagonal_witness(ctx, m, 0xA11CE + i)
        sizes[i] = m
    setup_s = time.perf_counter() - t0
    prover = G.Prover(ctx)
    # at most 24 requests per group: a burst spreads over the slots, so one group's latency-bound
    # reductions overlap another's accumulation (on the 128-request burst 24 measured ~5% above 64)
    svc = serve.ProverService(prover, keys, wits, budget_bytes=48 << 30, max_batch=24, slots=3)
    weights = [0.5] + [1.0] * (len(grid) - 2) + [0.5]
    svc.warm()
    # closed-loop capacity: a burst of requests all present at t = 0
    closed = serve.poisson_trace(1e9, 128, list(keys), seed=2, weights=weights)
    cap = {}
    for mode, tr in (("continuous", closed), ("batch", closed), ("plain", closed)):
        runs = []
        for _ in range(3):  # the median of three runs of the burst
            t1 = time.perf_counter()
            res = svc.run(tr, mode)
            runs.append(len(tr) / (time.perf_counter() - t1))
        cap[mode] = statistics.median(runs)
        if mode == "continuous":
            cap_proofs = res.proofs
    # The accumulation floor of the burst: its CSR entries (fixed-base mode: ceil(255 / c)
    # per point and query) times the accumulation kernel's time per entry, measured on one
    # large MSM of the largest resident key (G1 l-query, G2 b-query). No mode can prove the
    # burst faster than this, so plain_time / floor bounds the batched / plain ratio.
    from pyzkp_gb300 import synth
    from pyzkp_gb300.plugin import fixed_base_window

    def _entries(q):
        return q.count * -(-255 // fixed_base_window(q.count)) if q.count else 0

    e_g1 = sum(_entries(q) for a in closed for q in (keys[a.key_id].a, keys[a.key_id].b1, keys[a.key_id].l,
                                                      keys[a.key_id].h))
    e_g2 = sum(_entries(keys[a.key_id].b2) for a in closed)
    big = keys[max(keys, key=lambda i: sizes[i])]
    per_entry = {}
    for name, q, fn in (("g1", big.l, ctx.msm_g1), ("g2", big.b2, ctx.msm_g2)):
        sc = ctx.to_device(synth.fr_uniform(77, q.count))
        ctx.fr_to_mont(sc, sc, q.count)
        fn(q.bases, sc, q.count)
        ctx.sync()
        ctx.prof_reset()
        ctx.prof_enable(True)
        fn(q.bases, sc, q.count)
        ctx.sync()
        tab = ctx.prof_table()
        ctx.prof_enable(False)
        per_entry[name] = tab["msm_accumulate"][1] / ctx.msm_last_stats()["entries"]
        del sc
    floor_ms = e_g1 * per_entry["g1"] + e_g2 * per_entry["g2"]
    plain_ms = len(closed) / cap["plain"] * 1e3
    floor = {"g1_entries": e_g1, "g2_entries": e_g2,
             "ns_per_entry": {k: round(v * 1e6, 3) for k, v in per_entry.items()},
             "burst_ms": round(floor_ms, 2), "plain_burst_ms": round(plain_ms, 2),
             "continuous_burst_ms": round(len(closed) / cap["continuous"] * 1e3, 2),
             "max_ratio_over_plain": round(plain_ms / floor_ms, 2)}
    sweep = []
    exact = True
    verify_jobs = []

    def collect(trace, res):
        for a, p in zip(trace, res.proofs):
            if p is not None:
                k = keys[a.key_id]
                vk = (k.vk.alpha_g1, k.vk.beta_g2, k.vk.gamma_g2, k.vk.delta_g2, k.vk.ic)
                verify_jobs.append((a.key_id, vk, pubs[a.key_id], (p.a, p.b, p.c)))

    collect(closed, type("R", (), {"proofs": cap_proofs})())
    for frac in (0.25, 0.5, 0.9):
        rate = frac * cap["continuous"]
        tr = serve.poisson_trace(rate, requests, list(keys), seed=int(frac * 1000), weights=weights)
        rc = svc.run(tr, "continuous")
        rb = svc.run(tr, "batch")
        rp = svc.run(tr, "plain")
        exact = exact and rc.proofs == rp.proofs and rb.proofs == rp.proofs and all(p is not None for p in rc.proofs)
        collect(tr, rc)
        sweep.append({"rate_per_s": round(rate, 1), "continuous": rc.summary(), "batch": rb.summary(),
                      "plain": rp.summary()})
    svc.close()
    _SERVE_VERIFY_JOBS[:] = verify_jobs
    mean_m = sum(w * sizes[i] for i, w in zip(sorted(sizes), weights)) / sum(weights)
    return {
        "workload": "Groth16 prove, diagonal R1CS, m = round(2^U), U ~ U[10,18] on a 0.5 grid, Poisson arrivals",
        "circuits": len(grid), "constraints": [sizes[i] for i in sorted(sizes)], "mean_constraints": round(mean_m),
        "setup_s": round(setup_s, 2), "key_bytes": sum(k.device_bytes() for k in keys.values()),
        "capacity_proofs_s": {k: round(v, 1) for k, v in cap.items()},
        "capacity_continuous_over_plain": round(cap["continuous"] / cap["plain"], 2),
        "capacity_batch_over_plain": round(cap["batch"] / cap["plain"], 2),
        "accumulation_floor": floor,
        "sweep": sweep, "bit_exact_all_modes": exact,
        "proofs_total": len(verify_jobs), "proofs_verified": None,
        "note": "latency = completion - arrival on the wall clock; proof assembly (5 host scalar "
                "multiplications per proof) runs on host threads; proofs_verified is filled by the CPU leg",
    }


def _verify_chunk(jobs):
    from oracle import groth16_verify as V

    return V.verify_many(jobs)


def cpu_verify_serve(jobs) -> dict:
    """Every served proof through the reference's verification equation (protocols/groth16/
    verify.py:11-23) with the stand-in pairing, in a spawned process pool (off the timed path)."""
    import multiprocessing as mp

    if not jobs:
        return {"proofs_verified": 0, "proofs_total": 0}
    t0 = time.perf_counter()
    workers = max(1, min(16, (os.cpu_count() or 2) - 1))
    # chunks grouped by key so that each worker builds few verifiers
    jobs = sorted(jobs, key=lambda j: j[0])
    chunks = [jobs[i::workers * 2] for i in range(workers * 2)]
    with mp.get_context("spawn").Pool(workers) as pool:
        res = [ok for part in pool.map(_verify_chunk, chunks) for ok in part]
    return {"proofs_verified": int(sum(res)), "proofs_total": len(res), "verify_s": round(time.perf_counter() - t0, 1),
            "verifier": "reference verification equation (protocols/groth16/verify.py:11-23), py_ecc stand-in "
                        f"pairing, {workers} host processes"}


def load_peaks() -> dict:
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


# ------------------------------------------------------------------------------ CPU (oracle port)
def cpu_msm_sample(log_n: int, budget_s: float = 10.0, full_size: bool = False):
    """The reference's Pippenger (restated in C, all host threads) on the same workload."""
    from oracle import oracle as O
    from pyzkp_gb300 import synth

    n = 1 << log_n
    seed = synth.seed_for(2, log_n)
    k = synth.base_dlogs(seed, n)
    s = synth.fr_uniform(seed, n)
    bases = O.g1_fixed_base_mul(O.G1_GENERATOR, k)
    w = O.msm_window_rule(n)
    runs, t0 = 0, time.perf_counter()
    while True:
        O.msm_pippenger(bases, s, w)
        runs += 1
        el = time.perf_counter() - t0
        if el >= budget_s or full_size:
            break
    return n * runs / el / 1e6, runs, el


def cpu_ntt_sample(log_n: int, budget_s: float = 5.0):
    from oracle import oracle as O
    from pyzkp_gb300 import synth

    n = 1 << log_n
    v = synth.fr_uniform(synth.seed_for(1, log_n), n)
    om = O.omega_for_size(n)
    runs, t0 = 0, time.perf_counter()
    while True:
        O.ntt_op(0, v, n, om)
        runs += 1
        el = time.perf_counter() - t0
        if el >= budget_s:
            break
    return n * runs / el / 1e6, runs, el


def cpu_check_plonk(samples: dict) -> bool:
    """Checks the GPU arm's gathered PLONK quotient samples: at each sampled index i the
    numerator is the oracle formula applied to the 15 gathered evaluations at
    x = shift * omega_m^i, and Z_H(x) = shift^n * omega_m^(n i) - 1."""
    from oracle import oracle as O
    from pyzkp_gb300 import synth

    R = synth.FR_MODULUS
    got, n, om_m = samples["got"], samples["n"], samples["om_m"]
    alpha, beta, gamma, k1, k2 = samples["params"]
    ok = True
    for s_i, i in enumerate(samples["idx"]):
        vecs = [[got[j][s_i]] for j in range(15)]
        x = samples["shift"] * pow(om_m, i, R) % R
        e_num, _ = O.plonk_t_quotient_evals(vecs, n, om_m, x, samples["shift_n"], alpha, beta, gamma, k1, k2)
        e_zh = (samples["shift_n"] * pow(pow(om_m, n, R), i, R) - 1) % R
        ok = ok and e_num[0] == got[15][s_i] and e_zh == got[16][s_i]
    return ok


def cpu_msm_4096(gpu_row: dict, budget_s: float = 3.0) -> dict:
    """The 4096-point MSM on the host: the C restatement of crypto/msm/pippenger.py with the
    reference's window rule, timed over repeated runs, and the GPU arm's result against the
    known answer [sum k_i s_i]G and against this Pippenger."""
    from oracle import oracle as O
    from pyzkp_gb300 import synth

    n, seed = gpu_row["n"], gpu_row["seed"]
    k, s = synth.base_dlogs(seed, n), synth.fr_uniform(seed, n)
    bases = O.g1_fixed_base_mul(O.G1_GENERATOR, k)
    w = O.msm_window_rule(n)
    runs, t0 = 0, time.perf_counter()
    while True:
        got = O.msm_pippenger(bases, s, w)
        runs += 1
        el = time.perf_counter() - t0
        if el >= budget_s:
            break
    pip = O.affine_to_ints(got)
    known = O.affine_to_ints(O.msm_known_answer(k, s))
    return {"value": round(n * runs / el / 1e6, 4), "unit": "Mpts/s", "ms": round(el / runs * 1e3, 3),
            "window_bits": w, "runs": runs,
            "gpu_result_matches_known_answer": [hex(known[0]), hex(known[1])] == gpu_row["msm_result"],
            "pippenger_matches_known_answer": pip == known}


def cpu_reference_python(gpu_4096: Optional[dict], msm_logs=(12, 16), ntt_logs=(16, 20)) -> Optional[dict]:
    """The reference's own Python CPU path (crypto/msm/pippenger.py:msm_pippenger with the
    window rule of runtime/kernels/cpu/kernels.py:_msm_g1_impl, crypto/poly/ntt.py:ntt), run
    unmodified from the pip install in baseline/_ref with the py_ecc stand-in, single-threaded
    (it is pure Python), on the same seeds as the GPU arm. The 4096-point result is compared
    with the GPU's. None when the reference is not installed next to the repository."""
    import importlib

    sys.path.insert(0, os.path.join(REPO, "tests"))
    try:
        import reference_env

        reference_env.add_to_path()
        pip = importlib.import_module("crypto.msm.pippenger")
        rntt = importlib.import_module("crypto.poly.ntt")
    except ImportError:
        return None
    from oracle import oracle as O
    from py_ecc import optimized_bn128 as bn
    from pyzkp_gb300 import synth

    out = {"kind": "reference", "cores": 1, "host_cpus": os.cpu_count(),
           "source": "unmodified reference (baseline/_ref) + py_ecc stand-in, one Python thread"}
    msm = {}
    for lg in msm_logs:
        n = 1 << lg
        seed = synth.seed_for(0 if lg == 12 else 2, lg)
        xy = O.g1_fixed_base_mul(O.G1_GENERATOR, synth.base_dlogs(seed, n))
        pts = [(bn.FQ(x), bn.FQ(y), bn.FQ(1)) for x, y in (O.affine_to_ints(row) for row in xy)]
        sc = synth.limbs_to_ints(synth.fr_uniform(seed, n))
        w = max(4, min(16, n.bit_length() - 2))
        t0 = time.perf_counter()
        res = bn.normalize(pip.msm_pippenger(pts, sc, w))
        el = time.perf_counter() - t0
        row = {"Mpts_s": round(n / el / 1e6, 6), "s": round(el, 2), "window_bits": w}
        if lg == 12 and gpu_4096 is not None:
            row["gpu_result_equal"] = [hex(int(res[0])), hex(int(res[1]))] == gpu_4096.get("msm_result")
        msm[f"2^{lg}"] = row
    big = msm.get(f"2^{max(msm_logs)}")
    if big:
        # 2^20 not run: n / (n at the largest size run) times its time, and windows 254/w scaled
        lg = max(msm_logs)
        w20, w_big = 16, big["window_bits"]
        est = big["s"] * (1 << (20 - lg)) * (-(-254 // w20)) / (-(-254 // w_big))
        msm["2^20"] = {"Mpts_s": round((1 << 20) / est / 1e6, 6), "s": round(est, 1),
                       "extrapolated": f"from 2^{lg}: x n, x windows (ceil(254/16) / ceil(254/{w_big}))"}
    nt = {}
    for lg in ntt_logs:
        n = 1 << lg
        v = synth.limbs_to_ints(synth.fr_uniform(synth.seed_for(1, lg), n))
        t0 = time.perf_counter()
        rntt.ntt(v, rntt.omega_for_size(n))
        el = time.perf_counter() - t0
        nt[f"2^{lg}"] = {"Melem_s": round(n / el / 1e6, 4), "s": round(el, 2)}
    out["msm"] = msm
    out["ntt_forward"] = nt
    return out


def cpu_check_g2(row: dict) -> bool:
    """The GPU arm's G2 MSM result against the known answer [sum k_i s_i]G2."""
    from oracle import oracle as O
    from pyzkp_gb300 import synth

    n, seed = row["n"], row["seed"]
    k, s = synth.base_dlogs(seed, n), synth.fr_uniform(seed, n)
    known = synth.limbs_to_ints(O.g2_mul(O.G2_GENERATOR, O.fr_dot(k, s)).reshape(4, 4))
    return row.get("msm_result") == [hex(v) for v in known]


def cpu_baseline(log_n: int, gpu_result) -> dict:
    """CPU baseline leg (rank 0, N=1): the oracle port timed on a bounded sample; it also
    checks the GPU arm's MSM result against the known answer [sum k_i s_i]G."""
    from oracle import oracle as O
    from pyzkp_gb300 import synth

    n = 1 << log_n
    seed = synth.seed_for(2, log_n)
    known = O.affine_to_ints(O.msm_known_answer(synth.base_dlogs(seed, n), synth.fr_uniform(seed, n)))
    mp, runs, el = cpu_msm_sample(log_n, 10.0)
    ne, nruns, nel = cpu_ntt_sample(20, 5.0)
    return {"value": round(mp, 4), "unit": "Mpts/s", "cores": O.num_threads(), "kind": "port",
            "gpu_result_matches_known_answer": (None if gpu_result is None
                                                else [hex(known[0]), hex(known[1])] == gpu_result),
            "sample": f"C restatement of crypto/msm/pippenger.py (window rule w={O.msm_window_rule(1 << log_n)}), "
                      f"full n=2^{log_n} MSM x{runs} in {el:.1f}s on all host threads",
            "ntt": {"value": round(ne, 3), "unit": "Melem/s",
                    "sample": f"C restatement of crypto/poly/ntt.py, forward n=2^20 x{nruns} in {nel:.1f}s"}}


def run_reference(args, ranks: Ranks) -> dict:
    from oracle import oracle as O
    from pyzkp_gb300 import synth

    log_n = args.log_n
    n = 1 << log_n
    seed = synth.seed_for(2, log_n)
    k = synth.base_dlogs(seed, n)
    s = synth.fr_uniform(seed, n)
    bases = O.g1_fixed_base_mul(O.G1_GENERATOR, k)
    w = O.msm_window_rule(n)
    for _ in range(args.warmup):
        O.msm_pippenger(bases, s, w)
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.msm_pippenger(bases, s, w)
        ts.append(time.perf_counter() - t0)
    total = sum(ts)
    value = n * args.steps / total / 1e6
    ne, nruns, nel = cpu_ntt_sample(20, 3.0)
    return {
        "metric": METRIC, "value": round(value, 4), "unit": "Mpts/s", "impl": "reference", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total / args.steps * 1e3, 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64 limbs (exact)",
        "data": "synthetic (same seeds as the gb300 arm)",
        "config": {"workload": f"G1 MSM n=2^{log_n} (uniform scalars) + Fr NTT n=2^20", "n": n, "seed": seed,
                   "window_bits": w},
        "cpu_baseline": {"value": round(value, 4), "unit": "Mpts/s", "cores": O.num_threads(), "kind": "port",
                         "sample": f"full n=2^{log_n} MSM per step, C restatement of crypto/msm/pippenger.py"},
        "e2e": {"value": round(value, 4), "unit": "Mpts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "ntt": {"value": round(ne, 3), "unit": "Melem/s", "sample": f"forward n=2^20 x{nruns} in {nel:.1f}s"},
    }


def main() -> None:
    args = parse()
    if args.warmup < 3:
        args.warmup = 3
    ranks = Ranks(args.gpus)
    try:
        if args.impl == "reference":
            if ranks.rank == 0:
                print(json.dumps(run_reference(args, ranks)), flush=True)
            return
        res = run_gpu(args, ranks)
        if ranks.rank == 0:
            plonk = res.get("plonk_quotient_2_20") or {}
            samples = plonk.pop("_samples", None)
            if ranks.world == 1 and not args.no_cpu_baseline:
                if args.only in ("all", "msm"):
                    res["cpu_baseline"] = cpu_baseline(args.log_n, res.get("msm_result"))
                if res.get("msm_2_12"):
                    res["cpu_baseline"]["msm_2_12"] = cpu_msm_4096(res["msm_2_12"])
                g2 = res.get("msm_g2") or {}
                big = max(g2, key=lambda key: g2[key]["n"]) if g2 else None
                if big and "cpu_baseline" in res:
                    res["cpu_baseline"]["g2_result_matches_known_answer"] = cpu_check_g2(g2[big])
                elif big:
                    res["g2_result_matches_known_answer"] = cpu_check_g2(g2[big])
                if samples is not None:
                    plonk["sampled_check_ok"] = cpu_check_plonk(samples)
                if args.only == "all" and "cpu_baseline" in res:
                    res["cpu_baseline"]["reference_python"] = cpu_reference_python(res.get("msm_2_12"))
                if res.get("groth16_serve") and _SERVE_VERIFY_JOBS:
                    res["groth16_serve"].update(cpu_verify_serve(_SERVE_VERIFY_JOBS))
            print(json.dumps(res), flush=True)
    finally:
        ranks.close()


if __name__ == "__main__":
    main()
