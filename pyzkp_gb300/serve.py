"""Continuous batching of Groth16 proof requests on one GPU.

The reference proves one witness at a time (protocols/groth16/prove.py:30-126), or a list
of witnesses for one key in sequence (prove_batch, :133-246). A serving process instead
sees requests arrive over time, for many circuits. ProverService runs the arrival trace
on the wall clock and, whenever the GPU is free, admits every request that has arrived,
oldest first, while the batch's estimated device memory stays under a budget, then proves
the admitted requests together (groth16.Prover.prove_batch: one batched NTT call per
QAP stage, one batched G1 MSM call and one G2 MSM call for all of them). A request's
latency is its completion time minus its arrival time. The same trace run with batches
of one is the plain (sequential) baseline; a request's proof does not depend on what it
was batched with.
"""

from __future__ import annotations

import statistics
import time
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import groth16 as G


@dataclass
class Arrival:
    t: float  # seconds after the start of the trace
    key_id: int
    r: int
    s: int


@dataclass
class TraceResult:
    proofs: List[Optional[G.Proof]]
    latency_s: List[float]
    makespan_s: float
    batches: List[int] = field(default_factory=list)

    def summary(self) -> dict:
        lat = sorted(self.latency_s)

        def pct(p):
            if not lat:
                return None
            k = min(len(lat) - 1, max(0, int(round(p / 100.0 * (len(lat) - 1)))))
            return lat[k]

        return {
            "requests": len(self.latency_s),
            "proofs_per_s": round(len(self.latency_s) / self.makespan_s, 2) if self.makespan_s > 0 else None,
            "p50_ms": round(pct(50) * 1e3, 2) if lat else None,
            "p99_ms": round(pct(99) * 1e3, 2) if lat else None,
            "mean_ms": round(statistics.mean(lat) * 1e3, 2) if lat else None,
            "batches": len(self.batches),
            "mean_batch": round(statistics.mean(self.batches), 2) if self.batches else None,
            "max_batch": max(self.batches) if self.batches else None,
        }


def poisson_trace(rate_per_s: float, count: int, key_ids: Sequence[int], seed: int,
                  weights: Optional[Sequence[float]] = None) -> List[Arrival]:
    """`count` arrivals with exponential gaps of mean 1 / rate; key and (r, s) seeded."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_per_s, size=count)
    times = np.cumsum(gaps) - gaps[0]
    p = None if weights is None else np.asarray(weights, dtype=float) / float(np.sum(weights))
    keys = rng.choice(np.asarray(key_ids), size=count, p=p)
    rs = rng.integers(1, 1 << 62, size=(count, 2))
    return [Arrival(float(t), int(k), int(a), int(b)) for t, k, (a, b) in zip(times, keys, rs)]


class ProverService:
    """Batches proof requests for resident keys under a device-memory budget."""

    def __init__(self, prover: G.Prover, keys: dict, witnesses: dict, budget_bytes: int = 32 << 30,
                 max_batch: int = 64) -> None:
        self.prover = prover
        self.keys = keys
        self.witnesses = witnesses
        self.budget = int(budget_bytes)
        self.max_batch = int(max_batch)

    @staticmethod
    def request_bytes(key: G.DeviceKey) -> int:
        """Device memory one request holds during its batch: the witness, the three QAP
        vectors, the gathered MSM scalars, and the MSM pipeline scratch (about 12 bytes per
        CSR entry at 16 windows, plus its share of the buckets)."""
        n, nv = key.n, key.r1cs.n_vars
        scalars = key.a.count + key.b1.count + key.l.count + key.h.count
        vectors = 32 * (nv + 3 * n + key.a.count + key.b1.count + key.l.count)
        msm = scalars * 16 * 12 + key.b2.count * 16 * 12
        return vectors + msm + (64 << 20)

    def run(self, trace: Sequence[Arrival], batched: bool = True) -> TraceResult:
        n = len(trace)
        order = sorted(range(n), key=lambda i: trace[i].t)
        proofs: List[Optional[G.Proof]] = [None] * n
        done = [0.0] * n
        batches: List[int] = []
        nxt = 0
        t0 = time.perf_counter()
        while nxt < n:
            now = time.perf_counter() - t0
            if trace[order[nxt]].t > now:
                time.sleep(min(trace[order[nxt]].t - now, 0.01))
                continue
            # admit every arrived request, oldest first, within the memory budget
            take, used = [], 0
            cap = self.max_batch if batched else 1
            while nxt < n and len(take) < cap and trace[order[nxt]].t <= now:
                need = self.request_bytes(self.keys[trace[order[nxt]].key_id])
                if take and used + need > self.budget:
                    break
                take.append(order[nxt])
                used += need
                nxt += 1
            reqs = [G.Request(self.keys[trace[i].key_id], self.witnesses[trace[i].key_id], trace[i].r, trace[i].s)
                    for i in take]
            out = self.prover.prove_batch(reqs)
            t_done = time.perf_counter() - t0
            for i, p in zip(take, out):
                proofs[i] = p
                done[i] = t_done
            batches.append(len(take))
        makespan = max(done) - min(a.t for a in trace) if n else 0.0
        return TraceResult(proofs, [done[i] - trace[i].t for i in range(n)], makespan, batches)
