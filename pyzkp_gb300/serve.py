"""Continuous batching of Groth16 proof requests on one GPU.

The reference proves one witness at a time (protocols/groth16/prove.py:30-126), or a list
of witnesses for one key in sequence (prove_batch, :133-246). A serving process instead
sees requests arrive over time, for many circuits. ``ProverService.run`` replays an
arrival trace on the wall clock in one of three modes:

* ``"continuous"`` -- continuous batching. The GPU is shared by ``slots`` contexts, each
  with its own CUDA streams; slot 0 has the most urgent stream priority and takes only
  small requests (at most ``small_constraints`` constraints), the others take any. Whenever
  a slot is free, the requests that have arrived are admitted, oldest first, while the
  device memory of everything in flight stays under the budget, and their device work is
  enqueued at once (``groth16.Prover.submit``: nothing waits for the device). Requests
  that arrive while others are on the GPU are admitted as slots and memory free up; their
  kernels overlap the earlier ones' on the device, and a small request does not wait for
  a large batch to finish. A group retires when its own device work is done; its proofs
  are assembled on host threads while the loop goes on.
* ``"batch"`` -- batch at a time: everything that has arrived is proved together, and the
  next batch starts when the previous one has finished (the earlier design, kept as a
  comparison).
* ``"plain"`` -- one request at a time, synchronously (the reference's shape).

Failures stay with their request: an unsatisfied witness, a bad argument, a request larger
than the whole memory budget (rejected at admission) or a cancelled request (``cancel_at``
in its arrival: dropped if it has not been admitted by then, its result discarded if it
has) gives that request an error and the loop goes on. A request's latency is its
completion time minus its arrival time; its proof does not depend on what it was batched
with or which slot ran it.
"""

from __future__ import annotations

import collections
import statistics
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import _native as N
from . import groth16 as G


@dataclass
class Arrival:
    t: float  # seconds after the start of the trace
    key_id: int
    r: int
    s: int
    witness: Optional[np.ndarray] = None  # default: the service's witness of key_id
    cancel_at: Optional[float] = None     # seconds after the start: cancel the request then


class Cancelled(Exception):
    """The request was cancelled before its proof was delivered."""


@dataclass
class TraceResult:
    proofs: List[Optional[G.Proof]]
    errors: List[Optional[Exception]]
    latency_s: List[float]
    makespan_s: float
    batches: List[int] = field(default_factory=list)
    mode: str = ""

    def summary(self) -> dict:
        ok = [lat for lat, p in zip(self.latency_s, self.proofs) if p is not None]
        lat = sorted(ok)

        def pct(p):
            k = min(len(lat) - 1, max(0, int(round(p / 100.0 * (len(lat) - 1)))))
            return lat[k]

        return {
            "mode": self.mode,
            "requests": len(self.latency_s),
            "proved": len(ok),
            "failed": sum(1 for e in self.errors if e is not None),
            "proofs_per_s": round(len(ok) / self.makespan_s, 2) if self.makespan_s > 0 else None,
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


@dataclass
class _Group:
    slot: int
    pending: G.PendingProofs
    members: List[int]
    nbytes: int


class ProverService:
    """Proves arrival traces for resident keys under a device-memory budget (module docstring)."""

    def __init__(self, prover: G.Prover, keys: dict, witnesses: dict, budget_bytes: int = 32 << 30,
                 max_batch: int = 24, slots: int = 3, small_constraints: int = 1 << 14,
                 contexts: Optional[list] = None, pin_witnesses: bool = True) -> None:
        """``contexts``: the slot contexts to use (default: created on first use, slot 0 at the
        most urgent stream priority); ``pin_witnesses``: keep page-locked copies of the
        witnesses so that uploads do not wait for the device."""
        if contexts is not None:
            slots = len(contexts)
        if slots < 2:
            raise ValueError("continuous batching needs at least 2 slots (one urgent, one general)")
        self.prover = prover
        self.keys = keys
        self.witnesses = {k: G.pin_witness(w) for k, w in witnesses.items()} if pin_witnesses else dict(witnesses)
        self.budget = int(budget_bytes)
        self.max_batch = int(max_batch)
        self.nslots = int(slots)
        self.small = int(small_constraints)
        self._contexts: Optional[list] = list(contexts) if contexts is not None else None
        self._own_contexts = contexts is None
        self._finisher = ThreadPoolExecutor(max_workers=2, thread_name_prefix="zk-proof-assembly")

    # -- resources ------------------------------------------------------------------------
    def contexts(self) -> List[N.Context]:
        """Slot contexts on the prover's device: slot 0 at the most urgent stream priority."""
        if self._contexts is None:
            least, greatest = N.stream_priority_range()
            dev = self.prover.ctx.device
            self._contexts = [N.Context(dev, priority=greatest)] + \
                [N.Context(dev, priority=least) for _ in range(self.nslots - 1)]
        return self._contexts

    @staticmethod
    def request_bytes(key: G.DeviceKey) -> int:
        """Device memory one request holds while in flight: the witness, the three QAP
        vectors, the gathered MSM scalars, and the MSM pipeline scratch (about 12 bytes per
        CSR entry at 16 windows, plus its share of the buckets)."""
        n, nv = key.n, key.r1cs.n_vars
        scalars = key.a.count + key.b1.count + key.l.count + key.h.count
        vectors = 32 * (nv + 3 * n + key.a.count + key.b1.count + key.l.count)
        msm = scalars * 16 * 12 + key.b2.count * 16 * 12
        return vectors + msm + (64 << 20)

    def warm(self) -> None:
        """Prove every key once on every slot context and once one at a time (untimed):
        builds each context's NTT tables and memory pools before a measured run."""
        reqs = [G.Request(self.keys[k], self.witnesses[k], 1, 1) for k in self.keys]
        for c in self.contexts():
            self.prover.submit(reqs, ctx=c).results()
        for q in reqs:
            self.prover.submit([q]).results()

    def _request(self, a: Arrival) -> G.Request:
        w = a.witness if a.witness is not None else self.witnesses[a.key_id]
        return G.Request(self.keys[a.key_id], w, a.r, a.s)

    # -- trace replay -----------------------------------------------------------------------
    def run(self, trace: Sequence[Arrival], mode: str = "continuous") -> TraceResult:
        if mode == "continuous":
            return self._run_continuous(trace)
        if mode in ("batch", "plain"):
            return self._run_blocking(trace, batched=(mode == "batch"))
        raise ValueError(f"unknown mode {mode!r}")

    def _run_blocking(self, trace: Sequence[Arrival], batched: bool) -> TraceResult:
        n = len(trace)
        order = sorted(range(n), key=lambda i: trace[i].t)
        proofs: List[Optional[G.Proof]] = [None] * n
        errors: List[Optional[Exception]] = [None] * n
        done = [0.0] * n
        batches: List[int] = []
        nxt = 0
        t0 = time.perf_counter()
        while nxt < n:
            now = time.perf_counter() - t0
            if trace[order[nxt]].t > now:
                time.sleep(min(trace[order[nxt]].t - now, 0.002))
                continue
            take, used = [], 0
            cap = self.max_batch if batched else 1
            while nxt < n and len(take) < cap and trace[order[nxt]].t <= now:
                i = order[nxt]
                need = self.request_bytes(self.keys[trace[i].key_id])
                if need > self.budget:
                    errors[i] = MemoryError("request needs more device memory than the whole budget")
                    done[i] = now
                    nxt += 1
                    continue
                if take and used + need > self.budget:
                    break
                take.append(i)
                used += need
                nxt += 1
            if not take:
                continue
            try:
                res = self.prover.submit([self._request(trace[i]) for i in take]).results()
            except Exception as e:  # noqa: BLE001 -- a host failure fails this batch only
                res = [e] * len(take)
            t_done = time.perf_counter() - t0
            for i, p in zip(take, res):
                if isinstance(p, Exception):
                    errors[i] = p
                else:
                    proofs[i] = p
                done[i] = t_done
            batches.append(len(take))
        makespan = max(done) - min(a.t for a in trace) if n else 0.0
        return TraceResult(proofs, errors, [done[i] - trace[i].t for i in range(n)], makespan, batches,
                           "batch" if batched else "plain")

    def _run_continuous(self, trace: Sequence[Arrival]) -> TraceResult:
        ctxs = self.contexts()
        n = len(trace)
        order = sorted(range(n), key=lambda i: trace[i].t)
        proofs: List[Optional[G.Proof]] = [None] * n
        errors: List[Optional[Exception]] = [None] * n
        done: List[Optional[float]] = [None] * n
        batches: List[int] = []
        lock = threading.Lock()
        pending: collections.deque = collections.deque()
        inflight: List[_Group] = []
        free = list(range(len(ctxs)))
        used = 0
        nxt = 0
        t0 = time.perf_counter()
        clock = lambda: time.perf_counter() - t0  # noqa: E731

        def finish(i: int, proof, err) -> None:
            with lock:
                if done[i] is not None:
                    return
                if err is None and trace[i].cancel_at is not None and trace[i].cancel_at <= clock():
                    err, proof = Cancelled("cancelled while in flight"), None
                proofs[i], errors[i] = proof, err
                done[i] = clock()

        def assemble(g: _Group) -> None:
            try:
                res = g.pending.finish_host()
            except Exception as e:  # noqa: BLE001
                res = [e] * len(g.members)
            for i, p in zip(g.members, res):
                finish(i, None if isinstance(p, Exception) else p, p if isinstance(p, Exception) else None)

        futures = []
        while True:
            with lock:
                if all(d is not None for d in done):
                    break
            now = clock()
            busy = False
            while nxt < n and trace[order[nxt]].t <= now:
                pending.append(order[nxt])
                nxt += 1
            # cancellations of requests not admitted yet
            if any(trace[i].cancel_at is not None for i in pending):
                keep = collections.deque()
                for i in pending:
                    if trace[i].cancel_at is not None and trace[i].cancel_at <= now:
                        finish(i, None, Cancelled("cancelled before admission"))
                    else:
                        keep.append(i)
                pending = keep
            # retire the groups whose device work is done; assemble their proofs off this thread
            for g in list(inflight):
                if g.pending.done():
                    try:
                        g.pending.finish_device()
                    except Exception as e:  # noqa: BLE001 -- a device failure fails this group only
                        for i in g.members:
                            finish(i, None, e)
                    else:
                        futures.append(self._finisher.submit(assemble, g))
                    inflight.remove(g)
                    free.append(g.slot)
                    used -= g.nbytes
                    busy = True
            # admit: the urgent slot takes small requests, the others any, oldest first
            while pending and free:
                head = pending[0]
                if self.request_bytes(self.keys[trace[head].key_id]) > self.budget:
                    pending.popleft()
                    finish(head, None, MemoryError("request needs more device memory than the whole budget"))
                    continue
                small_head = self.keys[trace[head].key_id].r1cs.n <= self.small
                if 0 in free and (small_head or len(free) == 1):
                    slot = 0
                elif any(s != 0 for s in free):
                    slot = next(s for s in free if s != 0)
                else:
                    break
                take, nbytes = [], 0
                rest = collections.deque()
                while pending and len(take) < self.max_batch:
                    i = pending.popleft()
                    key = self.keys[trace[i].key_id]
                    need = self.request_bytes(key)
                    if (slot == 0 and key.r1cs.n > self.small) or used + nbytes + need > self.budget:
                        rest.append(i)
                        if used + nbytes + need > self.budget and slot != 0:
                            break  # oldest first on the general slots: stop at the first that does not fit
                        continue
                    take.append(i)
                    nbytes += need
                pending = rest + pending
                if not take:
                    break
                free.remove(slot)
                try:
                    pp = self.prover.submit([self._request(trace[i]) for i in take], ctx=ctxs[slot])
                except Exception as e:  # noqa: BLE001 -- a host failure fails this group only
                    for i in take:
                        finish(i, None, e)
                    free.append(slot)
                    continue
                inflight.append(_Group(slot, pp, take, nbytes))
                used += nbytes
                batches.append(len(take))
                busy = True
            if not busy:
                wait = 0.0002
                if nxt < n and not inflight:
                    wait = max(0.0, min(trace[order[nxt]].t - clock(), 0.002))
                time.sleep(wait)
        for f in futures:
            f.result()
        t_end = [d for d in done if d is not None]
        makespan = max(t_end) - min(a.t for a in trace) if n else 0.0
        return TraceResult(proofs, errors, [done[i] - trace[i].t for i in range(n)], makespan, batches, "continuous")

    def close(self) -> None:
        self._finisher.shutdown(wait=True)
        if self._contexts and self._own_contexts:
            for c in self._contexts:
                c.close()
        self._contexts = None
