"""The serving loop's scheduling and failure handling on the CPU (pyzkp_gb300.serve).

A fake prover stands in for the GPU: ``submit`` returns at once and its batch "finishes"
after a wall-clock delay proportional to its work, like the device queue; a witness marked
bad fails only its own request, and a marked key makes ``submit`` itself raise (a host
failure). Nothing here touches a GPU.
"""

import time
from types import SimpleNamespace

import pytest

from pyzkp_gb300 import serve

MB = 1 << 20


def _key(n, kid):
    q = SimpleNamespace(count=n)
    return SimpleNamespace(n=n, r1cs=SimpleNamespace(n=n, n_vars=3 * n + 1), a=q, b1=q, l=q, h=q, b2=q, kid=kid)


class _Pending:
    def __init__(self, reqs, seconds, log):
        self.reqs, self.t_done, self.log = reqs, time.perf_counter() + seconds, log
        self.device_done = False

    def __len__(self):
        return len(self.reqs)

    def done(self):
        return time.perf_counter() >= self.t_done

    def finish_device(self):
        while not self.done():
            time.sleep(0.0002)
        self.device_done = True

    def finish_host(self):
        assert self.device_done
        out = []
        for q in self.reqs:
            if q.witness == "bad":
                out.append(ValueError("witness does not satisfy R1CS (non-zero remainder)"))
            else:
                out.append(("proof", q.key.kid, q.r, q.s))
        return out

    def results(self):
        self.finish_device()
        return self.finish_host()


class _FakeProver:
    """submit(reqs, ctx) -> a batch done after 20 us per 1000 constraints (+ 0.5 ms)."""

    def __init__(self):
        self.ctx = SimpleNamespace(device=0)
        self.log = []

    def submit(self, reqs, ctx=None):
        if any(q.key.kid == "explode" for q in reqs):
            raise RuntimeError("host failure while enqueueing")
        self.log.append((ctx, [q.key.kid for q in reqs], time.perf_counter()))
        work = sum(q.key.n for q in reqs)
        return _Pending(reqs, 0.0005 + 20e-6 * work / 1000, self.log)


def _service(keys, budget=1 << 40, slots=3):
    wits = {k: "ok" for k in keys}
    ctxs = [f"slot{i}" for i in range(slots)]
    return serve.ProverService(_FakeProver(), keys, wits, budget_bytes=budget, max_batch=8, contexts=ctxs,
                               pin_witnesses=False, small_constraints=1 << 12)


def test_continuous_admits_mid_flight_and_small_requests_finish_first():
    keys = {0: _key(1 << 20, 0), 1: _key(1 << 10, 1)}  # ~21 ms and ~0.5 ms of fake device time
    svc = _service(keys)
    trace = [serve.Arrival(0.0, 0, 1, 2), serve.Arrival(0.003, 1, 3, 4)]
    res = svc.run(trace, "continuous")
    assert res.errors == [None, None]
    # the small request was admitted while the large one was in flight, on the urgent slot
    ctx_of = {kids[0]: ctx for ctx, kids, _ in svc.prover.log}
    assert ctx_of[0] != "slot0" and ctx_of[1] == "slot0"
    assert res.latency_s[1] + trace[1].t < res.latency_s[0]  # done before the large one
    # batch at a time: it waits for the large batch
    res_b = svc.run(trace, "batch")
    assert res_b.latency_s[1] + trace[1].t > res_b.latency_s[0]
    assert res.proofs == res_b.proofs == [("proof", 0, 1, 2), ("proof", 1, 3, 4)]
    svc.close()


def test_one_bad_witness_fails_only_its_request():
    keys = {0: _key(1000, 0)}
    svc = _service(keys)
    trace = [serve.Arrival(0.0, 0, i, i + 1) for i in range(5)]
    trace[2].witness = "bad"
    for mode in ("continuous", "batch", "plain"):
        res = svc.run(trace, mode)
        assert isinstance(res.errors[2], ValueError), mode
        assert [e is None for e in res.errors] == [True, True, False, True, True], mode
        assert res.proofs[2] is None and all(res.proofs[i] == ("proof", 0, i, i + 1) for i in (0, 1, 3, 4))
        assert res.summary()["failed"] == 1 and res.summary()["proved"] == 4
    svc.close()


def test_host_exception_fails_its_group_and_the_loop_goes_on():
    keys = {0: _key(1000, 0), 1: _key(1000, "explode")}
    svc = _service(keys)
    trace = [serve.Arrival(0.0, 1, 1, 1), serve.Arrival(0.002, 0, 2, 2), serve.Arrival(0.004, 0, 3, 3)]
    for mode in ("continuous", "batch", "plain"):
        res = svc.run(trace, mode)
        assert isinstance(res.errors[0], RuntimeError), mode
        assert res.proofs[1:] == [("proof", 0, 2, 2), ("proof", 0, 3, 3)], mode
    svc.close()


def test_request_larger_than_the_budget_is_rejected_not_admitted():
    keys = {0: _key(1000, 0), 1: _key(1 << 22, 1)}
    need_small = serve.ProverService.request_bytes(keys[0])
    svc = _service(keys, budget=need_small * 3)
    trace = [serve.Arrival(0.0, 1, 1, 1)] + [serve.Arrival(0.001 * i, 0, i, i) for i in range(1, 6)]
    for mode in ("continuous", "batch"):
        res = svc.run(trace, mode)
        assert isinstance(res.errors[0], MemoryError), mode
        assert all(res.proofs[i] == ("proof", 0, i, i) for i in range(1, 6)), mode
    # in flight, the budget holds at most 3 of the small requests at once
    res = svc.run([serve.Arrival(0.0, 0, i, i) for i in range(9)], "continuous")
    assert all(e is None for e in res.errors) and max(res.batches) <= 3
    svc.close()


def test_cancellation_before_and_during_flight():
    keys = {0: _key(1 << 20, 0), 1: _key(1000, 1)}
    svc = _service(keys, slots=2)
    trace = [serve.Arrival(0.0, 0, 1, 1, cancel_at=0.005),  # in flight (~21 ms) when cancelled
             serve.Arrival(0.0, 0, 2, 2, cancel_at=0.001),  # waits for the general slot: cancelled first
             serve.Arrival(0.001, 1, 3, 3)]
    svc.max_batch = 1
    res = svc.run(trace, "continuous")
    assert isinstance(res.errors[0], serve.Cancelled) and isinstance(res.errors[1], serve.Cancelled)
    assert res.proofs[2] == ("proof", 1, 3, 3)
    kids = [k for _, ks, _ in svc.prover.log for k in ks]
    assert kids.count(0) == 1  # the second large request never reached the device
    svc.close()


def test_service_needs_two_slots():
    with pytest.raises(ValueError):
        serve.ProverService(_FakeProver(), {}, {}, contexts=["only"], pin_witnesses=False)
