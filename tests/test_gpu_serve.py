"""Continuous batching on the GPU (pyzkp_gb300.serve): a request admitted while a large one
is in flight completes first, with the same proof it gets alone; every mode gives the same
proofs; a bad witness fails only its own request."""

import pytest

from pyzkp_gb300 import groth16 as G
from pyzkp_gb300 import serve

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def service(gpu_ctx):
    sizes = {0: 1 << 18, 1: 1 << 10, 2: 3000}
    keys, wits, pubs = {}, {}, {}
    for k, m in sizes.items():
        keys[k] = G.setup(gpu_ctx, G.diagonal_r1cs(m), G.Trapdoors.seeded(0x5E0 + k))
        wits[k], pubs[k] = G.diagonal_witness(gpu_ctx, m, 0xB0B + k)
    svc = serve.ProverService(G.Prover(gpu_ctx), keys, wits, budget_bytes=16 << 30, max_batch=16, slots=3,
                              small_constraints=1 << 14)
    svc.warm()
    yield svc, wits, pubs
    svc.close()


def test_request_admitted_mid_flight_finishes_first_with_its_solo_proof(service):
    svc, _, _ = service
    trace = [serve.Arrival(0.0, 0, 11, 12), serve.Arrival(0.001, 1, 13, 14)]
    solo = [svc.prover.prove(svc.keys[a.key_id], svc.witnesses[a.key_id], a.r, a.s) for a in trace]
    res = svc.run(trace, "continuous")
    assert res.errors == [None, None]
    assert res.proofs == solo
    small_done, large_done = trace[1].t + res.latency_s[1], trace[0].t + res.latency_s[0]
    assert small_done < large_done, (small_done, large_done)
    # batch at a time, the small request waits for the large batch to finish
    res_b = svc.run(trace, "batch")
    assert res_b.proofs == solo
    assert trace[1].t + res_b.latency_s[1] > trace[0].t + res_b.latency_s[0]


def test_all_modes_give_the_same_proofs_and_proofs_verify(service):
    svc, _, pubs = service
    trace = serve.poisson_trace(400.0, 24, list(svc.keys), seed=7, weights=[0.2, 1.0, 1.0])
    out = {m: svc.run(trace, m) for m in ("continuous", "batch", "plain")}
    for m, r in out.items():
        assert all(e is None for e in r.errors), m
    assert out["continuous"].proofs == out["plain"].proofs == out["batch"].proofs
    # two of them through the reference's verification equation (oracle/groth16_verify.py)
    from oracle import groth16_verify as V

    for a, p in list(zip(trace, out["continuous"].proofs))[:2]:
        k = svc.keys[a.key_id]
        v = V.Groth16Verifier(k.vk.alpha_g1, k.vk.beta_g2, k.vk.gamma_g2, k.vk.delta_g2, k.vk.ic)
        assert v.verify(pubs[a.key_id], p.a, p.b, p.c)


def test_bad_witness_fails_only_its_request_in_a_group(service):
    svc, wits, _ = service
    bad = wits[2].copy()
    bad[5, 0] ^= 1  # x_4 changes, z_4 does not: constraint 4 fails
    trace = [serve.Arrival(0.0, 2, 1, 2), serve.Arrival(0.0, 2, 3, 4, witness=G.pin_witness(bad)),
             serve.Arrival(0.0, 1, 5, 6)]
    res = svc.run(trace, "continuous")
    assert isinstance(res.errors[1], ValueError) and res.proofs[1] is None
    assert res.errors[0] is None and res.errors[2] is None
    assert res.proofs[0] == svc.prover.prove(svc.keys[2], wits[2], 1, 2)
