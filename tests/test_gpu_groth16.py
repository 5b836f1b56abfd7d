"""GPU parity of the Groth16 prover (pyzkp_gb300.groth16) through the C ABI.

Pinned three ways:
  * against the reference itself: tests/golden/groth16_reference.json holds the proving
    key and proof that the unmodified reference's setup / prove produced
    (make_groth16_golden.py, seeded trapdoors and r, s); the device setup must rebuild every
    key point and the device prover the proof, bit for bit;
  * by the pairing equation of verify.py:11-23, through the py_ecc stand-in;
  * by exponents: with the trapdoors known, A = [alpha + sum w_i A_i(tau) + r delta] G1 and
    likewise B and C, computed with plain integers (an independent check at 2^16).
"""

import json
import os
import sys

import numpy as np
import pytest

from pyzkp_gb300 import groth16 as G
from pyzkp_gb300 import synth

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
R = synth.FR_MODULUS


def _golden():
    with open(os.path.join(HERE, "golden", "groth16_reference.json")) as f:
        return json.load(f)["circuits"]


def _h(v):
    return int(v, 16)


def _g1(p):
    return None if p is None else (_h(p[0]), _h(p[1]))


def _g2(p):
    return None if p is None else ((_h(p[0][0]), _h(p[0][1])), (_h(p[1][0]), _h(p[1][1])))


def _r1cs(c):
    rows = lambda m: [{int(k): _h(v) for k, v in row} for row in m]  # noqa: E731
    return G.R1CS.from_rows(c["n"], c["n_vars"], c["one_id"], c["public_ids"], c["aux_ids"], rows(c["a_rows"]),
                            rows(c["b_rows"]), rows(c["c_rows"]))


def _td(c):
    t = c["trapdoors"]
    return G.Trapdoors(*[_h(t[k]) for k in ("tau", "alpha", "beta", "gamma", "delta")])


def test_setup_and_prove_match_reference(gpu_ctx):
    for c in _golden():
        key = G.setup(gpu_ctx, _r1cs(c), _td(c), keep_exponents=True)
        pk = c["pk"]
        pts = G.query_points(gpu_ctx, key)
        for name in ("a_query", "b_query_g1", "h_query", "l_query"):
            assert pts[name] == [_g1(p) for p in pk[name]], (c["name"], name)
        assert pts["b_query_g2"] == [_g2(p) for p in pk["b_query_g2"]], c["name"]
        assert key.vk.alpha_g1 == _g1(pk["alpha_g1"]) and key.beta_g1 == _g1(pk["beta_g1"])
        assert key.delta_g1 == _g1(pk["delta_g1"])
        assert key.vk.beta_g2 == _g2(pk["beta_g2"]) and key.vk.gamma_g2 == _g2(pk["gamma_g2"])
        assert key.vk.delta_g2 == _g2(pk["delta_g2"])
        assert key.vk.ic == [_g1(p) for p in pk["ic"]], c["name"]
        w = synth.ints_to_limbs([_h(v) for v in c["witness"]])
        proof = G.Prover(gpu_ctx).prove(key, w, _h(c["r"]), _h(c["s"]))
        assert proof.a == _g1(c["proof"]["a"]), c["name"]
        assert proof.b == _g2(c["proof"]["b"]), c["name"]
        assert proof.c == _g1(c["proof"]["c"]), c["name"]


def _shim():
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle", "py_ecc_shim"))
    from py_ecc import optimized_bn128 as b

    return b


def _verify(vk, public_values, proof) -> bool:
    """verify.py:11-23 with the stand-in's pairing."""
    b = _shim()

    def p1(p):
        return b.Z1 if p is None else (b.FQ(p[0]), b.FQ(p[1]), b.FQ(1))

    def p2(p):
        return b.Z2 if p is None else (b.FQ2(list(p[0])), b.FQ2(list(p[1])), b.FQ2.one())

    vk_x = b.Z1
    for s, pt in zip(public_values, vk.ic):
        vk_x = b.add(vk_x, b.multiply(p1(pt), s % R))
    left = b.pairing(p2(proof.b), p1(proof.a))
    right = b.pairing(p2(vk.beta_g2), p1(vk.alpha_g1))
    right = right * b.pairing(p2(vk.gamma_g2), vk_x)
    right = right * b.pairing(p2(vk.delta_g2), p1(proof.c))
    return left == right


def test_diagonal_proof_verifies_and_wrong_public_fails(gpu_ctx):
    m = 37
    key = G.setup(gpu_ctx, G.diagonal_r1cs(m), G.Trapdoors.seeded(11))
    w, pub = G.diagonal_witness(gpu_ctx, m, 12)
    proof = G.Prover(gpu_ctx).prove(key, w, 123456789, 987654321)
    assert _verify(key.vk, pub, proof)
    assert not _verify(key.vk, [1, (pub[1] + 1) % R], proof)


def test_batch_equals_alone_and_unsatisfied_witness(gpu_ctx):
    prover = G.Prover(gpu_ctx)
    reqs = []
    for j, m in enumerate((1, 5, 64, 1000, 3000)):
        key = G.setup(gpu_ctx, G.diagonal_r1cs(m), G.Trapdoors.seeded(100 + j))
        w, _ = G.diagonal_witness(gpu_ctx, m, 200 + j)
        reqs.append(G.Request(key, w, 1000 + j, 2000 + j))
    for c in _golden():
        key = G.setup(gpu_ctx, _r1cs(c), _td(c))
        reqs.append(G.Request(key, synth.ints_to_limbs([_h(v) for v in c["witness"]]), _h(c["r"]), _h(c["s"])))
    together = prover.prove_batch(reqs)
    alone = [prover.prove(q.key, q.witness, q.r, q.s) for q in reqs]
    assert together == alone
    assert together[-1].a == _g1(_golden()[-1]["proof"]["a"])
    bad = reqs[3].witness.copy()
    bad[5, 0] ^= 1  # x_4 changes, z_4 does not: constraint 4 fails
    with pytest.raises(ValueError):
        prover.prove(reqs[3].key, bad, 1, 2)
    with pytest.raises(ValueError):
        prover.prove(reqs[3].key, bad[:-1], 1, 2)


def test_large_diagonal_proof_by_exponents(gpu_ctx):
    """2^16 constraints: every proof element equals [its exponent] G from the trapdoors."""
    from pyzkp_gb300 import _native as N

    m = 1 << 16
    td = G.Trapdoors.seeded(77)
    r1 = G.diagonal_r1cs(m)
    key = G.setup(gpu_ctx, r1, td, keep_exponents=True)
    w, _ = G.diagonal_witness(gpu_ctx, m, 78)
    rr, ss = 31337, 271828
    proof = G.Prover(gpu_ctx).prove(key, w, rr, ss)
    wv = synth.limbs_to_ints(w)
    ua = synth.limbs_to_ints(key.exps["a"])
    ub = synth.limbs_to_ints(key.exps["b"])
    # diagonal circuit: u^C of z_i is L_i(tau) = u^A of x_i
    n, x0, y0 = r1.n, 1, 1 + m
    a_tau = sum(wv[i] * ua[i] for i in range(len(wv))) % R
    b_tau = sum(wv[i] * ub[i] for i in range(len(wv))) % R
    c_tau = sum(wv[x0 + i] * wv[y0 + i] % R * ua[x0 + i] for i in range(m)) % R  # z_i L_i
    l_sum = sum(wv[i] * v for i, v in zip(r1.aux_ids, synth.limbs_to_ints(key.exps["l"]))) % R
    a_exp = (td.alpha + a_tau + rr * td.delta) % R
    b_exp = (td.beta + b_tau + ss * td.delta) % R
    inv_d = pow(td.delta, R - 2, R)
    c_exp = (l_sum + (a_tau * b_tau - c_tau) * inv_d + ss * a_exp + rr * b_exp - rr * ss * td.delta) % R
    assert n == m
    assert proof.a == N.host_g1_mul(G.G1_GEN, a_exp)
    assert proof.b == N.host_g2_mul(G.G2_GEN, b_exp)
    assert proof.c == N.host_g1_mul(G.G1_GEN, c_exp)
