"""The oracle pinned against the reference's own outputs (CPU only).

tests/golden/*.json were produced by running the unmodified reference
(tests/golden/make_golden.py); the C oracle (oracle/bn254_oracle.c) must reproduce
every vector, and its Pippenger must agree with the independent known-answer
identity MSM([k_i]G, s) = [sum k_i s_i]G. The test-only py_ecc stand-in is checked
by curve identities and pairing bilinearity.
"""

import hashlib
import json
import os
import sys

import numpy as np
import pytest

from oracle import oracle as O
from pyzkp_gb300 import synth

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle", "py_ecc_shim"))


def _golden(name):
    with open(os.path.join(HERE, "golden", name)) as f:
        return json.load(f)


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u8").tobytes()).hexdigest()


def _limbs(hexes, w=4):
    return synth.ints_to_limbs([int(v, 16) for v in hexes]).reshape(-1, w)


def test_ntt_fixtures():
    for fx in _golden("ntt_reference.json")["fixtures"]:
        out = O.ntt_op(fx["mode"], _limbs(fx["input"]), fx["n"], int(fx["omega"], 16), int(fx["shift"], 16))
        assert synth.limbs_to_ints(out) == [int(v, 16) for v in fx["output"]], fx["name"]


def test_ntt_seeded_and_pad_truncate():
    g = _golden("ntt_reference.json")
    for rec in g["seeded"]:
        v = synth.fr_uniform(rec["seed"], rec["n"])
        assert _sha(v) == rec["input_sha256"]
        out = O.ntt_op(rec["mode"], v, rec["n"], int(rec["omega"], 16), int(rec["shift"], 16))
        assert _sha(out) == rec["output_sha256"]
        if "output" in rec:
            assert synth.limbs_to_ints(out) == [int(x, 16) for x in rec["output"]]
    for rec in g["pad_truncate"]:
        v = synth.fr_uniform(rec["seed"], rec["in_len"])
        out = O.ntt_op(rec["mode"], v, rec["n"], int(rec["omega"], 16), int(rec["shift"], 16))
        assert _sha(out) == rec["output_sha256"]


def test_omega_for_size_matches_reference_constant():
    # ROOT_2_28 (crypto/poly/ntt.py:8) has order exactly 2^28
    r = O.FR_MODULUS
    assert pow(O.ROOT_2_28, 1 << 28, r) == 1 and pow(O.ROOT_2_28, 1 << 27, r) == r - 1
    assert O.omega_for_size(1) == 1
    with pytest.raises(ValueError):
        O.omega_for_size(12)


def test_msm_cases():
    for case in _golden("msm_reference.json")["cases"]:
        bases = _limbs([c for p in case["bases"] for c in p], 8)
        sc = synth.ints_to_limbs([int(s, 16) for s in case["scalars"]])
        exp = tuple(int(x, 16) for x in case["result"])
        for w in (1, 4, 7, O.msm_window_rule(len(sc)), 16, 20):
            assert O.affine_to_ints(O.msm_pippenger(bases, sc, w)) == exp, (case["name"], w)


def test_msm_workloads_and_known_answer():
    for wl in _golden("msm_reference.json")["workloads"]:
        n, seed = wl["n"], wl["seed"]
        k = synth.base_dlogs(seed, n)
        s = synth.fr_uniform(seed, n) if wl["scalars"] == "uniform" else synth.fr_witness_like(seed, n)
        assert _sha(k) == wl["dlogs_sha256"] and _sha(s) == wl["scalars_sha256"]
        bases = O.g1_fixed_base_mul(O.G1_GENERATOR, k)
        assert _sha(bases) == wl["bases_sha256"]
        exp = tuple(int(x, 16) for x in wl["result"])
        assert O.affine_to_ints(O.msm_pippenger(bases, s, wl["window_bits_reference"])) == exp
        assert O.affine_to_ints(O.msm_known_answer(k, s)) == exp


def test_msm_errors():
    with pytest.raises(ValueError):
        O.msm_pippenger(np.zeros((2, 8), np.uint64), np.zeros((3, 4), np.uint64), 8)
    with pytest.raises(ValueError):
        O.msm_pippenger(np.zeros((2, 8), np.uint64), np.zeros((2, 4), np.uint64), 21)
    assert O.affine_to_ints(O.msm_pippenger(np.zeros((0, 8), np.uint64), np.zeros((0, 4), np.uint64), 8)) == (0, 0)


def test_shim_curve_identities_and_pairing():
    from py_ecc import optimized_bn128 as b

    assert b.is_on_curve(b.G1, b.b) and b.is_on_curve(b.G2, b.b2)
    assert b.is_inf(b.multiply(b.G1, b.curve_order)) and b.is_inf(b.multiply(b.G2, b.curve_order))
    # 2G equals the published alt_bn128 doubling vector (EIP-196 test vectors)
    two = b.normalize(b.double(b.G1))
    assert int(two[0]) == 0x030644E72E131A029B85045B68181585D97816A916871CA8D3C208C16D87CFD3
    e = b.pairing(b.G2, b.G1)
    assert e != b.FQ12.one() and e ** b.curve_order == b.FQ12.one()
    assert b.pairing(b.multiply(b.G2, 3), b.multiply(b.G1, 5)) == e ** 15
    # the oracle's group law agrees with the stand-in's
    p = O.g1_mul(O.G1_GENERATOR, 123456789)
    q = b.normalize(b.multiply(b.G1, 123456789))
    assert O.affine_to_ints(p) == (int(q[0]), int(q[1]))


def test_oracle_g2_matches_shim_and_known_answer():
    """G2 (crypto/ecc/bn254.py g2_mul / g2_add over py_ecc FQ2): the oracle's Jacobian Fq2
    arithmetic agrees with the stand-in, and its MSM_G2 with the dlog identity."""
    from py_ecc import optimized_bn128 as b

    def shim(k):
        p = b.normalize(b.multiply(b.G2, k))
        return (int(p[0].coeffs[0]), int(p[0].coeffs[1])), (int(p[1].coeffs[0]), int(p[1].coeffs[1]))

    for k in (1, 2, 3, 0xDEADBEEF, O.FR_MODULUS - 1, (1 << 250) + 12345):
        assert O.g2_to_ints(O.g2_mul(O.G2_GENERATOR, k)) == shim(k), k
    assert not O.g2_mul(O.G2_GENERATOR, O.FR_MODULUS).any()  # r G2 = infinity
    p5, p7 = O.g2_mul(O.G2_GENERATOR, 5), O.g2_mul(O.G2_GENERATOR, 7)
    assert (O.g2_add(p5, p7) == O.g2_mul(O.G2_GENERATOR, 12)).all()
    assert (O.g2_add(p5, p5) == O.g2_mul(O.G2_GENERATOR, 10)).all()
    assert not O.g2_add(p5, O.g2_mul(O.G2_GENERATOR, O.FR_MODULUS - 5)).any()
    k = synth.base_dlogs(31, 200)
    k[7] = 0
    bases = O.g2_fixed_base_mul(O.G2_GENERATOR, k)
    assert (bases[3] == O.g2_mul(O.G2_GENERATOR, int(synth.limbs_to_ints(k[3:4])[0]))).all()
    assert not bases[7].any()
    s = synth.fr_witness_like(32, 200)
    assert (O.g2_msm(bases, s) == O.g2_msm_known_answer(k, s)).all()


PLONK_INPUTS = 15


def plonk_quotient_case_inputs(rec):
    """The 15 input vectors and the attrs of a ``plonk_reference.json`` quotient record."""
    m = rec["m"]
    vecs = [synth.limbs_to_ints(synth.fr_uniform(rec["seed"] + j, m)) for j in range(PLONK_INPUTS)]
    attrs = {k: (v if isinstance(v, int) else int(v, 16)) for k, v in rec["attrs"].items()}
    return vecs, attrs


def _fr_sha(vals):
    return hashlib.sha256(b"".join(int(v).to_bytes(32, "little") for v in vals)).hexdigest()


def test_plonk_quotient_oracle_matches_reference_golden():
    """oracle/oracle.py's restatement of _plonk_t_quotient_evals (runtime/kernels/cpu/kernels.py:607-693)
    reproduces the reference's own outputs (tests/golden/make_plonk_golden.py)."""
    for rec in _golden("plonk_reference.json")["quotient"]:
        vecs, a = plonk_quotient_case_inputs(rec)
        num, zh = O.plonk_t_quotient_evals(vecs, a["n"], a["omega_m"], a["shift"], a["shift_n"], a["alpha"],
                                           a["beta"], a["gamma"], a["k1"], a["k2"])
        assert _fr_sha(num) == rec["num_sha256"], rec["m"]
        assert _fr_sha(zh) == rec["zh_sha256"], rec["m"]
        for i, v in rec["num_at"].items():
            assert num[int(i)] == int(v, 16)
