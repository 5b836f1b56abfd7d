"""CPU tests of the Groth16 host side: R1CS layout, the library's host curve arithmetic
(no GPU needed), and the serving trace. The GPU prover is covered by test_gpu_groth16.py."""

import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from pyzkp_gb300 import groth16 as G
from pyzkp_gb300 import serve, synth

HERE = os.path.dirname(os.path.abspath(__file__))
R = synth.FR_MODULUS


def test_host_curve_ops_match_oracle():
    from pyzkp_gb300 import _native as N

    for k in (1, 2, 0xFFFF, R - 1, R + 5, (1 << 255) + 3):
        assert N.host_g1_mul(G.G1_GEN, k) == (O.affine_to_ints(O.g1_mul(O.G1_GENERATOR, k)) if k % R else None)
        exp = O.g2_mul(O.G2_GENERATOR, k)
        assert N.host_g2_mul(G.G2_GEN, k) == (O.g2_to_ints(exp) if exp.any() else None)
    p = N.host_g1_mul(G.G1_GEN, 77)
    assert N.host_g1_add(p, p) == N.host_g1_mul(G.G1_GEN, 154)
    assert N.host_g1_add(p, None) == p and N.host_g1_add(None, None) is None
    assert N.host_g1_add(p, N.host_g1_mul(G.G1_GEN, R - 77)) is None
    q = N.host_g2_mul(G.G2_GEN, 99)
    assert N.host_g2_add(q, q) == N.host_g2_mul(G.G2_GEN, 198)
    assert N.host_g2_add(q, None) == q


def test_diagonal_r1cs_layout_and_transpose():
    m = 6
    r1 = G.diagonal_r1cs(m)
    assert (r1.n, r1.n_vars, r1.one_id) == (8, 3 * m + 1, 3 * m)
    assert r1.public_ids == [3 * m, 0] and r1.aux_ids == list(range(1, 3 * m))
    # row i of A is x_i (var 1 + i); of B y_i (1 + m + i); of C z_i (0, then 1 + 2m + i - 1)
    assert list(r1.a.cols) == [1 + i for i in range(m)]
    assert list(r1.b.cols) == [1 + m + i for i in range(m)]
    assert list(r1.c.cols) == [0] + [1 + 2 * m + i for i in range(m - 1)]
    assert list(np.diff(r1.a.row_ptr)) == [1] * m + [0] * (r1.n - m)
    t = r1.c.transpose(r1.n_vars)
    assert t.row_ptr[1] - t.row_ptr[0] == 1 and t.cols[0] == 0  # z_0 appears in constraint 0
    assert int(t.row_ptr[-1]) == m


def test_r1cs_from_golden_rows_matches_reference_layout():
    with open(os.path.join(HERE, "golden", "groth16_reference.json")) as f:
        c = json.load(f)["circuits"][1]
    rows = lambda mm: [{int(k): int(v, 16) for k, v in row} for row in mm]  # noqa: E731
    r1 = G.R1CS.from_rows(c["n"], c["n_vars"], c["one_id"], c["public_ids"], c["aux_ids"], rows(c["a_rows"]),
                          rows(c["b_rows"]), rows(c["c_rows"]))
    # A w, B w, C w of the witness satisfy the constraints (eval_r1cs_vectors, r1cs.py:84-92)
    w = [int(v, 16) for v in c["witness"]]

    def ev(m, i):
        lo, hi = int(m.row_ptr[i]), int(m.row_ptr[i + 1])
        vals = synth.limbs_to_ints(m.vals[lo:hi])
        return sum(w[int(k)] * v for k, v in zip(m.cols[lo:hi], vals)) % R

    for i in range(r1.n):
        assert ev(r1.a, i) * ev(r1.b, i) % R == ev(r1.c, i)


@pytest.mark.reference
def test_r1cs_from_reference_compile_r1cs():
    import reference_env

    reference_env.require()
    from frontend.api import compile_circuit
    from frontend.circuit.schema import public, secret
    from protocols.groth16.r1cs import compile_r1cs

    class Cubic:
        def __init__(self):
            self.x = secret("x")
            self.y = public("y")

        def define(self, api):
            api.AssertIsEqual(self.y, api.Add(api.Mul(self.x, self.x, self.x), self.x, 5))

    inst = compile_r1cs(compile_circuit(Cubic(), R))
    r1 = G.R1CS.from_reference(inst)
    with open(os.path.join(HERE, "golden", "groth16_reference.json")) as f:
        c = json.load(f)["circuits"][0]
    assert (r1.n, r1.n_vars, r1.one_id, r1.public_ids, r1.aux_ids) == (c["n"], c["n_vars"], c["one_id"],
                                                                     c["public_ids"], c["aux_ids"])
    for mat, key in ((r1.a, "a_rows"), (r1.b, "b_rows"), (r1.c, "c_rows")):
        got = [[[int(k), v] for k, v in zip(mat.cols[mat.row_ptr[i]:mat.row_ptr[i + 1]],
                                            synth.limbs_to_ints(mat.vals[mat.row_ptr[i]:mat.row_ptr[i + 1]]))]
               for i in range(r1.n)]
        assert got == [[[k, int(v, 16)] for k, v in row] for row in c[key]]


def test_poisson_trace_and_percentiles():
    tr = serve.poisson_trace(100.0, 2000, [3, 4, 5], seed=9, weights=[1, 2, 1])
    gaps = np.diff([a.t for a in tr])
    assert tr[0].t == 0.0 and (gaps >= 0).all() and abs(gaps.mean() - 0.01) < 0.001
    counts = np.bincount([a.key_id for a in tr], minlength=6)[3:]
    assert abs(counts[1] / len(tr) - 0.5) < 0.05
    res = serve.TraceResult(proofs=["p"] * 4, errors=[None] * 4, latency_s=[0.004, 0.001, 0.003, 0.002],
                            makespan_s=2.0, batches=[1, 3])
    s = res.summary()
    assert s["p50_ms"] in (2.0, 3.0) and s["p99_ms"] == 4.0 and s["proofs_per_s"] == 2.0 and s["mean_batch"] == 2
