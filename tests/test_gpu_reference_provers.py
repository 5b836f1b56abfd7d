"""The reference's own provers, unmodified, running on GB300 through ``plugin.install()``.

``install()`` points the reference's ``MetalContext.create_default`` and
``runtime.kernels.metal.register_metal_kernels`` at the GB300 implementation, so
``RuntimeConfig(backend=Backend.METAL)`` makes the reference's Groth16 and PLONK provers
(protocols/groth16/prove.py:30-248, protocols/plonk/prove.py:31-438) and its Executor
(runtime/executor.py:84-218) run their MSM / NTT / quotient nodes as GB300 kernels. With
the provers' randomness seeded as in tests/golden/make_groth16_golden.py and
make_plonk_golden.py, every proof must equal, bit for bit, the proof the reference made
on its CPU path (the committed goldens), and verify under the reference's verifier.

The reference comes from ``PYZKP_REFERENCE`` or ``baseline/_ref`` (tests/reference_env.py).
"""

import json
import os
import sys

import pytest

import reference_env

HERE = os.path.dirname(os.path.abspath(__file__))
R = reference_env.runtime()
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_groth16_golden as MG  # noqa: E402
import make_plonk_golden as MP  # noqa: E402
from crypto.field.fr import FR_MODULUS  # noqa: E402
from frontend.api import build_witness, compile_circuit  # noqa: E402
from protocols import plonk as PL  # noqa: E402

from pyzkp_gb300 import plugin  # noqa: E402

pytestmark = pytest.mark.gpu


def _golden(name):
    with open(os.path.join(HERE, "golden", name)) as f:
        return json.load(f)


def _metal():
    plugin.install()
    return R.RuntimeConfig(backend=R.Backend.METAL)


class _Trace:
    """Records which device each node ran on (the ``trace`` argument of Executor.run)."""

    def __init__(self):
        self.events = []

    def add(self, ev):
        self.events.append(ev)


def _g16_case(name):
    for c in _golden("groth16_reference.json")["circuits"]:
        if c["name"] == name:
            return c
    raise KeyError(name)


def _g16_setup(name):
    """The reference's setup with the golden's seeded fr_rand; returns (ir, pk, witness, public, golden case)."""
    c = _g16_case(name)
    seed = {"cubic": 0x6A0716, "mixed": 0x6A0717}[name]
    fr = reference_env.seeded_fr_rand(seed)
    MG.setup_mod.fr_rand = fr
    MG.prove_mod.fr_rand = fr
    if name == "cubic":
        circuit, assignment = MG.CubicCircuit(), {"x": 9, "y": int(c["public_values"][1], 16)}
    else:
        circuit = MG.MixedCircuit()
        assignment = {"x": 7, "w": 11, "z": 13, "y1": int(c["public_values"][1], 16),
                      "y2": int(c["public_values"][2], 16)}
    ir = compile_circuit(circuit, FR_MODULUS)
    wit = build_witness(ir, assignment)
    pk = MG.setup_mod.setup(ir)
    return ir, pk, wit, [int(v, 16) for v in c["public_values"]], c


@pytest.mark.parametrize("name", ["cubic", "mixed"])
def test_reference_groth16_prove_on_gb300_matches_reference_proof(name):
    ir, pk, wit, public, c = _g16_setup(name)
    trace = _Trace()
    proof = MG.prove_mod.prove(ir, pk, wit, runtime_config=_metal(), runtime_trace=trace)
    assert MG.g1(proof.a) == c["proof"]["a"]
    assert MG.g2(proof.b) == c["proof"]["b"]
    assert MG.g1(proof.c) == c["proof"]["c"]
    assert MG.verify(pk.vk, public, proof)
    # the MSMs ran as GB300 kernels (prove() keeps the QAP on the CPU, prove.py:98)
    ran = {(ev.op, ev.device) for ev in trace.events}
    assert (R.OpType.MSM_G1, R.Device.METAL) in ran and (R.OpType.MSM_G2, R.Device.METAL) in ran


def test_reference_groth16_prove_batch_on_gb300_matches_reference_proof():
    """prove_batch (prove.py:133-248) forwards the context to the QAP, so the iNTTs, POLY_MUL_NTT,
    POLY_SUB and DIV_XN_MINUS_1 of protocols/groth16/qap.py:78-91 run on the device too and
    qap.py:93-97 reads the kept device buffers. One witness: the reference's Executor cannot
    run a second one on a device backend (see test_reference_runtime.py)."""
    ir, pk, wit, public, c = _g16_setup("mixed")
    trace = _Trace()
    (proof,) = MG.prove_mod.prove_batch(ir, pk, [wit], runtime_config=_metal(), runtime_trace=trace)
    assert (MG.g1(proof.a), MG.g2(proof.b), MG.g1(proof.c)) == (c["proof"]["a"], c["proof"]["b"], c["proof"]["c"])
    assert MG.verify(pk.vk, public, proof)
    ran = {(ev.op, ev.device) for ev in trace.events}
    for op in (R.OpType.ROOTS_COEFFS_FROM_EVALS, R.OpType.POLY_MUL_NTT, R.OpType.POLY_SUB, R.OpType.DIV_XN_MINUS_1,
               R.OpType.MSM_G1, R.OpType.MSM_G2, R.OpType.TO_DEVICE):
        assert any(o == op for o, _ in ran), op
    assert (R.OpType.DIV_XN_MINUS_1, R.Device.METAL) in ran


def test_reference_groth16_rejects_unsatisfied_witness_on_gb300():
    """The device QAP leaves a remainder for a witness that breaks a constraint, and the
    reference raises (qap.py:98-99)."""
    import dataclasses

    ir, pk, wit, _, _ = _g16_setup("cubic")
    vals = list(wit.values)
    vals[-1] = (vals[-1] + 1) % FR_MODULUS  # the last internal wire no longer satisfies its constraint
    bad = dataclasses.replace(wit, values=tuple(vals))
    with pytest.raises(ValueError):
        MG.prove_mod.prove_batch(ir, pk, [bad], runtime_config=_metal())


@pytest.mark.parametrize("idx", [0, 1])
def test_reference_plonk_prove_on_gb300_matches_reference_proof(idx):
    """protocols/plonk/prove.py with the METAL config: KZG_BATCH_COMMIT, the 15 coset NTTs at
    4n, PLONK_T_QUOTIENT_EVALS, BATCH_INV, POINTWISE_MUL and the coset iNTT on GB300."""
    c = _golden("plonk_reference.json")["proofs"][idx]
    if c["name"] == "cubic":
        circuit = MP.CubicCircuit()
    else:
        circuit = MP.ChainCircuit(20)
    assignment = {k: int(v, 16) for k, v in c["assignment"].items()}
    public = [int(v, 16) for v in c["public_values"]]
    ir = compile_circuit(circuit, FR_MODULUS)
    wit = build_witness(ir, assignment)
    trace = _Trace()
    with reference_env.seeded_plonk_randomness(c["seed"]):
        pk = PL.setup(ir)
        prf = PL.prove(pk, wit, public_values=public, runtime_config=_metal(), runtime_trace=trace)
    for k in ("cm_a", "cm_b", "cm_c", "cm_z", "cm_t1", "cm_t2", "cm_t3", "pi_zeta", "pi_zeta_omega"):
        assert MP.g1(getattr(prf, k)) == c["proof"][k], k
    assert {str(k): hex(v) for k, v in dict(prf.evals_zeta).items()} == c["proof"]["evals_zeta"]
    assert hex(prf.eval_zeta_omega) == c["proof"]["eval_zeta_omega"]
    assert PL.verify(pk.vk, prf, public_values=public)
    ran = {(ev.op, ev.device) for ev in trace.events}
    for op in (R.OpType.KZG_BATCH_COMMIT, R.OpType.COSET_EVALS_FROM_COEFFS, R.OpType.PLONK_T_QUOTIENT_EVALS,
               R.OpType.BATCH_INV, R.OpType.COSET_COEFFS_FROM_EVALS):
        assert (op, R.Device.METAL) in ran, op


def test_reference_metal_test_shapes_through_reference_executor():
    """The graphs of the reference's Metal tests (tests/correctness/metal/test_runtime_metal_mix.py
    style: NTT -> pointwise -> iNTT chains with automatic transfers) on the reference Executor."""
    from crypto.poly import omega_for_size

    reg = R.KernelRegistry()
    R.register_cpu_kernels(reg, backend=R.Backend.METAL)
    plugin.register_gb300_kernels(reg)
    exe = R.Executor(registry=reg)
    n = 64
    om = omega_for_size(n)
    a = [(i * i + 3) % FR_MODULUS for i in range(n)]
    b = [(7 * i + 1) % FR_MODULUS for i in range(n)]
    g = R.Graph()
    g.add_buffer(id="a", device=R.Device.CPU, dtype=R.DType.FR, data=list(a))
    g.add_buffer(id="b", device=R.Device.CPU, dtype=R.DType.FR, data=list(b))
    g.add_node(op=R.OpType.ROOTS_EVALS_FROM_COEFFS, inputs=["a"], outputs=["ea"], attrs={"n": n, "omega": om})
    g.add_node(op=R.OpType.ROOTS_EVALS_FROM_COEFFS, inputs=["b"], outputs=["eb"], attrs={"n": n, "omega": om})
    g.add_node(op=R.OpType.POINTWISE_MUL, inputs=["ea", "eb"], outputs=["ec"])
    g.add_node(op=R.OpType.ROOTS_COEFFS_FROM_EVALS, inputs=["ec"], outputs=["c"], attrs={"omega": om})
    g.add_node(op=R.OpType.FROM_DEVICE, inputs=["c"], outputs=["c_host"])
    pool = R.MemoryPool()
    exe.run(g, runtime_config=_metal(), pool=pool, keep=["c_host"])
    # cyclic convolution mod x^n - 1
    exp = [0] * n
    for i, x in enumerate(a):
        for j, y in enumerate(b):
            exp[(i + j) % n] = (exp[(i + j) % n] + x * y) % FR_MODULUS
    assert g.buffers["c_host"].data == exp
    # everything not kept was released (runtime/executor.py:155-165), device buffers through the pool
    assert set(g.buffers) == {"c_host"}
    assert pool.metal_stats.alloc_calls >= 3 and pool.metal_stats.in_use < pool.metal_stats.alloc_calls
    # a coset round trip through the automatic TO_DEVICE of its input
    g2 = R.Graph()
    g2.add_buffer(id="x", device=R.Device.CPU, dtype=R.DType.FR, data=list(a))
    g2.add_node(op=R.OpType.COSET_EVALS_FROM_COEFFS, inputs=["x"], outputs=["ex"], attrs={"n": n, "omega": om,
                                                                                            "shift": 5})
    g2.add_node(op=R.OpType.COSET_COEFFS_FROM_EVALS, inputs=["ex"], outputs=["y"], attrs={"omega": om, "shift": 5})
    exe.run(g2, runtime_config=_metal(), keep=["y"])
    assert list(g2.buffers["y"].data) == a
