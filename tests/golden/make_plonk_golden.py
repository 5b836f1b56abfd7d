"""Generate PLONK golden vectors by running the unmodified reference (fzybravery/pyZKP).

Needs the reference: ``PYZKP_REFERENCE`` (a checkout or install directory) or the pip
install in ``baseline/_ref``; py_ecc is the stand-in under ``oracle/py_ecc_shim``.

    PYZKP_REFERENCE=<reference checkout> python tests/golden/make_plonk_golden.py

Two parts, written to ``plonk_reference.json`` beside this script:

* ``quotient``: the reference's CPU KernelFn ``_plonk_t_quotient_evals``
  (runtime/kernels/cpu/kernels.py:607-693) run through its own ``Executor`` on seeded
  extended-coset evaluations (15 vectors from ``pyzkp_gb300.synth.fr_uniform(seed + j, m)``)
  and seeded challenges, for m = 2^6 .. 2^10, 2^12 and a ragged m = 100. Each record keeps
  the attrs, the SHA-256 of the outputs (32-byte little-endian canonical values, ``num``
  then ``zh`` separately) and the values at a few indices.
* ``proofs``: the reference's PLONK ``setup`` / ``prove`` / ``verify``
  (protocols/plonk/setup.py:10, prove.py:31-160, verify.py:12) on the cubic circuit of
  tests/correctness/cpu/test_plonk_e2e.py (domain 16) and a 20-step chain (domain 128),
  with its randomness (``secrets.randbelow`` in protocols/plonk/domain.py and
  prove.py:325, ``fr_rand`` in crypto/kzg/cpu_ref.py:31) drawn from a seeded generator:
  the proof's commitments and evaluations and the verifier's verdicts for the right and
  a wrong public input.
"""

from __future__ import annotations

import hashlib
import json
import os
import random
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "tests"))
sys.path.insert(0, REPO)

import reference_env  # noqa: E402

reference_env.add_to_path()

from crypto.field.fr import FR_MODULUS  # noqa: E402
from crypto.poly import omega_for_size  # noqa: E402
from frontend.api import build_witness, check_r1cs, compile_circuit  # noqa: E402
from frontend.circuit.schema import public, secret  # noqa: E402
from protocols.plonk import prove, setup, verify  # noqa: E402
from py_ecc import optimized_bn128 as bn  # noqa: E402
from runtime import Executor, KernelRegistry  # noqa: E402
from runtime.ir import Device, DType, Graph, OpType  # noqa: E402
from runtime.kernels.cpu import register_cpu_kernels  # noqa: E402

from pyzkp_gb300 import synth  # noqa: E402

QUOTIENT_INPUTS = ("a", "b", "c", "z", "pi", "ql", "qr", "qm", "qo", "qc", "s1", "s2", "s3", "zshift", "l1")
SAMPLE_AT = (0, 1, 31, 32, 33, 511, 512, 4095)


def hx(v: int) -> str:
    return hex(int(v))


def digest(vals) -> str:
    return hashlib.sha256(b"".join((int(v) % FR_MODULUS).to_bytes(32, "little") for v in vals)).hexdigest()


def quotient_case(m: int, n: int, omega_m: int, seed: int, shift_n_override: bool = False) -> dict:
    rng = random.Random(seed)
    ch = {k: rng.randrange(1, FR_MODULUS) for k in ("shift", "alpha", "beta", "gamma", "k1", "k2")}
    shift_n = rng.randrange(1, FR_MODULUS) if shift_n_override else pow(ch["shift"], n, FR_MODULUS)
    attrs = {"n": n, "m": m, "omega_m": omega_m, "shift": ch["shift"], "shift_n": shift_n, "alpha": ch["alpha"],
             "beta": ch["beta"], "gamma": ch["gamma"], "k1": ch["k1"], "k2": ch["k2"]}
    reg = KernelRegistry()
    register_cpu_kernels(reg)
    g = Graph()
    for j, name in enumerate(QUOTIENT_INPUTS):
        g.add_buffer(id=name, device=Device.CPU, dtype=DType.FR,
                     data=synth.limbs_to_ints(synth.fr_uniform(seed + j, m)))
    g.add_node(op=OpType.PLONK_T_QUOTIENT_EVALS, inputs=list(QUOTIENT_INPUTS), outputs=["num", "zh"], attrs=attrs)
    Executor(registry=reg).run(g, keep=["num", "zh"])
    num, zh = list(g.buffers["num"].data), list(g.buffers["zh"].data)
    return {
        "m": m,
        "seed": seed,
        "input_seeds": f"pyzkp_gb300.synth.fr_uniform(seed + j, m) for j, name in enumerate({list(QUOTIENT_INPUTS)})",
        "attrs": {k: (hx(v) if k not in ("n", "m") else v) for k, v in attrs.items()},
        "num_sha256": digest(num),
        "zh_sha256": digest(zh),
        "num_at": {str(i): hx(num[i]) for i in SAMPLE_AT if i < m},
        "zh_at": {str(i): hx(zh[i]) for i in SAMPLE_AT if i < m},
    }


class CubicCircuit:
    """tests/correctness/cpu/test_plonk_e2e.py:12-19: y = x^3 + x + 5."""

    def __init__(self):
        self.x = secret("x")
        self.y = public("y")

    def define(self, api):
        x3 = api.Mul(self.x, self.x, self.x)
        api.AssertIsEqual(self.y, api.Add(x3, self.x, 5))


class ChainCircuit:
    """A longer circuit: v_0 = x, v_{i+1} = v_i^2 + (i + 1), y = v_steps (domain 2^7 for 20 steps)."""

    def __init__(self, steps: int = 20):
        self.steps = steps
        self.x = secret("x")
        self.y = public("y")

    def define(self, api):
        v = self.x
        for i in range(self.steps):
            v = api.Add(api.Mul(v, v), i + 1)
        api.AssertIsEqual(self.y, v)


def g1(p):
    if bn.is_inf(p):
        return None
    q = bn.normalize(p)
    return [hx(int(q[0])), hx(int(q[1]))]


def proof_case(name: str, circuit, assignment: dict, public_values: list, seed: int) -> dict:
    ir = compile_circuit(circuit, FR_MODULUS)
    wit = build_witness(ir, assignment)
    check_r1cs(ir, wit)
    with reference_env.seeded_plonk_randomness(seed):
        pk = setup(ir)
        prf = prove(pk, wit, public_values=public_values)
    ok = verify(pk.vk, prf, public_values=public_values)
    bad = verify(pk.vk, prf, public_values=[public_values[0]] + [(v + 1) % FR_MODULUS for v in public_values[1:]])
    return {
        "name": name,
        "seed": seed,
        "assignment": {k: hx(v) for k, v in assignment.items()},
        "public_values": [hx(v) for v in public_values],
        "domain_n": pk.circuit.domain.n,
        "proof": {
            **{k: g1(getattr(prf, k)) for k in ("cm_a", "cm_b", "cm_c", "cm_z", "cm_t1", "cm_t2", "cm_t3",
                                                  "pi_zeta", "pi_zeta_omega")},
            "evals_zeta": {str(k): hx(v) for k, v in dict(prf.evals_zeta).items()} if isinstance(prf.evals_zeta, dict)
            else [hx(v) for v in prf.evals_zeta],
            "eval_zeta_omega": hx(prf.eval_zeta_omega),
        },
        "verify": ok,
        "verify_wrong_public": bad,
    }


def main() -> None:
    quotient = []
    for lg in (6, 7, 8, 9, 10, 12):
        m = 1 << lg
        quotient.append(quotient_case(m, m // 4, omega_for_size(m), seed=0x9105 + lg))
    # ragged m (the op takes any m and any omega_m), and a shift_n that is not shift^n
    quotient.append(quotient_case(100, 25, omega_for_size(128), seed=0x9171))
    quotient.append(quotient_case(1 << 9, 1 << 7, omega_for_size(1 << 9), seed=0x9172, shift_n_override=True))
    x = 9
    y = (x ** 3 + x + 5) % FR_MODULUS
    proofs = [proof_case("cubic", CubicCircuit(), {"x": x, "y": y}, [1, y], seed=0x91A6)]
    v = 3
    for i in range(20):
        v = (v * v + i + 1) % FR_MODULUS
    proofs.append(proof_case("chain20", ChainCircuit(20), {"x": 3, "y": v}, [1, v], seed=0x91A7))
    for p in proofs:
        assert p["verify"] and not p["verify_wrong_public"], p["name"]
    with open(os.path.join(HERE, "plonk_reference.json"), "w") as f:
        json.dump({"source": "reference _plonk_t_quotient_evals and PLONK setup / prove / verify with seeded "
                             "randomness (make_plonk_golden.py)",
                   "quotient": quotient, "proofs": proofs}, f, indent=1)
    print("wrote plonk_reference.json")


if __name__ == "__main__":
    main()
