"""Generate Groth16 golden vectors by running the unmodified reference (fzybravery/pyZKP).

Needs the reference: ``PYZKP_REFERENCE`` (a checkout or install directory) or the pip
install in ``baseline/_ref`` (tests/reference_env.py finds it):

    python tests/golden/make_groth16_golden.py

The reference's setup and prove draw their randomness from ``fr_rand`` (crypto/field/fr.py:37-42,
``secrets``); here the module attributes ``protocols.groth16.setup.fr_rand`` and
``protocols.groth16.prove.fr_rand`` are replaced by a seeded generator so that the
trapdoors (tau, alpha, beta, gamma, delta) and the prover's (r, s) are reproducible. Everything
else runs unmodified: compile_circuit / build_witness / check_r1cs (frontend/api),
compile_r1cs (protocols/groth16/r1cs.py:39-81), setup (setup.py:25-121), prove
(prove.py:30-126) and verify (verify.py:11-23, through the py_ecc stand-in's pairing).

Output: groth16_reference.json beside this script (ints as hex strings): per circuit the
R1CS rows, the witness (with the trailing 1), the trapdoors, r and s, the proving key's
points, the proof, and the verifier's verdict.
"""

from __future__ import annotations

import json
import os
import random
import sys
from dataclasses import dataclass

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "tests"))

import reference_env  # noqa: E402

reference_env.add_to_path()

import importlib  # noqa: E402

# the package re-exports the functions setup / prove under the submodules' names
setup_mod = importlib.import_module("protocols.groth16.setup")
prove_mod = importlib.import_module("protocols.groth16.prove")
from crypto.field.fr import FR_MODULUS  # noqa: E402
from frontend.api import build_witness, check_r1cs, compile_circuit  # noqa: E402
from frontend.circuit.schema import public, secret  # noqa: E402
from protocols.groth16 import verify  # noqa: E402
from protocols.groth16.r1cs import compile_r1cs  # noqa: E402
from py_ecc import optimized_bn128 as bn  # noqa: E402


def hx(v: int) -> str:
    return hex(int(v))


def g1(p):
    q = bn.normalize(p)
    if bn.is_inf(p):
        return None
    return [hx(int(q[0])), hx(int(q[1]))]


def g2(p):
    if bn.is_inf(p):
        return None
    q = bn.normalize(p)
    return [[hx(int(q[0].coeffs[0])), hx(int(q[0].coeffs[1]))], [hx(int(q[1].coeffs[0])), hx(int(q[1].coeffs[1]))]]


@dataclass
class CubicCircuit:
    """tests/correctness/cpu/test_groth16_e2e.py:11-24: y = x^3 + x + 5."""

    x: object
    y: object

    def __init__(self):
        self.x = secret("x")
        self.y = public("y")

    def define(self, api):
        x3 = api.Mul(self.x, self.x, self.x)
        api.AssertIsEqual(self.y, api.Add(x3, self.x, 5))


class MixedCircuit:
    """Two public outputs and several products: y1 = x^5 + 3x + w z, y2 = (w + 2)(z - x) w."""

    def __init__(self):
        self.y1 = public("y1")
        self.y2 = public("y2")
        self.x = secret("x")
        self.w = secret("w")
        self.z = secret("z")

    def define(self, api):
        x5 = api.Mul(self.x, self.x, self.x, self.x, self.x)
        api.AssertIsEqual(self.y1, api.Add(x5, api.Mul(self.x, 3), api.Mul(self.w, self.z)))
        api.AssertIsEqual(self.y2, api.Mul(api.Add(self.w, 2), api.Sub(self.z, self.x), self.w))


def run(name, circuit, assignment, public_values, seed):
    rng = random.Random(seed)

    def fr_rand(nonzero: bool = True) -> int:
        while True:
            x = rng.randrange(FR_MODULUS)
            if nonzero and x == 0:
                continue
            return x

    setup_mod.fr_rand = fr_rand
    prove_mod.fr_rand = fr_rand
    ir = compile_circuit(circuit, FR_MODULUS)
    wit = build_witness(ir, assignment)
    check_r1cs(ir, wit)
    r1cs = compile_r1cs(ir)
    pk = setup_mod.setup(ir)
    # prove() draws r then s (prove.py:84-85): record them by replaying the generator state
    state = rng.getstate()
    r = fr_rand(True)
    s = fr_rand(True)
    rng.setstate(state)
    proof = prove_mod.prove(ir, pk, wit)
    ok = verify(pk.vk, public_values, proof)
    bad = verify(pk.vk, [public_values[0]] + [(v + 1) % FR_MODULUS for v in public_values[1:]], proof)
    rows = lambda m: [[[int(k), hx(v)] for k, v in sorted(row.items())] for row in m]  # noqa: E731
    return {
        "name": name,
        "n": r1cs.n_constraints,
        "n_vars": r1cs.n_vars,
        "one_id": r1cs.one_id,
        "public_ids": r1cs.public_ids,
        "aux_ids": r1cs.aux_ids,
        "a_rows": rows(r1cs.a_rows),
        "b_rows": rows(r1cs.b_rows),
        "c_rows": rows(r1cs.c_rows),
        "witness": [hx(v) for v in list(wit.values) + [1]],
        "public_values": [hx(v) for v in public_values],
        "trapdoors": {k: hx(getattr(pk, "trapdoor_" + k)) for k in ("tau", "alpha", "beta", "gamma", "delta")},
        "r": hx(r),
        "s": hx(s),
        "pk": {
            "alpha_g1": g1(pk.vk.alpha_g1),
            "beta_g1": g1(pk.beta_g1),
            "delta_g1": g1(pk.delta_g1),
            "beta_g2": g2(pk.vk.beta_g2),
            "gamma_g2": g2(pk.vk.gamma_g2),
            "delta_g2": g2(pk.vk.delta_g2),
            "ic": [g1(p) for p in pk.vk.ic],
            "a_query": [g1(p) for p in pk.a_query],
            "b_query_g1": [g1(p) for p in pk.b_query_g1],
            "b_query_g2": [g2(p) for p in pk.b_query_g2],
            "h_query": [g1(p) for p in pk.h_query],
            "l_query": [g1(p) for p in pk.l_query],
        },
        "proof": {"a": g1(proof.a), "b": g2(proof.b), "c": g1(proof.c)},
        "verify": ok,
        "verify_wrong_public": bad,
    }


def main() -> None:
    x = 9
    y = (x ** 3 + x + 5) % FR_MODULUS
    cubic = run("cubic", CubicCircuit(), {"x": x, "y": y}, [1, y], seed=0x6A0716)
    xv, wv, zv = 7, 11, 13
    y1 = (xv ** 5 + 3 * xv + wv * zv) % FR_MODULUS
    y2 = ((wv + 2) * (zv - xv) * wv) % FR_MODULUS
    mixed = run("mixed", MixedCircuit(), {"x": xv, "w": wv, "z": zv, "y1": y1, "y2": y2}, [1, y1, y2],
                seed=0x6A0717)
    for c in (cubic, mixed):
        assert c["verify"] and not c["verify_wrong_public"], c["name"]
    with open(os.path.join(HERE, "groth16_reference.json"), "w") as f:
        json.dump({"source": "reference setup / prove / verify with seeded fr_rand (make_groth16_golden.py)",
                   "circuits": [cubic, mixed]}, f, indent=1)
    print("wrote groth16_reference.json")


if __name__ == "__main__":
    main()
