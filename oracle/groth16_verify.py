"""Groth16 verification of proofs made on the GPU.

ORACLE / TEST INFRASTRUCTURE. Only ``tests/`` and the CPU-baseline leg of ``bench.py``
use it, to check served proofs off the timed path; it is not part of the product.

It restates the reference's verifier, protocols/groth16/verify.py:11-23: with
vk_x = sum_i public_i IC_i, a proof (A, B, C) is accepted iff

    e(A, B) == e(alpha, beta) * e(vk_x, gamma) * e(C, delta)

over the optimal ate pairing of the test-only py_ecc stand-in (oracle/py_ecc_shim). The
same equation is evaluated as FE(ML(B, A) ML(gamma, -vk_x) ML(delta, -C)) == e(alpha, beta),
with ML the Miller loop and FE the final exponentiation (one FE per proof instead of four,
and e(alpha, beta) computed once per key). Inputs are canonical affine ints as the GPU
prover returns them: G1 (x, y), G2 ((x0, x1), (y0, y1)) with x = x0 + x1 u, None for the
point at infinity.
"""

from __future__ import annotations

import os
import sys
from typing import Dict, Optional, Sequence, Tuple

HERE = os.path.dirname(os.path.abspath(__file__))
_SHIM = os.path.join(HERE, "py_ecc_shim")
if _SHIM not in sys.path:
    sys.path.insert(0, _SHIM)

from py_ecc import optimized_bn128 as bn  # noqa: E402

FR_MODULUS = 21888242871839275222246405745257275088548364400416034343698204186575808495617
FQ_MODULUS = 21888242871839275222246405745257275088696311157297823662689037894645226208583


def _g1(p) -> Optional[tuple]:
    """Canonical affine ints -> the stand-in's projective point (None = infinity)."""
    if p is None:
        return None
    return (bn.FQ(int(p[0])), bn.FQ(int(p[1])), bn.FQ(1))


def _g2_affine(q) -> Optional[tuple]:
    if q is None:
        return None
    (x0, x1), (y0, y1) = q
    return (bn.FQ2([int(x0), int(x1)]), bn.FQ2([int(y0), int(y1)]))


def _ml(q2, p1) -> "bn.FQ12":
    """Miller loop of G2 affine q2 and G1 point p1 (identity for infinity on either side)."""
    if q2 is None or p1 is None or bn.is_inf(p1):
        return bn.FQ12.one()
    pa = bn.normalize(p1)
    return bn.miller_loop(q2, (pa[0].n, pa[1].n))


class Groth16Verifier:
    """verify.py:11-23 for one verifying key (alpha_g1, beta_g2, gamma_g2, delta_g2, ic)."""

    def __init__(self, alpha_g1, beta_g2, gamma_g2, delta_g2, ic: Sequence) -> None:
        self.ic = [_g1(p) for p in ic]
        self.gamma = _g2_affine(gamma_g2)
        self.delta = _g2_affine(delta_g2)
        self.e_alpha_beta = bn.final_exponentiate(_ml(_g2_affine(beta_g2), _g1(alpha_g1)))

    def verify(self, public_values: Sequence[int], a, b, c) -> bool:
        if len(public_values) != len(self.ic):
            return False
        vk_x = bn.Z1
        for s, p in zip(public_values, self.ic):
            if p is not None:
                vk_x = bn.add(vk_x, bn.multiply(p, int(s) % FR_MODULUS))
        neg = lambda p: None if p is None or bn.is_inf(p) else bn.neg(p)  # noqa: E731
        f = _ml(_g2_affine(b), _g1(a)) * _ml(self.gamma, neg(vk_x)) * _ml(self.delta, neg(_g1(c)))
        return bn.final_exponentiate(f) == self.e_alpha_beta


_VERIFIERS: Dict[int, Groth16Verifier] = {}


def verify_many(jobs: Sequence[Tuple[int, tuple, Sequence[int], tuple]]) -> list:
    """jobs: (key id, (alpha_g1, beta_g2, gamma_g2, delta_g2, ic), public values, (A, B, C)).
    Verifiers are cached per key id within the calling process. Returns one bool per job."""
    out = []
    for kid, vk, pub, proof in jobs:
        v = _VERIFIERS.get(kid)
        if v is None:
            v = _VERIFIERS[kid] = Groth16Verifier(*vk)
        out.append(bool(v.verify(pub, *proof)))
    return out
