"""The GLV constants of the G1 MSM (pyzkp_gb300/csrc/msm.cu), checked from the source text.

The MSM splits every scalar k < r as k = k1 + k2 * lambda (mod r) and sums k1 P + k2 phi(P)
with phi(x, y) = (beta x, y) = [lambda](x, y). The result is the same group element, so the
GPU parity tests cover the split end to end; this file pins the constants and the bound
|k1|, |k2| < 2^127 that the window count W = ceil(128 / c) relies on, by restating the
device arithmetic (Babai rounding with 2^256-scaled reciprocals, two's complement mod 2^256).
"""

import os
import random
import re

import numpy as np

from oracle import oracle as O
from pyzkp_gb300 import synth

R = synth.FR_MODULUS
Q = 0x30644E72E131A029B85045B68181585D97816A916871CA8D3C208C16D87CFD47
SRC = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "pyzkp_gb300", "csrc", "msm.cu")


def _limbs(name: str, text: str) -> int:
    m = re.search(r"uint32_t " + name + r"\[\d+\] = \{([^}]*)\}", text)
    assert m, name
    words = [int(w.strip().rstrip("u"), 16) for w in m.group(1).split(",") if w.strip()]
    return sum(w << (32 * i) for i, w in enumerate(words))


def _consts():
    text = open(SRC).read()
    beta = int(re.search(r"beta = (0x[0-9a-f]+), the cube root", text).group(1), 16)
    lam = int(re.search(r"for lambda = (0x[0-9a-f]+)", text).group(1), 16)
    return {
        "g1": _limbs("kGlvG1", text), "g2": _limbs("kGlvG2", text), "a1": _limbs("kGlvA1", text),
        "a2": _limbs("kGlvA2", text), "b1": _limbs("kGlvB1", text), "beta": beta, "lam": lam,
    }


def _split(k: int, K: dict):
    """The device's glv_split on Python integers: (k1, k2) as signed integers."""
    M = 1 << 256
    c1 = (k * K["g1"] + (1 << 255)) >> 256
    c2 = (k * K["g2"] + (1 << 255)) >> 256
    k1 = (k - c1 * K["a1"] - c2 * K["a2"]) % M
    k2 = (c1 * K["b1"] - c2 * K["a1"]) % M
    signed = lambda x: x - M if x >> 255 else x
    return signed(k1), signed(k2)


def test_endomorphism_constants():
    K = _consts()
    lam, beta = K["lam"], K["beta"]
    assert lam != 1 and pow(lam, 3, R) == 1
    assert beta != 1 and pow(beta, 3, Q) == 1
    # [lambda]G == (beta * Gx, Gy) on the oracle's scalar multiplication
    p = O.g1_fixed_base_mul(O.G1_GENERATOR, synth.ints_to_limbs([lam]))
    x, y = O.affine_to_ints(p[0])
    assert (x, y) == (beta * 1 % Q, 2)


def test_lattice_basis_and_reciprocals():
    K = _consts()
    a1, a2, b1, lam = K["a1"], K["a2"], K["b1"], K["lam"]
    b2 = a1
    assert (a1 - b1 * lam) % R == 0  # v1 = (a1, -b1)
    assert (a2 + b2 * lam) % R == 0  # v2 = (a2, b2)
    assert a1 * b2 + a2 * b1 == R
    assert K["g1"] == (((1 << 256) * b2) + R // 2) // R
    assert K["g2"] == (((1 << 256) * b1) + R // 2) // R


def test_split_identity_and_bound():
    K = _consts()
    rng = random.Random(1234)
    cases = [0, 1, 2, R - 1, R - 2, K["lam"], R - K["lam"], (R - 1) // 2, R // 3, (2 * R) // 3]
    cases += [rng.randrange(R) for _ in range(20000)]
    seeds = synth.limbs_to_ints(synth.fr_uniform(77, 2000))
    worst = 0
    for k in cases + seeds:
        k1, k2 = _split(k, K)
        assert (k1 + k2 * K["lam"] - k) % R == 0
        worst = max(worst, abs(k1).bit_length(), abs(k2).bit_length())
    assert worst <= 127  # W * c >= 128 windows hold every half with its signed-digit carry
    assert np.log2(0.6 * (K["a1"] + K["a2"])) < 126.2  # the analytic bound behind it
