"""The library's host-side field code (pyzkp_gb300/csrc/host_field.hpp: the final MSM
combination and the NTT tables use it) built for the host and checked against Python
integers for Fr and Fq: Montgomery product, inverse (of a Montgomery form), sum, difference
and conversion; and the G1 XYZZ addition and doubling of the window combination against
affine integer arithmetic."""

import os
import random
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MODULI = {
    "fr": 21888242871839275222246405745257275088548364400416034343698204186575808495617,
    "fq": 21888242871839275222246405745257275088696311157297823662689037894645226208583,
}


def _build(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "host_field_check"
    res = subprocess.run([cxx, "-std=c++17", "-O2", os.path.join(REPO, "tests", "host_field_check.cpp"), "-o",
                          str(exe)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return exe


@pytest.mark.parametrize("name", ["fr", "fq"])
def test_host_field_matches_integers(tmp_path, name):
    exe = _build(tmp_path)
    p = MODULI[name]
    rinv = pow(2**256, -1, p)
    rng = random.Random(0x40F7 + len(name))
    edges = [0, 1, 2, p - 2, p - 1, 2**64 - 1, 2**64, 2**128 + 1, 2**192 - 1, 2**253]
    recs = [(rng.choice(edges), rng.choice(edges)) for _ in range(200)]
    recs += [(rng.randrange(p), rng.randrange(p)) for _ in range(3000)]
    src = tmp_path / "in.bin"
    dst = tmp_path / "out.bin"
    src.write_bytes(b"".join(x.to_bytes(32, "little") for r in recs for x in r))
    res = subprocess.run([str(exe), name, str(src), str(dst)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    raw = dst.read_bytes()
    assert len(raw) == 160 * len(recs)
    for i, (a, b) in enumerate(recs):
        got = [int.from_bytes(raw[160 * i + 32 * k:160 * i + 32 * k + 32], "little") for k in range(5)]
        # inv acts on Montgomery forms: (a / R)^-1 R = R^2 / a
        want = [a * b * rinv % p, pow(a, -1, p) * 2**512 % p if a else 0, (a + b) % p, (a - b) % p, a * 2**256 % p]
        assert got == want, (i, a, b)


def _affine_mul(k, q):
    """[k] (1, 2) on y^2 = x^3 + 3 over F_q by affine double-and-add (None = infinity)."""
    def add(P, Q):
        if P is None:
            return Q
        if Q is None:
            return P
        if P[0] == Q[0]:
            if (P[1] + Q[1]) % q == 0:
                return None
            lam = 3 * P[0] * P[0] * pow(2 * P[1], -1, q) % q
        else:
            lam = (Q[1] - P[1]) * pow(Q[0] - P[0], -1, q) % q
        x = (lam * lam - P[0] - Q[0]) % q
        return x, (lam * (P[0] - x) - P[1]) % q
    R, A = None, (1, 2)
    while k:
        if k & 1:
            R = add(R, A)
        A = add(A, A)
        k >>= 1
    return R


def test_host_doubling_chain_matches_integers(tmp_path):
    """XYZZ double-and-add, then n XYZZ doublings (the 2^c window shifts of the combination),
    give [2^n k] G1 for random 64-bit k and n < 48."""
    exe = _build(tmp_path)
    q = MODULI["fq"]
    rng = random.Random(0xD0B1)
    recs = [(rng.randrange(1, 2**64), n) for n in list(range(48)) + [rng.randrange(48) for _ in range(32)]]
    src = tmp_path / "in.bin"
    dst = tmp_path / "out.bin"
    src.write_bytes(b"".join(k.to_bytes(32, "little") + n.to_bytes(32, "little") for k, n in recs))
    res = subprocess.run([str(exe), "g1", str(src), str(dst)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    raw = dst.read_bytes()
    assert len(raw) == 64 * len(recs)
    for i, (k, n) in enumerate(recs):
        vals = [int.from_bytes(raw[64 * i + 32 * j:64 * i + 32 * j + 32], "little") for j in range(2)]
        assert vals == list(_affine_mul(k << n, q)), (i, k, n)


def test_host_fq2_square_matches_integers(tmp_path):
    """The host Fq2 square (2 products) against the product a * a and against (a0^2 - a1^2,
    2 a0 a1) over the integers (u^2 = -1)."""
    exe = _build(tmp_path)
    q = MODULI["fq"]
    rng = random.Random(0xF02)
    recs = [(0, 0), (1, 0), (0, 1), (q - 1, q - 1), (q - 1, 1)] + [(rng.randrange(q), rng.randrange(q))
                                                                   for _ in range(500)]
    src = tmp_path / "in.bin"
    dst = tmp_path / "out.bin"
    src.write_bytes(b"".join(a.to_bytes(32, "little") + b.to_bytes(32, "little") for a, b in recs))
    res = subprocess.run([str(exe), "fq2", str(src), str(dst)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    raw = dst.read_bytes()
    assert len(raw) == 128 * len(recs)
    for i, (a0, a1) in enumerate(recs):
        vals = [int.from_bytes(raw[128 * i + 32 * j:128 * i + 32 * j + 32], "little") for j in range(4)]
        want = [(a0 * a0 - a1 * a1) % q, 2 * a0 * a1 % q]
        assert vals[:2] == want and vals[2:] == want, (i, a0, a1)
