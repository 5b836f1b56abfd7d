"""The separated Fq forms of field.cuh (square, a b + c d, a b - c d, a b with one Montgomery
reduction, and the lazily reduced Fq2 product) built for the host and checked against Python
integers: congruence with x * 2^-256 mod q and the lazy bound [0, 2q) on random inputs and
on the edges of [0, 2q)."""

import os
import random
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
Q = 21888242871839275222246405745257275088696311157297823662689037894645226208583
RINV = pow(2**256, -1, Q)


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return None


def test_separated_forms_match_integers(tmp_path):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not found")
    exe = tmp_path / "field_sos_host"
    res = subprocess.run([nvcc, "-std=c++17", "-O2", "-x", "cu", os.path.join(REPO, "tests", "field_sos_host.cu"),
                          "-o", str(exe)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    rng = random.Random(0x50515)
    edges = [0, 1, 2, Q - 1, Q, Q + 1, 2 * Q - 2, 2 * Q - 1, 2**32 - 1, 2**64 - 1, 2**128, 2**253, 2**254 - 1]
    edges = [e for e in edges if e < 2 * Q]
    recs = [tuple(rng.choice(edges) for _ in range(4)) for _ in range(400)]
    recs += [tuple(rng.randrange(2 * Q) for _ in range(4)) for _ in range(4000)]
    recs += [(2 * Q - 1,) * 4, (0,) * 4, (2 * Q - 1, 2 * Q - 1, 0, 2 * Q - 1)]
    src = tmp_path / "in.bin"
    dst = tmp_path / "out.bin"
    src.write_bytes(b"".join(x.to_bytes(32, "little") for r in recs for x in r))
    res = subprocess.run([str(exe), str(src), str(dst)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    raw = dst.read_bytes()
    assert len(raw) == 192 * len(recs)
    for i, (a, b, c, d) in enumerate(recs):
        sq, madd, msub, mul, f0, f1 = (int.from_bytes(raw[192 * i + 32 * k:192 * i + 32 * k + 32], "little")
                                       for k in range(6))
        for got, want in ((sq, a * a), (madd, a * b + c * d), (msub, a * b - c * d), (mul, a * b),
                          (f0, a * c - b * d), (f1, a * d + b * c)):
            assert got < 2 * Q, (i, a, b, c, d)
            assert got % Q == want * RINV % Q, (i, a, b, c, d)
