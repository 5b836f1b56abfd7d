"""The library's host-side field code (pyzkp_gb300/csrc/host_field.hpp: the final MSM
combination and the NTT tables use it) built for the host and checked against Python
integers for Fr and Fq: Montgomery product, inverse (of a Montgomery form), sum, difference
and conversion."""

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


@pytest.mark.parametrize("name", ["fr", "fq"])
def test_host_field_matches_integers(tmp_path, name):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "host_field_check"
    res = subprocess.run([cxx, "-std=c++17", "-O2", os.path.join(REPO, "tests", "host_field_check.cpp"), "-o",
                          str(exe)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
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
