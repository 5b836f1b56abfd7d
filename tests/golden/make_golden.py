"""Generate golden vectors by running the unmodified reference (fzybravery/pyZKP).

Needs the reference: ``PYZKP_REFERENCE`` (a checkout or install directory) or the pip
install in ``baseline/_ref`` (tests/reference_env.py finds it):

    python tests/golden/make_golden.py

The reference imports ``py_ecc.optimized_bn128``, which is not installed offline,
so the test-only stand-in under ``oracle/py_ecc_shim`` is put on ``sys.path``.
Outputs (JSON, ints as hex strings) land beside this script and are committed;
the GPU machine never needs the reference.

Sources of each vector (paths within the reference):
  * NTT: crypto/poly/ntt.py evals_from_coeffs_on_roots / coeffs_from_evals_on_roots /
    evals_from_coeffs_on_coset / coeffs_from_evals_on_coset (:103-146), with the
    fixtures of tests/correctness/metal/test_runtime_metal_fr_ntt.py:22-24,44-45 and
    test_runtime_metal_fr_coset.py:22-25 (i^2 and (i+3)*7, n = 16, shift = 5) plus
    seeded uniform inputs.
  * MSM: runtime/kernels/cpu/kernels.py:_msm_g1_impl (:553-571) -> msm_pippenger
    (crypto/msm/pippenger.py:10-64) or msm_naive_g1 below the 64-point threshold, on
    the fixture of tests/correctness/metal/test_runtime_metal_g1_msm.py:33-37
    (scalars (i*12345+6789) mod r, bases (i+1)G), the n = 4096 workload, and edge cases.
"""

from __future__ import annotations

import hashlib
import importlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "tests"))

import reference_env  # noqa: E402

reference_env.add_to_path()

import numpy as np  # noqa: E402

from pyzkp_gb300 import synth  # noqa: E402

RN = importlib.import_module("crypto.poly.ntt")
from crypto.ecc.bn254 import G1_GENERATOR, G1_ZERO, g1_mul, g1_neg  # noqa: E402
from crypto.field.fr import FR_MODULUS  # noqa: E402
from py_ecc import optimized_bn128 as bn  # noqa: E402
from runtime.kernels.cpu.kernels import _msm_g1_impl  # noqa: E402


def hx(v: int) -> str:
    return hex(int(v))


def digest_ints(vals) -> str:
    h = hashlib.sha256()
    for v in vals:
        h.update(int(v).to_bytes(32, "little"))
    return h.hexdigest()


def digest_array(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u8").tobytes()).hexdigest()


def affine(p):
    x, y = bn.normalize(p)
    return [hx(int(x)), hx(int(y))]


def ntt_vectors() -> dict:
    out = {"source": "crypto/poly/ntt.py:103-146", "fixtures": [], "seeded": [], "pad_truncate": []}
    n = 16
    om = RN.omega_for_size(n)
    coeff = [i * i % FR_MODULUS for i in range(n)]
    ev = [(i + 3) * 7 % FR_MODULUS for i in range(n)]
    out["fixtures"].append({"name": "roots_evals_i2", "mode": 0, "n": n, "omega": hx(om), "shift": hx(1),
                            "input": [hx(v) for v in coeff],
                            "output": [hx(v) for v in RN.evals_from_coeffs_on_roots(coeff, n, om)]})
    out["fixtures"].append({"name": "roots_coeffs_i3x7", "mode": 1, "n": n, "omega": hx(om), "shift": hx(1),
                            "input": [hx(v) for v in ev],
                            "output": [hx(v) for v in RN.coeffs_from_evals_on_roots(ev, om)]})
    out["fixtures"].append({"name": "coset_evals_i2_shift5", "mode": 2, "n": n, "omega": hx(om), "shift": hx(5),
                            "input": [hx(v) for v in coeff],
                            "output": [hx(v) for v in RN.evals_from_coeffs_on_coset(coeff, n=n, omega=om, shift=5)]})
    out["fixtures"].append({"name": "coset_coeffs_i3x7_shift5", "mode": 3, "n": n, "omega": hx(om), "shift": hx(5),
                            "input": [hx(v) for v in ev],
                            "output": [hx(v) for v in RN.coeffs_from_evals_on_coset(ev, omega=om, shift=5)]})
    for log_n in (1, 2, 3, 5, 8, 10, 12):
        n = 1 << log_n
        seed = synth.seed_for(1, log_n)
        v = synth.fr_uniform(seed, n)
        vi = synth.limbs_to_ints(v)
        om = RN.omega_for_size(n)
        res = {
            0: RN.evals_from_coeffs_on_roots(vi, n, om),
            1: RN.coeffs_from_evals_on_roots(vi, om),
            2: RN.evals_from_coeffs_on_coset(vi, n=n, omega=om, shift=5),
            3: RN.coeffs_from_evals_on_coset(vi, omega=om, shift=5),
        }
        for mode, vals in res.items():
            rec = {"seed": seed, "n": n, "mode": mode, "omega": hx(om), "shift": hx(5 if mode >= 2 else 1),
                   "input_sha256": digest_array(v), "output_sha256": digest_ints(vals)}
            if n <= 32:
                rec["output"] = [hx(x) for x in vals]
            out["seeded"].append(rec)
    # forward ops pad (in_len < n) or truncate (in_len > n): runtime/kernels/cpu/kernels.py:181-188
    for in_len, n in ((700, 1024), (1500, 1024), (3, 8)):
        seed = 0xC0FFEE + 77 + in_len
        v = synth.fr_uniform(seed, in_len)
        vi = synth.limbs_to_ints(v)
        om = RN.omega_for_size(n)
        for mode, vals in ((0, RN.evals_from_coeffs_on_roots(vi, n, om)),
                           (2, RN.evals_from_coeffs_on_coset(vi, n=n, omega=om, shift=5))):
            out["pad_truncate"].append({"seed": seed, "in_len": in_len, "n": n, "mode": mode, "omega": hx(om),
                                        "shift": hx(5 if mode == 2 else 1), "input_sha256": digest_array(v),
                                        "output_sha256": digest_ints(vals)})
    return out


def msm_case(name: str, points, scalars, attrs=None, extra=None) -> dict:
    res = _msm_g1_impl(points, scalars, dict(attrs or {}))
    rec = {"name": name, "n": len(points),
           "bases": [affine(p) if p[2] != 0 else [hx(0), hx(0)] for p in points],
           "scalars": [hx(s) for s in scalars],
           "result": affine(res) if res[2] != 0 else [hx(0), hx(0)]}
    if extra:
        rec.update(extra)
    return rec


def msm_vectors() -> dict:
    out = {"source": "runtime/kernels/cpu/kernels.py:553-571 -> crypto/msm/pippenger.py:10-64", "cases": [],
           "workloads": []}
    # fixture of tests/correctness/metal/test_runtime_metal_g1_msm.py:33-37 (default window 16 there)
    n = 100
    scalars = [(i * 12345 + 6789) % FR_MODULUS for i in range(n)]
    points = [g1_mul(G1_GENERATOR, i + 1) for i in range(n)]
    out["cases"].append(msm_case("metal_test_fixture_n100", points, scalars, {"window_bits": 16}))

    # edge cases (small sizes run msm_naive_g1 below the 64-point threshold; the result is the same group element)
    g = G1_GENERATOR
    p5 = g1_mul(g, 5)
    out["cases"].append(msm_case("single_point", [p5], [12345]))
    out["cases"].append(msm_case("all_zero_scalars", [g1_mul(g, i + 2) for i in range(70)], [0] * 70))
    out["cases"].append(msm_case("scalars_r_minus_1_r_r_plus_1_2^256-1",
                                 [g1_mul(g, 3), g1_mul(g, 7), g1_mul(g, 11), g1_mul(g, 13)],
                                 [FR_MODULUS - 1, FR_MODULUS, FR_MODULUS + 1, (1 << 256) - 1]))
    pts = [g1_mul(g, 9)] * 40 + [g1_mul(g, 17)] * 40
    out["cases"].append(msm_case("duplicate_bases_same_scalar", pts, [424242] * 80))
    pts = [p5, g1_neg(p5)] * 40
    out["cases"].append(msm_case("p_and_minus_p", pts, [777] * 80))
    pts = [g1_mul(g, i + 1) if i % 3 else G1_ZERO for i in range(96)]
    sc = [(i * 0x1234567890ABCDEF1234567 + 99) % FR_MODULUS for i in range(96)]
    out["cases"].append(msm_case("infinity_bases", pts, sc))
    sc = [1] * 64 + [2] * 32 + [FR_MODULUS - 1] * 32
    pts = [g1_mul(g, 1000 + i) for i in range(128)]
    out["cases"].append(msm_case("skewed_small_digits", pts, sc))
    # top-window carries of a signed-digit decomposition: scalars with many ones in high bits
    sc = [FR_MODULUS - 1 - (1 << k) for k in range(0, 128, 2)]
    pts = [g1_mul(g, 31 + i) for i in range(len(sc))]
    out["cases"].append(msm_case("high_bits_set", pts, sc))

    # seeded workloads: bases [k_i]G with k_i uniform in [1, r), scalars uniform / witness-like
    for name, log_n, kind in (("uniform_n1024", 10, "uniform"), ("witness_like_n1024", 10, "witness"),
                              ("config0_n4096", 12, "uniform")):
        n = 1 << log_n
        cfg = 0 if name.startswith("config0") else 2
        seed = synth.seed_for(cfg, log_n)
        k = synth.base_dlogs(seed, n)
        s = synth.fr_uniform(seed, n) if kind == "uniform" else synth.fr_witness_like(seed, n)
        ki = synth.limbs_to_ints(k)
        si = synth.limbs_to_ints(s)
        points = tuple(bn.multiply(bn.G1, kk) for kk in ki)
        pts_aff = np.zeros((n, 8), dtype=np.uint64)
        for i, p in enumerate(points):
            x, y = bn.normalize(p)
            pts_aff[i, :4] = synth.int_to_limbs(int(x))
            pts_aff[i, 4:] = synth.int_to_limbs(int(y))
        res = _msm_g1_impl(points, si, {})
        out["workloads"].append({"name": name, "seed": seed, "n": n, "scalars": kind,
                                 "window_bits_reference": max(4, min(16, n.bit_length() - 2)),
                                 "bases_sha256": digest_array(pts_aff), "scalars_sha256": digest_array(s),
                                 "dlogs_sha256": digest_array(k), "result": affine(res)})
        print(name, "done", flush=True)
    return out


def main() -> None:
    ntt = ntt_vectors()
    with open(os.path.join(HERE, "ntt_reference.json"), "w") as f:
        json.dump(ntt, f, indent=1)
    print("ntt vectors written", flush=True)
    msm = msm_vectors()
    with open(os.path.join(HERE, "msm_reference.json"), "w") as f:
        json.dump(msm, f, indent=1)
    print("msm vectors written", flush=True)


if __name__ == "__main__":
    main()
