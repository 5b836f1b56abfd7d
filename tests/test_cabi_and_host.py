"""CPU-only checks of the C ABI library and the host-side logic (no GPU compute)."""

import os
import re
import subprocess

import numpy as np
import pytest

from pyzkp_gb300 import _native as N
from pyzkp_gb300 import plugin, synth

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_symbols():
    with open(os.path.join(REPO, "include", "zkgpu.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(zk_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = N.load()
    declared = _header_symbols()
    assert declared, "no declarations parsed"
    for name in declared:
        assert hasattr(L, name), name
    assert set(declared) == set(N.EXPORTED_SYMBOLS)
    # dynamic symbol table of the .so (no device needed)
    out = subprocess.run(["nm", "-D", "--defined-only", N.LIB_PATH], capture_output=True, text=True).stdout
    for name in declared:
        assert re.search(rf"\bT {name}\b", out), name


def test_header_is_plain_c_and_links(tmp_path):
    """include/zkgpu.h compiles as strict C99 and every declared entry point links against the
    library (what a cgo / FFI binding of the reference's side would do); nothing is called."""
    names = _header_symbols()
    src = tmp_path / "abi.c"
    refs = ",\n    ".join(f"(void (*)(void)){n}" for n in names)
    src.write_text('#include "zkgpu.h"\n#include <stdio.h>\n'
                   f"void (*const zk_all[])(void) = {{\n    {refs}\n}};\n"
                   "int main(void) { printf(\"%d\\n\", (int)(sizeof zk_all / sizeof zk_all[0])); return 0; }\n")
    lib_dir = os.path.dirname(N.LIB_PATH)
    lib_name = os.path.basename(N.LIB_PATH)[3:-3]  # libX.so -> X
    exe = tmp_path / "abi"
    res = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic",
                          "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe), "-L", lib_dir,
                          f"-l{lib_name}", f"-Wl,-rpath,{lib_dir}"], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    assert len(names) > 60


def test_null_arguments_map_to_value_error():
    L = N.load()
    with pytest.raises(ValueError):
        N.check(L.zk_ctx_sync(None), "zk_ctx_sync")
    assert "null" in L.zk_last_error().decode()
    assert L.zk_version() == 1


def test_synth_generators_are_deterministic_and_in_range():
    a = synth.fr_uniform(123, 1000)
    b = synth.fr_uniform(123, 1000)
    assert (a == b).all()
    ints = synth.limbs_to_ints(a)
    assert all(0 <= v < synth.FR_MODULUS for v in ints) and len(set(ints)) == 1000
    k = synth.base_dlogs(123, 500)
    assert all(0 < v < synth.FR_MODULUS for v in synth.limbs_to_ints(k))
    w = synth.limbs_to_ints(synth.fr_witness_like(7, 20000))
    frac01 = sum(1 for v in w if v in (0, 1)) / len(w)
    frac64 = sum(1 for v in w if 1 < v < (1 << 64)) / len(w)
    assert 0.08 < frac01 < 0.12 and 0.55 < frac64 < 0.65
    assert synth.seed_for(2, 20) == 0xC0FFEE + 2020


def test_plugin_host_helpers():
    vals = [0, 1, synth.FR_MODULUS - 1, synth.FR_MODULUS + 5, -1]
    raw = np.frombuffer(plugin._ints_to_bytes(vals), dtype=np.uint8)
    back = plugin._bytes_to_ints(raw, len(vals))
    assert back == [v % synth.FR_MODULUS for v in vals]
    assert plugin._log2_exact(1) == 0 and plugin._log2_exact(1 << 20) == 20
    for bad in (0, 3, 1 << 29):
        with pytest.raises(ValueError):
            plugin._log2_exact(bad)
    gb = plugin.GpuBuffer(dtype="fr_mont_u64x4", n=7, mtl_buffer=None)
    assert len(gb) == 7


def test_points_to_affine_array_handles_infinity_and_projective():
    import sys

    sys.path.insert(0, os.path.join(REPO, "oracle", "py_ecc_shim"))
    from py_ecc import optimized_bn128 as bn

    pts = [bn.G1, bn.Z1, bn.multiply(bn.G1, 7), (bn.FQ(1), bn.FQ(2), bn.FQ(1))]
    arr = plugin.points_to_affine_array(pts)
    assert arr.shape == (4, 8)
    assert synth.limbs_to_ints(arr[:, :4]) == [1, 0, int(bn.normalize(pts[2])[0]), 1]
    assert synth.limbs_to_ints(arr[:, 4:]) == [2, 0, int(bn.normalize(pts[2])[1]), 2]
