"""Build the zkgpu shared library (CUDA, sm_103a) in-tree.

``python -m pyzkp_gb300.build`` compiles every ``csrc/*.cu`` translation unit in
parallel with nvcc for ``sm_103a`` and links ``pyzkp_gb300/_lib/libzkgpu.so``
(CUDA runtime linked statically, so the library needs only the driver).
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from typing import List

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(LIB_DIR, "obj")
LIB_PATH = os.path.join(LIB_DIR, "libzkgpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources() -> List[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers_mtime() -> float:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))]
    hs.append(os.path.join(INCLUDE, "zkgpu.h"))
    return max(os.path.getmtime(h) for h in hs)


def _compile(src: str, extra: List[str], obj_dir: str) -> str:
    obj = os.path.join(obj_dir, os.path.basename(src) + ".o")
    newest = max(os.path.getmtime(src), _headers_mtime())
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest:
        return obj
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + extra + ["-c", src, "-o", obj + ".tmp"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    if res.stderr.strip():
        sys.stderr.write(res.stderr)
    os.replace(obj + ".tmp", obj)
    return obj


def build(force: bool = False, verbose_ptxas: bool = False, defines: List[str] = (), lib_path: str = "") -> str:
    """Compile and link; ``defines`` (e.g. ["ZK_MUL_STYLE=1"]) build a variant into ``lib_path``."""
    obj_dir, out_path = OBJ_DIR, LIB_PATH
    if defines or lib_path:
        tag = "_".join(d.replace("=", "") for d in defines) or "custom"
        obj_dir = os.path.join(LIB_DIR, "obj_" + tag)
        out_path = lib_path or os.path.join(LIB_DIR, f"libzkgpu_{tag}.so")
    os.makedirs(obj_dir, exist_ok=True)
    if force:
        for f in os.listdir(obj_dir):
            os.remove(os.path.join(obj_dir, f))
    extra = (["-Xptxas", "-v"] if verbose_ptxas else []) + [f"-D{d}" for d in defines]
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, obj_dir), srcs))
    if force or not os.path.exists(out_path) or os.path.getmtime(out_path) < max(os.path.getmtime(o) for o in objs):
        tmp = out_path + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, out_path)
    return out_path


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
