"""Locate and import the unmodified reference (fzybravery/pyZKP) for tests and fixture scripts.

The reference is pure Python with top-level packages ``crypto``, ``runtime``, ``protocols``
and ``frontend``; it imports ``py_ecc.optimized_bn128``, which tests replace with the
stand-in under ``oracle/py_ecc_shim``. Where it lives:

* ``PYZKP_REFERENCE`` (a checkout or an install directory), else
* ``baseline/_ref`` in this repository: the reference installed with pip ``--target``
  (not committed; it travels with the working tree to machines that run the GPU tests).

Tests that need it skip when neither is present.
"""

from __future__ import annotations

import os
import random
import secrets
import sys
from contextlib import contextmanager

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(REPO, "oracle", "py_ecc_shim")
FR_MODULUS = 21888242871839275222246405745257275088548364400416034343698204186575808495617


def reference_root():
    """Directory holding the reference's ``runtime`` package, or None."""
    for p in (os.environ.get("PYZKP_REFERENCE"), os.path.join(REPO, "baseline", "_ref")):
        if p and os.path.isdir(os.path.join(p, "runtime")) and os.path.isdir(os.path.join(p, "protocols")):
            return p
    return None


def add_to_path() -> str:
    """Put the py_ecc stand-in and the reference on ``sys.path``; returns the reference root.

    Raises ``ImportError`` when the reference is not available.
    """
    root = reference_root()
    if root is None:
        raise ImportError("reference not found: set PYZKP_REFERENCE or install it into baseline/_ref")
    sys.dont_write_bytecode = True
    for p in (root, SHIM):
        if p not in sys.path:
            sys.path.insert(0, p)
    return root


def require():
    """``add_to_path`` for pytest: skips the calling test (or module) when the reference is absent."""
    import pytest

    try:
        return add_to_path()
    except ImportError as e:
        pytest.skip(str(e), allow_module_level=True)


def runtime():
    """The reference's runtime types in one namespace (skips the caller when absent):
    Graph / Node (runtime/ir/graph.py), Buffer / Device / Backend / DType (runtime/ir/types.py),
    OpType (runtime/ir/ops.py), Executor, KernelRegistry, RuntimeConfig, CPUContext,
    MemoryPool (runtime/memory.py) and register_cpu_kernels."""
    import types

    require()
    import runtime as rt
    import runtime.ir as ir
    from runtime.kernels.cpu import register_cpu_kernels
    from runtime.memory import MemoryPool

    return types.SimpleNamespace(
        ir=ir, Graph=ir.Graph, Node=ir.Node, Buffer=ir.Buffer, Device=ir.Device, Backend=ir.Backend, DType=ir.DType,
        OpType=ir.OpType, Executor=rt.Executor, KernelRegistry=rt.KernelRegistry, RuntimeConfig=rt.RuntimeConfig,
        CPUContext=rt.CPUContext, MemoryPool=MemoryPool, register_cpu_kernels=register_cpu_kernels)


def seeded_fr_rand(seed: int):
    """A drop-in for ``crypto.field.fr.fr_rand`` (crypto/field/fr.py:37-42) drawing from ``random.Random(seed)``."""
    rng = random.Random(seed)

    def fr_rand(nonzero: bool = True) -> int:
        while True:
            x = rng.randrange(FR_MODULUS)
            if nonzero and x == 0:
                continue
            return x

    fr_rand.rng = rng
    return fr_rand


@contextmanager
def seeded_plonk_randomness(seed: int):
    """Make the reference's PLONK setup and prover deterministic.

    The PLONK code draws from ``secrets.randbelow`` (protocols/plonk/domain.py:46-59 for the
    coset factors k1, k2; protocols/plonk/prove.py:325 for the quotient coset shift) and
    from ``fr_rand`` (crypto/kzg/cpu_ref.py:31 for the SRS trapdoor). Inside this context
    both come from one ``random.Random(seed)``.
    """
    import importlib

    kzg = importlib.import_module("crypto.kzg.cpu_ref")
    rng = random.Random(seed)
    old_randbelow, old_fr_rand = secrets.randbelow, kzg.fr_rand

    def randbelow(k: int) -> int:
        return rng.randrange(k)

    def fr_rand(nonzero: bool = True) -> int:
        while True:
            x = rng.randrange(FR_MODULUS)
            if nonzero and x == 0:
                continue
            return x

    secrets.randbelow = randbelow
    kzg.fr_rand = fr_rand
    try:
        yield rng
    finally:
        secrets.randbelow = old_randbelow
        kzg.fr_rand = old_fr_rand
