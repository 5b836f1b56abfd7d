"""Test-only stand-in for the third-party ``py_ecc`` package (not installed here).

ORACLE / TEST INFRASTRUCTURE. Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import anything under ``oracle/``.

The reference (fzybravery/pyZKP) imports ``from py_ecc import optimized_bn128``
(crypto/field/fr.py:5, crypto/ecc/bn254.py:5, crypto/pairing/bn254.py:5,
runtime/metal/msm.py:16,37).  py_ecc is unpinned there (README.md:75 names it
without a version) and absent offline, so this package provides the surface the
reference uses, written from the BN254 mathematics (not from py_ecc's source).
"""

from . import optimized_bn128  # noqa: F401

__all__ = ["optimized_bn128"]
