"""ctypes front-end of the C oracle (``oracle/bn254_oracle.c``).

ORACLE / TEST INFRASTRUCTURE. Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of ``bench.py`` may import this module. It is the checker the
CUDA path is compared against, never the product path.

Each function names the reference function it restates (paths within
fzybravery/pyZKP). Arrays are numpy ``uint64`` with 4 limbs per field element
(canonical, little endian) and 8 limbs per affine G1 point, (0, 0) = infinity.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "bn254_oracle.c")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")

FR_MODULUS = 21888242871839275222246405745257275088548364400416034343698204186575808495617
FQ_MODULUS = 21888242871839275222246405745257275088696311157297823662689037894645226208583
ROOT_2_28 = 19103219067921713944291392827692070036145651957329286315305642004821462161904  # crypto/poly/ntt.py:8

# NTT op modes of orc_ntt_op
EVALS_FROM_COEFFS_ON_ROOTS = 0
COEFFS_FROM_EVALS_ON_ROOTS = 1
EVALS_FROM_COEFFS_ON_COSET = 2
COEFFS_FROM_EVALS_ON_COSET = 3

_lib: Optional[ctypes.CDLL] = None


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (portable C, pthreads); returns the .so path."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(SRC):
        tmp = LIB_PATH + ".tmp"
        subprocess.check_call(["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-o", tmp, SRC, "-lpthread"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        L.orc_ntt_op.argtypes = [ctypes.c_int, P, ctypes.c_size_t, P, ctypes.c_size_t, P, P, ctypes.c_int]
        L.orc_msm_pippenger.argtypes = [P, P, ctypes.c_size_t, ctypes.c_int, P, ctypes.c_int]
        L.orc_g1_fixed_base_mul.argtypes = [P, P, ctypes.c_size_t, P, ctypes.c_int]
        L.orc_g1_mul.argtypes = [P, P, P]
        L.orc_g1_add.argtypes = [P, P, P]
        L.orc_fr_dot.argtypes = [P, P, ctypes.c_size_t, P]
        L.orc_to_from_mont.argtypes = [ctypes.c_int, ctypes.c_int, P, P, ctypes.c_size_t, ctypes.c_int]
        L.orc_g2_mul.argtypes = [P, P, P]
        L.orc_g2_add.argtypes = [P, P, P]
        L.orc_g2_fixed_base_mul.argtypes = [P, P, ctypes.c_size_t, P, ctypes.c_int]
        L.orc_g2_msm.argtypes = [P, P, ctypes.c_size_t, P, ctypes.c_int]
        for f in (L.orc_ntt_op, L.orc_msm_pippenger, L.orc_g1_fixed_base_mul, L.orc_g1_mul, L.orc_g1_add,
                  L.orc_fr_dot, L.orc_to_from_mont, L.orc_num_threads, L.orc_g2_mul, L.orc_g2_add,
                  L.orc_g2_fixed_base_mul, L.orc_g2_msm):
            f.restype = ctypes.c_int
        _lib = L
    return _lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def _limbs(v: int, n: int = 4) -> np.ndarray:
    return np.array([(v >> (64 * i)) & 0xFFFFFFFFFFFFFFFF for i in range(n)], dtype=np.uint64)


def num_threads() -> int:
    return int(lib().orc_num_threads())


def omega_for_size(n: int) -> int:
    """crypto/poly/ntt.py:13-26: omega_n = ROOT_2_28^(2^(28 - log2 n))."""
    if n <= 0 or n & (n - 1):
        raise ValueError("n must be a power of two")
    logn = n.bit_length() - 1
    if logn > 28:
        raise ValueError("domain too large for BN254 root of unity")
    return pow(ROOT_2_28, 1 << (28 - logn), FR_MODULUS)


def ntt_op(mode: int, values: np.ndarray, n: int, omega: int, shift: int = 1, nthreads: int = 0) -> np.ndarray:
    """One of the four transforms of crypto/poly/ntt.py:103-146 (see mode constants).

    ``values``: uint64[m, 4] canonical; forward modes pad/truncate to n, inverse
    modes need m == n. Returns uint64[n, 4] canonical.
    """
    v = np.ascontiguousarray(values, dtype=np.uint64).reshape(-1, 4)
    out = np.zeros((n, 4), dtype=np.uint64)
    om = _limbs(omega % FR_MODULUS)
    sh = _limbs(shift % FR_MODULUS)
    rc = lib().orc_ntt_op(int(mode), _ptr(v), v.shape[0], _ptr(out), int(n), _ptr(om), _ptr(sh), int(nthreads))
    if rc != 0:
        raise ValueError(f"orc_ntt_op failed ({rc})")
    return out


def msm_pippenger(bases: np.ndarray, scalars: np.ndarray, window_bits: int, nthreads: int = 0) -> np.ndarray:
    """crypto/msm/pippenger.py:10-64. bases uint64[n, 8] affine canonical, scalars uint64[n, 4]."""
    b = np.ascontiguousarray(bases, dtype=np.uint64).reshape(-1, 8)
    s = np.ascontiguousarray(scalars, dtype=np.uint64).reshape(-1, 4)
    if b.shape[0] != s.shape[0]:
        raise ValueError("points and scalars length mismatch")
    out = np.zeros(8, dtype=np.uint64)
    rc = lib().orc_msm_pippenger(_ptr(b), _ptr(s), b.shape[0], int(window_bits), _ptr(out), int(nthreads))
    if rc != 0:
        raise ValueError(f"orc_msm_pippenger failed ({rc})")
    return out


def msm_window_rule(n: int) -> int:
    """runtime/kernels/cpu/kernels.py:559: max(4, min(16, bitlen(n) - 2))."""
    return max(4, min(16, int(n).bit_length() - 2))


def g1_fixed_base_mul(point: np.ndarray, k: np.ndarray, nthreads: int = 0) -> np.ndarray:
    """[k_i] P for many k_i (the synthetic bases [k_i]G)."""
    p = np.ascontiguousarray(point, dtype=np.uint64).reshape(8)
    kk = np.ascontiguousarray(k, dtype=np.uint64).reshape(-1, 4)
    out = np.zeros((kk.shape[0], 8), dtype=np.uint64)
    rc = lib().orc_g1_fixed_base_mul(_ptr(p), _ptr(kk), kk.shape[0], _ptr(out), int(nthreads))
    if rc != 0:
        raise ValueError(f"orc_g1_fixed_base_mul failed ({rc})")
    return out


def g1_mul(point: np.ndarray, k: int) -> np.ndarray:
    p = np.ascontiguousarray(point, dtype=np.uint64).reshape(8)
    kk = _limbs(k % FR_MODULUS)
    out = np.zeros(8, dtype=np.uint64)
    lib().orc_g1_mul(_ptr(p), _ptr(kk), _ptr(out))
    return out


def g1_add(p: np.ndarray, q: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(p, dtype=np.uint64).reshape(8)
    b = np.ascontiguousarray(q, dtype=np.uint64).reshape(8)
    out = np.zeros(8, dtype=np.uint64)
    lib().orc_g1_add(_ptr(a), _ptr(b), _ptr(out))
    return out


def fr_dot(a: np.ndarray, b: np.ndarray) -> int:
    x = np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 4)
    y = np.ascontiguousarray(b, dtype=np.uint64).reshape(-1, 4)
    out = np.zeros(4, dtype=np.uint64)
    lib().orc_fr_dot(_ptr(x), _ptr(y), x.shape[0], _ptr(out))
    return int.from_bytes(out.astype("<u8").tobytes(), "little")


def to_mont(values: np.ndarray, field: str = "fr") -> np.ndarray:
    v = np.ascontiguousarray(values, dtype=np.uint64).reshape(-1, 4)
    out = np.zeros_like(v)
    lib().orc_to_from_mont(1 if field == "fq" else 0, 1, _ptr(v), _ptr(out), v.shape[0], 0)
    return out


def from_mont(values: np.ndarray, field: str = "fr") -> np.ndarray:
    v = np.ascontiguousarray(values, dtype=np.uint64).reshape(-1, 4)
    out = np.zeros_like(v)
    lib().orc_to_from_mont(1 if field == "fq" else 0, 0, _ptr(v), _ptr(out), v.shape[0], 0)
    return out


G1_GENERATOR = np.array([1, 0, 0, 0, 2, 0, 0, 0], dtype=np.uint64)


def msm_known_answer(dlogs: np.ndarray, scalars: np.ndarray) -> np.ndarray:
    """Independent exact check for bases P_i = [k_i]G: MSM(P, s) = [sum k_i s_i mod r] G."""
    return g1_mul(G1_GENERATOR, fr_dot(dlogs, scalars))


# G2 generator (crypto/ecc/bn254.py G2_GENERATOR = py_ecc G2; the EIP-197 constants):
# x = x0 + x1 u, y = y0 + y1 u as 16 limbs (x0, x1, y0, y1)
G2_GENERATOR = np.concatenate([_limbs(v) for v in (
    10857046999023057135944570762232829481370756359578518086990519993285655852781,
    11559732032986387107991004021392285783925812861821192530917403151452391805634,
    8495653923123431417604973247489272438418190587263600148770280649306958101930,
    4082367875863433681332203403145435568316851327593401208105741076214120093531)])


def g2_mul(point: np.ndarray, k: int) -> np.ndarray:
    """[k] P on G2 (affine canonical 16 limbs; all zero = infinity)."""
    p = np.ascontiguousarray(point, dtype=np.uint64).reshape(16)
    kk = _limbs(k % FR_MODULUS)
    out = np.zeros(16, dtype=np.uint64)
    lib().orc_g2_mul(_ptr(p), _ptr(kk), _ptr(out))
    return out


def g2_add(p: np.ndarray, q: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(p, dtype=np.uint64).reshape(16)
    b = np.ascontiguousarray(q, dtype=np.uint64).reshape(16)
    out = np.zeros(16, dtype=np.uint64)
    lib().orc_g2_add(_ptr(a), _ptr(b), _ptr(out))
    return out


def g2_fixed_base_mul(point: np.ndarray, k: np.ndarray, nthreads: int = 0) -> np.ndarray:
    """[k_i] P on G2 for many k_i (synthetic G2 bases [k_i]G2)."""
    p = np.ascontiguousarray(point, dtype=np.uint64).reshape(16)
    kk = np.ascontiguousarray(k, dtype=np.uint64).reshape(-1, 4)
    out = np.zeros((kk.shape[0], 16), dtype=np.uint64)
    rc = lib().orc_g2_fixed_base_mul(_ptr(p), _ptr(kk), kk.shape[0], _ptr(out), int(nthreads))
    if rc != 0:
        raise ValueError(f"orc_g2_fixed_base_mul failed ({rc})")
    return out


def g2_msm(bases: np.ndarray, scalars: np.ndarray, nthreads: int = 0) -> np.ndarray:
    """MSM_G2 (runtime/kernels/cpu/kernels.py:574-582) as the plain sum of [s_i] P_i."""
    b = np.ascontiguousarray(bases, dtype=np.uint64).reshape(-1, 16)
    s = np.ascontiguousarray(scalars, dtype=np.uint64).reshape(-1, 4)
    if b.shape[0] != s.shape[0]:
        raise ValueError("points and scalars length mismatch")
    out = np.zeros(16, dtype=np.uint64)
    rc = lib().orc_g2_msm(_ptr(b), _ptr(s), b.shape[0], _ptr(out), int(nthreads))
    if rc != 0:
        raise ValueError(f"orc_g2_msm failed ({rc})")
    return out


def g2_msm_known_answer(dlogs: np.ndarray, scalars: np.ndarray) -> np.ndarray:
    """For G2 bases [k_i]G2: MSM = [sum k_i s_i mod r] G2."""
    return g2_mul(G2_GENERATOR, fr_dot(dlogs, scalars))


def g2_to_ints(p: np.ndarray):
    """16 limbs -> ((x0, x1), (y0, y1)) canonical ints."""
    b = np.ascontiguousarray(p, dtype="<u8").tobytes()
    v = [int.from_bytes(b[32 * i:32 * i + 32], "little") for i in range(4)]
    return (v[0], v[1]), (v[2], v[3])


def affine_to_ints(p: np.ndarray):
    b = np.ascontiguousarray(p, dtype="<u8").tobytes()
    return int.from_bytes(b[:32], "little"), int.from_bytes(b[32:64], "little")


def plonk_t_quotient_evals(vecs, n: int, omega_m: int, shift: int, shift_n: int, alpha: int, beta: int,
                           gamma: int, k1: int, k2: int):
    """runtime/kernels/cpu/kernels.py:_plonk_t_quotient_evals restated with plain ints (small m):
    vecs = [a, b, c, z, pi, ql, qr, qm, qo, qc, s1, s2, s3, zshift, l1] (lists of ints).
    Returns (num, zh)."""
    r = FR_MODULUS
    a_, b_, c_, z_, pi_, ql, qr, qm, qo, qc, s1, s2, s3, zs, l1 = vecs
    m = len(a_)
    alpha, beta, gamma, k1, k2 = (v % r for v in (alpha, beta, gamma, k1, k2))
    u = pow(omega_m % r, n, r)
    x, upow = shift % r, 1
    num, zh = [], []
    for i in range(m):
        a, b, c, z = a_[i] % r, b_[i] % r, c_[i] % r, z_[i] % r
        gate = (ql[i] * a + qr[i] * b + qm[i] * a * b + qo[i] * c + qc[i] + pi_[i]) % r
        left = (a + beta * x + gamma) * (b + beta * k1 * x + gamma) * (c + beta * k2 * x + gamma) * z % r
        right = (a + beta * s1[i] + gamma) * (b + beta * s2[i] + gamma) * (c + beta * s3[i] + gamma) * zs[i] % r
        boundary = (z - 1) * l1[i] % r
        num.append((gate + alpha * (left - right) + alpha * alpha * boundary) % r)
        zh.append((shift_n * upow - 1) % r)
        upow = upow * u % r
        x = x * omega_m % r
    return num, zh
