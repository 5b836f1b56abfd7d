"""Seeded synthetic inputs for the BN254 MSM / Fr NTT workloads.

Every workload is synthetic (the reference measures on no dataset): scalars and
NTT inputs are uniform field elements drawn from ``numpy.random.Generator(PCG64)``.
Elements are returned as ``uint64[n, 4]`` little-endian limbs of the canonical
value (the byte layout of ``runtime/kernels/cpu/kernels.py:135-141`` before the
Montgomery conversion).

Draw rule (fixed, so the GPU machine regenerates the same inputs from a seed):
candidates are 4 uint64 words per element with the top word masked to 62 bits
(a 254-bit value); a candidate is accepted iff it is below the bound; rejected
candidates are redrawn in further batches, accepted values are kept in draw order.
"""

from __future__ import annotations

import numpy as np

FR_MODULUS = 21888242871839275222246405745257275088548364400416034343698204186575808495617
FQ_MODULUS = 21888242871839275222246405745257275088696311157297823662689037894645226208583

_MASK62 = np.uint64((1 << 62) - 1)


def seed_for(family: int, log_n: int) -> int:
    """Seed of a synthetic input: 0xC0FFEE + 1000*family + log2(n), with the workload family
    0 = the 4096-point MSM case, 1 = NTTs, 2 = MSM sweeps, 3 = batches, 5 = PLONK quotient,
    6 = G2 MSMs."""
    return 0xC0FFEE + 1000 * int(family) + int(log_n)


def int_to_limbs(v: int) -> np.ndarray:
    return np.array([(v >> (64 * i)) & 0xFFFFFFFFFFFFFFFF for i in range(4)], dtype=np.uint64)


def _less_than(c: np.ndarray, bound: int) -> np.ndarray:
    """Row-wise c < bound for c of shape (m, 4) uint64 limbs (little endian)."""
    b = int_to_limbs(bound)
    lt = np.zeros(c.shape[0], dtype=bool)
    eq = np.ones(c.shape[0], dtype=bool)
    for limb in (3, 2, 1, 0):
        lt |= eq & (c[:, limb] < b[limb])
        eq &= c[:, limb] == b[limb]
    return lt


def uniform_below(rng: np.random.Generator, n: int, bound: int, *, nonzero: bool = False) -> np.ndarray:
    """n values uniform in [0, bound) (or [1, bound) if nonzero) as uint64[n, 4]."""
    out = np.empty((n, 4), dtype=np.uint64)
    filled = 0
    while filled < n:
        need = n - filled
        batch = max(64, int(need * 1.4) + 16)
        c = rng.integers(0, np.iinfo(np.uint64).max, size=(batch, 4), dtype=np.uint64, endpoint=True)
        c[:, 3] &= _MASK62
        ok = _less_than(c, bound)
        if nonzero:
            ok &= (c != 0).any(axis=1)
        acc = c[ok][:need]
        out[filled:filled + acc.shape[0]] = acc
        filled += acc.shape[0]
    return out


def fr_uniform(seed: int, n: int) -> np.ndarray:
    """n scalars uniform in [0, r)."""
    return uniform_below(np.random.Generator(np.random.PCG64(seed)), n, FR_MODULUS)


def fr_witness_like(seed: int, n: int) -> np.ndarray:
    """Witness-like scalar mix: 10% in {0, 1} (half each), 60% uniform below 2^64, the rest uniform in [0, r)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    kind = rng.random(n)
    full = uniform_below(rng, n, FR_MODULUS)
    small = rng.integers(0, np.iinfo(np.uint64).max, size=n, dtype=np.uint64, endpoint=True)
    bit = rng.integers(0, 2, size=n, dtype=np.uint64)
    out = full.copy()
    sel01 = kind < 0.10
    sel64 = (kind >= 0.10) & (kind < 0.70)
    out[sel01] = 0
    out[sel01, 0] = bit[sel01]
    out[sel64] = 0
    out[sel64, 0] = small[sel64]
    return out


def base_dlogs(seed: int, n: int) -> np.ndarray:
    """Discrete logs k_i uniform in [1, r) of the MSM bases P_i = [k_i]G."""
    return uniform_below(np.random.Generator(np.random.PCG64(seed ^ 0x5EED_BA5E)), n, FR_MODULUS, nonzero=True)


def limbs_to_ints(a: np.ndarray) -> list:
    """uint64[n, 4] -> list of Python ints."""
    b = np.ascontiguousarray(a, dtype="<u8").tobytes()
    return [int.from_bytes(b[32 * i:32 * i + 32], "little") for i in range(a.shape[0])]


def ints_to_limbs(vals) -> np.ndarray:
    """Sequence of non-negative ints < 2^256 -> uint64[n, 4]."""
    buf = b"".join(int(v).to_bytes(32, "little") for v in vals)
    return np.frombuffer(buf, dtype="<u8").reshape(-1, 4).astype(np.uint64)
