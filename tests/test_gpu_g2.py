"""GPU parity of the G2 MSM (zk_msm_g2, zk_msm_g2_batch) through the C ABI.

MSM_G2 is CPU-only in the reference (_msm_g2_impl, runtime/kernels/cpu/kernels.py:574-582,
used for Groth16's b_query_g2 * w, protocols/groth16/prove.py:76-77). Results are checked
bit-exactly against the oracle: its plain sum of scalar multiples (oracle/bn254_oracle.c
orc_g2_msm, pinned against the py_ecc stand-in) and the dlog identity
MSM([k_i]G2, s) = [sum k_i s_i]G2.
"""

import numpy as np
import pytest

from oracle import oracle as O
from pyzkp_gb300 import synth

pytestmark = pytest.mark.gpu


def _g2(p: np.ndarray):
    return None if not p.any() else O.g2_to_ints(p)


def _dev(ctx, s: np.ndarray, mont: bool = True):
    d = ctx.to_device(s if s.shape[0] else np.zeros((1, 4), dtype=np.uint64))
    if mont and s.shape[0]:
        ctx.fr_to_mont(d, d, s.shape[0])
    return d


@pytest.mark.parametrize("kind", ["uniform", "witness"])
def test_msm_g2_matches_oracle(gpu_ctx, kind):
    n = 3000
    k = synth.base_dlogs(4100, n)
    k[11] = 0  # an infinity base
    xy = O.g2_fixed_base_mul(O.G2_GENERATOR, k)
    s = synth.fr_uniform(4101, n) if kind == "uniform" else synth.fr_witness_like(4101, n)
    exp = _g2(O.g2_msm(xy, s))
    assert exp == _g2(O.g2_msm_known_answer(k, s))
    b = gpu_ctx.bases_g2_from_host(xy)
    ds = _dev(gpu_ctx, s)
    for c in (0, 4, 7, 11, 16):
        assert gpu_ctx.msm_g2(b, ds, n, window_bits=c) == exp, c
    dc = _dev(gpu_ctx, s, mont=False)
    assert gpu_ctx.msm_g2(b, dc, n, scalars_mont=False) == exp
    m = 1234
    assert gpu_ctx.msm_g2(b, ds, m, offset=17) == _g2(O.g2_msm_known_answer(k[17:17 + m], s[:m]))


def test_msm_g2_edge_cases_and_batch(gpu_ctx):
    n = 1 << 13
    k = synth.base_dlogs(4200, n)
    xy = O.g2_fixed_base_mul(O.G2_GENERATOR, k)
    b = gpu_ctx.bases_g2_from_host(xy)
    # P + (-P) = infinity; repeated points (doubling inside a bucket)
    neg1 = synth.ints_to_limbs([O.FR_MODULUS - 1])
    one = synth.ints_to_limbs([1])
    two_pts = gpu_ctx.bases_g2_from_host(np.stack([xy[0], xy[0]]))
    assert gpu_ctx.msm_g2(two_pts, _dev(gpu_ctx, np.concatenate([one, neg1])), 2) is None
    assert gpu_ctx.msm_g2(two_pts, _dev(gpu_ctx, np.concatenate([one, one])), 2) == _g2(
        O.g2_mul(xy[0], 2))
    assert gpu_ctx.msm_g2(b, _dev(gpu_ctx, synth.fr_uniform(1, 4)), 0) is None
    sizes = [0, 1, 100, 4096, n, 777]
    scal = [synth.fr_uniform(4300 + j, m) for j, m in enumerate(sizes)]
    got = gpu_ctx.msm_g2_batch(b, [_dev(gpu_ctx, x) for x in scal], sizes)
    assert got == [None if m == 0 else _g2(O.g2_msm_known_answer(k[:m], x)) for m, x in zip(sizes, scal)]
    # G1 and G2 handles are not interchangeable
    g1 = gpu_ctx.bases_from_host(O.g1_fixed_base_mul(O.G1_GENERATOR, k[:4]))
    with pytest.raises(ValueError):
        gpu_ctx.msm_g2(g1, _dev(gpu_ctx, scal[2][:4]), 4)
    with pytest.raises(ValueError):
        gpu_ctx.msm_g1(b, _dev(gpu_ctx, scal[2][:4]), 4)
    with pytest.raises(ValueError):
        gpu_ctx.msm_g2(b, _dev(gpu_ctx, scal[2]), n + 1)


def test_g2_fixed_base_mul_matches_oracle(gpu_ctx):
    n = 2000
    k = synth.base_dlogs(4400, n)
    k[9] = 0  # [0]G2 = infinity
    dk = gpu_ctx.to_device(k)
    out = gpu_ctx.alloc(n * 128)
    gen = O.g2_to_ints(O.G2_GENERATOR)
    gpu_ctx.g2_fixed_base_mul(gen, dk, n, out)
    got = out.download().view("<u8").reshape(n, 16)
    assert (got == O.g2_fixed_base_mul(O.G2_GENERATOR, k)).all()


def test_msm_g2_glv_edge_scalars(gpu_ctx):
    """G2 MSMs use the GLV split with phi(x, y) = (beta^2 x, y) = [lambda](x, y) on the twist:
    scalars at the ends of the range, lambda, its negation and rounding midpoints."""
    R = O.FR_MODULUS
    lam = 0xB3C4D79D41A917585BFC41088D8DAAA78B17EA66B99C90DD
    vals = [0, 1, 2, R - 1, R - 2, lam, R - lam, lam + 1, (R - 1) // 2, (R + 1) // 2, R // 3, (2 * R) // 3,
            (1 << 127) - 1, 1 << 127, (1 << 253) - 1]
    vals += [int(x) for x in synth.limbs_to_ints(synth.fr_uniform(4343, 17))]
    n = len(vals)
    s = synth.ints_to_limbs(vals)
    k = synth.base_dlogs(4344, n)
    k[3] = 0  # an infinity base
    xy = O.g2_fixed_base_mul(O.G2_GENERATOR, k)
    exp = _g2(O.g2_msm_known_answer(k, s))
    b = gpu_ctx.bases_g2_from_host(xy)
    ds = _dev(gpu_ctx, s)
    for c in (0, 4, 5, 8, 13, 16):
        assert gpu_ctx.msm_g2(b, ds, n, window_bits=c) == exp, c
    for i in range(15):  # one scalar at a time, on its own base
        one = _dev(gpu_ctx, s[i:i + 1])
        assert gpu_ctx.msm_g2(b, one, 1, offset=i) == _g2(O.g2_msm_known_answer(k[i:i + 1], s[i:i + 1])), i


def test_msm_g2_fixed_base_rows(gpu_ctx):
    """Window-shifted G2 rows (zk_bases_precompute on a G2 handle): the same points as the
    plain path, for several windows, with offsets and in a batch beside plain instances."""
    n = 1500
    k = synth.base_dlogs(4400, n)
    k[7] = 0  # an infinity base
    xy = O.g2_fixed_base_mul(O.G2_GENERATOR, k)
    s = synth.fr_uniform(4401, n)
    exp = _g2(O.g2_msm_known_answer(k, s))
    b = gpu_ctx.bases_g2_from_host(xy)
    ds = _dev(gpu_ctx, s)
    for c in (5, 10, 16):
        gpu_ctx.bases_precompute(b, c)
        assert gpu_ctx.msm_g2(b, ds, n) == exp, c
        m = 333
        assert gpu_ctx.msm_g2(b, ds, m, offset=40) == _g2(O.g2_msm_known_answer(k[40:40 + m], s[:m])), c
    plain = gpu_ctx.bases_g2_from_host(xy[:600])
    got = gpu_ctx.msm_g2_batch([b, plain, b], [ds, ds, ds], [n, 600, 100])
    assert got == [exp, _g2(O.g2_msm_known_answer(k[:600], s[:600])), _g2(O.g2_msm_known_answer(k[:100], s[:100]))]

