"""zk_ntt_noalloc -- the NTT entry point that allocates no device memory.

It serves callers that cannot allocate while they transform (a process that reserved
its device memory budget up front, or a latency-critical path that must avoid
cudaMalloc's implicit synchronisation). Its scratch is one static device array of the
library, so it is limited to n <= 2^16. This file is collected last so that, if it
fails, a run that stops at the first failure has already run every other test; it
also passes when run alone in a fresh process.

Each call goes through the C ABI (ctypes on include/zkgpu.h) and must give bit for
bit the output of the allocating entry point zk_ntt on the same input, for two calls
in a row (the static array keeps the previous call's contents).
"""

import ctypes

import numpy as np
import pytest

from pyzkp_gb300 import _native as N
from pyzkp_gb300 import synth

pytestmark = pytest.mark.gpu

ROOT_2_28 = 19103219067921713944291392827692070036145651957329286315305642004821462161904


def _omega(n: int) -> int:
    return pow(ROOT_2_28, 1 << (28 - (n.bit_length() - 1)), synth.FR_MODULUS)


def _call(fn_name, ctx, mode, out, inp, in_len, log_n, omega, shift):
    fn = getattr(N.load(), fn_name)
    rc = fn(ctx.handle, int(mode), out.ptr, inp.ptr, int(in_len), int(log_n), int(omega).to_bytes(32, "little"),
            int(shift).to_bytes(32, "little"))
    N.check(rc, fn_name)


def _both(ctx, mode, values, log_n, shift):
    n = 1 << log_n
    m = values.shape[0]
    d = ctx.to_device(values)
    ctx.fr_to_mont(d, d, m)
    ref = ctx.alloc(n * 32)
    new = ctx.alloc(n * 32)
    ctx.memset(new, 0xAB)  # stale bytes in the output must not matter
    om = _omega(n)
    _call("zk_ntt", ctx, mode, ref, d, m, log_n, om, shift)
    _call("zk_ntt_noalloc", ctx, mode, new, d, m, log_n, om, shift)
    ctx.sync()
    return ref.download(), new.download()


@pytest.mark.parametrize("log_n", [0, 3, 11, 12, 14, 16])
def test_noalloc_matches_zk_ntt_two_calls_in_a_row(gpu_ctx, log_n):
    n = 1 << log_n
    for call, mode in enumerate((N.NTT_EVALS_FROM_COEFFS, N.NTT_COSET_COEFFS_FROM_EVALS,
                                 N.NTT_COSET_EVALS_FROM_COEFFS, N.NTT_COEFFS_FROM_EVALS)):
        # forward transforms also take a shorter (zero-padded) input
        m = n if mode in (N.NTT_COEFFS_FROM_EVALS, N.NTT_COSET_COEFFS_FROM_EVALS) else max(1, n - n // 3)
        v = synth.fr_uniform(1000 * log_n + call, m)
        ref, new = _both(gpu_ctx, mode, v, log_n, 5 if mode >= 2 else 1)
        assert np.array_equal(ref, new), (log_n, mode)


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu_ctx):
    d = gpu_ctx.alloc(32)
    with pytest.raises(ValueError, match="2\\^16"):
        _call("zk_ntt_noalloc", gpu_ctx, N.NTT_EVALS_FROM_COEFFS, d, d, 1, 17, _omega(1 << 17), 1)
    assert "2^16" in N.load().zk_last_error().decode()


def test_noalloc_exported_through_the_header():
    with open(N.os.path.join(N.os.path.dirname(N.HERE), "include", "zkgpu.h")) as f:
        assert "int zk_ntt_noalloc(" in f.read()
    assert isinstance(N.load().zk_ntt_noalloc, ctypes._CFuncPtr)
