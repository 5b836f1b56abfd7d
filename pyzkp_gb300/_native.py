"""ctypes binding of ``libzkgpu.so`` (the C ABI declared in ``include/zkgpu.h``).

The library is built in-tree (``pyzkp_gb300/_lib/libzkgpu.so``) by
``pyzkp_gb300.build``. There is no fallback: if the library or a CUDA device is
missing, the calls raise, the way the reference's Metal path raises
``RuntimeError`` without Metal (runtime/context.py:33-34).
"""

from __future__ import annotations

import ctypes
import os
import threading
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("ZKGPU_LIB") or os.path.join(HERE, "_lib", "libzkgpu.so")

ZK_OK, ZK_EINVAL, ZK_ECUDA, ZK_ENOMEM, ZK_ENODEV, ZK_ETIMEOUT = 0, 1, 2, 3, 4, 5

NTT_PLAN_GRAPH, NTT_PLAN_QUEUE = 1, 2
MSM_PLAN_GRAPH, MSM_PLAN_QUEUE = 1, 2

NTT_EVALS_FROM_COEFFS = 0
NTT_COEFFS_FROM_EVALS = 1
NTT_COSET_EVALS_FROM_COEFFS = 2
NTT_COSET_COEFFS_FROM_EVALS = 3

EXPORTED_SYMBOLS = (
    "zk_last_error", "zk_version", "zk_ctx_create", "zk_ctx_destroy", "zk_ctx_sync", "zk_ctx_stream",
    "zk_ctx_num_sms", "zk_alloc", "zk_free", "zk_h2d", "zk_d2h", "zk_host_alloc", "zk_host_free",
    "zk_fr_to_mont", "zk_fr_from_mont", "zk_fq_to_mont", "zk_fq_from_mont", "zk_fr_mul", "zk_fr_sub", "zk_ntt",
    "zk_bases_create", "zk_bases_create_dev", "zk_bases_destroy", "zk_bases_count", "zk_msm_g1", "zk_msm_g1_host", "zk_msm_g1_batch_submit",
    "zk_msm_g2_batch_submit", "zk_batch_wait", "zk_batch_destroy",
    "zk_g1_fixed_base_mul", "zk_memset", "zk_launch_count", "zk_prof_enable", "zk_prof_reset", "zk_prof_count",
    "zk_prof_get", "zk_timer_start", "zk_timer_stop", "zk_msm_last_stats", "zk_imad_peak", "zk_d2d",
    "zk_fr_trimmed_len", "zk_ntt_noalloc", "zk_imad_probe", "zk_bases_precompute", "zk_msm_g1_batch",
    "zk_msm_plan_create", "zk_msm_plan_scalars", "zk_msm_plan_run", "zk_msm_plan_launches", "zk_msm_plan_destroy",
    "zk_ntt_batch", "zk_ntt_plan_create", "zk_ntt_plan_run", "zk_ntt_plan_launches", "zk_ntt_plan_destroy",
    "zk_tune_set_msm_window", "zk_tune_get_msm_window", "zk_tune_set_ntt_split", "zk_tune_get_ntt_split",
    "zk_autotune_msm", "zk_autotune_ntt", "zk_autotune_save", "zk_autotune_load", "zk_bases_g2_create",
    "zk_msm_g2", "zk_msm_g2_batch", "zk_g2_fixed_base_mul", "zk_fr_spmv", "zk_fr_r1cs_check",
    "zk_fr_qap_quotient", "zk_fr_gather", "zk_fr_scale", "zk_fr_powers", "zk_fr_div_xn_minus_1", "zk_host_g1_mul",
    "zk_host_g1_add", "zk_host_g2_mul", "zk_host_g2_add", "zk_fr_add", "zk_bases_g2_create_dev", "zk_fr_batch_inv",
    "zk_plonk_quotient_evals", "zk_ctx_create_prio", "zk_stream_priority_range", "zk_h2d_async", "zk_d2h_async",
    "zk_fence_record", "zk_fence_wait", "zk_fence_destroy", "zk_fr_r1cs_check_async",
    "zk_ntt_batch_set_queue", "zk_ntt_queue_status", "zk_ntt_queue_selftest", "zk_msm_batch_set_queue",
    "zk_msm_queue_test_limit", "zk_msm_g1_host_submit", "zk_ntt_host_submit",
)

_lib: Optional[ctypes.CDLL] = None
_lock = threading.Lock()


class ZkError(RuntimeError):
    pass


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load the library and declare the signatures (no device is touched)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise RuntimeError(f"zkgpu library not built: {path} (run python -m pyzkp_gb300.build)")
        L = ctypes.CDLL(path)
        P, S, I, U32 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_uint32
        PP = ctypes.POINTER(ctypes.c_void_p)
        sig = {
            "zk_last_error": ([], ctypes.c_char_p),
            "zk_version": ([], I),
            "zk_ctx_create": ([I, PP], I),
            "zk_ctx_destroy": ([P], I),
            "zk_ctx_sync": ([P], I),
            "zk_ctx_stream": ([P, PP], I),
            "zk_ctx_num_sms": ([P, ctypes.POINTER(ctypes.c_int)], I),
            "zk_alloc": ([P, S, PP], I),
            "zk_free": ([P, P], I),
            "zk_h2d": ([P, P, P, S], I),
            "zk_d2h": ([P, P, P, S], I),
            "zk_host_alloc": ([S, PP], I),
            "zk_host_free": ([P], I),
            "zk_fr_to_mont": ([P, P, P, S], I),
            "zk_fr_from_mont": ([P, P, P, S], I),
            "zk_fq_to_mont": ([P, P, P, S], I),
            "zk_fq_from_mont": ([P, P, P, S], I),
            "zk_fr_mul": ([P, P, P, P, S], I),
            "zk_fr_sub": ([P, P, P, P, S], I),
            "zk_ntt": ([P, I, P, P, S, U32, P, P], I),
            "zk_bases_create": ([P, P, S, PP], I),
            "zk_bases_create_dev": ([P, P, S, PP], I),
            "zk_bases_destroy": ([P], I),
            "zk_bases_count": ([P, ctypes.POINTER(ctypes.c_size_t)], I),
            "zk_msm_g1": ([P, P, S, P, S, I, U32, P, ctypes.POINTER(ctypes.c_int)], I),
            "zk_msm_g1_host": ([P, P, P, S, I, U32, P, ctypes.POINTER(ctypes.c_int)], I),
            "zk_g1_fixed_base_mul": ([P, P, P, S, P], I),
            "zk_memset": ([P, P, I, S], I),
            "zk_launch_count": ([P, ctypes.POINTER(ctypes.c_uint64)], I),
            "zk_prof_enable": ([P, I], I),
            "zk_prof_reset": ([P], I),
            "zk_prof_count": ([P, ctypes.POINTER(ctypes.c_int)], I),
            "zk_prof_get": ([P, I, ctypes.c_char_p, S, ctypes.POINTER(ctypes.c_uint64),
                             ctypes.POINTER(ctypes.c_double)], I),
            "zk_timer_start": ([P], I),
            "zk_timer_stop": ([P, ctypes.POINTER(ctypes.c_double)], I),
            "zk_msm_last_stats": ([P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint32),
                                   ctypes.POINTER(ctypes.c_uint32)], I),
            "zk_imad_peak": ([P, ctypes.POINTER(ctypes.c_double)], I),
            "zk_d2d": ([P, P, P, S], I),
            "zk_fr_trimmed_len": ([P, P, S, ctypes.POINTER(ctypes.c_size_t)], I),
            "zk_ntt_noalloc": ([P, I, P, P, S, U32, P, P], I),
            "zk_imad_probe": ([P, I, ctypes.POINTER(ctypes.c_double)], I),
            "zk_bases_precompute": ([P, P, U32], I),
            "zk_msm_g1_batch": ([P, S, PP, P, PP, P, I, U32, P, P], I),
            "zk_msm_plan_create": ([P, S, PP, P, P, I, U32, I, PP], I),
            "zk_msm_plan_scalars": ([P, S, PP], I),
            "zk_msm_plan_run": ([P, P, P], I),
            "zk_msm_plan_launches": ([P, ctypes.POINTER(ctypes.c_uint64)], I),
            "zk_msm_plan_destroy": ([P], I),
            "zk_ntt_batch": ([P, S, P, PP, PP, P, P, P, P], I),
            "zk_ntt_plan_create": ([P, S, P, PP, PP, P, P, P, P, I, PP], I),
            "zk_ntt_plan_run": ([P], I),
            "zk_ntt_batch_set_queue": ([P, I], I),
            "zk_msm_batch_set_queue": ([P, I], I),
            "zk_msm_g1_host_submit": ([P, P, P, S, I, U32, P, P, PP], I),
            "zk_ntt_host_submit": ([P, I, P, P, S, U32, P, P, PP], I),
            "zk_msm_queue_test_limit": ([P, ctypes.c_uint64], I),
            "zk_ntt_queue_status": ([P], I),
            "zk_ntt_queue_selftest": ([P, ctypes.c_uint64, ctypes.POINTER(U32)], I),
            "zk_ntt_plan_launches": ([P, ctypes.POINTER(ctypes.c_uint64)], I),
            "zk_ntt_plan_destroy": ([P], I),
            "zk_tune_set_msm_window": ([P, U32, U32], I),
            "zk_tune_get_msm_window": ([P, ctypes.c_uint64, ctypes.POINTER(U32)], I),
            "zk_tune_set_ntt_split": ([P, U32, U32, P], I),
            "zk_tune_get_ntt_split": ([P, U32, ctypes.POINTER(U32), P], I),
            "zk_autotune_msm": ([P, P, P, U32, I, ctypes.POINTER(U32), ctypes.POINTER(ctypes.c_double)], I),
            "zk_autotune_ntt": ([P, P, U32, I, ctypes.POINTER(U32), P, ctypes.POINTER(ctypes.c_double)], I),
            "zk_autotune_save": ([P, ctypes.c_char_p], I),
            "zk_autotune_load": ([P, ctypes.c_char_p], I),
            "zk_bases_g2_create": ([P, P, S, PP], I),
            "zk_msm_g2": ([P, P, S, P, S, I, U32, P, ctypes.POINTER(ctypes.c_int)], I),
            "zk_msm_g2_batch": ([P, S, PP, P, PP, P, I, U32, P, P], I),
            "zk_msm_g1_batch_submit": ([P, S, PP, P, PP, P, I, U32, P, P, ctypes.POINTER(ctypes.c_void_p)], I),
            "zk_msm_g2_batch_submit": ([P, S, PP, P, PP, P, I, U32, P, P, ctypes.POINTER(ctypes.c_void_p)], I),
            "zk_batch_wait": ([P, I], I),
            "zk_batch_destroy": ([P], I),
            "zk_g2_fixed_base_mul": ([P, P, P, S, P], I),
            "zk_fr_spmv": ([P, U32, P, P, P, P, P], I),
            "zk_fr_r1cs_check": ([P, P, P, P, S, ctypes.POINTER(ctypes.c_uint64)], I),
            "zk_fr_r1cs_check_async": ([P, P, P, P, S, P], I),
            "zk_ctx_create_prio": ([I, I, PP], I),
            "zk_stream_priority_range": ([ctypes.POINTER(I), ctypes.POINTER(I)], I),
            "zk_h2d_async": ([P, P, P, S], I),
            "zk_d2h_async": ([P, P, P, S], I),
            "zk_fence_record": ([P, PP], I),
            "zk_fence_wait": ([P, I], I),
            "zk_fence_destroy": ([P], I),
            "zk_fr_qap_quotient": ([P, P, P, P, P, S, P], I),
            "zk_fr_gather": ([P, P, P, P, S], I),
            "zk_fr_scale": ([P, P, P, P, S], I),
            "zk_fr_powers": ([P, P, P, S], I),
            "zk_fr_div_xn_minus_1": ([P, P, S, S, P, P, ctypes.POINTER(ctypes.c_size_t),
                                      ctypes.POINTER(ctypes.c_size_t)], I),
            "zk_host_g1_mul": ([P, P, P], I),
            "zk_host_g1_add": ([P, P, P], I),
            "zk_host_g2_mul": ([P, P, P], I),
            "zk_host_g2_add": ([P, P, P], I),
            "zk_fr_add": ([P, P, P, P, S], I),
            "zk_bases_g2_create_dev": ([P, P, S, PP], I),
            "zk_fr_batch_inv": ([P, P, P, S], I),
            "zk_plonk_quotient_evals": ([P, PP, S, ctypes.c_uint64, P, P, P, P, P, P, P, P, P, P], I),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
        return L


def check(rc: int, what: str = "") -> None:
    if rc == ZK_OK:
        return
    msg = load().zk_last_error().decode(errors="replace")
    text = f"{what}: {msg}" if what else msg
    if rc == ZK_EINVAL:
        raise ValueError(text)
    if rc == ZK_ENOMEM:
        raise MemoryError(text)
    if rc == ZK_ETIMEOUT:
        raise TimeoutError(text)
    raise ZkError(text)


class MsmBatch:
    """An in-flight asynchronous MSM batch (zk_batch)."""

    def __init__(self, handle, count, g2, out, inf, keep) -> None:
        self.handle, self.count, self.g2, self._out, self._inf, self._keep = handle, count, g2, out, inf, keep

    def wait(self, timeout_ms: int = -1):
        """Results once the batch is done (TimeoutError if timeout_ms >= 0 passes first)."""
        check(load().zk_batch_wait(self.handle, int(timeout_ms)), "zk_batch_wait")
        if self.g2:
            return [None if self._inf[k] else _g2_from(self._out[k].tobytes()) for k in range(self.count)]
        return _points_from(self._out[:self.count], self._inf[:self.count])

    def done(self) -> bool:
        try:
            check(load().zk_batch_wait(self.handle, 0), "zk_batch_wait")
            return True
        except TimeoutError:
            return False

    def destroy(self) -> None:
        if self.handle is not None:
            load().zk_batch_destroy(self.handle)
            self.handle = None
            self._keep = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class DeviceArray:
    """An owned device allocation of ``nbytes`` (freed with the context's pool)."""

    __slots__ = ("ctx", "ptr", "nbytes", "owned", "__weakref__")

    def __init__(self, ctx: "Context", nbytes: int, ptr: Optional[int] = None, owned: bool = True) -> None:
        """Allocate ``nbytes``; or, with ``ptr`` given and ``owned=False``, view memory that
        something else owns (a plan's scalar slot), which free() leaves alone."""
        self.ctx = ctx
        self.nbytes = int(nbytes)
        self.owned = owned
        if ptr is not None:
            self.ptr = ptr
            return
        p = ctypes.c_void_p()
        check(load().zk_alloc(ctx.handle, max(16, self.nbytes), ctypes.byref(p)), "zk_alloc")
        self.ptr = p.value

    def free(self) -> None:
        if self.owned and self.ptr is not None and self.ctx.handle is not None:
            load().zk_free(self.ctx.handle, self.ptr)
        self.ptr = None

    def __del__(self) -> None:
        try:
            self.free()
        except Exception:
            pass

    def length(self) -> int:
        """Byte size (the MTLBuffer.length() protocol used by MemoryPool.release_metal)."""
        return self.nbytes

    def upload(self, host: np.ndarray) -> None:
        buf = np.ascontiguousarray(host)
        if buf.nbytes > self.nbytes:
            raise ValueError("host array larger than device allocation")
        check(load().zk_h2d(self.ctx.handle, self.ptr, buf.ctypes.data, buf.nbytes), "zk_h2d")

    def download(self, nbytes: Optional[int] = None) -> np.ndarray:
        nb = self.nbytes if nbytes is None else int(nbytes)
        out = np.empty(nb, dtype=np.uint8)
        check(load().zk_d2h(self.ctx.handle, out.ctypes.data, self.ptr, nb), "zk_d2h")
        return out


class PinnedBuffer:
    """Page-locked host memory exposed as a numpy uint8 array (``.array``)."""

    def __init__(self, nbytes: int) -> None:
        p = ctypes.c_void_p()
        check(load().zk_host_alloc(max(16, int(nbytes)), ctypes.byref(p)), "zk_host_alloc")
        self.ptr = p.value
        self.nbytes = int(nbytes)
        self.array = np.ctypeslib.as_array((ctypes.c_uint8 * max(16, self.nbytes)).from_address(self.ptr))[:self.nbytes]

    def free(self) -> None:
        if self.ptr is not None:
            self.array = None
            load().zk_host_free(self.ptr)
            self.ptr = None

    def __del__(self) -> None:
        try:
            self.free()
        except Exception:
            pass


class PinnedArray(np.ndarray):
    """A numpy array in page-locked host memory; it keeps its ``PinnedBuffer`` alive."""

    def __array_finalize__(self, obj) -> None:
        self._pin = getattr(obj, "_pin", None)


def pinned_copy(a: np.ndarray) -> PinnedArray:
    """A C-contiguous copy of ``a`` in page-locked host memory."""
    a = np.ascontiguousarray(a)
    buf = PinnedBuffer(a.nbytes)
    out = buf.array.view(a.dtype).reshape(a.shape).view(PinnedArray)
    out[...] = a
    out._pin = buf
    return out


class Bases:
    """Resident affine G1 bases in Montgomery form on the device."""

    def __init__(self, ctx: "Context", handle: int, n: int) -> None:
        self.ctx = ctx
        self.handle = handle
        self.n = n

    def free(self) -> None:
        if self.handle is not None:
            load().zk_bases_destroy(self.handle)
            self.handle = None

    def __del__(self) -> None:
        try:
            self.free()
        except Exception:
            pass


def _points_from(out: np.ndarray, inf: np.ndarray):
    res = []
    for k in range(out.shape[0]):
        if inf[k]:
            res.append(None)
        else:
            b = out[k].tobytes()
            res.append((int.from_bytes(b[:32], "little"), int.from_bytes(b[32:], "little")))
    return res


def host_g1_mul(p, k: int):
    """[k] P on the host; p = (x, y) canonical ints or None (infinity); returns the same form."""
    out = (ctypes.c_uint8 * 64)()
    check(load().zk_host_g1_mul(_g1_bytes(p), _fr_bytes(k), out), "zk_host_g1_mul")
    return _g1_from(bytes(out))


def host_g1_add(p, q):
    out = (ctypes.c_uint8 * 64)()
    check(load().zk_host_g1_add(_g1_bytes(p), _g1_bytes(q), out), "zk_host_g1_add")
    return _g1_from(bytes(out))


def host_g2_mul(p, k: int):
    """[k] P on G2; p = ((x0, x1), (y0, y1)) canonical ints or None."""
    out = (ctypes.c_uint8 * 128)()
    check(load().zk_host_g2_mul(_g2_bytes(p), _fr_bytes(k), out), "zk_host_g2_mul")
    b = bytes(out)
    return None if not any(b) else _g2_from(b)


def host_g2_add(p, q):
    out = (ctypes.c_uint8 * 128)()
    check(load().zk_host_g2_add(_g2_bytes(p), _g2_bytes(q), out), "zk_host_g2_add")
    b = bytes(out)
    return None if not any(b) else _g2_from(b)


def _g1_bytes(p) -> bytes:
    if p is None:
        return bytes(64)
    return int(p[0]).to_bytes(32, "little") + int(p[1]).to_bytes(32, "little")


def _g1_from(b: bytes):
    if not any(b):
        return None
    return int.from_bytes(b[:32], "little"), int.from_bytes(b[32:], "little")


def _g2_bytes(p) -> bytes:
    if p is None:
        return bytes(128)
    (x0, x1), (y0, y1) = p
    return b"".join(int(v).to_bytes(32, "little") for v in (x0, x1, y0, y1))


def _g2_from(b: bytes):
    v = [int.from_bytes(b[32 * i:32 * i + 32], "little") for i in range(4)]
    return (v[0], v[1]), (v[2], v[3])


def _fr_bytes(v: int) -> bytes:
    return (int(v) % (1 << 256)).to_bytes(32, "little")


class NttPlan:
    """A prepared NTT batch (zk_ntt_plan_*); run() is asynchronous on the context stream."""

    def __init__(self, ctx: "Context", handle: int, buffers) -> None:
        self.ctx = ctx
        self.handle = handle
        self._buffers = buffers  # keep the device buffers alive as long as the plan

    def run(self) -> None:
        check(load().zk_ntt_plan_run(self.handle), "zk_ntt_plan_run")

    def launches(self) -> int:
        v = ctypes.c_uint64()
        check(load().zk_ntt_plan_launches(self.handle, ctypes.byref(v)), "zk_ntt_plan_launches")
        return int(v.value)

    def free(self) -> None:
        if self.handle is not None:
            load().zk_ntt_plan_destroy(self.handle)
            self.handle = None

    def __del__(self) -> None:
        try:
            self.free()
        except Exception:
            pass


class MsmPlan:
    """A prepared MSM batch (zk_msm_plan_*): plan-owned scalar slots, optional CUDA graph."""

    def __init__(self, ctx: "Context", handle: int, sizes, bases) -> None:
        self.ctx = ctx
        self.handle = handle
        self.sizes = sizes
        self._bases = bases  # keep the bases alive as long as the plan

    def slot(self, index: int) -> DeviceArray:
        """Device view of instance ``index``'s scalar slot (sizes[index] elements)."""
        p = ctypes.c_void_p()
        check(load().zk_msm_plan_scalars(self.handle, int(index), ctypes.byref(p)), "zk_msm_plan_scalars")
        return DeviceArray(self.ctx, self.sizes[index] * 32, ptr=p.value or 0, owned=False)

    def run(self):
        count = len(self.sizes)
        out = np.zeros((max(count, 1), 64), dtype=np.uint8)
        inf = np.zeros(max(count, 1), dtype=np.int32)
        check(load().zk_msm_plan_run(self.handle, out.ctypes.data, inf.ctypes.data), "zk_msm_plan_run")
        return _points_from(out[:count], inf[:count])

    def launches(self) -> int:
        v = ctypes.c_uint64()
        check(load().zk_msm_plan_launches(self.handle, ctypes.byref(v)), "zk_msm_plan_launches")
        return int(v.value)

    def free(self) -> None:
        if self.handle is not None:
            load().zk_msm_plan_destroy(self.handle)
            self.handle = None

    def __del__(self) -> None:
        try:
            self.free()
        except Exception:
            pass


class Fence:
    """A point on a context's stream (zk_fence): ``done()`` asks, ``wait()`` blocks."""

    def __init__(self, handle) -> None:
        self.handle = handle

    def wait(self, timeout_ms: int = -1) -> None:
        check(load().zk_fence_wait(self.handle, int(timeout_ms)), "zk_fence_wait")

    def done(self) -> bool:
        try:
            self.wait(0)
            return True
        except TimeoutError:
            return False

    def destroy(self) -> None:
        if self.handle is not None:
            load().zk_fence_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def stream_priority_range():
    """(least, greatest) CUDA stream priorities of the device (greatest = most urgent)."""
    lo, hi = ctypes.c_int(), ctypes.c_int()
    check(load().zk_stream_priority_range(ctypes.byref(lo), ctypes.byref(hi)), "zk_stream_priority_range")
    return int(lo.value), int(hi.value)


class Context:
    """One GPU, one stream (zk_ctx); ``priority`` sets the CUDA priority of its streams."""

    def __init__(self, device: int = 0, priority: Optional[int] = None) -> None:
        L = load()
        h = ctypes.c_void_p()
        if priority is None:
            check(L.zk_ctx_create(int(device), ctypes.byref(h)), "zk_ctx_create")
        else:
            check(L.zk_ctx_create_prio(int(device), int(priority), ctypes.byref(h)), "zk_ctx_create_prio")
        self.handle = h.value
        self.device = device
        self.priority = priority

    def ntt_host_submit(self, mode: int, out_host, in_host, in_len: int, log_n: int, omega: int,
                        shift: int = 1) -> Fence:
        """zk_ntt_host_submit: canonical host input (in_len x 32 bytes) -> canonical host output
        (2^log_n x 32 bytes), asynchronous; the returned Fence passes when the output is
        written. ``out_host`` / ``in_host``: PinnedBuffer or pinned arrays (anything with a
        ``ptr``), which must stay alive and unchanged until then."""
        om = np.frombuffer(_fr_bytes(omega), dtype=np.uint8).copy()
        sh = np.frombuffer(_fr_bytes(shift), dtype=np.uint8).copy()
        h = ctypes.c_void_p()
        check(load().zk_ntt_host_submit(self.handle, int(mode), out_host.ptr, in_host.ptr if in_len else None,
                                        int(in_len), int(log_n), om.ctypes.data, sh.ctypes.data, ctypes.byref(h)),
              "zk_ntt_host_submit")
        return Fence(h.value)

    def fence(self) -> Fence:
        h = ctypes.c_void_p()
        check(load().zk_fence_record(self.handle, ctypes.byref(h)), "zk_fence_record")
        return Fence(h.value)

    def h2d_async(self, dst, src: np.ndarray, nbytes: Optional[int] = None) -> None:
        """Enqueue a host-to-device copy; ``src`` must stay unchanged until the stream passes it."""
        if not src.flags.c_contiguous:
            raise ValueError("h2d_async needs a C-contiguous host array")
        nb = src.nbytes if nbytes is None else int(nbytes)
        check(load().zk_h2d_async(self.handle, getattr(dst, "ptr", dst), src.ctypes.data, nb), "zk_h2d_async")

    def d2h_async(self, dst: np.ndarray, src, nbytes: Optional[int] = None) -> None:
        """Enqueue a device-to-host copy; ``dst`` is valid once the stream has passed it."""
        if not dst.flags.c_contiguous:
            raise ValueError("d2h_async needs a C-contiguous host array")
        nb = dst.nbytes if nbytes is None else int(nbytes)
        check(load().zk_d2h_async(self.handle, dst.ctypes.data, getattr(src, "ptr", src), nb), "zk_d2h_async")

    def close(self) -> None:
        if self.handle is not None:
            load().zk_ctx_destroy(self.handle)
            self.handle = None

    def sync(self) -> None:
        check(load().zk_ctx_sync(self.handle), "zk_ctx_sync")

    def num_sms(self) -> int:
        v = ctypes.c_int()
        check(load().zk_ctx_num_sms(self.handle, ctypes.byref(v)))
        return v.value

    # ---- measurement ----
    def memset(self, d: DeviceArray, value: int = 0) -> None:
        check(load().zk_memset(self.handle, d.ptr, int(value), d.nbytes), "zk_memset")

    def launch_count(self) -> int:
        v = ctypes.c_uint64()
        check(load().zk_launch_count(self.handle, ctypes.byref(v)))
        return int(v.value)

    def prof_enable(self, on: bool) -> None:
        check(load().zk_prof_enable(self.handle, 1 if on else 0), "zk_prof_enable")

    def prof_reset(self) -> None:
        check(load().zk_prof_reset(self.handle), "zk_prof_reset")

    def prof_table(self) -> dict:
        """{kernel name: (launches, total device ms)} accumulated since the last reset."""
        L = load()
        cnt = ctypes.c_int()
        check(L.zk_prof_count(self.handle, ctypes.byref(cnt)))
        out = {}
        buf = ctypes.create_string_buffer(128)
        for i in range(cnt.value):
            la, ms = ctypes.c_uint64(), ctypes.c_double()
            check(L.zk_prof_get(self.handle, i, buf, 128, ctypes.byref(la), ctypes.byref(ms)))
            out[buf.value.decode()] = (int(la.value), float(ms.value))
        return out

    def timer_start(self) -> None:
        check(load().zk_timer_start(self.handle), "zk_timer_start")

    def timer_stop(self) -> float:
        """Milliseconds since timer_start, from CUDA events on the context stream."""
        v = ctypes.c_double()
        check(load().zk_timer_stop(self.handle, ctypes.byref(v)), "zk_timer_stop")
        return float(v.value)

    def msm_last_stats(self) -> dict:
        e, c, w = ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_uint32()
        check(load().zk_msm_last_stats(self.handle, ctypes.byref(e), ctypes.byref(c), ctypes.byref(w)))
        return {"entries": int(e.value), "window_bits": int(c.value), "windows": int(w.value)}

    def imad_probe(self, mode: int) -> float:
        v = ctypes.c_double()
        check(load().zk_imad_probe(self.handle, int(mode), ctypes.byref(v)), "zk_imad_probe")
        return float(v.value)

    def imad_peak(self) -> float:
        """Measured 32-bit IMAD throughput, 10^12 instructions/s."""
        v = ctypes.c_double()
        check(load().zk_imad_peak(self.handle, ctypes.byref(v)), "zk_imad_peak")
        return float(v.value)

    # ---- memory ----
    def pinned(self, nbytes: int) -> "PinnedBuffer":
        return PinnedBuffer(nbytes)

    def alloc(self, nbytes: int) -> DeviceArray:
        return DeviceArray(self, nbytes)

    def to_device(self, host: np.ndarray) -> DeviceArray:
        buf = np.ascontiguousarray(host)
        d = DeviceArray(self, buf.nbytes)
        d.upload(buf)
        return d

    # ---- field vectors (n elements of 32 bytes) ----
    def fr_to_mont(self, out: DeviceArray, inp: DeviceArray, n: int) -> None:
        check(load().zk_fr_to_mont(self.handle, out.ptr, inp.ptr, n), "zk_fr_to_mont")

    def fr_from_mont(self, out: DeviceArray, inp: DeviceArray, n: int) -> None:
        check(load().zk_fr_from_mont(self.handle, out.ptr, inp.ptr, n), "zk_fr_from_mont")

    def d2d(self, dst: DeviceArray, src: DeviceArray, nbytes: int) -> None:
        check(load().zk_d2d(self.handle, dst.ptr, src.ptr, int(nbytes)), "zk_d2d")

    def fr_trimmed_len(self, a: DeviceArray, n: int) -> int:
        v = ctypes.c_size_t()
        check(load().zk_fr_trimmed_len(self.handle, a.ptr, int(n), ctypes.byref(v)), "zk_fr_trimmed_len")
        return int(v.value)

    def fr_mul(self, out: DeviceArray, a: DeviceArray, b: DeviceArray, n: int) -> None:
        check(load().zk_fr_mul(self.handle, out.ptr, a.ptr, b.ptr, n), "zk_fr_mul")

    def fr_sub(self, out: DeviceArray, a: DeviceArray, b: DeviceArray, n: int) -> None:
        check(load().zk_fr_sub(self.handle, out.ptr, a.ptr, b.ptr, n), "zk_fr_sub")

    def fr_add(self, out, a, b, n: int) -> None:
        check(load().zk_fr_add(self.handle, getattr(out, "ptr", out), getattr(a, "ptr", a), getattr(b, "ptr", b),
                               int(n)), "zk_fr_add")

    def ntt(self, mode: int, out: DeviceArray, inp: Optional[DeviceArray], in_len: int, log_n: int, omega: int,
            shift: int = 1) -> None:
        om = int(omega).to_bytes(32, "little")
        sh = int(shift).to_bytes(32, "little")
        check(load().zk_ntt(self.handle, int(mode), out.ptr, inp.ptr if inp is not None else None, int(in_len),
                            int(log_n), om, sh), "zk_ntt")

    # ---- G1 ----
    def bases_from_host(self, xy: np.ndarray) -> Bases:
        a = np.ascontiguousarray(xy, dtype=np.uint64).reshape(-1, 8)
        h = ctypes.c_void_p()
        check(load().zk_bases_create(self.handle, a.ctypes.data, a.shape[0], ctypes.byref(h)), "zk_bases_create")
        return Bases(self, h.value, a.shape[0])

    def bases_g2_from_host(self, xy: np.ndarray) -> Bases:
        """G2 bases: rows of 16 uint64 limbs (x.c0, x.c1, y.c0, y.c1 canonical; zero = infinity)."""
        a = np.ascontiguousarray(xy, dtype=np.uint64).reshape(-1, 16)
        h = ctypes.c_void_p()
        check(load().zk_bases_g2_create(self.handle, a.ctypes.data, a.shape[0], ctypes.byref(h)),
              "zk_bases_g2_create")
        return Bases(self, h.value, a.shape[0])

    def bases_g2_from_device(self, xy: DeviceArray, n: int) -> Bases:
        h = ctypes.c_void_p()
        check(load().zk_bases_g2_create_dev(self.handle, xy.ptr, int(n), ctypes.byref(h)), "zk_bases_g2_create_dev")
        return Bases(self, h.value, int(n))

    def msm_g2(self, bases: Bases, scalars: DeviceArray, n: int, *, offset: int = 0, scalars_mont: bool = True,
               window_bits: int = 0):
        """Returns ((x0, x1), (y0, y1)) canonical ints, or None for the point at infinity."""
        out = (ctypes.c_uint8 * 128)()
        inf = ctypes.c_int()
        check(load().zk_msm_g2(self.handle, bases.handle, int(offset), scalars.ptr, int(n), 1 if scalars_mont else 0,
                               int(window_bits), out, ctypes.byref(inf)), "zk_msm_g2")
        return None if inf.value else _g2_from(bytes(out))

    def msm_g2_batch(self, bases, scalars, sizes, *, offsets=None, scalars_mont: bool = True,
                     window_bits: int = 0):
        count = len(sizes)
        if isinstance(bases, Bases):
            bases = [bases] * count
        bh = (ctypes.c_void_p * count)(*[b.handle for b in bases])
        sp = (ctypes.c_void_p * count)(*[getattr(s, "ptr", s) for s in scalars])
        sz = np.ascontiguousarray(sizes, dtype=np.uint64)
        off = None if offsets is None else np.ascontiguousarray(offsets, dtype=np.uint64)
        out = np.zeros((max(count, 1), 128), dtype=np.uint8)
        inf = np.zeros(max(count, 1), dtype=np.int32)
        check(load().zk_msm_g2_batch(self.handle, count, bh, None if off is None else off.ctypes.data, sp,
                                     sz.ctypes.data, 1 if scalars_mont else 0, int(window_bits), out.ctypes.data,
                                     inf.ctypes.data), "zk_msm_g2_batch")
        return [None if inf[k] else _g2_from(out[k].tobytes()) for k in range(count)]

    def msm_batch_submit(self, bases, scalars, sizes, *, g2: bool = False, offsets=None,
                         scalars_mont: bool = True, window_bits: int = 0) -> "MsmBatch":
        """Asynchronous batched MSM (zk_msm_g1_batch_submit / zk_msm_g2_batch_submit): returns
        at once; ``MsmBatch.wait(timeout_ms)`` gives the results of msm_g1_batch / msm_g2_batch."""
        count = len(sizes)
        if isinstance(bases, Bases):
            bases = [bases] * count
        bh = (ctypes.c_void_p * count)(*[b.handle for b in bases])
        sp = (ctypes.c_void_p * count)(*[getattr(s, "ptr", s) for s in scalars])
        sz = np.ascontiguousarray(sizes, dtype=np.uint64)
        off = None if offsets is None else np.ascontiguousarray(offsets, dtype=np.uint64)
        out = np.zeros((max(count, 1), 128 if g2 else 64), dtype=np.uint8)
        inf = np.zeros(max(count, 1), dtype=np.int32)
        h = ctypes.c_void_p()
        fn = load().zk_msm_g2_batch_submit if g2 else load().zk_msm_g1_batch_submit
        check(fn(self.handle, count, bh, None if off is None else off.ctypes.data, sp, sz.ctypes.data,
                 1 if scalars_mont else 0, int(window_bits), out.ctypes.data, inf.ctypes.data, ctypes.byref(h)),
              "zk_msm_batch_submit")
        # the arrays the library reads or writes until the batch completes stay referenced
        return MsmBatch(h.value, count, g2, out, inf, keep=(bh, sp, sz, off, scalars, bases))

    def bases_precompute(self, bases: "Bases", window_bits: int) -> None:
        """Window-shifted rows for fixed-base MSMs on ``bases`` (zk_bases_precompute)."""
        check(load().zk_bases_precompute(self.handle, bases.handle, int(window_bits)), "zk_bases_precompute")

    def bases_from_device(self, xy: DeviceArray, n: int) -> Bases:
        h = ctypes.c_void_p()
        check(load().zk_bases_create_dev(self.handle, xy.ptr, int(n), ctypes.byref(h)), "zk_bases_create_dev")
        return Bases(self, h.value, int(n))

    def msm_g1(self, bases: Bases, scalars: DeviceArray, n: int, *, offset: int = 0, scalars_mont: bool = True,
               window_bits: int = 0):
        """Returns (x, y) canonical ints, or None for the point at infinity."""
        out = (ctypes.c_uint8 * 64)()
        inf = ctypes.c_int()
        check(load().zk_msm_g1(self.handle, bases.handle, int(offset), scalars.ptr, int(n), 1 if scalars_mont else 0,
                               int(window_bits), out, ctypes.byref(inf)), "zk_msm_g1")
        if inf.value:
            return None
        b = bytes(out)
        return int.from_bytes(b[:32], "little"), int.from_bytes(b[32:], "little")

    def msm_g1_host_submit(self, xy, scalars, n: int, *, scalars_mont: bool = False,
                           window_bits: int = 0) -> "MsmBatch":
        """msm_g1_host, asynchronous (zk_msm_g1_host_submit): returns an MsmBatch whose wait()
        gives [point]. The host buffers stay referenced until the batch is destroyed; they
        must not change before it completes (PinnedBuffer / pinned arrays keep the copies
        asynchronous, so one call's uploads overlap the previous call's MSM)."""
        keep = [xy, scalars]

        def _ptr(a):
            if hasattr(a, "ptr"):
                return a.ptr
            a = np.ascontiguousarray(a)
            keep.append(a)
            return a.ctypes.data
        out = np.zeros((1, 64), dtype=np.uint8)
        inf = np.zeros(1, dtype=np.int32)
        h = ctypes.c_void_p()
        check(load().zk_msm_g1_host_submit(self.handle, _ptr(xy), _ptr(scalars), int(n), 1 if scalars_mont else 0,
                                           int(window_bits), out.ctypes.data, inf.ctypes.data, ctypes.byref(h)),
              "zk_msm_g1_host_submit")
        return MsmBatch(h.value, 1, False, out, inf, keep=keep)

    def msm_g1_host(self, xy, scalars, n: int, *, scalars_mont: bool = False, window_bits: int = 0):
        """One-call MSM from host memory (zk_msm_g1_host): ``xy`` canonical affine points
        (n x 64 bytes), ``scalars`` n x 32 bytes; numpy arrays or PinnedBuffer (pinned memory
        makes the copies asynchronous). Returns (x, y) canonical ints, or None for infinity."""
        def _ptr(a):
            if hasattr(a, "ptr"):
                return a.ptr
            a = np.ascontiguousarray(a)
            keep.append(a)
            return a.ctypes.data
        keep = []
        out = (ctypes.c_uint8 * 64)()
        inf = ctypes.c_int()
        check(load().zk_msm_g1_host(self.handle, _ptr(xy), _ptr(scalars), int(n), 1 if scalars_mont else 0,
                                    int(window_bits), out, ctypes.byref(inf)), "zk_msm_g1_host")
        if inf.value:
            return None
        b = bytes(out)
        return int.from_bytes(b[:32], "little"), int.from_bytes(b[32:], "little")

    def msm_g1_batch(self, bases, scalars, sizes, *, offsets=None, scalars_mont: bool = True,
                     window_bits: int = 0):
        """Batched MSM (zk_msm_g1_batch). ``bases``: one Bases or a list (one per instance);
        ``scalars``: list of DeviceArray (or device pointers); ``sizes``: list of lengths.
        Returns a list of (x, y) canonical ints or None (infinity)."""
        count = len(sizes)
        if isinstance(bases, Bases):
            bases = [bases] * count
        bh = (ctypes.c_void_p * count)(*[b.handle for b in bases])
        sp = (ctypes.c_void_p * count)(*[getattr(s, "ptr", s) for s in scalars])
        sz = np.ascontiguousarray(sizes, dtype=np.uint64)
        off = None if offsets is None else np.ascontiguousarray(offsets, dtype=np.uint64)
        out = np.zeros((max(count, 1), 64), dtype=np.uint8)
        inf = np.zeros(max(count, 1), dtype=np.int32)
        check(load().zk_msm_g1_batch(self.handle, count, bh, None if off is None else off.ctypes.data, sp,
                                     sz.ctypes.data, 1 if scalars_mont else 0, int(window_bits), out.ctypes.data,
                                     inf.ctypes.data), "zk_msm_g1_batch")
        return _points_from(out[:count], inf[:count])

    def msm_plan(self, bases, sizes, *, offsets=None, scalars_mont: bool = True, window_bits: int = 0,
                 use_graph: bool = True, queue: bool = False) -> "MsmPlan":
        """A prepared G1 batch; ``queue``: its work-queue form (sorts, then one persistent launch)."""
        count = len(sizes)
        if isinstance(bases, Bases):
            bases = [bases] * count
        bh = (ctypes.c_void_p * count)(*[b.handle for b in bases])
        sz = np.ascontiguousarray(sizes, dtype=np.uint64)
        off = None if offsets is None else np.ascontiguousarray(offsets, dtype=np.uint64)
        h = ctypes.c_void_p()
        check(load().zk_msm_plan_create(self.handle, count, bh, None if off is None else off.ctypes.data,
                                        sz.ctypes.data, 1 if scalars_mont else 0, int(window_bits),
                                        (MSM_PLAN_GRAPH if use_graph else 0) | (MSM_PLAN_QUEUE if queue else 0),
                                        ctypes.byref(h)), "zk_msm_plan_create")
        return MsmPlan(self, h.value, [int(x) for x in sizes], list(bases))

    @staticmethod
    def _ntt_args(jobs):
        """jobs: (mode, out, inp, in_len, log_n, omega, shift) tuples -> ctypes arrays."""
        count = len(jobs)
        modes = np.array([j[0] for j in jobs], dtype=np.int32)
        outs = (ctypes.c_void_p * count)(*[getattr(j[1], "ptr", j[1]) for j in jobs])
        ins = (ctypes.c_void_p * count)(*[getattr(j[2], "ptr", j[2]) for j in jobs])
        lens = np.array([j[3] for j in jobs], dtype=np.uint64)
        logs = np.array([j[4] for j in jobs], dtype=np.uint32)
        om = np.frombuffer(b"".join(_fr_bytes(j[5]) for j in jobs) or b"\0", dtype=np.uint8).copy()
        sh = np.frombuffer(b"".join(_fr_bytes(j[6] if len(j) > 6 else 1) for j in jobs) or b"\0",
                           dtype=np.uint8).copy()
        return count, modes, outs, ins, lens, logs, om, sh

    def ntt_batch(self, jobs) -> None:
        """Many transforms, one launch per pass level (zk_ntt_batch); asynchronous like ntt()."""
        count, modes, outs, ins, lens, logs, om, sh = self._ntt_args(jobs)
        check(load().zk_ntt_batch(self.handle, count, modes.ctypes.data, outs, ins, lens.ctypes.data,
                                  logs.ctypes.data, om.ctypes.data, sh.ctypes.data), "zk_ntt_batch")

    def ntt_plan(self, jobs, *, use_graph: bool = True, queue: bool = False) -> "NttPlan":
        """A prepared batch; ``queue``: its work-queue form (one persistent launch)."""
        count, modes, outs, ins, lens, logs, om, sh = self._ntt_args(jobs)
        h = ctypes.c_void_p()
        flags = (NTT_PLAN_GRAPH if use_graph else 0) | (NTT_PLAN_QUEUE if queue else 0)
        check(load().zk_ntt_plan_create(self.handle, count, modes.ctypes.data, outs, ins, lens.ctypes.data,
                                        logs.ctypes.data, om.ctypes.data, sh.ctypes.data, flags,
                                        ctypes.byref(h)), "zk_ntt_plan_create")
        return NttPlan(self, h.value, [j[1] for j in jobs] + [j[2] for j in jobs])

    def msm_batch_set_queue(self, on: bool) -> None:
        """G1 MSM batches (and their asynchronous form) in the work-queue form when on."""
        check(load().zk_msm_batch_set_queue(self.handle, 1 if on else 0), "zk_msm_batch_set_queue")

    def msm_queue_test_limit(self, limit_us: int) -> None:
        """Arms the next MSM work-queue launch with a wait that cannot succeed and this limit
        (zk_msm_queue_test_limit): that call then raises TimeoutError."""
        check(load().zk_msm_queue_test_limit(self.handle, int(limit_us)), "zk_msm_queue_test_limit")

    def ntt_batch_set_queue(self, on: bool) -> None:
        """ntt_batch in its work-queue form (one persistent launch) when on."""
        check(load().zk_ntt_batch_set_queue(self.handle, 1 if on else 0), "zk_ntt_batch_set_queue")

    def ntt_queue_status(self) -> None:
        """Waits for the context stream; raises TimeoutError if a work-queue launch gave up."""
        check(load().zk_ntt_queue_status(self.handle), "zk_ntt_queue_status")

    def ntt_queue_selftest(self, limit_us: int) -> int:
        """Runs a work-queue launch whose wait cannot succeed (zk_ntt_queue_selftest); returns
        1 + the queue entry whose wait ran out. Raises if the launch did not time out."""
        e = ctypes.c_uint32()
        rc = load().zk_ntt_queue_selftest(self.handle, int(limit_us), ctypes.byref(e))
        if rc != ZK_ETIMEOUT:
            check(rc, "zk_ntt_queue_selftest")
            raise ZkError("zk_ntt_queue_selftest: the wait did not run out")
        return int(e.value)

    # ---- tuning
    def tune_set_msm_window(self, log_n: int, window_bits: int) -> None:
        check(load().zk_tune_set_msm_window(self.handle, int(log_n), int(window_bits)), "zk_tune_set_msm_window")

    def tune_msm_window(self, n: int) -> int:
        v = ctypes.c_uint32()
        check(load().zk_tune_get_msm_window(self.handle, int(n), ctypes.byref(v)), "zk_tune_get_msm_window")
        return int(v.value)

    def tune_set_ntt_split(self, log_n: int, bits) -> None:
        arr = np.ascontiguousarray(list(bits) or [0], dtype=np.uint32)
        check(load().zk_tune_set_ntt_split(self.handle, int(log_n), len(bits), arr.ctypes.data),
              "zk_tune_set_ntt_split")

    def tune_ntt_split(self, log_n: int):
        np_ = ctypes.c_uint32()
        bits = np.zeros(4, dtype=np.uint32)
        check(load().zk_tune_get_ntt_split(self.handle, int(log_n), ctypes.byref(np_), bits.ctypes.data),
              "zk_tune_get_ntt_split")
        return [int(b) for b in bits[: np_.value]]

    def autotune_msm(self, bases: "Bases", scalars: DeviceArray, log_n: int, reps: int = 2):
        c = ctypes.c_uint32()
        ms = ctypes.c_double()
        check(load().zk_autotune_msm(self.handle, bases.handle, scalars.ptr, int(log_n), int(reps), ctypes.byref(c),
                                     ctypes.byref(ms)), "zk_autotune_msm")
        return int(c.value), float(ms.value)

    def autotune_ntt(self, data: DeviceArray, log_n: int, reps: int = 3):
        np_ = ctypes.c_uint32()
        bits = np.zeros(4, dtype=np.uint32)
        ms = ctypes.c_double()
        check(load().zk_autotune_ntt(self.handle, data.ptr, int(log_n), int(reps), ctypes.byref(np_),
                                     bits.ctypes.data, ctypes.byref(ms)), "zk_autotune_ntt")
        return [int(b) for b in bits[: np_.value]], float(ms.value)

    def autotune_save(self, path: str) -> None:
        check(load().zk_autotune_save(self.handle, os.fsencode(path)), "zk_autotune_save")

    def autotune_load(self, path: str) -> None:
        check(load().zk_autotune_load(self.handle, os.fsencode(path)), "zk_autotune_load")

    # ---- Groth16 prover vectors (Montgomery device arrays)
    def fr_spmv(self, nrows: int, row_ptr: DeviceArray, cols: DeviceArray, coeffs: DeviceArray, x, out) -> None:
        check(load().zk_fr_spmv(self.handle, int(nrows), row_ptr.ptr, cols.ptr, coeffs.ptr, getattr(x, "ptr", x),
                                getattr(out, "ptr", out)), "zk_fr_spmv")

    def fr_r1cs_check(self, a, b, c, n: int) -> int:
        bad = ctypes.c_uint64()
        check(load().zk_fr_r1cs_check(self.handle, getattr(a, "ptr", a), getattr(b, "ptr", b), getattr(c, "ptr", c),
                                      int(n), ctypes.byref(bad)), "zk_fr_r1cs_check")
        return int(bad.value)

    def fr_r1cs_check_async(self, a, b, c, n: int, bad_dev) -> None:
        """Adds #{i : a[i] b[i] != c[i]} to the uint64 at ``bad_dev`` (device) without waiting."""
        check(load().zk_fr_r1cs_check_async(self.handle, getattr(a, "ptr", a), getattr(b, "ptr", b),
                                            getattr(c, "ptr", c), int(n), getattr(bad_dev, "ptr", bad_dev)),
              "zk_fr_r1cs_check_async")

    def fr_qap_quotient(self, out, a, b, c, n: int, zinv: int) -> None:
        check(load().zk_fr_qap_quotient(self.handle, getattr(out, "ptr", out), getattr(a, "ptr", a),
                                        getattr(b, "ptr", b), getattr(c, "ptr", c), int(n), _fr_bytes(zinv)),
              "zk_fr_qap_quotient")

    def fr_gather(self, out, inp, idx: DeviceArray, n: int) -> None:
        check(load().zk_fr_gather(self.handle, getattr(out, "ptr", out), getattr(inp, "ptr", inp), idx.ptr, int(n)),
              "zk_fr_gather")

    def fr_scale(self, out, inp, s: int, n: int) -> None:
        check(load().zk_fr_scale(self.handle, getattr(out, "ptr", out), getattr(inp, "ptr", inp), _fr_bytes(s),
                                 int(n)), "zk_fr_scale")

    def fr_powers(self, out, base: int, n: int) -> None:
        check(load().zk_fr_powers(self.handle, getattr(out, "ptr", out), _fr_bytes(base), int(n)), "zk_fr_powers")

    def fr_batch_inv(self, out, inp, n: int) -> None:
        check(load().zk_fr_batch_inv(self.handle, getattr(out, "ptr", out), getattr(inp, "ptr", inp), int(n)),
              "zk_fr_batch_inv")

    def plonk_quotient_evals(self, inputs, m: int, n: int, omega_m: int, shift: int, shift_n: int, alpha: int,
                             beta: int, gamma: int, k1: int, k2: int, num_out, zh_out) -> None:
        if len(inputs) != 15:
            raise ValueError("PLONK quotient takes 15 evaluation vectors")
        arr = (ctypes.c_void_p * 15)(*[getattr(x, "ptr", x) for x in inputs])
        check(load().zk_plonk_quotient_evals(self.handle, arr, int(m), int(n), _fr_bytes(omega_m), _fr_bytes(shift),
                                             _fr_bytes(shift_n), _fr_bytes(alpha), _fr_bytes(beta),
                                             _fr_bytes(gamma), _fr_bytes(k1), _fr_bytes(k2),
                                             getattr(num_out, "ptr", num_out), getattr(zh_out, "ptr", zh_out)),
              "zk_plonk_quotient_evals")

    def fr_div_xn_minus_1(self, a, length: int, n: int, q_out, r_out):
        ql, rl = ctypes.c_size_t(), ctypes.c_size_t()
        check(load().zk_fr_div_xn_minus_1(self.handle, getattr(a, "ptr", a), int(length), int(n),
                                          getattr(q_out, "ptr", q_out), getattr(r_out, "ptr", r_out),
                                          ctypes.byref(ql), ctypes.byref(rl)), "zk_fr_div_xn_minus_1")
        return int(ql.value), int(rl.value)

    def g2_fixed_base_mul(self, point, k: DeviceArray, n: int, out: DeviceArray) -> None:
        """out[i] = [k_i] P on G2; point = ((x0, x1), (y0, y1)) canonical."""
        (x0, x1), (y0, y1) = point
        pb = b"".join(int(v).to_bytes(32, "little") for v in (x0, x1, y0, y1))
        check(load().zk_g2_fixed_base_mul(self.handle, pb, k.ptr, int(n), out.ptr), "zk_g2_fixed_base_mul")

    def g1_fixed_base_mul(self, point_xy, k: DeviceArray, n: int, out: DeviceArray) -> None:
        x, y = point_xy
        pb = int(x).to_bytes(32, "little") + int(y).to_bytes(32, "little")
        check(load().zk_g1_fixed_base_mul(self.handle, pb, k.ptr, int(n), out.ptr), "zk_g1_fixed_base_mul")


_default: Optional[Context] = None


def default_context() -> Context:
    global _default
    with _lock:
        pass
    if _default is None:
        _default = Context(int(os.environ.get("ZKGPU_DEVICE", "0")))
    return _default
