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

ZK_OK, ZK_EINVAL, ZK_ECUDA, ZK_ENOMEM, ZK_ENODEV = 0, 1, 2, 3, 4

NTT_EVALS_FROM_COEFFS = 0
NTT_COEFFS_FROM_EVALS = 1
NTT_COSET_EVALS_FROM_COEFFS = 2
NTT_COSET_COEFFS_FROM_EVALS = 3

EXPORTED_SYMBOLS = (
    "zk_last_error", "zk_version", "zk_ctx_create", "zk_ctx_destroy", "zk_ctx_sync", "zk_ctx_stream",
    "zk_ctx_num_sms", "zk_alloc", "zk_free", "zk_h2d", "zk_d2h", "zk_host_alloc", "zk_host_free",
    "zk_fr_to_mont", "zk_fr_from_mont", "zk_fq_to_mont", "zk_fq_from_mont", "zk_fr_mul", "zk_fr_sub", "zk_ntt",
    "zk_bases_create", "zk_bases_create_dev", "zk_bases_destroy", "zk_bases_count", "zk_msm_g1",
    "zk_g1_fixed_base_mul", "zk_memset", "zk_launch_count", "zk_prof_enable", "zk_prof_reset", "zk_prof_count",
    "zk_prof_get", "zk_timer_start", "zk_timer_stop", "zk_msm_last_stats", "zk_imad_peak", "zk_d2d",
    "zk_fr_trimmed_len", "zk_ntt_noalloc", "zk_imad_probe", "zk_bases_precompute",
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
    raise ZkError(text)


class DeviceArray:
    """An owned device allocation of ``nbytes`` (freed with the context's pool)."""

    __slots__ = ("ctx", "ptr", "nbytes", "__weakref__")

    def __init__(self, ctx: "Context", nbytes: int) -> None:
        self.ctx = ctx
        self.nbytes = int(nbytes)
        p = ctypes.c_void_p()
        check(load().zk_alloc(ctx.handle, max(16, self.nbytes), ctypes.byref(p)), "zk_alloc")
        self.ptr = p.value

    def free(self) -> None:
        if self.ptr is not None and self.ctx.handle is not None:
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


class Context:
    """One GPU, one stream (zk_ctx)."""

    def __init__(self, device: int = 0) -> None:
        L = load()
        h = ctypes.c_void_p()
        check(L.zk_ctx_create(int(device), ctypes.byref(h)), "zk_ctx_create")
        self.handle = h.value
        self.device = device

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
