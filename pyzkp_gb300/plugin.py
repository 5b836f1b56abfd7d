"""GB300 KernelFns for pyZKP's ``KernelRegistry`` -- the drop-in for the Metal backend.

``register_gb300_kernels(registry)`` installs KernelFns under the keys of
``register_metal_kernels`` (runtime/kernels/metal/kernels.py:12-20), i.e.
``(OpType.X, Device.METAL, Backend.METAL)`` for POINTWISE_MUL, POLY_SUB,
ROOTS_EVALS_FROM_COEFFS, ROOTS_COEFFS_FROM_EVALS, COSET_EVALS_FROM_COEFFS,
COSET_COEFFS_FROM_EVALS, MSM_G1, KZG_BATCH_COMMIT (plus MSM_G1_BATCH, and MSM_G2,
POLY_MUL_NTT, DIV_XN_MINUS_1, BATCH_INV and PLONK_T_QUOTIENT_EVALS, which the reference
runs on the CPU only), and
replaces the transfer kernels (TO_DEVICE on CPU, FROM_DEVICE on CPU and METAL,
runtime/kernels/cpu/kernels.py:75-77,98-172) so that device data lives in GB300
memory. ``Executor._run_node`` (runtime/executor.py:167-218) calls them unchanged.

Semantics follow the reference op contract, the CPU KernelFns
(runtime/kernels/cpu/kernels.py:175-250, 271-309, 325-335, 441-496): forward NTTs
pad or truncate to ``attrs["n"]`` (the Metal versions ignore it,
runtime/kernels/metal/kernels.py:427,509), inverse NTTs keep the input length,
POLY_SUB pads to the longer input and trims trailing zeros, MSM results are
returned on the CPU as ``(FQ(x), FQ(y), FQ(1))`` like runtime/metal/msm.py:36-63.
Errors: ``ValueError`` for dtype / length / power-of-two violations,
``RuntimeError`` when no GB300 context is present (runtime/kernels/metal/kernels.py:92-110).

``install()`` redirects the reference's ``MetalContext.create_default`` to
``GpuContext.create_default`` and its ``runtime.kernels.metal.register_metal_kernels``
to ``register_gb300_kernels``, so the reference's provers
(protocols/groth16/prove.py:56-62, qap.py:70-76, plonk/prove.py:64-69) run on GB300
with ``RuntimeConfig(backend=Backend.METAL)`` and no other change.
"""

from __future__ import annotations

import importlib
import sys
from dataclasses import dataclass
from typing import Any, Dict, List, Optional, Tuple

import numpy as np

from pyzkp_gb300 import _native as N

FR_MODULUS = 21888242871839275222246405745257275088548364400416034343698204186575808495617
_MAX_LOG_N = 28


# ------------------------------------------------------------------------------ buffers
@dataclass
class GpuBuffer:
    """Device FR vector, the counterpart of ``MetalBuffer`` (runtime/metal/buffer.py:7-15).

    ``mtl_buffer`` is the device allocation (``_native.DeviceArray``); the executor
    releases it through ``pool.release_metal(buf.data.mtl_buffer)`` (executor.py:139-140).
    """

    dtype: str
    n: int
    mtl_buffer: Any
    host_cache: Optional[list] = None

    def __len__(self) -> int:
        return int(self.n)

    def to_host(self) -> List[int]:
        """The canonical values (one device-to-host read; Montgomery -> canonical on the device)."""
        n = int(self.n)
        if n == 0:
            return []
        zk = self.mtl_buffer.ctx
        tmp = zk.alloc(n * 32)
        zk.fr_from_mont(tmp, self.mtl_buffer, n)
        vals = _bytes_to_ints(tmp.download(n * 32), n)
        tmp.free()
        return vals

    # Callers that read kept device outputs as lists (protocols/groth16/qap.py:93-97 does
    # list(g.buffers[...].data)) get the canonical values.
    def __iter__(self):
        return iter(self.to_host())

    def __getitem__(self, i):
        return self.to_host()[i]


class _DeviceAllocator:
    """The ``rt.device.newBufferWithLength_options_`` protocol used by MemoryPool.alloc_metal
    (runtime/memory.py:56-81), backed by GB300 memory."""

    def __init__(self, zk: N.Context) -> None:
        self._zk = zk

    def newBufferWithLength_options_(self, size_bytes: int, _options: int = 0) -> N.DeviceArray:
        return self._zk.alloc(int(size_bytes))


class GpuRuntime:
    """Counterpart of ``MetalRuntime`` (runtime/metal/runtime.py:469-629): the device
    handle plus the resident-base cache of the MSM ops."""

    def __init__(self, zk: N.Context, bases_budget_bytes: int = 64 << 30) -> None:
        self.zk = zk
        self.device = _DeviceAllocator(zk)
        self._bases: Dict[Any, Tuple[Any, N.Bases, int]] = {}
        self._bases_order: List[Any] = []
        self._bases_budget = int(bases_budget_bytes)
        self._bases_bytes = 0

    @staticmethod
    def create_default(device: int = 0) -> "GpuRuntime":
        return GpuRuntime(N.Context(device))

    # -- resident bases ------------------------------------------------------
    def bases_for(self, points, g2: bool = False) -> N.Bases:
        """Montgomery affine copy of ``points`` (G1, or G2 with ``g2``) on the device.

        Tuples (the reference's ``cached_points_tuple`` form, runtime/warmup.py:17-26)
        are cached by identity while a reference is held; lists by identity plus a
        fingerprint of sampled coordinates, since they can be mutated in place.
        """
        tag = "t2" if g2 else "t"
        key = (tag, id(points)) if isinstance(points, tuple) else ("l" + tag, id(points), _fingerprint(points))
        hit = self._bases.get(key)
        if hit is not None and hit[0] is points:
            self._bases_order.remove(key)
            self._bases_order.append(key)
            return hit[1]
        xy = points_g2_to_affine_array(points) if g2 else points_to_affine_array(points)
        b = self.zk.bases_g2_from_host(xy) if g2 else self.zk.bases_from_host(xy)
        size = xy.nbytes
        while self._bases_order and self._bases_bytes + size > self._bases_budget:
            old = self._bases_order.pop(0)
            _, ob, osz = self._bases.pop(old)
            ob.free()
            self._bases_bytes -= osz
        self._bases[key] = (points, b, size)
        self._bases_order.append(key)
        self._bases_bytes += size
        return b


def fixed_base_window(n: int) -> int:
    """Window of the fixed-base mode. Its rows [2^(c j)] P_i share one bucket set, so the work
    is about n ceil(255/c) mixed additions (10 Fq products) plus 2^(c-1) buckets to reduce
    (~28): the c in 8..20 that minimises it (20 at n = 2^20: 13 rows)."""
    n = max(1, int(n))
    return min(range(8, 21), key=lambda c: (n * -(-255 // c) * 10 + (1 << (c - 1)) * 28, c))


def _fingerprint(points) -> int:
    n = len(points)
    idx = sorted(set([0, n - 1] + [i * n // 16 for i in range(16)])) if n else []
    acc = [n]
    for i in idx:
        p = points[i]
        for c in p:
            coeffs = getattr(c, "coeffs", None)
            acc.extend(int(v) for v in coeffs) if coeffs is not None else acc.append(int(c))
    return hash(tuple(acc))


def _py_ecc():
    """The curve module of the points (the reference's dependency py_ecc.optimized_bn128)."""
    return importlib.import_module("py_ecc.optimized_bn128")


def points_to_affine_array(points) -> np.ndarray:
    """Sequence of py_ecc G1 points -> uint64[n, 8] affine canonical, (0, 0) for infinity
    (the conversion _pack_g1_point does per call, runtime/metal/msm.py:13-34)."""
    n = len(points)
    out = bytearray(64 * n)
    b = None
    for i, p in enumerate(points):
        if int(p[2]) == 0:
            continue
        if int(p[2]) == 1:
            x, y = int(p[0]), int(p[1])
        else:
            if b is None:
                b = _py_ecc()
            ax, ay = b.normalize(p)
            x, y = int(ax), int(ay)
        out[64 * i:64 * i + 32] = x.to_bytes(32, "little")
        out[64 * i + 32:64 * i + 64] = y.to_bytes(32, "little")
    return np.frombuffer(bytes(out), dtype="<u8").reshape(n, 8).astype(np.uint64) if n else np.zeros((0, 8), np.uint64)


def points_g2_to_affine_array(points) -> np.ndarray:
    """Sequence of py_ecc G2 points (FQ2 coordinates) -> uint64[n, 16] affine canonical
    (x.c0, x.c1, y.c0, y.c1), all zero for infinity."""
    n = len(points)
    out = bytearray(128 * n)
    b = None
    for i, p in enumerate(points):
        z = p[2]
        if all(int(v) == 0 for v in z.coeffs):
            continue
        if int(z.coeffs[0]) == 1 and int(z.coeffs[1]) == 0:
            x, y = p[0], p[1]
        else:
            if b is None:
                b = _py_ecc()
            x, y = b.normalize(p)
        vals = (int(x.coeffs[0]), int(x.coeffs[1]), int(y.coeffs[0]), int(y.coeffs[1]))
        out[128 * i:128 * i + 128] = b"".join(v.to_bytes(32, "little") for v in vals)
    return np.frombuffer(bytes(out), dtype="<u8").reshape(n, 16).astype(np.uint64) if n else np.zeros((0, 16),
                                                                                                     np.uint64)


def _g2_point(res):
    """((x0, x1), (y0, y1)) or None -> the reference's G2 object (FQ2 coordinates)."""
    b = _py_ecc()
    if res is None:
        return b.Z2
    (x0, x1), (y0, y1) = res
    return (b.FQ2([x0, x1]), b.FQ2([y0, y1]), b.FQ2.one())


def _omega_for_size(n: int) -> int:
    """crypto/poly/ntt.py:13-24 (ROOT_2_28 of ntt.py:8)."""
    root = 19103219067921713944291392827692070036145651957329286315305642004821462161904
    return pow(root, 1 << (_MAX_LOG_N - _log2_exact(n)), FR_MODULUS)


def _g1_point(res):
    """Affine canonical (x, y) or None -> the reference's G1 object (runtime/metal/msm.py:45-63)."""
    b = _py_ecc()
    if res is None:
        return b.Z1
    return (b.FQ(res[0]), b.FQ(res[1]), b.FQ(1))


# ------------------------------------------------------------------------------ context
def _ir_for(registry) -> Any:
    """The module holding OpType / Device / Backend / DType / Buffer of ``registry``'s runtime
    (the reference's ``runtime.ir`` for ``runtime.kernels.registry.KernelRegistry``)."""
    modname = type(registry).__module__
    if modname.endswith(".kernels.registry"):
        return importlib.import_module(modname[: -len(".kernels.registry")] + ".ir")
    return importlib.import_module(modname)


@dataclass
class GpuContext:
    """Counterpart of ``MetalContext`` (runtime/context.py:25-36): ``metal`` holds the GB300
    runtime so code that tests ``getattr(context, "metal", None)`` keeps working."""

    backend: Any = None
    device: Any = None
    pool: Any = None
    config: Any = None
    metal: Any = None

    @staticmethod
    def create_default(*, pool=None, config=None, ir: Any = None, device: int = 0) -> "GpuContext":
        if ir is None:
            ir = _default_ir()
        rt = _shared_runtime(device)
        return GpuContext(backend=ir.Backend.METAL, device=ir.Device.METAL, pool=pool, config=config, metal=rt)


_RUNTIMES: Dict[int, GpuRuntime] = {}


def _shared_runtime(device: int = 0) -> GpuRuntime:
    rt = _RUNTIMES.get(device)
    if rt is None:
        rt = GpuRuntime.create_default(device)
        _RUNTIMES[device] = rt
    return rt


def _default_ir():
    """The reference's ``runtime.ir`` (its IR types); the plugin has no runtime of its own."""
    if "runtime.ir" in sys.modules:
        return sys.modules["runtime.ir"]
    try:
        return importlib.import_module("runtime.ir")
    except ImportError as e:
        raise ImportError("pyZKP's runtime (runtime.ir) is not importable: put the reference on sys.path, "
                          "or pass its runtime.ir module as ir=") from e


# ------------------------------------------------------------------------------ helpers
def _runtime(ctx: Dict[str, Any], what: str) -> GpuRuntime:
    c = ctx.get("context")
    rt = getattr(c, "metal", None) if c is not None else None
    if not isinstance(rt, GpuRuntime):
        raise RuntimeError(f"gb300 {what} requires GpuContext with a GB300 runtime")
    return rt


def _alloc(ctx: Dict[str, Any], rt: GpuRuntime, nbytes: int) -> N.DeviceArray:
    pool = ctx.get("pool")
    if pool is not None and hasattr(pool, "alloc_metal"):
        buf = pool.alloc_metal(rt, nbytes)
        if isinstance(buf, N.DeviceArray) and buf.nbytes >= nbytes:
            return buf
    return rt.zk.alloc(nbytes)


def _ints_to_bytes(values) -> bytes:
    r = FR_MODULUS
    return b"".join((int(v) % r).to_bytes(32, "little") for v in values)


def _bytes_to_ints(raw: np.ndarray, n: int) -> List[int]:
    mv = memoryview(raw.tobytes())
    fb = int.from_bytes
    return [fb(mv[32 * i:32 * i + 32], "little") for i in range(n)]


def _device_fr(ctx: Dict[str, Any], buf, what: str) -> GpuBuffer:
    if not isinstance(buf.data, GpuBuffer):
        raise ValueError(f"gb300 {what} expects a device FR buffer")
    return buf.data


def _log2_exact(n: int) -> int:
    if n <= 0 or n & (n - 1):
        raise ValueError("n must be a power of two")
    lg = n.bit_length() - 1
    if lg > _MAX_LOG_N:
        raise ValueError("domain too large for BN254 root of unity")
    return lg


# ------------------------------------------------------------------------------ registration
def register_gb300_kernels(registry, *, ir: Any = None) -> None:
    """Register the GB300 KernelFns into ``registry`` (the reference's ``KernelRegistry``)."""
    ir = ir or _ir_for(registry)
    OpType, Device, Backend, DType, Buffer = ir.OpType, ir.Device, ir.Backend, ir.DType, ir.Buffer
    METAL, BM = Device.METAL, Backend.METAL

    def to_device(ctx):
        node = ctx["node"]
        inp = ctx["inputs"][0]
        out_id = node.outputs[0]
        if inp.dtype != DType.FR:
            if inp.dtype in (DType.OBJ, DType.G1, DType.G2):
                return {"outputs": {out_id: Buffer(id=out_id, device=METAL, dtype=inp.dtype, data=inp.data)}}
            raise ValueError(f"to_device supports FR only, got {inp.dtype}")
        rt = _runtime(ctx, "to_device")
        host = inp.data
        n = len(host)
        d = _alloc(ctx, rt, n * 32)
        if n:
            d.upload(np.frombuffer(_ints_to_bytes(host), dtype=np.uint8))
            rt.zk.fr_to_mont(d, d, n)
        gb = GpuBuffer(dtype="fr_mont_u64x4", n=n, mtl_buffer=d)
        return {"outputs": {out_id: Buffer(id=out_id, device=METAL, dtype=inp.dtype, data=gb, meta={"n": n})}}

    def from_device(ctx):
        node = ctx["node"]
        inp = ctx["inputs"][0]
        out_id = node.outputs[0]
        if inp.device == Device.CPU:
            return {"outputs": {out_id: Buffer(id=out_id, device=Device.CPU, dtype=inp.dtype, data=inp.data)}}
        if inp.dtype != DType.FR:
            if inp.dtype in (DType.OBJ, DType.G1, DType.G2):
                return {"outputs": {out_id: Buffer(id=out_id, device=Device.CPU, dtype=inp.dtype, data=inp.data)}}
            raise ValueError("from_device supports FR only")
        if not isinstance(inp.data, GpuBuffer):
            raise ValueError("from_device expects a device FR buffer")
        rt = _runtime(ctx, "from_device")
        n = int(inp.data.n)
        vals: List[int] = []
        if n:
            tmp = rt.zk.alloc(n * 32)
            rt.zk.fr_from_mont(tmp, inp.data.mtl_buffer, n)
            vals = _bytes_to_ints(tmp.download(n * 32), n)
            tmp.free()
        return {"outputs": {out_id: Buffer(id=out_id, device=Device.CPU, dtype=inp.dtype, data=vals, meta={"n": n})}}

    def _ntt(ctx, mode: int, what: str):
        node = ctx["node"]
        inp = ctx["inputs"][0]
        out_id = node.outputs[0]
        attrs = ctx["attrs"]
        if inp.dtype != DType.FR:
            raise ValueError(f"gb300 {what} supports FR only")
        src = _device_fr(ctx, inp, what)
        rt = _runtime(ctx, what)
        omega = int(attrs["omega"]) % FR_MODULUS
        inverse = mode in (N.NTT_COEFFS_FROM_EVALS, N.NTT_COSET_COEFFS_FROM_EVALS)
        n = int(src.n) if inverse else int(attrs["n"])
        shift = int(attrs["shift"]) if mode in (N.NTT_COSET_EVALS_FROM_COEFFS, N.NTT_COSET_COEFFS_FROM_EVALS) else 1
        if n <= 0:
            out = rt.zk.alloc(16)
            gb = GpuBuffer(dtype="fr_mont_u64x4", n=0, mtl_buffer=out)
        else:
            log_n = _log2_exact(n)
            out = _alloc(ctx, rt, n * 32)
            rt.zk.ntt(mode, out, src.mtl_buffer, int(src.n), log_n, omega, shift % FR_MODULUS)
            gb = GpuBuffer(dtype="fr_mont_u64x4", n=n, mtl_buffer=out)
        if mode == N.NTT_EVALS_FROM_COEFFS:
            meta = {"n": n, "omega": int(attrs["omega"])}
        elif mode == N.NTT_COEFFS_FROM_EVALS:
            meta = {"omega": int(attrs["omega"])}
        elif mode == N.NTT_COSET_EVALS_FROM_COEFFS:
            meta = {"n": n, "omega": int(attrs["omega"]), "shift": int(attrs["shift"])}
        else:
            meta = {"omega": int(attrs["omega"]), "shift": int(attrs["shift"])}
        return {"outputs": {out_id: Buffer(id=out_id, device=METAL, dtype=DType.FR, data=gb, meta=meta)}}

    def roots_evals_from_coeffs(ctx):
        return _ntt(ctx, N.NTT_EVALS_FROM_COEFFS, "roots_evals_from_coeffs")

    def roots_coeffs_from_evals(ctx):
        return _ntt(ctx, N.NTT_COEFFS_FROM_EVALS, "roots_coeffs_from_evals")

    def coset_evals_from_coeffs(ctx):
        return _ntt(ctx, N.NTT_COSET_EVALS_FROM_COEFFS, "coset_evals_from_coeffs")

    def coset_coeffs_from_evals(ctx):
        return _ntt(ctx, N.NTT_COSET_COEFFS_FROM_EVALS, "coset_coeffs_from_evals")

    def pointwise_mul(ctx):
        node = ctx["node"]
        a, b = ctx["inputs"][0], ctx["inputs"][1]
        out_id = node.outputs[0]
        if a.dtype != DType.FR or b.dtype != DType.FR:
            raise ValueError("gb300 pointwise_mul supports FR only")
        ga, gb_ = _device_fr(ctx, a, "pointwise_mul"), _device_fr(ctx, b, "pointwise_mul")
        if len(ga) != len(gb_):
            raise ValueError("length mismatch")
        rt = _runtime(ctx, "pointwise_mul")
        n = int(ga.n)
        out = _alloc(ctx, rt, max(1, n) * 32)
        rt.zk.fr_mul(out, ga.mtl_buffer, gb_.mtl_buffer, n)
        res = GpuBuffer(dtype="fr_mont_u64x4", n=n, mtl_buffer=out)
        return {"outputs": {out_id: Buffer(id=out_id, device=METAL, dtype=DType.FR, data=res, meta={"n": n})}}

    def poly_sub(ctx):
        node = ctx["node"]
        a, b = ctx["inputs"][0], ctx["inputs"][1]
        out_id = node.outputs[0]
        if a.dtype != DType.FR or b.dtype != DType.FR:
            raise ValueError("gb300 poly_sub supports FR only")
        ga, gb_ = _device_fr(ctx, a, "poly_sub"), _device_fr(ctx, b, "poly_sub")
        rt = _runtime(ctx, "poly_sub")
        na, nb = int(ga.n), int(gb_.n)
        n = max(na, nb)
        out = _alloc(ctx, rt, max(1, n) * 32)
        if n:
            # out = pad(a) - pad(b), then trim trailing zeros (crypto/poly/cpu_ref.py:18-25)
            rt.zk.memset(out, 0)
            rt.zk.d2d(out, ga.mtl_buffer, na * 32)
            rt.zk.fr_sub(out, out, gb_.mtl_buffer, nb)
            n = rt.zk.fr_trimmed_len(out, n)
        res = GpuBuffer(dtype="fr_mont_u64x4", n=n, mtl_buffer=out)
        return {"outputs": {out_id: Buffer(id=out_id, device=METAL, dtype=DType.FR, data=res, meta={"n": n})}}

    def _window_hint(attrs) -> int:
        w = int(attrs.get("window_bits", 0) or 0)
        return w if 4 <= w <= 20 else 0  # any valid window yields the same point

    def _fixed_base(rt: GpuRuntime, bases: N.Bases, num: int, attrs) -> None:
        """Fixed-base mode when the op asks for it (attrs fixed_base True, or the policy "on",
        runtime/kernels/cpu/kernels.py:560-569 / runtime/warmup.py:125-150): window-shifted rows
        of the resident bases, computed once per base set. The point is the same either way."""
        if not (attrs.get("fixed_base") is True or attrs.get("fixed_base_policy") == "on"):
            return
        c = fixed_base_window(bases.n)
        if getattr(bases, "fixed_c", None) != c:
            rt.zk.bases_precompute(bases, c)
            bases.fixed_c = c

    def msm_g1(ctx):
        node = ctx["node"]
        points, scalars = ctx["inputs"][0], ctx["inputs"][1]
        out_id = node.outputs[0]
        rt = _runtime(ctx, "msm_g1")
        if scalars.dtype != DType.FR:
            raise ValueError("gb300 msm_g1 scalars must be FR")
        gs = _device_fr(ctx, scalars, "msm_g1")
        num = int(gs.n)
        if num > len(points.data):
            raise ValueError("scalars length exceeds points length")
        if num == 0:
            pt = _g1_point(None)
        else:
            bases = rt.bases_for(points.data)
            _fixed_base(rt, bases, num, ctx["attrs"])
            pt = _g1_point(rt.zk.msm_g1(bases, gs.mtl_buffer, num, window_bits=_window_hint(ctx["attrs"])))
        return {"outputs": {out_id: Buffer(id=out_id, device=Device.CPU, dtype=DType.G1, data=pt)}}

    def msm_g2(ctx):
        """MSM_G2 (runtime/kernels/cpu/kernels.py:338-348,574-582; CPU-only in the reference)."""
        node = ctx["node"]
        points, scalars = ctx["inputs"][0], ctx["inputs"][1]
        out_id = node.outputs[0]
        rt = _runtime(ctx, "msm_g2")
        if scalars.dtype != DType.FR:
            raise ValueError("gb300 msm_g2 scalars must be FR")
        gs = _device_fr(ctx, scalars, "msm_g2")
        num = int(gs.n)
        if num > len(points.data):
            raise ValueError("scalars length exceeds points length")
        if num == 0:
            pt = _g2_point(None)
        else:
            bases = rt.bases_for(points.data, g2=True)
            pt = _g2_point(rt.zk.msm_g2(bases, gs.mtl_buffer, num, window_bits=_window_hint(ctx["attrs"])))
        return {"outputs": {out_id: Buffer(id=out_id, device=Device.CPU, dtype=DType.G2, data=pt)}}

    def poly_mul_ntt(ctx):
        """POLY_MUL_NTT (runtime/kernels/cpu/kernels.py:288-298 -> crypto/poly/ntt.py:149-162):
        a * b through NTTs of size 2^ceil(log2(len a + len b - 1)), trailing zeros trimmed."""
        node = ctx["node"]
        a, b = ctx["inputs"][0], ctx["inputs"][1]
        out_id = node.outputs[0]
        if a.dtype != DType.FR or b.dtype != DType.FR:
            raise ValueError("gb300 poly_mul_ntt supports FR only")
        ga, gb_ = _device_fr(ctx, a, "poly_mul_ntt"), _device_fr(ctx, b, "poly_mul_ntt")
        rt = _runtime(ctx, "poly_mul_ntt")
        na, nb = int(ga.n), int(gb_.n)
        if na == 0 or nb == 0:
            res = GpuBuffer(dtype="fr_mont_u64x4", n=0, mtl_buffer=rt.zk.alloc(16))
            return {"outputs": {out_id: Buffer(id=out_id, device=METAL, dtype=DType.FR, data=res, meta={"n": 0})}}
        need = na + nb - 1
        n = 1 << (need - 1).bit_length()
        lg, om = _log2_exact(n), _omega_for_size(n)
        ea = _alloc(ctx, rt, n * 32)
        eb = rt.zk.alloc(n * 32)
        rt.zk.ntt_batch([(N.NTT_EVALS_FROM_COEFFS, ea, ga.mtl_buffer, na, lg, om, 1),
                         (N.NTT_EVALS_FROM_COEFFS, eb, gb_.mtl_buffer, nb, lg, om, 1)])
        rt.zk.fr_mul(ea, ea, eb, n)
        rt.zk.ntt(N.NTT_COEFFS_FROM_EVALS, ea, ea, n, lg, om)
        out_n = rt.zk.fr_trimmed_len(ea, need)
        eb.free()
        res = GpuBuffer(dtype="fr_mont_u64x4", n=out_n, mtl_buffer=ea)
        return {"outputs": {out_id: Buffer(id=out_id, device=METAL, dtype=DType.FR, data=res, meta={"n": out_n})}}

    def div_xn_minus_1(ctx):
        """DIV_XN_MINUS_1 (runtime/kernels/cpu/kernels.py:312-323 -> crypto/poly/fast.py:8-37):
        quotient and remainder by X^n - 1, both trimmed."""
        node = ctx["node"]
        inp = ctx["inputs"][0]
        n = int(ctx["attrs"]["n"])
        if n <= 0:
            raise ValueError("n must be positive")
        if inp.dtype != DType.FR:
            raise ValueError("gb300 div_xn_minus_1 supports FR only")
        g = _device_fr(ctx, inp, "div_xn_minus_1")
        rt = _runtime(ctx, "div_xn_minus_1")
        length = int(g.n)
        q = _alloc(ctx, rt, max(1, length - n) * 32)
        r = _alloc(ctx, rt, n * 32)
        ql, rl = rt.zk.fr_div_xn_minus_1(g.mtl_buffer, length, n, q, r)
        q_id, r_id = node.outputs[0], node.outputs[1]
        qb = GpuBuffer(dtype="fr_mont_u64x4", n=ql, mtl_buffer=q)
        rb = GpuBuffer(dtype="fr_mont_u64x4", n=rl, mtl_buffer=r)
        return {"outputs": {q_id: Buffer(id=q_id, device=METAL, dtype=DType.FR, data=qb, meta={"n": ql}),
                            r_id: Buffer(id=r_id, device=METAL, dtype=DType.FR, data=rb, meta={"n": rl})}}

    def batch_inv(ctx):
        """BATCH_INV (runtime/kernels/cpu/kernels.py:_batch_inv): inverses, 0 for 0."""
        node = ctx["node"]
        inp = ctx["inputs"][0]
        out_id = node.outputs[0]
        if inp.dtype != DType.FR:
            raise ValueError("gb300 batch_inv supports FR only")
        g = _device_fr(ctx, inp, "batch_inv")
        rt = _runtime(ctx, "batch_inv")
        n = int(g.n)
        out = _alloc(ctx, rt, max(1, n) * 32)
        rt.zk.fr_batch_inv(out, g.mtl_buffer, n)
        res = GpuBuffer(dtype="fr_mont_u64x4", n=n, mtl_buffer=out)
        return {"outputs": {out_id: Buffer(id=out_id, device=METAL, dtype=DType.FR, data=res, meta=inp.meta)}}

    def plonk_t_quotient_evals(ctx):
        """PLONK_T_QUOTIENT_EVALS (runtime/kernels/cpu/kernels.py:_plonk_t_quotient_evals), fused."""
        node = ctx["node"]
        attrs = ctx["attrs"]
        rt = _runtime(ctx, "plonk_t_quotient_evals")
        m = int(attrs["m"])
        bufs = [_device_fr(ctx, b, "plonk_t_quotient_evals") for b in ctx["inputs"][:15]]
        if len(bufs) != 15 or any(int(b.n) != m for b in bufs):
            raise ValueError("eval length mismatch")
        num = _alloc(ctx, rt, max(1, m) * 32)
        zh = _alloc(ctx, rt, max(1, m) * 32)
        rt.zk.plonk_quotient_evals([b.mtl_buffer for b in bufs], m, int(attrs["n"]), int(attrs["omega_m"]),
                                   int(attrs["shift"]), int(attrs["shift_n"]), int(attrs["alpha"]),
                                   int(attrs["beta"]), int(attrs["gamma"]), int(attrs["k1"]), int(attrs["k2"]),
                                   num, zh)
        o_num, o_zh = node.outputs[0], node.outputs[1]
        return {"outputs": {
            o_num: Buffer(id=o_num, device=METAL, dtype=DType.FR,
                          data=GpuBuffer(dtype="fr_mont_u64x4", n=m, mtl_buffer=num), meta={"m": m}),
            o_zh: Buffer(id=o_zh, device=METAL, dtype=DType.FR,
                         data=GpuBuffer(dtype="fr_mont_u64x4", n=m, mtl_buffer=zh), meta={"m": m})}}

    def _msm_many(rt: GpuRuntime, points, scalar_lists, attrs) -> List[Any]:
        """Instance k = MSM of scalar_lists[k] over points[:len(scalar_lists[k])]
        (msm_pippenger_batch semantics, crypto/msm/pippenger.py:124-214): one batched call,
        one pipeline per window size (zk_msm_g1_batch)."""
        lens = [len(s) for s in scalar_lists]
        total = sum(lens)
        if total == 0:
            return [_g1_point(None) for _ in scalar_lists]
        bases = rt.bases_for(points)
        _fixed_base(rt, bases, max(lens), attrs)
        flat = rt.zk.alloc(total * 32)
        flat.upload(np.frombuffer(_ints_to_bytes(v for s in scalar_lists for v in s), dtype=np.uint8))
        ptrs, off = [], 0
        for ln in lens:
            ptrs.append(flat.ptr + 32 * off)
            off += ln
        res = rt.zk.msm_g1_batch(bases, ptrs, lens, scalars_mont=False, window_bits=_window_hint(attrs))
        flat.free()
        return [_g1_point(r) for r in res]

    def kzg_batch_commit(ctx):
        node = ctx["node"]
        srs, polys = ctx["inputs"][0], ctx["inputs"][1]
        out_id = node.outputs[0]
        rt = _runtime(ctx, "kzg_batch_commit")
        s = srs.data
        scalar_lists = [[int(x) % FR_MODULUS for x in coeffs] for coeffs in polys.data]
        max_len = max((len(sc) for sc in scalar_lists), default=0)
        if max_len > len(s.g1_powers):
            raise ValueError("SRS too small for polynomial degree")
        outs = _msm_many(rt, s.g1_powers, scalar_lists, ctx["attrs"])
        return {"outputs": {out_id: Buffer(id=out_id, device=Device.CPU, dtype=DType.OBJ, data=outs)}}

    def msm_g1_batch(ctx):
        node = ctx["node"]
        points, scalars_list = ctx["inputs"][0], ctx["inputs"][1]
        out_id = node.outputs[0]
        rt = _runtime(ctx, "msm_g1_batch")
        lists = [[int(c) % FR_MODULUS for c in sc] for sc in scalars_list.data]
        if max((len(sc) for sc in lists), default=0) > len(points.data):
            raise ValueError("points and scalars length mismatch")
        outs = _msm_many(rt, points.data, lists, ctx["attrs"])
        return {"outputs": {out_id: Buffer(id=out_id, device=Device.CPU, dtype=DType.OBJ, data=outs)}}

    kernels = {
        (OpType.POINTWISE_MUL, METAL): pointwise_mul,
        (OpType.POLY_SUB, METAL): poly_sub,
        (OpType.ROOTS_EVALS_FROM_COEFFS, METAL): roots_evals_from_coeffs,
        (OpType.ROOTS_COEFFS_FROM_EVALS, METAL): roots_coeffs_from_evals,
        (OpType.COSET_EVALS_FROM_COEFFS, METAL): coset_evals_from_coeffs,
        (OpType.COSET_COEFFS_FROM_EVALS, METAL): coset_coeffs_from_evals,
        (OpType.MSM_G1, METAL): msm_g1,
        (OpType.KZG_BATCH_COMMIT, METAL): kzg_batch_commit,
        (OpType.MSM_G1_BATCH, METAL): msm_g1_batch,
        (OpType.MSM_G2, METAL): msm_g2,
        (OpType.POLY_MUL_NTT, METAL): poly_mul_ntt,
        (OpType.DIV_XN_MINUS_1, METAL): div_xn_minus_1,
        (OpType.BATCH_INV, METAL): batch_inv,
        (OpType.PLONK_T_QUOTIENT_EVALS, METAL): plonk_t_quotient_evals,
        (OpType.TO_DEVICE, Device.CPU): to_device,
        (OpType.FROM_DEVICE, Device.CPU): from_device,
        (OpType.FROM_DEVICE, METAL): from_device,
    }
    for (op, dev), fn in kernels.items():
        # register() raises on duplicates (runtime/kernels/registry.py:33-36); the transfer
        # kernels replace the CPU ones registered by register_cpu_kernels(backend=METAL).
        registry._kernels[(op, dev, BM)] = fn


GB300_OPS = ("POINTWISE_MUL", "POLY_SUB", "ROOTS_EVALS_FROM_COEFFS", "ROOTS_COEFFS_FROM_EVALS",
             "COSET_EVALS_FROM_COEFFS", "COSET_COEFFS_FROM_EVALS", "MSM_G1", "KZG_BATCH_COMMIT", "MSM_G1_BATCH",
             "MSM_G2", "POLY_MUL_NTT", "DIV_XN_MINUS_1", "BATCH_INV", "PLONK_T_QUOTIENT_EVALS")


def install() -> None:
    """Point the reference's Metal entry points at the GB300 implementation (see module docstring)."""
    ctx_mod = importlib.import_module("runtime.context")
    metal_mod = importlib.import_module("runtime.kernels.metal")
    ir = importlib.import_module("runtime.ir")

    def create_default(*, pool=None, config=None):
        return GpuContext.create_default(pool=pool, config=config, ir=ir)

    ctx_mod.MetalContext.create_default = staticmethod(create_default)
    metal_mod.register_metal_kernels = register_gb300_kernels
