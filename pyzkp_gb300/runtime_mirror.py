"""Stand-alone mirror of the reference runtime's public API for the hot path.

The plugin (``pyzkp_gb300.plugin``) registers into whatever ``KernelRegistry`` it is
given: the reference's own (fzybravery/pyZKP ``runtime``) when that package is
importable, otherwise this mirror. The mirror keeps the reference's names,
argument meanings and error behaviour so code written against the reference runs
unchanged on a machine that has only this package:

* ``Device``, ``Backend``, ``DType``, ``Buffer``      -- runtime/ir/types.py:8-32
* ``OpType``                                           -- runtime/ir/ops.py:6-26
* ``Node``, ``GraphAnalysis``, ``Graph``               -- runtime/ir/graph.py:22-153
* ``KernelRegistry`` (register raises on duplicates, get raises KeyError)
                                                       -- runtime/kernels/registry.py:22-53
* ``Executor`` (device placement by registry lookup, automatic TO_DEVICE /
  FROM_DEVICE insertion with cached "{id}_{device}" copies, use-count release
  of intermediates with ``keep``)                      -- runtime/executor.py:27-218
* ``PoolStats``, ``MemoryPool`` (alloc_metal / release_metal keyed by byte size)
                                                       -- runtime/memory.py:9-113
* ``DeviceContext``, ``CPUContext``                    -- runtime/context.py:10-23
* ``RuntimeConfig`` (backend, runtime attrs, make_context)  -- runtime/config.py:10-54

Only the CPU kernels of the reference (crypto/*) are not mirrored: ops that have no
GPU kernel need the reference itself.
"""

from __future__ import annotations

import sys
import time
from dataclasses import dataclass, field
from enum import Enum
from typing import Any, Callable, Dict, List, Optional, Sequence, Tuple


class Device(str, Enum):
    CPU = "cpu"
    METAL = "metal"


class Backend(str, Enum):
    CPU = "cpu"
    METAL = "metal"


class DType(str, Enum):
    FR = "fr"
    G1 = "g1"
    G2 = "g2"
    BYTES = "bytes"
    OBJ = "obj"


@dataclass
class Buffer:
    id: str
    device: Device
    dtype: DType
    data: Any
    meta: Optional[Dict[str, Any]] = None


class OpType(str, Enum):
    TO_DEVICE = "to_device"
    FROM_DEVICE = "from_device"
    ROOTS_EVALS_FROM_COEFFS = "roots_evals_from_coeffs"
    ROOTS_COEFFS_FROM_EVALS = "roots_coeffs_from_evals"
    COSET_EVALS_FROM_COEFFS = "coset_evals_from_coeffs"
    COSET_COEFFS_FROM_EVALS = "coset_coeffs_from_evals"
    BATCH_INV = "batch_inv"
    POINTWISE_MUL = "pointwise_mul"
    POLY_MUL_NTT = "poly_mul_ntt"
    POLY_SUB = "poly_sub"
    DIV_XN_MINUS_1 = "div_xn_minus_1"
    PLONK_T_QUOTIENT_EVALS = "plonk_t_quotient_evals"
    MSM_G1 = "msm_g1"
    MSM_G2 = "msm_g2"
    MSM_G1_BATCH = "msm_g1_batch"
    KZG_COMMIT = "kzg_commit"
    KZG_OPEN = "kzg_open"
    KZG_OPEN_PREP_BATCH = "kzg_open_prep_batch"
    KZG_BATCH_COMMIT = "kzg_batch_commit"
    KZG_BATCH_OPEN = "kzg_batch_open"


@dataclass(frozen=True)
class Node:
    op: OpType
    inputs: List[str]
    outputs: List[str]
    attrs: Dict[str, Any]


@dataclass(frozen=True)
class GraphAnalysis:
    producers: Dict[str, int]
    topo_order: Tuple[int, ...]
    initial: Tuple[str, ...]


class Graph:
    def __init__(self) -> None:
        self.buffers: Dict[str, Buffer] = {}
        self.nodes: List[Node] = []
        self.meta: Dict[str, Any] = {}
        self._version = 0
        self._cache: Optional[GraphAnalysis] = None
        self._cache_version = -1

    def add_buffer(self, *, id: str, device: Device, dtype: DType, data: Any,
                   meta: Optional[Dict[str, Any]] = None) -> Buffer:
        if id in self.buffers:
            raise ValueError(f"buffer already exists: {id}")
        buf = Buffer(id=id, device=device, dtype=dtype, data=data, meta=meta)
        self.buffers[id] = buf
        self._version += 1
        return buf

    def add_node(self, *, op: OpType, inputs: Sequence[str], outputs: Sequence[str],
                 attrs: Optional[Dict[str, Any]] = None) -> Node:
        node = Node(op=op, inputs=list(inputs), outputs=list(outputs), attrs=attrs or {})
        self.nodes.append(node)
        self._version += 1
        return node

    def analyze(self) -> GraphAnalysis:
        producers: Dict[str, int] = {}
        initial = set(self.buffers)
        for idx, node in enumerate(self.nodes):
            if not node.outputs:
                raise ValueError(f"node has no outputs: {idx}")
            for out in node.outputs:
                if out in initial:
                    raise ValueError(f"node output overwrites existing buffer: {out}")
                if out in producers:
                    raise ValueError(f"buffer produced by multiple nodes: {out}")
                producers[out] = idx
        indeg = [0] * len(self.nodes)
        succ: List[List[int]] = [[] for _ in self.nodes]
        for j, node in enumerate(self.nodes):
            if not node.inputs:
                raise ValueError(f"node has no inputs: {j}")
            for inp in node.inputs:
                if inp in producers:
                    succ[producers[inp]].append(j)
                    indeg[j] += 1
                elif inp not in initial:
                    raise ValueError(f"missing input buffer: {inp}")
        ready = [i for i, d in enumerate(indeg) if d == 0]
        order: List[int] = []
        while ready:
            i = ready.pop()
            order.append(i)
            for j in succ[i]:
                indeg[j] -= 1
                if indeg[j] == 0:
                    ready.append(j)
        if len(order) != len(self.nodes):
            raise ValueError("graph has cycle or unresolved dependencies")
        return GraphAnalysis(producers=producers, topo_order=tuple(order), initial=tuple(sorted(initial)))

    def analyze_cached(self) -> GraphAnalysis:
        if self._cache is None or self._cache_version != self._version:
            self._cache = self.analyze()
            self._cache_version = self._version
        return self._cache

    def reset_to_initial(self, analysis: GraphAnalysis) -> None:
        keep = set(analysis.initial)
        for k in list(self.buffers):
            if k not in keep:
                del self.buffers[k]


KernelFn = Callable[[Dict[str, Any]], Dict[str, Any]]


class KernelRegistry:
    def __init__(self) -> None:
        self._kernels: Dict[Tuple[OpType, Device, Backend], KernelFn] = {}

    def register(self, op: OpType, device: Device, fn: KernelFn, *, backend: Backend = Backend.CPU) -> None:
        key = (op, device, backend)
        if key in self._kernels:
            raise ValueError(f"kernel already registered: {op} on {device} ({backend})")
        self._kernels[key] = fn

    def get(self, op: OpType, device: Device, *, backend: Backend = Backend.CPU) -> KernelFn:
        key = (op, device, backend)
        if key not in self._kernels:
            raise KeyError(f"kernel not found: {op} on {device} ({backend})")
        return self._kernels[key]

    def has(self, op: OpType, device: Device, *, backend: Backend = Backend.CPU) -> bool:
        return (op, device, backend) in self._kernels


@dataclass
class PoolStats:
    alloc_calls: int = 0
    reuse_calls: int = 0
    in_use: int = 0
    peak_in_use: int = 0


class MemoryPool:
    """CPU list[int] free lists keyed by (dtype, n); device buffers keyed by byte size."""

    def __init__(self) -> None:
        self._free_cpu: Dict[Tuple[DType, int], List[List[int]]] = {}
        self._owned_cpu: set = set()
        self.cpu_stats = PoolStats()
        self._free_metal: Dict[int, List[Any]] = {}
        self._owned_metal: set = set()
        self.metal_stats = PoolStats()

    def alloc_fr(self, n: int) -> List[int]:
        return self.alloc_cpu(DType.FR, n)

    def alloc_cpu(self, dtype: DType, n: int) -> List[int]:
        st = self.cpu_stats
        st.alloc_calls += 1
        st.in_use += 1
        st.peak_in_use = max(st.peak_in_use, st.in_use)
        lst = self._free_cpu.get((dtype, int(n)))
        if lst:
            st.reuse_calls += 1
            out = lst.pop()
            for i in range(len(out)):
                out[i] = 0
        else:
            out = [0] * int(n)
        self._owned_cpu.add(id(out))
        return out

    def release_cpu(self, dtype: DType, arr: List[int]) -> None:
        if id(arr) not in self._owned_cpu:
            return
        self.cpu_stats.in_use -= 1
        self._free_cpu.setdefault((dtype, len(arr)), []).append(arr)

    def alloc_metal(self, rt: Any, size_bytes: int) -> Any:
        st = self.metal_stats
        st.alloc_calls += 1
        st.in_use += 1
        st.peak_in_use = max(st.peak_in_use, st.in_use)
        lst = self._free_metal.get(size_bytes)
        if lst:
            st.reuse_calls += 1
            out = lst.pop()
        else:
            out = rt.device.newBufferWithLength_options_(size_bytes, 0)
            if out is None:
                raise RuntimeError(f"failed to allocate device buffer of size {size_bytes}")
        self._owned_metal.add(id(out))
        return out

    def release_metal(self, buf: Any) -> None:
        if id(buf) not in self._owned_metal:
            return
        self.metal_stats.in_use -= 1
        self._free_metal.setdefault(buf.length(), []).append(buf)


CPUMemoryPool = MemoryPool


@dataclass
class DeviceContext:
    backend: Backend = Backend.CPU
    device: Device = Device.CPU
    pool: Any = None
    config: Any = None


@dataclass
class CPUContext(DeviceContext):
    backend: Backend = Backend.CPU
    device: Device = Device.CPU


@dataclass(frozen=True)
class RuntimeConfig:
    backend: Backend = Backend.CPU
    fixed_base_policy: str = "off"
    fixed_base_window_bits: int = 8
    fixed_base_auto_min_points: int = 256
    fixed_base_auto_groth16_min_calls: int = 2
    metal_ntt_mode: str = "v1"
    metal_msm_mode: str = "v1"

    def runtime_attrs(self) -> Dict[str, Any]:
        return {
            "fixed_base_policy": str(self.fixed_base_policy),
            "fixed_base_window_bits": int(self.fixed_base_window_bits),
            "fixed_base_auto_min_points": int(self.fixed_base_auto_min_points),
            "fixed_base_auto_groth16_min_calls": int(self.fixed_base_auto_groth16_min_calls),
            "metal_ntt_mode": str(self.metal_ntt_mode),
            "metal_msm_mode": str(self.metal_msm_mode),
        }

    def with_overrides(self, overrides: Optional[Dict[str, Any]]) -> Dict[str, Any]:
        out = dict(self.runtime_attrs())
        out.update(dict(overrides or {}))
        return out

    def make_context(self, *, pool=None, context: Optional[DeviceContext] = None) -> DeviceContext:
        if context is not None:
            return context
        if self.backend == Backend.METAL:
            from pyzkp_gb300.plugin import GpuContext

            return GpuContext.create_default(pool=pool, config=self, ir=sys.modules[__name__])
        return CPUContext(pool=pool, backend=self.backend, config=self)


@dataclass
class TraceEvent:
    op: OpType
    device: Device
    backend: Backend
    start_ns: int
    end_ns: int
    attrs: Dict[str, Any] = field(default_factory=dict)
    input_sizes: List[int] = field(default_factory=list)
    output_sizes: List[int] = field(default_factory=list)


def _buffer_size(buf: Buffer) -> int:
    d = buf.data
    if isinstance(d, (list, tuple, bytes, bytearray)):
        return len(d)
    return 1


def _release(pool: Any, buf: Buffer) -> None:
    if pool is None:
        return
    if buf.device == Device.CPU and buf.dtype == DType.FR and isinstance(buf.data, list) and hasattr(pool, "release_cpu"):
        pool.release_cpu(DType.FR, buf.data)
    elif buf.device == Device.METAL and hasattr(buf.data, "mtl_buffer") and hasattr(pool, "release_metal"):
        pool.release_metal(buf.data.mtl_buffer)


@dataclass
class Executor:
    registry: KernelRegistry

    def run(self, graph: Graph, *, trace: Any = None, pool: Any = None, keep: Optional[List[str]] = None,
            backend: Backend = Backend.CPU, context: Optional[DeviceContext] = None,
            runtime_config: Optional[RuntimeConfig] = None) -> None:
        analysis = graph.analyze_cached()
        if context is not None:
            ctx = context
        elif runtime_config is not None:
            ctx = runtime_config.make_context(pool=pool)
        else:
            ctx = CPUContext(backend=backend, pool=pool)
        if ctx.pool is None:
            ctx.pool = pool
        self._run(graph, analysis, trace=trace, pool=ctx.pool, keep=keep, backend=ctx.backend, context=ctx)

    def _run(self, graph: Graph, analysis: GraphAnalysis, *, trace, pool, keep, backend, context) -> None:
        keep_set = set(keep) if keep is not None else None
        uses: Dict[str, int] = {}
        for node in graph.nodes:
            for inp in node.inputs:
                uses[inp] = uses.get(inp, 0) + 1
        for idx in analysis.topo_order:
            node = graph.nodes[idx]
            target = Device.CPU
            if backend != Backend.CPU and self.registry.has(node.op, context.device, backend=backend):
                target = context.device
            new_inputs: List[str] = []
            for inp_id in node.inputs:
                buf = graph.buffers[inp_id]
                if buf.device == target:
                    new_inputs.append(inp_id)
                    continue
                op = OpType.TO_DEVICE if target != Device.CPU else OpType.FROM_DEVICE
                moved = f"{inp_id}_{target.value}"
                if moved not in graph.buffers:
                    tnode = Node(op=op, inputs=[inp_id], outputs=[moved], attrs={})
                    self._run_node(graph, tnode, trace=trace, pool=pool, backend=backend, context=context,
                                   force_device=Device.CPU)
                uses[moved] = uses.get(moved, 0) + 1
                new_inputs.append(moved)
                if keep_set is not None:
                    uses[inp_id] = uses.get(inp_id, 0) - 1
                    if uses[inp_id] == 0 and inp_id in graph.buffers and inp_id not in keep_set:
                        _release(pool, graph.buffers[inp_id])
                        del graph.buffers[inp_id]
            if new_inputs != node.inputs:
                node = Node(op=node.op, inputs=new_inputs, outputs=node.outputs, attrs=node.attrs)
                graph.nodes[idx] = node
            self._run_node(graph, node, trace=trace, pool=pool, backend=backend, context=context,
                           force_device=target)
            if keep_set is not None:
                for inp in node.inputs:
                    uses[inp] = uses.get(inp, 0) - 1
                    if uses[inp] == 0 and inp in graph.buffers and inp not in keep_set:
                        _release(pool, graph.buffers[inp])
                        del graph.buffers[inp]

    def _run_node(self, graph: Graph, node: Node, *, trace, pool, backend, context, force_device=None) -> None:
        if not node.inputs:
            raise ValueError("node must have inputs")
        device = force_device if force_device is not None else graph.buffers[node.inputs[0]].device
        fn = self.registry.get(node.op, device, backend=backend)
        inputs = [graph.buffers[i] for i in node.inputs]
        ctx = {"graph": graph, "node": node, "inputs": inputs, "attrs": dict(node.attrs), "pool": pool,
               "context": context}
        t0 = time.perf_counter_ns()
        out = fn(ctx)
        t1 = time.perf_counter_ns()
        if "outputs" not in out:
            raise ValueError("kernel must return outputs")
        for bid, buf in out["outputs"].items():
            graph.buffers[bid] = buf
        if trace is not None:
            trace.append(TraceEvent(op=node.op, device=device, backend=backend, start_ns=t0, end_ns=t1,
                                    attrs=dict(node.attrs), input_sizes=[_buffer_size(b) for b in inputs],
                                    output_sizes=[_buffer_size(out["outputs"][k]) for k in node.outputs
                                                  if k in out["outputs"]]))
