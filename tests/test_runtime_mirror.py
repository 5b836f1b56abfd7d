"""The runtime mirror behaves like the reference runtime, and the plugin plugs into both (CPU only).

Where the reference checkout is present (it is not on the GPU machine) the same graphs
run through the reference's own Executor/KernelRegistry and the mirror and must
produce identical placements and results; fake kernels stand in for device work so
no GPU is touched.
"""

import os
import sys

import pytest

from pyzkp_gb300 import plugin
from pyzkp_gb300 import runtime_mirror as M

REF = os.environ.get("PYZKP_REFERENCE", "/root/reference")
REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _reference():
    if not os.path.isdir(os.path.join(REF, "runtime")):
        pytest.skip("reference checkout not present")
    for p in (os.path.join(REPO, "oracle", "py_ecc_shim"), REF):
        if p not in sys.path:
            sys.path.insert(0, p)
    sys.dont_write_bytecode = True
    import runtime  # noqa: F401
    from runtime import executor, ir
    from runtime.kernels import registry

    return ir, registry, executor


def _fake_kernels(ir, reg, log):
    """TO_DEVICE / FROM_DEVICE / a device op that only tag data, registered like the protocols do."""
    D, B, O, T = ir.Device, ir.Backend, ir.OpType, ir.DType

    def to_dev(ctx):
        inp = ctx["inputs"][0]
        log.append(("to", inp.id))
        o = ctx["node"].outputs[0]
        return {"outputs": {o: ir.Buffer(id=o, device=D.METAL, dtype=inp.dtype, data=("dev", inp.data))}}

    def from_dev(ctx):
        inp = ctx["inputs"][0]
        log.append(("from", inp.id))
        o = ctx["node"].outputs[0]
        data = inp.data[1] if isinstance(inp.data, tuple) else inp.data
        return {"outputs": {o: ir.Buffer(id=o, device=D.CPU, dtype=inp.dtype, data=data)}}

    def dev_add(ctx):
        a, b = ctx["inputs"]
        log.append(("add", a.id, b.id))
        o = ctx["node"].outputs[0]
        s = [x + y for x, y in zip(a.data[1], b.data[1])]
        return {"outputs": {o: ir.Buffer(id=o, device=D.METAL, dtype=T.FR, data=("dev", s))}}

    def cpu_neg(ctx):
        a = ctx["inputs"][0]
        log.append(("neg", a.id))
        o = ctx["node"].outputs[0]
        return {"outputs": {o: ir.Buffer(id=o, device=D.CPU, dtype=T.FR, data=[-x for x in a.data])}}

    reg.register(O.TO_DEVICE, D.CPU, to_dev, backend=B.METAL)
    reg.register(O.FROM_DEVICE, D.CPU, from_dev, backend=B.METAL)
    reg.register(O.FROM_DEVICE, D.METAL, from_dev, backend=B.METAL)
    reg.register(O.POLY_SUB, D.METAL, dev_add, backend=B.METAL)
    reg.register(O.BATCH_INV, D.CPU, cpu_neg, backend=B.METAL)


def _graph(ir, graph_mod):
    g = graph_mod.Graph()
    D, T, O = ir.Device, ir.DType, ir.OpType
    g.add_buffer(id="a", device=D.CPU, dtype=T.FR, data=[1, 2, 3])
    g.add_buffer(id="b", device=D.CPU, dtype=T.FR, data=[10, 20, 30])
    g.add_node(op=O.POLY_SUB, inputs=["a", "b"], outputs=["c"])
    g.add_node(op=O.BATCH_INV, inputs=["c"], outputs=["d"])
    g.add_node(op=O.POLY_SUB, inputs=["d", "a"], outputs=["e"])
    return g


def _run(ir, reg_mod, exe_mod, graph_mod, ctx_cls):
    log = []
    reg = reg_mod.KernelRegistry()
    _fake_kernels(ir, reg, log)
    g = _graph(ir, graph_mod)
    ctx = ctx_cls(backend=ir.Backend.METAL, device=ir.Device.METAL)
    exe_mod.Executor(registry=reg).run(g, context=ctx, keep=["e"])
    return log, sorted(g.buffers), g.buffers["e"].data


def test_mirror_registry_and_graph_errors():
    reg = M.KernelRegistry()
    reg.register(M.OpType.MSM_G1, M.Device.CPU, lambda c: c)
    with pytest.raises(ValueError):
        reg.register(M.OpType.MSM_G1, M.Device.CPU, lambda c: c)
    with pytest.raises(KeyError):
        reg.get(M.OpType.MSM_G2, M.Device.CPU)
    g = M.Graph()
    g.add_buffer(id="x", device=M.Device.CPU, dtype=M.DType.FR, data=[])
    g.add_node(op=M.OpType.POLY_SUB, inputs=["x", "missing"], outputs=["y"])
    with pytest.raises(ValueError):
        g.analyze()
    g2 = M.Graph()
    g2.add_buffer(id="x", device=M.Device.CPU, dtype=M.DType.FR, data=[])
    g2.add_node(op=M.OpType.POLY_SUB, inputs=["x"], outputs=["x"])
    with pytest.raises(ValueError):
        g2.analyze()


def test_mirror_executor_places_and_transfers():
    class Ctx(M.DeviceContext):
        pass

    log, bufs, e = _run(M, M, M, M, Ctx)
    assert e == ("dev", [-11 + 1, -22 + 2, -33 + 3])
    assert ("to", "a") in log and ("from", "c") in log and ("to", "d") in log
    assert "c" not in bufs and "d" not in bufs  # released by use count, not kept


def test_mirror_matches_reference_executor():
    ir, registry, executor = _reference()
    from runtime.context import DeviceContext
    from runtime.ir import graph as rgraph

    ref = _run(ir, registry, executor, rgraph, DeviceContext)
    mir = _run(M, M, M, M, M.DeviceContext)
    assert ref == mir


def test_plugin_registers_into_reference_registry():
    ir, registry, _ = _reference()
    from runtime.kernels.cpu import register_cpu_kernels

    reg = registry.KernelRegistry()
    register_cpu_kernels(reg, backend=ir.Backend.METAL)
    cpu_to_dev = reg.get(ir.OpType.TO_DEVICE, ir.Device.CPU, backend=ir.Backend.METAL)
    plugin.register_gb300_kernels(reg)
    for name in plugin.GB300_OPS:
        assert reg.has(getattr(ir.OpType, name), ir.Device.METAL, backend=ir.Backend.METAL), name
    assert reg.get(ir.OpType.TO_DEVICE, ir.Device.CPU, backend=ir.Backend.METAL) is not cpu_to_dev
    # ops without a GB300 kernel stay on the reference CPU kernels
    assert not reg.has(ir.OpType.KZG_OPEN, ir.Device.METAL, backend=ir.Backend.METAL)


def test_install_redirects_reference_metal_entry_points():
    ir, _, _ = _reference()
    import runtime.context as rctx
    import runtime.kernels.metal as rmetal

    old_create, old_reg = rctx.MetalContext.__dict__["create_default"], rmetal.register_metal_kernels
    try:
        plugin.install()
        assert rmetal.register_metal_kernels is plugin.register_gb300_kernels
        assert rctx.MetalContext.create_default is not old_create
    finally:
        rctx.MetalContext.create_default = old_create
        rmetal.register_metal_kernels = old_reg


def test_reference_hot_path_tests_pass_with_the_stand_in():
    """The reference's own CPU tests of the hot path (test_poly_ntt, test_msm_pippenger) pass."""
    _reference()
    import subprocess

    env = dict(os.environ, PYTHONDONTWRITEBYTECODE="1",
               PYTHONPATH=os.pathsep.join([os.path.join(REPO, "oracle", "py_ecc_shim"), REF]))
    out = subprocess.run([sys.executable, "-m", "unittest", "tests.correctness.cpu.test_poly_ntt",
                          "tests.correctness.cpu.test_msm_pippenger"], cwd=REF, env=env, capture_output=True,
                         text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
