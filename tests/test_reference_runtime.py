"""The plugin against the reference's own runtime, on the CPU (no GPU is touched).

The reference comes from ``PYZKP_REFERENCE`` or ``baseline/_ref`` (tests/reference_env.py);
every test here skips when it is absent. Fake device kernels, written from the KernelFn
contract (a ``ctx`` dict in, ``{"outputs": {id: Buffer}}`` out, runtime/executor.py:185-204),
stand in for device work where a test needs the Executor's device path without a GPU.
"""

import os
import subprocess
import sys

import pytest

import reference_env
from pyzkp_gb300 import plugin

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _fake_device_kernels(R, reg):
    """TO_DEVICE / FROM_DEVICE that only relabel the device, and device MSM_G1 / MSM_G2 that call
    the reference's CPU kernels: the Executor's device path with CPU arithmetic."""
    cpu = R.KernelRegistry()
    R.register_cpu_kernels(cpu)
    D, B = R.Device, R.Backend

    def relabel(device):
        def fn(ctx):
            b = ctx["inputs"][0]
            o = ctx["node"].outputs[0]
            data = list(b.data) if isinstance(b.data, list) else b.data
            return {"outputs": {o: R.Buffer(id=o, device=device, dtype=b.dtype, data=data)}}

        return fn

    def on_cpu(op):
        f = cpu.get(op, D.CPU)

        def fn(ctx):
            ins = [R.Buffer(id=b.id, device=D.CPU, dtype=b.dtype, data=b.data) for b in ctx["inputs"]]
            return f(dict(ctx, inputs=ins))

        return fn

    reg._kernels[(R.OpType.TO_DEVICE, D.CPU, B.METAL)] = relabel(D.METAL)
    reg._kernels[(R.OpType.FROM_DEVICE, D.CPU, B.METAL)] = relabel(D.CPU)
    reg._kernels[(R.OpType.FROM_DEVICE, D.METAL, B.METAL)] = relabel(D.CPU)
    for op in (R.OpType.MSM_G1, R.OpType.MSM_G2):
        reg._kernels[(op, D.METAL, B.METAL)] = on_cpu(op)


def test_plugin_registers_into_reference_registry():
    R = reference_env.runtime()
    reg = R.KernelRegistry()
    R.register_cpu_kernels(reg, backend=R.Backend.METAL)
    cpu_to_dev = reg.get(R.OpType.TO_DEVICE, R.Device.CPU, backend=R.Backend.METAL)
    plugin.register_gb300_kernels(reg)
    for name in plugin.GB300_OPS:
        assert reg.has(getattr(R.OpType, name), R.Device.METAL, backend=R.Backend.METAL), name
    assert reg.get(R.OpType.TO_DEVICE, R.Device.CPU, backend=R.Backend.METAL) is not cpu_to_dev
    # ops without a GB300 kernel stay on the reference CPU kernels
    assert not reg.has(R.OpType.KZG_OPEN, R.Device.METAL, backend=R.Backend.METAL)


def test_install_redirects_reference_metal_entry_points():
    reference_env.runtime()
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


def test_missing_gpu_context_raises_runtime_error():
    """A GB300 KernelFn called without a GB300 context raises RuntimeError, like the Metal
    kernels without a Metal runtime (runtime/kernels/metal/kernels.py:92-110)."""
    R = reference_env.runtime()
    reg = R.KernelRegistry()
    plugin.register_gb300_kernels(reg)
    fn = reg.get(R.OpType.MSM_G1, R.Device.METAL, backend=R.Backend.METAL)
    node = R.Node(op=R.OpType.MSM_G1, inputs=["p", "s"], outputs=["o"], attrs={})
    with pytest.raises(RuntimeError):
        fn({"node": node, "inputs": [None, None], "attrs": {}, "pool": None, "context": R.CPUContext()})


def test_reference_prove_batch_second_witness_fails_on_any_device_backend():
    """A property of the reference itself, independent of any kernel: on a device backend its
    Executor rewrites each node's inputs to the transfer ids in place (runtime/executor.py:147-149)
    and then deletes those transfer buffers once used (:155-165), so the second run of the same
    graph in protocols/groth16/prove.py:prove_batch finds a node input that no longer exists
    (KeyError at executor.py:114). With one witness it completes and verifies. The GB300 tests
    therefore run prove_batch with one witness per call."""
    R = reference_env.runtime()
    sys.path.insert(0, os.path.join(REPO, "tests", "golden"))
    import make_groth16_golden as MG
    from frontend.api import build_witness, compile_circuit
    import runtime.kernels.metal as rmetal

    fr = reference_env.seeded_fr_rand(7)
    MG.setup_mod.fr_rand = fr
    MG.prove_mod.fr_rand = fr
    r = MG.FR_MODULUS
    ir = compile_circuit(MG.CubicCircuit(), r)
    ws = [build_witness(ir, {"x": x, "y": (x ** 3 + x + 5) % r}) for x in (9, 10)]
    pk = MG.setup_mod.setup(ir)
    old = rmetal.register_metal_kernels
    rmetal.register_metal_kernels = lambda reg: _fake_device_kernels(R, reg)
    try:
        from runtime.context import DeviceContext

        ctx = DeviceContext(backend=R.Backend.METAL, device=R.Device.METAL)
        (one,) = MG.prove_mod.prove_batch(ir, pk, ws[:1], runtime_context=ctx)
        assert MG.verify(pk.vk, [1, (9 ** 3 + 9 + 5) % r], one)
        with pytest.raises(KeyError):
            MG.prove_mod.prove_batch(ir, pk, ws, runtime_context=ctx)
    finally:
        rmetal.register_metal_kernels = old


def test_reference_hot_path_tests_pass_with_the_stand_in():
    """The reference's own CPU tests of the hot path (test_poly_ntt, test_msm_pippenger) pass
    with the py_ecc stand-in. Needs the reference's tests package (a checkout, or an install
    that includes it)."""
    root = reference_env.require()
    if not os.path.isdir(os.path.join(root, "tests", "correctness", "cpu")):
        pytest.skip("reference tests not present")
    env = dict(os.environ, PYTHONDONTWRITEBYTECODE="1",
               PYTHONPATH=os.pathsep.join([reference_env.SHIM, root]))
    out = subprocess.run([sys.executable, "-m", "unittest", "tests.correctness.cpu.test_poly_ntt",
                          "tests.correctness.cpu.test_msm_pippenger"], cwd=root, env=env, capture_output=True,
                         text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
