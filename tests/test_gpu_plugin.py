"""GPU tests of the drop-in KernelFns (pyzkp_gb300.plugin) through the reference's own runtime.

They follow the reference's Metal tests (tests/correctness/metal/test_runtime_metal_*.py):
register the reference's CPU kernels and the GB300 kernels into the reference's
``KernelRegistry``, build a ``Graph`` with TO_DEVICE -> op -> FROM_DEVICE, run it with the
reference's ``Executor`` under ``RuntimeConfig(backend=METAL)`` (``plugin.install()`` makes
that config create a GB300 context), and compare with the reference's CPU result -- the
committed golden vectors made by running the reference (tests/golden/make_golden.py,
make_plonk_golden.py) or exact Python arithmetic. The reference comes from
``PYZKP_REFERENCE`` or ``baseline/_ref`` (tests/reference_env.py); py_ecc is the test-only
stand-in under oracle/py_ecc_shim.
"""

import json
import os
import sys

import pytest

import reference_env

HERE = os.path.dirname(os.path.abspath(__file__))
R = reference_env.runtime()

from py_ecc import optimized_bn128 as bn  # noqa: E402

from oracle import oracle as O  # noqa: E402
from pyzkp_gb300 import plugin, synth  # noqa: E402

pytestmark = pytest.mark.gpu
FR = synth.FR_MODULUS
plugin.install()


def _golden(name):
    with open(os.path.join(HERE, "golden", name)) as f:
        return json.load(f)


def _exe():
    """A registry set up the way the reference's provers do it (protocols/groth16/prove.py:56-62)."""
    reg = R.KernelRegistry()
    R.register_cpu_kernels(reg, backend=R.Backend.METAL)
    plugin.register_gb300_kernels(reg)
    return R.Executor(registry=reg), reg


def _cfg():
    return R.RuntimeConfig(backend=R.Backend.METAL)


def _run_unary(op, data, attrs):
    exe, _ = _exe()
    g = R.Graph()
    g.add_buffer(id="a", device=R.Device.CPU, dtype=R.DType.FR, data=list(data))
    g.add_node(op=R.OpType.TO_DEVICE, inputs=["a"], outputs=["a_m"])
    g.add_node(op=op, inputs=["a_m"], outputs=["o_m"], attrs=attrs)
    g.add_node(op=R.OpType.FROM_DEVICE, inputs=["o_m"], outputs=["o"])
    exe.run(g, runtime_config=_cfg(), keep=["o"])
    return g.buffers["o"].data


OPS = {0: R.OpType.ROOTS_EVALS_FROM_COEFFS, 1: R.OpType.ROOTS_COEFFS_FROM_EVALS,
       2: R.OpType.COSET_EVALS_FROM_COEFFS, 3: R.OpType.COSET_COEFFS_FROM_EVALS}


def test_ntt_ops_match_reference_fixtures():
    # tests/correctness/metal/test_runtime_metal_fr_ntt.py and ..._fr_coset.py (n = 16, shift 5)
    for fx in _golden("ntt_reference.json")["fixtures"]:
        attrs = {"n": fx["n"], "omega": int(fx["omega"], 16), "shift": int(fx["shift"], 16)}
        got = _run_unary(OPS[fx["mode"]], [int(v, 16) for v in fx["input"]], attrs)
        assert got == [int(v, 16) for v in fx["output"]], fx["name"]


def test_forward_ops_pad_and_truncate_to_attr_n():
    import hashlib

    for rec in _golden("ntt_reference.json")["pad_truncate"]:
        v = synth.limbs_to_ints(synth.fr_uniform(rec["seed"], rec["in_len"]))
        attrs = {"n": rec["n"], "omega": int(rec["omega"], 16), "shift": int(rec["shift"], 16)}
        got = _run_unary(OPS[rec["mode"]], v, attrs)
        h = hashlib.sha256(b"".join(x.to_bytes(32, "little") for x in got)).hexdigest()
        assert len(got) == rec["n"] and h == rec["output_sha256"]


def test_ntt_op_errors():
    exe, _ = _exe()
    g = R.Graph()
    g.add_buffer(id="a", device=R.Device.CPU, dtype=R.DType.FR, data=[1, 2, 3])
    g.add_node(op=R.OpType.ROOTS_COEFFS_FROM_EVALS, inputs=["a"], outputs=["o"], attrs={"omega": 1})
    with pytest.raises(ValueError):
        exe.run(g, runtime_config=_cfg())
    # empty input of an inverse transform gives an empty result, as the CPU op does
    assert _run_unary(R.OpType.ROOTS_COEFFS_FROM_EVALS, [], {"omega": 1}) == []


def test_pointwise_mul_and_poly_sub():
    exe, _ = _exe()
    n = 100
    a = [(i * 123 + 456) % FR for i in range(n)]
    b = [(i * 789 + 123) % FR for i in range(n)]
    for op, exp in ((R.OpType.POINTWISE_MUL, [(x * y) % FR for x, y in zip(a, b)]),
                    (R.OpType.POLY_SUB, [(x - y) % FR for x, y in zip(a, b)])):
        g = R.Graph()
        g.add_buffer(id="a", device=R.Device.CPU, dtype=R.DType.FR, data=list(a))
        g.add_buffer(id="b", device=R.Device.CPU, dtype=R.DType.FR, data=list(b))
        g.add_node(op=R.OpType.TO_DEVICE, inputs=["a"], outputs=["a_m"])
        g.add_node(op=R.OpType.TO_DEVICE, inputs=["b"], outputs=["b_m"])
        g.add_node(op=op, inputs=["a_m", "b_m"], outputs=["c_m"])
        g.add_node(op=R.OpType.FROM_DEVICE, inputs=["c_m"], outputs=["c"])
        exe.run(g, runtime_config=_cfg(), keep=["c"])
        assert g.buffers["c"].data == exp


def test_poly_sub_unequal_lengths_trims_like_cpu_ref():
    # crypto/poly/cpu_ref.py:18-25: pad to the longer input, trim trailing zeros
    a = [5, 6, 7, 8, 9]
    b = [1, 2, 3, 8, 9, 0, 0]
    exe, _ = _exe()
    g = R.Graph()
    g.add_buffer(id="a", device=R.Device.CPU, dtype=R.DType.FR, data=a)
    g.add_buffer(id="b", device=R.Device.CPU, dtype=R.DType.FR, data=b)
    g.add_node(op=R.OpType.POLY_SUB, inputs=["a", "b"], outputs=["c"])
    g.add_node(op=R.OpType.FROM_DEVICE, inputs=["c"], outputs=["d"])
    exe.run(g, runtime_config=_cfg(), keep=["d"])
    assert g.buffers["d"].data == [4, 4, 4]
    g2 = R.Graph()
    g2.add_buffer(id="a", device=R.Device.CPU, dtype=R.DType.FR, data=[1, 2])
    g2.add_buffer(id="b", device=R.Device.CPU, dtype=R.DType.FR, data=[0, 0, 5])
    g2.add_node(op=R.OpType.POLY_SUB, inputs=["a", "b"], outputs=["c"])
    exe.run(g2, runtime_config=_cfg(), keep=["c"])
    assert g2.buffers["c"].data.n == 3


def test_pointwise_length_mismatch_raises():
    exe, _ = _exe()
    g = R.Graph()
    g.add_buffer(id="a", device=R.Device.CPU, dtype=R.DType.FR, data=[1, 2])
    g.add_buffer(id="b", device=R.Device.CPU, dtype=R.DType.FR, data=[1, 2, 3])
    g.add_node(op=R.OpType.POINTWISE_MUL, inputs=["a", "b"], outputs=["c"])
    with pytest.raises(ValueError):
        exe.run(g, runtime_config=_cfg())


def _points_from_golden(case):
    pts = []
    for x, y in case["bases"]:
        x, y = int(x, 16), int(y, 16)
        pts.append(bn.Z1 if (x, y) == (0, 0) else (bn.FQ(x), bn.FQ(y), bn.FQ(1)))
    return pts


def _run_msm(points, scalars, attrs=None):
    exe, _ = _exe()
    g = R.Graph()
    g.add_buffer(id="points", device=R.Device.CPU, dtype=R.DType.OBJ, data=points)
    g.add_buffer(id="scalars", device=R.Device.CPU, dtype=R.DType.FR, data=list(scalars))
    g.add_node(op=R.OpType.MSM_G1, inputs=["points", "scalars"], outputs=["msm_res"], attrs=attrs or {})
    exe.run(g, context=_cfg().make_context())
    return g.buffers["msm_res"]


def test_msm_g1_matches_reference_cases():
    # tests/correctness/metal/test_runtime_metal_g1_msm.py fixture + edge cases, results from the reference
    for case in _golden("msm_reference.json")["cases"]:
        pts = _points_from_golden(case)
        sc = [int(s, 16) for s in case["scalars"]]
        out = _run_msm(pts, sc)
        assert out.device == R.Device.CPU and out.dtype == R.DType.G1
        exp = tuple(int(v, 16) for v in case["result"])
        got = bn.normalize(out.data)
        assert (int(got[0]), int(got[1])) == exp, case["name"]


def test_msm_g1_projective_points_and_resident_cache():
    # py_ecc points with Z != 1 are normalised; a second call reuses the resident bases
    pts = tuple(bn.multiply(bn.G1, k + 3) for k in range(200))
    sc = [(k * 7919 + 1) % FR for k in range(200)]
    exp = bn.normalize(bn.multiply(bn.G1, sum((k + 3) * s for k, s in zip(range(200), sc)) % FR))
    for _ in range(2):
        got = bn.normalize(_run_msm(pts, sc).data)
        assert got == exp
    # fewer scalars than points uses the prefix (runtime/kernels/metal/kernels.py:108-114)
    got = bn.normalize(_run_msm(pts, sc[:50]).data)
    assert got == bn.normalize(bn.multiply(bn.G1, sum((k + 3) * s for k, s in zip(range(50), sc[:50])) % FR))


def test_msm_g1_too_many_scalars_raises():
    with pytest.raises(ValueError):
        _run_msm([bn.G1], [1, 2])


def test_kzg_batch_commit_and_msm_batch():
    class SRS:
        def __init__(self, pts):
            self.g1_powers = pts

    ks = [k * 31 + 11 for k in range(300)]
    srs = SRS(tuple(bn.multiply(bn.G1, k) for k in ks))
    polys = [[(i * 17 + j) % FR for i in range(L)] for j, L in enumerate([300, 64, 1, 0, 129])]
    exe, _ = _exe()
    g = R.Graph()
    g.add_buffer(id="srs", device=R.Device.CPU, dtype=R.DType.OBJ, data=srs)
    g.add_buffer(id="polys", device=R.Device.CPU, dtype=R.DType.OBJ, data=polys)
    g.add_node(op=R.OpType.KZG_BATCH_COMMIT, inputs=["srs", "polys"], outputs=["cms"])
    exe.run(g, context=_cfg().make_context())
    outs = g.buffers["cms"].data
    for p, cm in zip(polys, outs):
        e = sum(k * c for k, c in zip(ks, p)) % FR
        exp = bn.normalize(bn.multiply(bn.G1, e)) if e else (bn.FQ(0), bn.FQ(0))
        assert bn.normalize(cm) == exp
    g2 = R.Graph()
    g2.add_buffer(id="pts", device=R.Device.CPU, dtype=R.DType.OBJ, data=srs.g1_powers)
    g2.add_buffer(id="sl", device=R.Device.CPU, dtype=R.DType.OBJ, data=polys)
    g2.add_node(op=R.OpType.MSM_G1_BATCH, inputs=["pts", "sl"], outputs=["outs"])
    exe.run(g2, context=_cfg().make_context())
    assert [bn.normalize(x) for x in g2.buffers["outs"].data] == [bn.normalize(x) for x in outs]


def test_pool_reuse_with_gb300_runtime():
    # tests/correctness/metal/test_runtime_metal_pool.py against GB300 memory
    pool = R.MemoryPool()
    rt = plugin.GpuContext.create_default(ir=R.ir).metal
    b1 = pool.alloc_metal(rt, 1024)
    b2 = pool.alloc_metal(rt, 1024)
    assert pool.metal_stats.alloc_calls == 2 and pool.metal_stats.in_use == 2
    pool.release_metal(b1)
    b3 = pool.alloc_metal(rt, 1024)
    assert pool.metal_stats.reuse_calls == 1 and id(b1) == id(b3)
    assert b2.length() == 1024


def test_executor_inserts_transfers_and_releases_with_pool():
    # runtime/executor.py:104-165: automatic TO_DEVICE / FROM_DEVICE and keep-based release
    exe, _ = _exe()
    pool = R.MemoryPool()
    n = 64
    om = O.omega_for_size(n)
    a = synth.limbs_to_ints(synth.fr_uniform(5, n))
    g = R.Graph()
    g.add_buffer(id="a", device=R.Device.CPU, dtype=R.DType.FR, data=list(a))
    g.add_node(op=R.OpType.ROOTS_EVALS_FROM_COEFFS, inputs=["a"], outputs=["ev"], attrs={"n": n, "omega": om})
    g.add_node(op=R.OpType.ROOTS_COEFFS_FROM_EVALS, inputs=["ev"], outputs=["back"], attrs={"omega": om})
    g.add_node(op=R.OpType.POLY_SUB, inputs=["back", "a"], outputs=["zero"])
    exe.run(g, runtime_config=_cfg(), pool=pool, keep=["zero"])
    assert "ev" not in g.buffers and g.buffers["zero"].data.n == 0
    assert pool.metal_stats.alloc_calls >= 3


def test_missing_gpu_context_raises_runtime_error():
    _, reg = _exe()
    fn = reg.get(R.OpType.MSM_G1, R.Device.METAL, backend=R.Backend.METAL)
    node = R.Node(op=R.OpType.MSM_G1, inputs=["p", "s"], outputs=["o"], attrs={})
    with pytest.raises(RuntimeError):
        fn({"node": node, "inputs": [None, None], "attrs": {}, "pool": None, "context": R.CPUContext()})


def _poly_mul(a, b):
    out = [0] * (len(a) + len(b) - 1)
    for i, x in enumerate(a):
        for j, y in enumerate(b):
            out[i + j] = (out[i + j] + x * y) % FR
    while out and out[-1] == 0:
        out.pop()
    return out


def _div_xn(a, n):
    """crypto/poly/fast.py:8-37 restated with plain ints."""
    a = [x % FR for x in a]
    while a and a[-1] == 0:
        a.pop()
    if not a:
        return [], []
    if len(a) <= n:
        return [], a
    q = [0] * (len(a) - n)
    for k in range(len(a) - 1, n - 1, -1):
        q[k - n] = (a[k] + (q[k] if k < len(q) else 0)) % FR
    r = [(a[i] + (q[i] if i < len(q) else 0)) % FR for i in range(n)]
    while q and q[-1] == 0:
        q.pop()
    while r and r[-1] == 0:
        r.pop()
    return q, r


def test_qap_graph_on_device_matches_cpu_algebra():
    """The node sequence of compute_h_from_abc_on_roots (protocols/groth16/qap.py:79-91):
    three iNTTs, POLY_MUL_NTT, POLY_SUB, DIV_XN_MINUS_1 -- all on the device."""
    n = 32
    om = O.omega_for_size(n)
    rng = synth.fr_uniform(901, 2 * n)
    a = synth.limbs_to_ints(rng[:n])
    b = synth.limbs_to_ints(rng[n:])
    c = [x * y % FR for x, y in zip(a, b)]
    for broken in (False, True):
        cc = list(c)
        if broken:
            cc[3] = (cc[3] + 1) % FR
        exe, _ = _exe()
        g = R.Graph()
        for name, v in (("a_eval", a), ("b_eval", b), ("c_eval", cc)):
            g.add_buffer(id=name, device=R.Device.CPU, dtype=R.DType.FR, data=list(v))
        for x in "abc":
            g.add_node(op=R.OpType.ROOTS_COEFFS_FROM_EVALS, inputs=[f"{x}_eval"], outputs=[f"{x}_coeff"],
                       attrs={"omega": om})
        g.add_node(op=R.OpType.POLY_MUL_NTT, inputs=["a_coeff", "b_coeff"], outputs=["ab_coeff"])
        g.add_node(op=R.OpType.POLY_SUB, inputs=["ab_coeff", "c_coeff"], outputs=["p_coeff"])
        g.add_node(op=R.OpType.DIV_XN_MINUS_1, inputs=["p_coeff"], outputs=["h_coeff", "rem"], attrs={"n": n})
        exe.run(g, runtime_config=_cfg(), keep=["a_coeff", "b_coeff", "c_coeff", "ab_coeff", "h_coeff", "rem"])
        coeff = {x: O.ntt_op(1, synth.ints_to_limbs(v), n, om) for x, v in (("a", a), ("b", b), ("c", cc))}
        ac, bc, ccf = (synth.limbs_to_ints(coeff[x]) for x in "abc")
        ab = _poly_mul(ac, bc)
        assert list(g.buffers["ab_coeff"].data) == ab
        p = [(x - (ccf[i] if i < len(ccf) else 0)) % FR for i, x in enumerate(ab)]
        while p and p[-1] == 0:
            p.pop()
        q, r = _div_xn(p, n)
        assert list(g.buffers["h_coeff"].data) == q
        assert list(g.buffers["rem"].data) == r
        assert (len(r) != 0) == broken


def test_div_xn_minus_1_edge_cases():
    exe, _ = _exe()
    for vals, n in (([], 4), ([5, 0, 0], 4), ([1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11], 3), ([0, 0, 7, 0, 0, 0, 9], 2)):
        g = R.Graph()
        g.add_buffer(id="p", device=R.Device.CPU, dtype=R.DType.FR, data=list(vals))
        g.add_node(op=R.OpType.DIV_XN_MINUS_1, inputs=["p"], outputs=["q", "r"], attrs={"n": n})
        exe.run(g, runtime_config=_cfg(), keep=["q", "r"])
        assert (list(g.buffers["q"].data), list(g.buffers["r"].data)) == _div_xn(vals, n), (vals, n)


def test_msm_g2_op_matches_oracle():
    n = 300
    k = synth.base_dlogs(902, n)
    pts = [bn.multiply(bn.G2, int(v)) for v in synth.limbs_to_ints(k[:20])]
    pts += [bn.normalize(p) + (bn.FQ2.one(),) for p in pts[:5]]  # affine (z = 1) forms too
    pts.append(bn.Z2)
    s = synth.limbs_to_ints(synth.fr_uniform(903, len(pts)))
    exe, _ = _exe()
    g = R.Graph()
    g.add_buffer(id="pts", device=R.Device.CPU, dtype=R.DType.G2, data=tuple(pts))
    g.add_buffer(id="s", device=R.Device.CPU, dtype=R.DType.FR, data=list(s))
    g.add_node(op=R.OpType.MSM_G2, inputs=["pts", "s"], outputs=["o"])
    exe.run(g, runtime_config=_cfg(), keep=["o"])
    got = bn.normalize(g.buffers["o"].data)
    exp = bn.Z2
    for p, v in zip(pts, s):
        exp = bn.add(exp, bn.multiply(p, v))
    exp = bn.normalize(exp)
    assert [int(c) for c in got[0].coeffs] == [int(c) for c in exp[0].coeffs]
    assert [int(c) for c in got[1].coeffs] == [int(c) for c in exp[1].coeffs]


def test_batch_inv_op_zero_maps_to_zero():
    vals = synth.limbs_to_ints(synth.fr_uniform(904, 1000))
    for i in (0, 17, 31, 32, 33, 999):
        vals[i] = 0
    got = _run_unary(R.OpType.BATCH_INV, vals, {})
    assert got == [pow(v, FR - 2, FR) if v else 0 for v in vals]


def _plonk_quotient_graph(vecs, attrs, exe):
    g = R.Graph()
    names = [f"v{j}" for j in range(15)]
    for name, v in zip(names, vecs):
        g.add_buffer(id=name, device=R.Device.CPU, dtype=R.DType.FR, data=list(v))
    g.add_node(op=R.OpType.PLONK_T_QUOTIENT_EVALS, inputs=names, outputs=["num", "zh"], attrs=attrs)
    g.add_node(op=R.OpType.BATCH_INV, inputs=["zh"], outputs=["inv_zh"])
    g.add_node(op=R.OpType.POINTWISE_MUL, inputs=["num", "inv_zh"], outputs=["t"])
    exe.run(g, runtime_config=_cfg(), keep=["num", "zh", "t"])
    return [list(g.buffers[k].data) for k in ("num", "zh", "t")]


def _fr_sha(vals):
    import hashlib

    return hashlib.sha256(b"".join(int(v).to_bytes(32, "little") for v in vals)).hexdigest()


def test_plonk_t_quotient_evals_op_matches_reference_golden():
    """PLONK_T_QUOTIENT_EVALS against the reference's own _plonk_t_quotient_evals
    (runtime/kernels/cpu/kernels.py:607-693) on its committed outputs: m = 2^6 .. 2^10, 2^12,
    a ragged m = 100 and a shift_n that is not shift^n, every element compared (SHA-256 of
    the whole vector, plus sampled values); then BATCH_INV and POINTWISE_MUL as in
    protocols/plonk/prove.py:412-414."""
    exe, _ = _exe()
    for rec in _golden("plonk_reference.json")["quotient"]:
        m = rec["m"]
        vecs = [synth.limbs_to_ints(synth.fr_uniform(rec["seed"] + j, m)) for j in range(15)]
        attrs = {k: (v if isinstance(v, int) else int(v, 16)) for k, v in rec["attrs"].items()}
        num, zh, t = _plonk_quotient_graph(vecs, attrs, exe)
        assert _fr_sha(num) == rec["num_sha256"], m
        assert _fr_sha(zh) == rec["zh_sha256"], m
        for i, v in rec["num_at"].items():
            assert num[int(i)] == int(v, 16), (m, i)
        assert t == [x * pow(z, FR - 2, FR) % FR if z else 0 for x, z in zip(num, zh)]


def test_plonk_t_quotient_evals_many_warps_every_element():
    """The quotient op past one warp table row: m = 70000 points (137 warps of 512 points, so
    the starting powers use warp-table indices up to 136 = 2 * 64 + 8) and a ragged last warp,
    every element against the oracle's restatement of _plonk_t_quotient_evals
    (runtime/kernels/cpu/kernels.py:607-693), itself pinned to the reference's outputs."""
    exe, _ = _exe()
    m, n = 70000, 1 << 14
    omega_m = O.omega_for_size(1 << 17)
    attrs = {"n": n, "m": m, "omega_m": omega_m, "shift": 5, "shift_n": pow(5, n, FR), "alpha": 0x1234567,
             "beta": 0xABCDEF, "gamma": 0x7654321, "k1": 7, "k2": 13}
    vecs = [synth.limbs_to_ints(synth.fr_uniform(9700 + j, m)) for j in range(15)]
    num, zh, _ = _plonk_quotient_graph(vecs, attrs, exe)
    e_num, e_zh = O.plonk_t_quotient_evals(vecs, n, omega_m, 5, attrs["shift_n"], attrs["alpha"], attrs["beta"],
                                           attrs["gamma"], 7, 13)
    assert zh == e_zh
    assert num == e_num
