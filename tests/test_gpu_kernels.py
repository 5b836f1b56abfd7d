"""GPU parity of the CUDA kernels, called through the C ABI (include/zkgpu.h).

Checked against (a) the golden vectors produced by running the reference itself
(tests/golden/*.json, see tests/golden/make_golden.py) and (b) the C oracle
(oracle/bn254_oracle.c) at sizes it finishes in seconds, and (c) size-independent
properties at the full sizes (round trips, known-answer MSM with bases [k_i]G).
Bit-exact: every comparison is on canonical integers / bytes.
"""

import hashlib
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from pyzkp_gb300 import _native as N
from pyzkp_gb300 import synth

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
R = synth.FR_MODULUS


def _sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u8").tobytes()).hexdigest()


def _hex_to_limbs(vals, width=4):
    return synth.ints_to_limbs([int(v, 16) for v in vals]).reshape(-1, width)


def gpu_ntt(ctx, mode, values: np.ndarray, n: int, omega: int, shift: int = 1) -> np.ndarray:
    """canonical uint64[m,4] -> canonical uint64[n,4] through to_mont / zk_ntt / from_mont on the device."""
    m = values.shape[0]
    din = ctx.alloc(max(1, m) * 32)
    if m:
        din.upload(values)
        ctx.fr_to_mont(din, din, m)
    dout = ctx.alloc(n * 32)
    ctx.ntt(mode, dout, din, m, n.bit_length() - 1, omega, shift)
    ctx.fr_from_mont(dout, dout, n)
    return dout.download(n * 32).view("<u8").reshape(n, 4).astype(np.uint64)


def gpu_msm(ctx, bases: np.ndarray, scalars: np.ndarray, window_bits: int = 0, mont: bool = True):
    b = ctx.bases_from_host(bases)
    n = scalars.shape[0]
    ds = ctx.to_device(scalars)
    if mont:
        ctx.fr_to_mont(ds, ds, n)
    res = ctx.msm_g1(b, ds, n, scalars_mont=mont, window_bits=window_bits)
    return (0, 0) if res is None else res


# ---------------------------------------------------------------------------- fields
def test_fr_montgomery_roundtrip(gpu_ctx):
    v = synth.fr_uniform(11, 5000)
    # values >= r (up to 2^256 - 1) reduce mod r like int(x) % FR_MODULUS
    big = synth.ints_to_limbs([R, R + 5, 2 * R + 1, (1 << 256) - 1, 5 * R + 7])
    v = np.concatenate([v, big])
    d = gpu_ctx.to_device(v)
    m = gpu_ctx.alloc(v.nbytes)
    gpu_ctx.fr_to_mont(m, d, v.shape[0])
    mont = m.download().view("<u8").reshape(-1, 4)
    assert (mont == O.to_mont(v)).all()
    gpu_ctx.fr_from_mont(d, m, v.shape[0])
    back = d.download().view("<u8").reshape(-1, 4)
    assert synth.limbs_to_ints(back) == [x % R for x in synth.limbs_to_ints(v)]


def test_fr_pointwise_mul_sub(gpu_ctx):
    n = 4099
    a = synth.fr_uniform(12, n)
    b = synth.fr_uniform(13, n)
    da, db, do = gpu_ctx.to_device(a), gpu_ctx.to_device(b), gpu_ctx.alloc(n * 32)
    gpu_ctx.fr_to_mont(da, da, n)
    gpu_ctx.fr_to_mont(db, db, n)
    gpu_ctx.fr_mul(do, da, db, n)
    gpu_ctx.fr_from_mont(do, do, n)
    ai, bi = synth.limbs_to_ints(a), synth.limbs_to_ints(b)
    got = synth.limbs_to_ints(do.download().view("<u8").reshape(-1, 4))
    assert got == [(x * y) % R for x, y in zip(ai, bi)]
    gpu_ctx.fr_sub(do, da, db, n)
    gpu_ctx.fr_from_mont(do, do, n)
    got = synth.limbs_to_ints(do.download().view("<u8").reshape(-1, 4))
    assert got == [(x - y) % R for x, y in zip(ai, bi)]


# ---------------------------------------------------------------------------- NTT
def _load(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def test_ntt_reference_fixtures(gpu_ctx):
    for fx in _load("ntt_reference.json")["fixtures"]:
        inp = _hex_to_limbs(fx["input"])
        out = gpu_ntt(gpu_ctx, fx["mode"], inp, fx["n"], int(fx["omega"], 16), int(fx["shift"], 16))
        assert synth.limbs_to_ints(out) == [int(x, 16) for x in fx["output"]], fx["name"]


def test_ntt_seeded_golden(gpu_ctx):
    for rec in _load("ntt_reference.json")["seeded"]:
        v = synth.fr_uniform(rec["seed"], rec["n"])
        assert _sha(v) == rec["input_sha256"]
        out = gpu_ntt(gpu_ctx, rec["mode"], v, rec["n"], int(rec["omega"], 16), int(rec["shift"], 16))
        assert _sha(out) == rec["output_sha256"], (rec["n"], rec["mode"])


def test_ntt_pad_truncate_golden(gpu_ctx):
    for rec in _load("ntt_reference.json")["pad_truncate"]:
        v = synth.fr_uniform(rec["seed"], rec["in_len"])
        assert _sha(v) == rec["input_sha256"]
        out = gpu_ntt(gpu_ctx, rec["mode"], v, rec["n"], int(rec["omega"], 16), int(rec["shift"], 16))
        assert _sha(out) == rec["output_sha256"], (rec["in_len"], rec["n"], rec["mode"])


@pytest.mark.parametrize("log_n", [0, 1, 4, 11, 12, 13, 16, 17, 20])
def test_ntt_matches_oracle(gpu_ctx, log_n):
    n = 1 << log_n
    v = synth.fr_uniform(synth.seed_for(1, log_n), n)
    om = O.omega_for_size(n)
    for mode in range(4):
        shift = 5 if mode >= 2 else 1
        exp = O.ntt_op(mode, v, n, om, shift)
        got = gpu_ntt(gpu_ctx, mode, v, n, om, shift)
        assert (got == exp).all(), (log_n, mode)


def test_ntt_host_submit_stream_matches_oracle(gpu_ctx):
    """zk_ntt_host_submit: canonical host input -> canonical host output, several calls in
    flight (three staging buffers in turn, three streams), sizes growing and shrinking, every
    mode, a zero-padded input, each result the oracle's."""
    cases = [(12, 0, 4096, 1), (16, 2, 65536, 5), (12, 1, 4096, 1), (20, 3, 1 << 20, 5), (10, 0, 700, 1),
             (16, 0, 50000, 1), (20, 0, 1 << 20, 1), (8, 2, 256, 5)]
    bufs, fences, exps = [], [], []
    for j, (lg, mode, in_len, shift) in enumerate(cases):
        n = 1 << lg
        v = synth.fr_uniform(8800 + j, in_len)
        pin_in = gpu_ctx.pinned(max(1, in_len) * 32)
        pin_in.array[:in_len * 32] = v.view(np.uint8).reshape(-1)
        pin_out = gpu_ctx.pinned(n * 32)
        om = O.omega_for_size(n)
        fences.append(gpu_ctx.ntt_host_submit(mode, pin_out, pin_in, in_len, lg, om, shift))
        bufs.append((pin_in, pin_out, n))
        exps.append(O.ntt_op(mode, v, n, om, shift))
    for f, (pin_in, pin_out, n), exp in zip(fences, bufs, exps):
        f.wait()
        f.destroy()
        got = pin_out.array[:n * 32].view("<u8").reshape(n, 4)
        assert (got == exp).all(), n
        pin_in.free()
        pin_out.free()


def test_ntt_host_submit_reduces_noncanonical_input(gpu_ctx):
    """zk_ntt_host_submit runs on the canonical values without Montgomery conversions; an
    input of any 256 bits (r, 2r + 7, 4r + 3, 2^256 - 1, ...) transforms as its value mod r,
    in every mode, at n = 1 and 2 and at one and two passes."""
    r = synth.FR_MODULUS
    for lg, mode, shift in ((0, 0, 1), (0, 3, 5), (1, 1, 1), (1, 2, 5), (10, 0, 1), (10, 3, 5), (14, 2, 5), (14, 1, 1)):
        n = 1 << lg
        base = synth.limbs_to_ints(synth.fr_uniform(9100 + lg + mode, n))
        extra = [r, r + 1, 2 * r + 7, 4 * r + 3, 5 * r, (1 << 256) - 1, (1 << 255) + 11]
        vals = [(v + r * (i % 5)) if (v + r * (i % 5)) < (1 << 256) else v for i, v in enumerate(base)]
        vals[:min(n, len(extra))] = extra[(lg + mode) % len(extra):][:n] if n < len(extra) else extra
        raw = synth.ints_to_limbs(vals)
        canon = synth.ints_to_limbs([v % r for v in vals])
        pin_in = gpu_ctx.pinned(n * 32)
        pin_in.array[:n * 32] = raw.view(np.uint8).reshape(-1)
        pin_out = gpu_ctx.pinned(n * 32)
        om = O.omega_for_size(n)
        f = gpu_ctx.ntt_host_submit(mode, pin_out, pin_in, n, lg, om, shift)
        f.wait()
        f.destroy()
        got = pin_out.array[:n * 32].view("<u8").reshape(n, 4)
        assert (got == O.ntt_op(mode, canon, n, om, shift)).all(), (lg, mode)
        pin_in.free()
        pin_out.free()


def test_ntt_2_22_oracle_and_roundtrip(gpu_ctx):
    log_n = 22
    n = 1 << log_n
    v = synth.fr_uniform(synth.seed_for(1, log_n), n)
    om = O.omega_for_size(n)
    exp = O.ntt_op(0, v, n, om)
    d = gpu_ctx.to_device(v)
    gpu_ctx.fr_to_mont(d, d, n)
    ev = gpu_ctx.alloc(n * 32)
    gpu_ctx.ntt(N.NTT_EVALS_FROM_COEFFS, ev, d, n, log_n, om)
    back = gpu_ctx.alloc(n * 32)
    gpu_ctx.ntt(N.NTT_COEFFS_FROM_EVALS, back, ev, n, log_n, om)
    gpu_ctx.ntt(N.NTT_COSET_EVALS_FROM_COEFFS, ev, back, n, log_n, om, 5)
    gpu_ctx.ntt(N.NTT_COSET_COEFFS_FROM_EVALS, back, ev, n, log_n, om, 5)
    gpu_ctx.fr_from_mont(back, back, n)
    assert (back.download().view("<u8").reshape(n, 4) == v).all()
    got = gpu_ntt(gpu_ctx, 0, v, n, om)
    assert (got == exp).all()


def test_ntt_2_23_sparse_sampled_and_roundtrip(gpu_ctx):
    """2^23: above the size whose plans keep full twiddle tables, so the two-level tables run.
    Sparse input (16 terms): every output is a 16-term sum, checked exactly at 128 sampled
    indices per mode; then a dense four-mode round trip."""
    log_n = 23
    n = 1 << log_n
    om = O.omega_for_size(n)
    rng = np.random.default_rng(2323)
    pos = sorted(set(int(x) for x in rng.integers(0, n, 16)))
    val = [int(x) for x in rng.integers(1, 1 << 62, len(pos))]
    v = np.zeros((n, 4), dtype=np.uint64)
    for p, x in zip(pos, val):
        v[p, 0] = x
    sample = [int(x) for x in rng.integers(0, n, 128)] + [0, n - 1]
    n_inv = pow(n, R - 2, R)
    for mode, shift in ((0, 1), (1, 1), (2, 5), (3, 5)):
        got = gpu_ntt(gpu_ctx, mode, v, n, om, shift)
        w = om if mode in (0, 2) else pow(om, R - 2, R)
        for i in sample:
            acc = sum(x * pow(w, i * p, R) for p, x in zip(pos, val))
            if mode == 2:
                acc = sum(x * pow(shift, p, R) * pow(w, i * p, R) for p, x in zip(pos, val))
            if mode in (1, 3):
                acc = acc * n_inv
            if mode == 3:
                acc = acc * pow(pow(shift, i, R), R - 2, R)
            acc %= R
            assert synth.limbs_to_ints(got[i : i + 1])[0] == acc, (mode, i)
    dense = synth.fr_uniform(synth.seed_for(1, log_n), n)
    d = gpu_ctx.to_device(dense)
    gpu_ctx.fr_to_mont(d, d, n)
    ev = gpu_ctx.alloc(n * 32)
    gpu_ctx.ntt(N.NTT_COSET_EVALS_FROM_COEFFS, ev, d, n, log_n, om, 5)
    gpu_ctx.ntt(N.NTT_COSET_COEFFS_FROM_EVALS, d, ev, n, log_n, om, 5)
    gpu_ctx.ntt(N.NTT_EVALS_FROM_COEFFS, ev, d, n, log_n, om)
    gpu_ctx.ntt(N.NTT_COEFFS_FROM_EVALS, d, ev, n, log_n, om)
    gpu_ctx.fr_from_mont(d, d, n)
    assert (d.download().view("<u8").reshape(n, 4) == dense).all()


def _gather_canonical(ctx, src, idx):
    didx = ctx.to_device(np.asarray(idx, dtype=np.uint32))
    g = ctx.alloc(len(idx) * 32)
    ctx.fr_gather(g, src, didx, len(idx))
    ctx.fr_from_mont(g, g, len(idx))
    return synth.limbs_to_ints(g.download().view("<u8").reshape(-1, 4))


def test_ntt_2_28_maximum_size_closed_form(gpu_ctx):
    """The largest domain (2^28, the 2-adicity of r, crypto/poly/ntt.py:9): input a_i = b^i
    generated on the device, whose transforms have closed forms -- forward
    sum_i (b w^k)^i = (b^n - 1) / (b w^k - 1), coset with s: the same with b s -- checked
    exactly at sampled indices; then the inverse brings the input back (sampled)."""
    log_n = 28
    n = 1 << log_n
    om = O.omega_for_size(n)
    b, s = 0x1234567890ABCDEF1234567, 5
    a = gpu_ctx.alloc(n * 32)
    gpu_ctx.fr_powers(a, b, n)  # Montgomery b^i
    ev = gpu_ctx.alloc(n * 32)
    rng = np.random.default_rng(28)
    idx = [0, 1, n // 2, n - 1] + [int(x) for x in rng.integers(0, n, 28)]
    for mode, base in ((N.NTT_EVALS_FROM_COEFFS, b), (N.NTT_COSET_EVALS_FROM_COEFFS, b * s % R)):
        gpu_ctx.ntt(mode, ev, a, n, log_n, om, s if mode == N.NTT_COSET_EVALS_FROM_COEFFS else 1)
        got = _gather_canonical(gpu_ctx, ev, idx)
        num = (pow(base, n, R) - 1) % R
        for k, g in zip(idx, got):
            assert g == num * pow((base * pow(om, k, R) - 1) % R, R - 2, R) % R, (mode, k)
    # forward then inverse (coset pair) restores the powers
    gpu_ctx.ntt(N.NTT_COSET_COEFFS_FROM_EVALS, ev, ev, n, log_n, om, s)
    back = _gather_canonical(gpu_ctx, ev, idx)
    assert back == [pow(b, k, R) for k in idx]


def test_ntt_coset_zero_shift_and_other_shift(gpu_ctx):
    n = 64
    v = synth.fr_uniform(99, n)
    om = O.omega_for_size(n)
    for shift in (0, 7, R - 1):
        for mode in (2, 3):
            assert (gpu_ntt(gpu_ctx, mode, v, n, om, shift) == O.ntt_op(mode, v, n, om, shift)).all(), (shift, mode)


def test_ntt_rejects_bad_arguments(gpu_ctx):
    n = 16
    d = gpu_ctx.alloc(n * 32)
    with pytest.raises(ValueError):
        gpu_ctx.ntt(0, d, d, n, 4, 5)  # 5 is not a primitive 16th root of unity
    with pytest.raises(ValueError):
        gpu_ctx.ntt(1, d, d, 8, 4, O.omega_for_size(16))  # inverse needs len == n
    with pytest.raises(ValueError):
        gpu_ctx.ntt(0, d, d, n, 29, 1)


# ---------------------------------------------------------------------------- MSM
def test_msm_reference_cases(gpu_ctx):
    for case in _load("msm_reference.json")["cases"]:
        bases = _hex_to_limbs([c for p in case["bases"] for c in p], 8)
        scal = synth.ints_to_limbs([int(s, 16) for s in case["scalars"]])
        exp = tuple(int(x, 16) for x in case["result"])
        # canonical scalars (reduced mod r on the device) and Montgomery scalars
        assert gpu_msm(gpu_ctx, bases, scal, mont=False) == exp, case["name"]
        assert gpu_msm(gpu_ctx, bases, scal, mont=True) == exp, case["name"]


def test_msm_reference_workloads(gpu_ctx):
    for wl in _load("msm_reference.json")["workloads"]:
        n, seed = wl["n"], wl["seed"]
        k = synth.base_dlogs(seed, n)
        assert _sha(k) == wl["dlogs_sha256"]
        s = synth.fr_uniform(seed, n) if wl["scalars"] == "uniform" else synth.fr_witness_like(seed, n)
        assert _sha(s) == wl["scalars_sha256"]
        bases = O.g1_fixed_base_mul(O.G1_GENERATOR, k)
        assert _sha(bases) == wl["bases_sha256"]
        exp = tuple(int(x, 16) for x in wl["result"])
        for c in (0, 5, 11, 16):
            assert gpu_msm(gpu_ctx, bases, s, window_bits=c) == exp, (wl["name"], c)


@pytest.mark.parametrize("kind", ["uniform", "witness"])
def test_msm_matches_oracle_2_16(gpu_ctx, kind):
    n = 1 << 16
    seed = synth.seed_for(2, 16)
    k = synth.base_dlogs(seed, n)
    s = synth.fr_uniform(seed, n) if kind == "uniform" else synth.fr_witness_like(seed, n)
    bases = O.g1_fixed_base_mul(O.G1_GENERATOR, k)
    exp = O.affine_to_ints(O.msm_pippenger(bases, s, O.msm_window_rule(n)))
    assert exp == O.affine_to_ints(O.msm_known_answer(k, s))
    for c in (0, 4, 9, 13, 16, 20):
        assert gpu_msm(gpu_ctx, bases, s, window_bits=c) == exp, c


def test_fixed_base_mul_matches_oracle(gpu_ctx):
    n = 3000
    k = synth.base_dlogs(7, n)
    k[5] = 0  # [0]G = infinity
    dk = gpu_ctx.to_device(k)
    out = gpu_ctx.alloc(n * 64)
    gpu_ctx.g1_fixed_base_mul((1, 2), dk, n, out)
    got = out.download().view("<u8").reshape(n, 8)
    assert (got == O.g1_fixed_base_mul(O.G1_GENERATOR, k)).all()


def test_msm_2_20_known_answer(gpu_ctx):
    """Full-size MSM: bases generated on the device, checked on a sample; result by the dlog identity."""
    log_n = 20
    n = 1 << log_n
    seed = synth.seed_for(2, log_n)
    k = synth.base_dlogs(seed, n)
    s = synth.fr_uniform(seed, n)
    dk = gpu_ctx.to_device(k)
    dxy = gpu_ctx.alloc(n * 64)
    gpu_ctx.g1_fixed_base_mul((1, 2), dk, n, dxy)
    sample = np.arange(0, n, 997)
    host_xy = dxy.download().view("<u8").reshape(n, 8)
    assert (host_xy[sample] == O.g1_fixed_base_mul(O.G1_GENERATOR, k[sample])).all()
    bases = gpu_ctx.bases_from_device(dxy, n)
    ds = gpu_ctx.to_device(s)
    gpu_ctx.fr_to_mont(ds, ds, n)
    exp = O.affine_to_ints(O.msm_known_answer(k, s))
    assert gpu_ctx.msm_g1(bases, ds, n) == exp
    # prefix (offset) MSM over the same resident bases
    m = 1000
    exp2 = O.affine_to_ints(O.msm_known_answer(k[7:7 + m], s[:m]))
    assert gpu_ctx.msm_g1(bases, ds, m, offset=7) == exp2


@pytest.mark.parametrize("log_n,c", [(16, 0), (16, 13), (18, 0), (20, 0)])
def test_msm_hot_digit_known_answer(gpu_ctx, log_n, c):
    """Scalars that crowd one bucket: all 1 (every entry in bucket 1 of window 0), then 1 and
    -1 with a share of uniform scalars. The hot bucket spans thousands of accumulation
    segments, so its pieces are summed in chunks by many CTAs and the chunk sums by the last
    of them; the result is the known answer [sum k_i s_i]G."""
    n = 1 << log_n
    seed = synth.seed_for(7, log_n)
    k = synth.base_dlogs(seed, n)
    dk = gpu_ctx.to_device(k)
    dxy = gpu_ctx.alloc(n * 64)
    gpu_ctx.g1_fixed_base_mul((1, 2), dk, n, dxy)
    bases = gpu_ctx.bases_from_device(dxy, n)
    ones = synth.ints_to_limbs([1] * n)
    rng = np.random.default_rng(seed)
    mixed_ints = synth.limbs_to_ints(synth.fr_uniform(seed + 1, n))
    pick = rng.random(n)
    mixed_ints = [1 if u < 0.45 else (R - 1 if u < 0.9 else v) for u, v in zip(pick, mixed_ints)]
    mixed = synth.ints_to_limbs(mixed_ints)
    for s in (ones, mixed):
        ds = gpu_ctx.to_device(s)
        gpu_ctx.fr_to_mont(ds, ds, n)
        assert gpu_ctx.msm_g1(bases, ds, n, window_bits=c) == O.affine_to_ints(O.msm_known_answer(k, s)), c


def test_msm_2_24_known_answer(gpu_ctx):
    """A large MSM (2^24 points: 2^25 GLV halves x 8 windows = 2^28 CSR entries) against the
    known answer; bases generated on the device."""
    log_n = 24
    n = 1 << log_n
    seed = synth.seed_for(2, log_n)
    k = synth.base_dlogs(seed, n)
    s = synth.fr_uniform(seed, n)
    dk = gpu_ctx.to_device(k)
    dxy = gpu_ctx.alloc(n * 64)
    gpu_ctx.g1_fixed_base_mul((1, 2), dk, n, dxy)
    del dk
    bases = gpu_ctx.bases_from_device(dxy, n)
    del dxy
    ds = gpu_ctx.to_device(s)
    gpu_ctx.fr_to_mont(ds, ds, n)
    assert gpu_ctx.msm_g1(bases, ds, n) == O.affine_to_ints(O.msm_known_answer(k, s))


def test_msm_g1_host_one_call(gpu_ctx):
    """zk_msm_g1_host (points and scalars from host memory, points uploaded on a second
    stream): same point as the oracle, from pinned and from pageable buffers, with
    infinity points, both scalar forms, and repeated calls on one context."""
    n = 1 << 15
    seed = synth.seed_for(2, 15) + 11
    k = synth.base_dlogs(seed, n)
    k[3] = 0  # an infinity point
    s = synth.fr_uniform(seed, n)
    s[9] = 0
    xy = O.g1_fixed_base_mul(O.G1_GENERATOR, k)
    exp = O.affine_to_ints(O.msm_known_answer(k, s))
    pin_xy = gpu_ctx.pinned(n * 64)
    pin_xy.array[:] = xy.view(np.uint8).reshape(-1)
    pin_s = gpu_ctx.pinned(n * 32)
    pin_s.array[:] = s.view(np.uint8).reshape(-1)
    for _ in range(3):
        assert gpu_ctx.msm_g1_host(pin_xy, pin_s, n) == exp
    assert gpu_ctx.msm_g1_host(xy, s, n) == exp  # pageable numpy buffers
    assert gpu_ctx.msm_g1_host(xy, s, n, window_bits=9) == exp
    # Montgomery-form scalars: to_mont on the device, read back
    ds = gpu_ctx.to_device(s)
    gpu_ctx.fr_to_mont(ds, ds, n)
    s_mont = ds.download().view("<u8").reshape(n, 4)
    assert gpu_ctx.msm_g1_host(xy, s_mont, n, scalars_mont=True) == exp
    m = 1000  # a prefix
    assert gpu_ctx.msm_g1_host(xy[:m], s[:m], m) == O.affine_to_ints(O.msm_known_answer(k[:m], s[:m]))
    assert gpu_ctx.msm_g1_host(xy, s, 0) is None
    pin_xy.free()
    pin_s.free()


def test_msm_g1_host_alternating_infinity_sets(gpu_ctx):
    """zk_msm_g1_host at 2^20 from pinned buffers, alternating a base set whose every second
    point is infinity with the full set (the same scratch buffers in turn): the points upload
    on a second stream while the digits are sorted, and each result must equal the known
    answer -- nothing before the accumulation may depend on the points' upload."""
    n = 1 << 20
    seed = synth.seed_for(2, 20) + 17
    k = synth.base_dlogs(seed, n)
    s = synth.fr_uniform(seed, n)
    dk = gpu_ctx.to_device(k)
    dxy = gpu_ctx.alloc(n * 64)
    gpu_ctx.g1_fixed_base_mul((1, 2), dk, n, dxy)
    full = dxy.download().view("<u8").reshape(n, 8)
    half = full.copy()
    half[1::2] = 0
    k_half = k.copy()
    k_half[1::2] = 0
    exp_full = O.affine_to_ints(O.msm_known_answer(k, s))
    exp_half = O.affine_to_ints(O.msm_known_answer(k_half, s))
    pin_full = gpu_ctx.pinned(n * 64)
    pin_full.array[:] = full.view(np.uint8).reshape(-1)
    pin_half = gpu_ctx.pinned(n * 64)
    pin_half.array[:] = half.view(np.uint8).reshape(-1)
    pin_s = gpu_ctx.pinned(n * 32)
    pin_s.array[:] = s.view(np.uint8).reshape(-1)
    for _ in range(2):
        assert gpu_ctx.msm_g1_host(pin_half, pin_s, n) == exp_half
        assert gpu_ctx.msm_g1_host(pin_full, pin_s, n) == exp_full
    # the asynchronous form, several calls in flight (two staging buffers used in turn, each
    # waiting for the MSM two calls back), then a larger call that grows a buffer, and a
    # smaller one: every result the known answer
    jobs = [gpu_ctx.msm_g1_host_submit(pin_half if j % 2 else pin_full, pin_s, n) for j in range(5)]
    for j, b in enumerate(jobs):
        assert b.wait() == [exp_half if j % 2 else exp_full], j
        b.destroy()
    m = (1 << 18) + 5
    exp_m = O.affine_to_ints(O.msm_known_answer(k[:m], s[:m]))
    first = gpu_ctx.msm_g1_host_submit(pin_full, pin_s, m)
    second = gpu_ctx.msm_g1_host_submit(pin_full, pin_s, n)
    third = gpu_ctx.msm_g1_host_submit(pin_half, pin_s, m)
    assert first.wait() == [exp_m] and second.wait() == [exp_full]
    assert third.wait() == [O.affine_to_ints(O.msm_known_answer(k_half[:m], s[:m]))]
    for b in (first, second, third):
        b.destroy()
    empty = gpu_ctx.msm_g1_host_submit(pin_full, pin_s, 0)
    assert empty.wait() == [None]
    empty.destroy()
    for b in (pin_full, pin_half, pin_s):
        b.free()


def test_msm_glv_edge_scalars(gpu_ctx):
    """G1 MSMs split every scalar k = k1 + k2 lambda (GLV): scalars at the ends of the range,
    lambda itself, its negation and rounding midpoints, on random bases, for every window
    size the split changes the window count of (W = ceil(128 / c))."""
    lam = 0xB3C4D79D41A917585BFC41088D8DAAA78B17EA66B99C90DD
    vals = [0, 1, 2, 3, R - 1, R - 2, lam, R - lam, lam + 1, (R - 1) // 2, (R + 1) // 2, R // 3, (2 * R) // 3,
            (1 << 127) - 1, 1 << 127, (1 << 253) - 1]
    vals += [int(x) for x in synth.limbs_to_ints(synth.fr_uniform(4242, 48))]
    n = len(vals)
    s = synth.ints_to_limbs(vals)
    k = synth.base_dlogs(31, n)
    k[5] = 0  # an infinity base
    bases = O.g1_fixed_base_mul(O.G1_GENERATOR, k)
    exp = O.affine_to_ints(O.msm_known_answer(k, s))
    for c in (0, 4, 5, 7, 8, 11, 13, 16, 20):
        assert gpu_msm(gpu_ctx, bases, s, window_bits=c) == exp, c
    st = gpu_ctx.msm_last_stats()
    assert st["window_bits"] == 20 and st["windows"] == (128 + 19) // 20
    # the same scalars through fixed-base rows (rows of P and of phi(P), one bucket set)
    b = gpu_ctx.bases_from_host(bases)
    ds = gpu_ctx.to_device(s)
    gpu_ctx.fr_to_mont(ds, ds, n)
    for c in (4, 7, 16, 19):
        gpu_ctx.bases_precompute(b, c)
        assert gpu_ctx.msm_g1(b, ds, n) == exp, ("fixed", c)
        assert gpu_ctx.msm_g1(b, ds, n - 9, offset=9) == O.affine_to_ints(O.msm_known_answer(k[9:], s[:n - 9]))
    # one scalar at a time (each half alone in its buckets)
    for v in vals[:16]:
        one = synth.ints_to_limbs([v])
        got = gpu_msm(gpu_ctx, bases[:1], one)
        assert got == O.affine_to_ints(O.msm_known_answer(k[:1], one)), hex(v)


def test_msm_canonical_scalars_at_or_above_r(gpu_ctx):
    """Canonical scalars are reduced mod r first, as msm_pippenger does (s % FR_MODULUS,
    crypto/msm/pippenger.py:28): r, r + 1, 2r - 1, 2^256 - 1 and friends give the MSM of
    their residues."""
    vals = [R, R + 1, 2 * R - 1, 2 * R, 3 * R + 12345, (1 << 256) - 1, (1 << 255) + 7, R - 1]
    n = len(vals)
    k = synth.base_dlogs(777, n)
    bases = O.g1_fixed_base_mul(O.G1_GENERATOR, k)
    raw = synth.ints_to_limbs(vals)
    red = synth.ints_to_limbs([v % R for v in vals])
    exp = O.affine_to_ints(O.msm_known_answer(k, red))
    assert gpu_msm(gpu_ctx, bases, raw, mont=False) == exp
    assert gpu_ctx.msm_g1_host(bases, raw, n) == exp


def test_msm_empty_and_errors(gpu_ctx):
    bases = gpu_ctx.bases_from_host(O.g1_fixed_base_mul(O.G1_GENERATOR, synth.base_dlogs(1, 4)))
    ds = gpu_ctx.to_device(synth.fr_uniform(1, 4))
    assert gpu_ctx.msm_g1(bases, ds, 0) is None
    with pytest.raises(ValueError):
        gpu_ctx.msm_g1(bases, ds, 5)
    with pytest.raises(ValueError):
        gpu_ctx.msm_g1(bases, ds, 4, window_bits=3)


@pytest.mark.parametrize("kind", ["uniform", "witness"])
def test_msm_fixed_base_precompute_matches_oracle(gpu_ctx, kind):
    """Window-shifted fixed-base rows (zk_bases_precompute) give the same point as plain Pippenger."""
    n = 1 << 14
    seed = synth.seed_for(2, 14) + 5
    k = synth.base_dlogs(seed, n)
    k[3] = 0  # an infinity base
    s = synth.fr_uniform(seed, n) if kind == "uniform" else synth.fr_witness_like(seed, n)
    bases_xy = O.g1_fixed_base_mul(O.G1_GENERATOR, k)
    exp = O.affine_to_ints(O.msm_known_answer(k, s))
    b = gpu_ctx.bases_from_host(bases_xy)
    ds = gpu_ctx.to_device(s)
    gpu_ctx.fr_to_mont(ds, ds, n)
    assert gpu_ctx.msm_g1(b, ds, n) == exp
    for c in (5, 8, 13, 16, 20):
        gpu_ctx.bases_precompute(b, c)
        assert gpu_ctx.msm_g1(b, ds, n) == exp, c
        assert gpu_ctx.msm_g1(b, ds, n, window_bits=c) == exp, c
        # a different explicit window falls back to the plain path
        assert gpu_ctx.msm_g1(b, ds, n, window_bits=12 if c != 12 else 11) == exp
        # prefix with offset over the shifted rows
        m = 777
        assert gpu_ctx.msm_g1(b, ds, m, offset=100) == O.affine_to_ints(O.msm_known_answer(k[100:100 + m], s[:m]))


def test_msm_zero_digit_after_carry(gpu_ctx):
    """A window whose bits are all ones and that receives the carry of a negative digit below
    yields digit 0 with a carry onwards (v = 2^c); every window size must skip that digit."""
    n = 64
    k = synth.base_dlogs(4700, n)
    bases = O.g1_fixed_base_mul(O.G1_GENERATOR, k)
    vals = []
    for c in range(4, 17):
        # window 0 above half (carry 1), window 1 all ones -> 2^c, then the same pattern higher up
        v = ((1 << (c - 1)) + 1) | (((1 << c) - 1) << c)
        v |= v << (4 * c)
        vals.append(v % R)
    vals += [(R - 1), (1 << 253) - 1, (1 << 200) - 1]
    s = synth.ints_to_limbs((vals * (n // len(vals) + 1))[:n])
    exp = O.affine_to_ints(O.msm_known_answer(k, s))
    for c in (0, 4, 5, 6, 7, 8, 11, 13, 16, 20):
        assert gpu_msm(gpu_ctx, bases, s, window_bits=c) == exp, c
