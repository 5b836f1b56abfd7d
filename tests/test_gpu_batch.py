"""GPU parity of the batched MSM engine (zk_msm_g1_batch, zk_msm_plan_*) through the C ABI.

Every instance is checked bit-exactly against the oracle: the known-answer identity
MSM([k_i]G, s) = [sum k_i s_i]G for all of them, and the oracle's Pippenger
(crypto/msm/pippenger.py:10-64 restated) on a sample. The batch semantics follow
MSM_G1_BATCH / KZG_BATCH_COMMIT (runtime/kernels/cpu/kernels.py:441-496): instance k
is the MSM of its scalars over the prefix points[:len(s_k)], empty instances give the
identity.
"""

import numpy as np
import pytest

from oracle import oracle as O
from pyzkp_gb300 import synth

pytestmark = pytest.mark.gpu


def _expect(k: np.ndarray, s: np.ndarray):
    if s.shape[0] == 0:
        return None
    p = O.affine_to_ints(O.msm_known_answer(k, s))
    return None if p == (0, 0) else p


def _bases(ctx, seed: int, n: int, zero_at=()):
    k = synth.base_dlogs(seed, n)
    for z in zero_at:
        k[z] = 0  # infinity bases
    return k, ctx.bases_from_host(O.g1_fixed_base_mul(O.G1_GENERATOR, k))


def _upload(ctx, s: np.ndarray, mont: bool = True):
    d = ctx.to_device(s if s.shape[0] else np.zeros((1, 4), dtype=np.uint64))
    if mont and s.shape[0]:
        ctx.fr_to_mont(d, d, s.shape[0])
    return d


def test_msm_batch_shared_prefix_mixed_sizes(gpu_ctx):
    n = 1 << 15
    k, b = _bases(gpu_ctx, 101, n, zero_at=(0, 17))
    sizes = [0, 1, 2, 5, 63, 64, 65, 1000, 4096, 777, (1 << 12) + 3, 20000, n, 0, 3]
    scal = []
    for j, m in enumerate(sizes):
        s = synth.fr_uniform(500 + j, m) if j % 2 else synth.fr_witness_like(500 + j, m)
        scal.append(s)
    dev = [_upload(gpu_ctx, s) for s in scal]
    got = gpu_ctx.msm_g1_batch(b, dev, sizes)
    exp = [_expect(k[:m], s) for m, s in zip(sizes, scal)]
    assert got == exp
    # one explicit window for every instance, and canonical (non-Montgomery) scalars
    assert gpu_ctx.msm_g1_batch(b, dev, sizes, window_bits=9) == exp
    dev_c = [_upload(gpu_ctx, s, mont=False) for s in scal]
    assert gpu_ctx.msm_g1_batch(b, dev_c, sizes, scalars_mont=False) == exp
    # the oracle's own Pippenger on a sample of instances
    for j in (4, 8, 11):
        m = sizes[j]
        bases_xy = O.g1_fixed_base_mul(O.G1_GENERATOR, k[:m])
        assert got[j] == O.affine_to_ints(O.msm_pippenger(bases_xy, scal[j], O.msm_window_rule(m)))


def test_msm_batch_many_base_sets_offsets_and_fixed_base(gpu_ctx):
    """Instances over different resident base sets, with offsets, some in fixed-base mode."""
    k1, b1 = _bases(gpu_ctx, 201, 5000)
    k2, b2 = _bases(gpu_ctx, 202, 9000, zero_at=(9,))
    k3, b3 = _bases(gpu_ctx, 203, 3000)
    gpu_ctx.bases_precompute(b3, 10)  # b3 instances run in fixed-base mode (c = 10)
    # (b2, k2, 0, 5000) reaches b2's infinity point and shares a pipeline (same window) with
    # the first b1 instance, whose set holds none
    spec = [(b1, k1, 0, 5000), (b2, k2, 100, 8000), (b3, k3, 0, 3000), (b1, k1, 4000, 1000), (b3, k3, 7, 2000),
            (b2, k2, 8999, 1), (b2, k2, 0, 0), (b2, k2, 0, 5000)]
    bases, offs, sizes, dev, exp = [], [], [], [], []
    for j, (b, k, off, m) in enumerate(spec):
        s = synth.fr_uniform(900 + j, m)
        bases.append(b)
        offs.append(off)
        sizes.append(m)
        dev.append(_upload(gpu_ctx, s))
        exp.append(_expect(k[off:off + m], s))
    assert gpu_ctx.msm_g1_batch(bases, dev, sizes, offsets=offs) == exp
    with pytest.raises(ValueError):  # a prefix beyond the base set
        gpu_ctx.msm_g1_batch([b1], [dev[0]], [5001])
    with pytest.raises(ValueError):
        gpu_ctx.msm_g1_batch([b2], [dev[1]], [10], offsets=[8995])
    with pytest.raises(ValueError):
        gpu_ctx.msm_g1_batch([b1], [dev[0]], [10], window_bits=3)


@pytest.mark.parametrize("use_graph", [True, False])
def test_msm_plan_replays_with_new_scalars(gpu_ctx, use_graph):
    n = 1 << 14
    k, b = _bases(gpu_ctx, 301, n)
    rng = np.random.default_rng(7)
    sizes = [int(round(2 ** u)) for u in rng.uniform(6, 14, size=24)] + [0, n]
    plan = gpu_ctx.msm_plan(b, sizes, use_graph=use_graph)
    assert plan.launches() > 0 if use_graph else plan.launches() == 0
    for rep in range(2):
        scal = [synth.fr_uniform(1000 * rep + j, m) for j, m in enumerate(sizes)]
        for j, s in enumerate(scal):
            if s.shape[0]:
                slot = plan.slot(j)
                slot.upload(s)
                gpu_ctx.fr_to_mont(slot, slot, s.shape[0])
        got = plan.run()
        assert got == [_expect(k[:m], s) for m, s in zip(sizes, scal)], rep
    plan.free()


def test_msm_batch_log_uniform_64(gpu_ctx):
    """A 64-instance batch with sizes 2^U, U ~ Uniform[10, 16] (the batched-engine workload, scaled down)."""
    n = 1 << 16
    k, b = _bases(gpu_ctx, 401, n)
    rng = np.random.default_rng(synth.seed_for(3, 16))
    sizes = [int(round(2 ** u)) for u in rng.uniform(10, 16, size=64)]
    scal = [synth.fr_uniform(2000 + j, m) for j, m in enumerate(sizes)]
    dev = [_upload(gpu_ctx, s) for s in scal]
    got = gpu_ctx.msm_g1_batch(b, dev, sizes)
    assert got == [_expect(k[:m], s) for m, s in zip(sizes, scal)]
    # the same instances one by one through zk_msm_g1
    for j in (0, 31, 63):
        assert gpu_ctx.msm_g1(b, dev[j], sizes[j]) == got[j]


# ----------------------------------------------------------------- MSM work queue (one launch)
def test_msm_work_queue_matches_known_answers(gpu_ctx):
    """The work-queue form (sorts, then every pipeline's later stages in one persistent launch)
    gives the same points: mixed sizes with infinity bases, witness-like scalars (hot buckets
    and long-bucket fixups), several base sets with offsets and a fixed-base set, the merge-round
    mode (window 8 at 2^16: ~1000 entries per bucket), single MSMs, and the asynchronous form."""
    k, b = _bases(gpu_ctx, 1101, 1 << 16, zero_at=(0, 17))
    k3, b3 = _bases(gpu_ctx, 1103, 3000)
    gpu_ctx.bases_precompute(b3, 10)
    sizes = [0, 1, 2, 5, 63, 64, 65, 1000, 4096, 777, (1 << 12) + 3, 20000, 1 << 16, 3]
    scal = [synth.fr_witness_like(1200 + j, m) if j % 3 == 0 else synth.fr_uniform(1200 + j, m)
            for j, m in enumerate(sizes)]
    dev = [_upload(gpu_ctx, s) for s in scal]
    exp = [_expect(k[:m], s) for m, s in zip(sizes, scal)]
    s3 = synth.fr_uniform(1300, 2000)
    d3 = _upload(gpu_ctx, s3)
    e3 = _expect(k3[7:2007], s3)
    try:
        gpu_ctx.msm_batch_set_queue(True)
        for rep in range(2):
            assert gpu_ctx.msm_g1_batch(b, dev, sizes) == exp, rep
        assert gpu_ctx.msm_g1_batch(b, dev, sizes, window_bits=9) == exp
        assert gpu_ctx.msm_g1_batch([b, b3, b], [dev[12], d3, dev[8]], [sizes[12], 2000, sizes[8]],
                                    offsets=[0, 7, 0]) == [exp[12], e3, exp[8]]
        # merge rounds instead of the fixup
        assert gpu_ctx.msm_g1_batch(b, [dev[12]], [sizes[12]], window_bits=8) == [exp[12]]
        assert gpu_ctx.msm_g1(b, dev[11], sizes[11]) == exp[11]
        job = gpu_ctx.msm_batch_submit(b, dev, sizes)
        try:
            assert job.wait() == exp
        finally:
            job.destroy()
    finally:
        gpu_ctx.msm_batch_set_queue(False)


@pytest.mark.parametrize("use_graph", [True, False])
def test_msm_queue_plan_replays(gpu_ctx, use_graph):
    n = 1 << 14
    k, b = _bases(gpu_ctx, 1401, n)
    rng = np.random.default_rng(17)
    sizes = [int(round(2 ** u)) for u in rng.uniform(6, 14, size=24)] + [0, n]
    plan = gpu_ctx.msm_plan(b, sizes, use_graph=use_graph, queue=True)
    for rep in range(2):
        scal = [synth.fr_uniform(1500 + 100 * rep + j, m) for j, m in enumerate(sizes)]
        for j, s in enumerate(scal):
            if s.shape[0]:
                slot = plan.slot(j)
                slot.upload(s)
                gpu_ctx.fr_to_mont(slot, slot, s.shape[0])
        assert plan.run() == [_expect(k[:m], s) for m, s in zip(sizes, scal)], rep
    plan.free()


def test_msm_queue_wait_limit_runs_out_and_context_survives(gpu_ctx):
    """A wait that can never succeed (the first waiting item of the queue waits for one item
    more than its dependency has) gives up at its limit: the call raises TimeoutError within
    the limit's order of magnitude and the context's next MSM is correct."""
    import time

    k, b = _bases(gpu_ctx, 1601, 5000)
    s = synth.fr_uniform(1602, 5000)
    d = _upload(gpu_ctx, s)
    try:
        gpu_ctx.msm_batch_set_queue(True)
        gpu_ctx.msm_queue_test_limit(20000)  # 20 ms
        t = time.perf_counter()
        with pytest.raises(TimeoutError):
            gpu_ctx.msm_g1_batch(b, [d], [5000])
        assert time.perf_counter() - t < 5.0
        assert gpu_ctx.msm_g1_batch(b, [d], [5000]) == [_expect(k, s)]  # the limit was used once
    finally:
        gpu_ctx.msm_batch_set_queue(False)
    assert gpu_ctx.msm_g1(b, d, 5000) == _expect(k, s)


# ---------------------------------------------------------------------------- NTT batches
def _omega(log_n: int) -> int:
    return O.omega_for_size(1 << log_n)


def _oracle_ntt(mode, values, log_n, shift=1):
    return O.ntt_op(mode, values, 1 << log_n, _omega(log_n), shift)


def _ntt_jobs(ctx, spec, seed):
    """spec: (mode, log_n, in_len, shift, in_place) -> jobs, host inputs, output buffers."""
    jobs, inputs, outs = [], [], []
    for j, (mode, log_n, in_len, shift, in_place) in enumerate(spec):
        n = 1 << log_n
        v = synth.fr_uniform(seed + j, in_len)
        din = ctx.alloc(max(n, in_len, 1) * 32)
        if in_len:
            din.upload(v)
            ctx.fr_to_mont(din, din, in_len)
        dout = din if in_place else ctx.alloc(n * 32)
        jobs.append((mode, dout, din, in_len, log_n, _omega(log_n), shift))
        inputs.append(v)
        outs.append(dout)
    return jobs, inputs, outs


def _download(ctx, d, n):
    ctx.fr_from_mont(d, d, n)
    return d.download(n * 32).view("<u8").reshape(n, 4).astype(np.uint64)


NTT_SPEC = [
    (0, 0, 1, 1, False), (1, 1, 2, 1, False), (2, 4, 16, 5, False), (3, 4, 16, 5, True), (0, 10, 700, 1, False),
    (0, 11, 2048, 1, True), (2, 12, 4000, 5, False), (1, 13, 8192, 1, True), (3, 16, 1 << 16, 7, False),
    (0, 17, 1 << 17, 1, False), (2, 20, 1 << 20, 5, True), (0, 12, 5000, 1, False), (0, 3, 0, 1, False),
]


def test_ntt_batch_matches_oracle(gpu_ctx):
    jobs, inputs, outs = _ntt_jobs(gpu_ctx, NTT_SPEC, 3100)
    gpu_ctx.ntt_batch(jobs)
    gpu_ctx.sync()
    for (mode, log_n, in_len, shift, _), v, d in zip(NTT_SPEC, inputs, outs):
        got = _download(gpu_ctx, d, 1 << log_n)
        assert (got == _oracle_ntt(mode, v, log_n, shift)).all(), (mode, log_n, in_len)


@pytest.mark.parametrize("use_graph", [True, False])
def test_ntt_plan_replays_with_new_inputs(gpu_ctx, use_graph):
    spec = [s for s in NTT_SPEC if not s[4]]  # out of place: the inputs stay valid for the next run
    jobs, _, outs = _ntt_jobs(gpu_ctx, spec, 3200)
    plan = gpu_ctx.ntt_plan(jobs, use_graph=use_graph)
    assert plan.launches() > 0 if use_graph else plan.launches() == 0
    for rep in range(2):
        inputs = []
        for j, (mode, log_n, in_len, shift, _) in enumerate(spec):
            v = synth.fr_uniform(4000 + 100 * rep + j, in_len)
            if in_len:
                jobs[j][2].upload(v)
                gpu_ctx.fr_to_mont(jobs[j][2], jobs[j][2], in_len)
            inputs.append(v)
        plan.run()
        gpu_ctx.sync()
        for (mode, log_n, in_len, shift, _), v, d in zip(spec, inputs, outs):
            got = _download(gpu_ctx, d, 1 << log_n)
            assert (got == _oracle_ntt(mode, v, log_n, shift)).all(), (rep, mode, log_n)
    plan.free()


def test_ntt_batch_work_queue_matches_oracle(gpu_ctx):
    """The work-queue form (one persistent launch) gives the per-transform results, in place and
    out of place, including 3-pass transforms (tuned split) whose middle pass reads data other
    CTAs wrote earlier in the same launch."""
    spec = NTT_SPEC + [(2, 14, 1 << 14, 5, True), (1, 15, 1 << 15, 1, False)]
    try:
        gpu_ctx.tune_set_ntt_split(14, [5, 5, 4])
        gpu_ctx.tune_set_ntt_split(15, [4, 6, 5])
        gpu_ctx.ntt_batch_set_queue(True)
        for rep in range(2):
            jobs, inputs, outs = _ntt_jobs(gpu_ctx, spec, 3300 + 50 * rep)
            gpu_ctx.ntt_batch(jobs)
            gpu_ctx.ntt_queue_status()
            for (mode, log_n, in_len, shift, _), v, d in zip(spec, inputs, outs):
                got = _download(gpu_ctx, d, 1 << log_n)
                assert (got == _oracle_ntt(mode, v, log_n, shift)).all(), (rep, mode, log_n, in_len)
    finally:
        gpu_ctx.ntt_batch_set_queue(False)
        gpu_ctx.tune_set_ntt_split(14, [])
        gpu_ctx.tune_set_ntt_split(15, [])


@pytest.mark.parametrize("use_graph", [True, False])
def test_ntt_queue_plan_replays_and_counts_one_kernel(gpu_ctx, use_graph):
    spec = [s for s in NTT_SPEC if not s[4]]
    jobs, _, outs = _ntt_jobs(gpu_ctx, spec, 3400)
    plan = gpu_ctx.ntt_plan(jobs, use_graph=use_graph, queue=True)
    if use_graph:
        assert plan.launches() == 1  # the whole batch is one kernel
    for rep in range(3):
        inputs = []
        for j, (mode, log_n, in_len, shift, _) in enumerate(spec):
            v = synth.fr_uniform(4400 + 100 * rep + j, in_len)
            if in_len:
                jobs[j][2].upload(v)
                gpu_ctx.fr_to_mont(jobs[j][2], jobs[j][2], in_len)
            inputs.append(v)
        plan.run()
        gpu_ctx.ntt_queue_status()
        for (mode, log_n, in_len, shift, _), v, d in zip(spec, inputs, outs):
            got = _download(gpu_ctx, d, 1 << log_n)
            assert (got == _oracle_ntt(mode, v, log_n, shift)).all(), (rep, mode, log_n)
    plan.free()


def test_ntt_queue_wait_limit_runs_out_and_context_survives(gpu_ctx):
    """A wait that can never succeed (a second pass waiting for one first-pass tile more than
    exist) gives up at its limit: the launch returns, the status names the waiting entry, and
    the context runs the next transform correctly."""
    import time

    t = time.perf_counter()
    entry = gpu_ctx.ntt_queue_selftest(20000)  # 20 ms limit
    assert time.perf_counter() - t < 5.0
    assert entry in (2, 3)  # 1 + queue entry 1 (the second pass), or 2 under a 3-pass split
    gpu_ctx.ntt_queue_status()  # the self-test's record is its own: nothing left over
    v = synth.fr_uniform(3500, 1 << 12)
    d = gpu_ctx.to_device(v)
    gpu_ctx.fr_to_mont(d, d, 1 << 12)
    gpu_ctx.ntt_batch_set_queue(True)
    try:
        gpu_ctx.ntt_batch([(0, d, d, 1 << 12, 12, _omega(12), 1)])
        gpu_ctx.ntt_queue_status()
    finally:
        gpu_ctx.ntt_batch_set_queue(False)
    assert (_download(gpu_ctx, d, 1 << 12) == _oracle_ntt(0, v, 12, 1)).all()


def test_ntt_tuned_splits_in_place_and_json(gpu_ctx, tmp_path):
    """A tuned radix split changes timing only: 3-pass in-place transforms, tuning file round trip."""
    try:
        gpu_ctx.tune_set_ntt_split(12, [4, 4, 4])
        gpu_ctx.tune_set_ntt_split(16, [11, 5])
        assert gpu_ctx.tune_ntt_split(12) == [4, 4, 4]
        assert gpu_ctx.tune_ntt_split(20) == [10, 10]  # the built-in split
        for log_n, mode, shift in ((12, 0, 1), (12, 3, 5), (16, 2, 5), (16, 1, 1)):
            n = 1 << log_n
            v = synth.fr_uniform(5000 + log_n + mode, n)
            d = gpu_ctx.to_device(v)
            gpu_ctx.fr_to_mont(d, d, n)
            gpu_ctx.ntt(mode, d, d, n, log_n, _omega(log_n), shift)  # in place
            assert (_download(gpu_ctx, d, n) == _oracle_ntt(mode, v, log_n, shift)).all(), (log_n, mode)
        gpu_ctx.tune_set_msm_window(14, 9)
        assert gpu_ctx.tune_msm_window(1 << 14) == 9
        assert gpu_ctx.tune_msm_window((1 << 13) + 1) == 9
        path = str(tmp_path / "tune.json")
        gpu_ctx.autotune_save(path)
        gpu_ctx.tune_set_ntt_split(12, [])
        gpu_ctx.tune_set_msm_window(14, 0)
        assert gpu_ctx.tune_ntt_split(12) == [6, 6]
        gpu_ctx.autotune_load(path)
        assert gpu_ctx.tune_ntt_split(12) == [4, 4, 4] and gpu_ctx.tune_msm_window(1 << 14) == 9
        with pytest.raises(ValueError):
            gpu_ctx.tune_set_ntt_split(12, [6, 5])  # does not sum to 12
        with pytest.raises(ValueError):
            gpu_ctx.tune_set_ntt_split(24, [12, 12])  # 12-bit passes exceed the 2^11 tile
        bad = tmp_path / "bad.json"
        bad.write_text('{"ntt_split": {"12": [6, 7]}}')
        with pytest.raises(ValueError):
            gpu_ctx.autotune_load(str(bad))
        assert gpu_ctx.tune_ntt_split(12) == [4, 4, 4]  # a rejected file changes nothing
    finally:
        gpu_ctx.tune_set_ntt_split(12, [])
        gpu_ctx.tune_set_ntt_split(16, [])
        gpu_ctx.tune_set_msm_window(14, 0)


def test_ntt_2_23_three_passes_in_place_round_trip(gpu_ctx):
    """n = 2^23 takes three passes by default: in place, forward then inverse gives the input back."""
    log_n = 23
    n = 1 << log_n
    v = synth.fr_uniform(6000, n)
    a = gpu_ctx.to_device(v)
    gpu_ctx.fr_to_mont(a, a, n)
    b = gpu_ctx.alloc(n * 32)
    gpu_ctx.ntt(2, b, a, n, log_n, _omega(log_n), 5)  # out of place
    gpu_ctx.ntt(2, a, a, n, log_n, _omega(log_n), 5)  # in place
    gpu_ctx.sync()
    assert np.array_equal(a.download(n * 32), b.download(n * 32))
    gpu_ctx.ntt(3, a, a, n, log_n, _omega(log_n), 5)
    assert (_download(gpu_ctx, a, n) == v).all()


def test_autotune_small_sizes(gpu_ctx):
    log_n = 14
    n = 1 << log_n
    try:
        d = gpu_ctx.to_device(synth.fr_uniform(7000, n))
        gpu_ctx.fr_to_mont(d, d, n)
        split, ms = gpu_ctx.autotune_ntt(d, log_n, reps=2)
        assert sum(split) == log_n and ms > 0 and gpu_ctx.tune_ntt_split(log_n) == split
        k, b = _bases(gpu_ctx, 7001, n)
        s = synth.fr_uniform(7002, n)
        ds = _upload(gpu_ctx, s)
        c, ms = gpu_ctx.autotune_msm(b, ds, log_n, reps=1)
        assert 4 <= c <= 20 and ms > 0 and gpu_ctx.tune_msm_window(n) == c
        assert gpu_ctx.msm_g1(b, ds, n) == _expect(k, s)
    finally:
        gpu_ctx.tune_set_ntt_split(log_n, [])
        gpu_ctx.tune_set_msm_window(log_n, 0)


def test_async_batches_match_sync(gpu_ctx):
    """zk_msm_g1_batch_submit / zk_msm_g2_batch_submit + zk_batch_wait: the same points as the
    synchronous batch calls, with two batches in flight at once, a time-limited wait, an
    empty batch, and other work enqueued on the context between submit and wait."""
    sizes = [3000, 0, 1, 4096, 777]
    k, b = _bases(gpu_ctx, 5150, max(sizes), zero_at=(2,))
    scal = [synth.fr_uniform(5151 + j, m) for j, m in enumerate(sizes)]
    dev = [_upload(gpu_ctx, s) for s in scal]
    exp = [_expect(k[:m], s) for m, s in zip(sizes, scal)]
    first = gpu_ctx.msm_batch_submit(b, dev, sizes)
    second = gpu_ctx.msm_batch_submit(b, dev[::-1], sizes[::-1])
    busy = gpu_ctx.alloc(64 << 20)  # unrelated work on the same stream
    gpu_ctx.memset(busy, 3)
    done = False
    for _ in range(2000):  # bounded polling with short waits
        try:
            got1 = first.wait(5)
            done = True
            break
        except TimeoutError:
            continue
    assert done
    assert got1 == exp
    assert second.wait() == exp[::-1]
    assert first.done() and second.done()
    first.destroy()
    second.destroy()
    empty = gpu_ctx.msm_batch_submit(b, [], [])
    assert empty.wait(0) == []
    empty.destroy()
    # G2
    n2 = 600
    k2 = synth.base_dlogs(5160, n2)
    b2 = gpu_ctx.bases_g2_from_host(O.g2_fixed_base_mul(O.G2_GENERATOR, k2))
    s2 = [synth.fr_uniform(5161, n2), synth.fr_uniform(5162, 250)]
    d2 = [_upload(gpu_ctx, s) for s in s2]
    g2 = gpu_ctx.msm_batch_submit(b2, d2, [n2, 250], g2=True)
    res = g2.wait()
    g2.destroy()
    for s, r in zip(s2, res):
        p = O.g2_msm_known_answer(k2[:s.shape[0]], s)
        assert r == (None if not p.any() else O.g2_to_ints(p))
