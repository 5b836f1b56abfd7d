"""Groth16 on the GB300: proving keys resident on the device, the QAP on the device, and
all of a batch's MSMs in one batched G1 call plus one batched G2 call.

Mirrors protocols/groth16 of the reference:
  * R1CS     -- the R1CSInstance of r1cs.py:25-36 (rows as sparse {var: coeff}, padded to
               n = 2^k constraints, the constant ONE at one_id = n_vars - 1, public ids
               first) held as three CSR matrices.
  * setup    -- setup.py:25-121 for given trapdoors (tau, alpha, beta, gamma, delta).
               Instead of interpolating every variable's column (O(vars n log n)), the
               Lagrange basis at tau is one inverse NTT of the powers of tau
               (L_j(tau) = n^-1 sum_k tau^k omega^(-jk)), and the column values are one
               sparse transposed product A^T L. Same exponents, hence the same points.
  * prove    -- prove.py:30-126 / prove_batch (:133-246) for given (r, s): A w, B w, C w
               (r1cs.py:84-92), the quotient H of qap.py:53-101 computed on the coset
               5 <omega>, and the MSMs a_query w, b_query_g1 w, b_query_g2 w, l_query aux,
               h_query h; the proof A, B, C assembled exactly as prove.py:87-124.
  * verifying key and proof -- types.py:9-41.
Query points that are infinity (a variable absent from A or B) are dropped from the
resident bases together with their scalars: every MSM keeps the same value.
"""

from __future__ import annotations

import random
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import _native as N
from .synth import FR_MODULUS, int_to_limbs, ints_to_limbs, limbs_to_ints  # noqa: F401

G1_GEN = (1, 2)
# crypto/ecc/bn254.py G2_GENERATOR (py_ecc G2): x = x0 + x1 u, y = y0 + y1 u
G2_GEN = ((10857046999023057135944570762232829481370756359578518086990519993285655852781,
           11559732032986387107991004021392285783925812861821192530917403151452391805634),
          (8495653923123431417604973247489272438418190587263600148770280649306958101930,
           4082367875863433681332203403145435568316851327593401208105741076214120093531))
ROOT_2_28 = 19103219067921713944291392827692070036145651957329286315305642004821462161904  # crypto/poly/ntt.py:8
COSET_SHIFT = 5

MODE_EVALS, MODE_COEFFS, MODE_COSET_EVALS, MODE_COSET_COEFFS = 0, 1, 2, 3


def omega_for_size(n: int) -> int:
    """crypto/poly/ntt.py:13-24."""
    if n <= 0 or n & (n - 1):
        raise ValueError("n must be a power of two")
    logn = n.bit_length() - 1
    if logn > 28:
        raise ValueError("domain too large for BN254 root of unity")
    return pow(ROOT_2_28, 1 << (28 - logn), FR_MODULUS)


# ------------------------------------------------------------------------------------ R1CS
@dataclass
class CSR:
    row_ptr: np.ndarray  # uint32, rows + 1
    cols: np.ndarray     # uint32
    vals: np.ndarray     # uint64[nnz, 4] canonical Fr

    @staticmethod
    def from_rows(rows: Sequence[Dict[int, int]]) -> "CSR":
        ptr, cols, vals = [0], [], []
        for row in rows:
            for k in sorted(row):
                v = int(row[k]) % FR_MODULUS
                if v:
                    cols.append(int(k))
                    vals.append(v)
            ptr.append(len(cols))
        return CSR(np.array(ptr, dtype=np.uint32), np.array(cols, dtype=np.uint32), ints_to_limbs(vals))

    def transpose(self, ncols: int) -> "CSR":
        """Column-major view: row i of the result lists (constraint j, coefficient)."""
        rows = np.repeat(np.arange(len(self.row_ptr) - 1, dtype=np.uint32), np.diff(self.row_ptr))
        order = np.argsort(self.cols, kind="stable")
        counts = np.bincount(self.cols, minlength=ncols) if len(self.cols) else np.zeros(ncols, np.int64)
        ptr = np.zeros(ncols + 1, dtype=np.uint32)
        np.cumsum(counts, out=ptr[1:])
        return CSR(ptr, rows[order].astype(np.uint32), self.vals[order])


@dataclass
class R1CS:
    """protocols/groth16/r1cs.py:25-36."""

    n: int
    n_vars: int
    one_id: int
    public_ids: List[int]
    aux_ids: List[int]
    a: CSR
    b: CSR
    c: CSR

    @staticmethod
    def from_rows(n: int, n_vars: int, one_id: int, public_ids, aux_ids, a_rows, b_rows, c_rows) -> "R1CS":
        if n & (n - 1) or len(a_rows) != n or len(b_rows) != n or len(c_rows) != n:
            raise ValueError("R1CS rows must be padded to a power of two")
        return R1CS(n, n_vars, one_id, list(public_ids), list(aux_ids), CSR.from_rows(a_rows),
                    CSR.from_rows(b_rows), CSR.from_rows(c_rows))

    @staticmethod
    def from_reference(inst) -> "R1CS":
        """From the reference's R1CSInstance (compile_r1cs, r1cs.py:39-81)."""
        return R1CS.from_rows(inst.n_constraints, inst.n_vars, inst.one_id, inst.public_ids, inst.aux_ids,
                              inst.a_rows, inst.b_rows, inst.c_rows)


def diagonal_r1cs(m: int) -> R1CS:
    """Synthetic circuit of m constraints x_i * y_i = z_i (padded to n = 2^ceil(log2 m)), with
    the variable layout of compile_r1cs: the public z_0 first (id 0), then x_0..x_{m-1},
    y_0..y_{m-1}, z_1..z_{m-1}, and ONE last. A w and B w are the x and y values, C w their
    products."""
    if m < 1:
        raise ValueError("m must be positive")
    n = 1 << (m - 1).bit_length()
    x0, y0, z1 = 1, 1 + m, 1 + 2 * m
    one_id = 3 * m
    zid = np.concatenate([[0], z1 + np.arange(m - 1)]).astype(np.uint32)
    ptr = np.zeros(n + 1, dtype=np.uint32)
    ptr[1:m + 1] = np.arange(1, m + 1, dtype=np.uint32)
    ptr[m + 1:] = m
    ones = np.zeros((m, 4), dtype=np.uint64)
    ones[:, 0] = 1
    a = CSR(ptr, (x0 + np.arange(m)).astype(np.uint32), ones)
    b = CSR(ptr.copy(), (y0 + np.arange(m)).astype(np.uint32), ones.copy())
    c = CSR(ptr.copy(), zid, ones.copy())
    return R1CS(n, one_id + 1, one_id, [one_id, 0], list(range(1, one_id)), a, b, c)


def diagonal_witness(ctx: N.Context, m: int, seed: int) -> Tuple[np.ndarray, List[int]]:
    """Witness of diagonal_r1cs(m) (seeded uniform x, y; z = x y computed on the device), as
    canonical limbs with the trailing ONE, and the public values [1, z_0] of verify.py."""
    from .synth import fr_uniform

    x = fr_uniform(seed, m)
    y = fr_uniform(seed ^ 0x5A5A5A5A, m)
    dx, dy = ctx.to_device(x), ctx.to_device(y)
    ctx.fr_to_mont(dx, dx, m)
    ctx.fr_to_mont(dy, dy, m)
    ctx.fr_mul(dx, dx, dy, m)
    ctx.fr_from_mont(dx, dx, m)
    z = dx.download(m * 32).view("<u8").reshape(m, 4).astype(np.uint64)
    one = np.array([[1, 0, 0, 0]], dtype=np.uint64)
    w = np.concatenate([z[:1], x, y, z[1:], one])
    return w, [1, limbs_to_ints(z[:1])[0]]


# ------------------------------------------------------------------------------------ keys
@dataclass
class Trapdoors:
    tau: int
    alpha: int
    beta: int
    gamma: int
    delta: int

    @staticmethod
    def seeded(seed: int) -> "Trapdoors":
        rng = random.Random(seed)
        return Trapdoors(*[rng.randrange(1, FR_MODULUS) for _ in range(5)])


@dataclass
class VerifyingKey:
    """types.py:18-24."""

    alpha_g1: tuple
    beta_g2: tuple
    gamma_g2: tuple
    delta_g2: tuple
    ic: List[Optional[tuple]]


@dataclass
class Proof:
    """types.py:9-13: A, C in G1 and B in G2 as canonical affine ints (None = infinity)."""

    a: Optional[tuple]
    b: Optional[tuple]
    c: Optional[tuple]


@dataclass
class Query:
    """One resident MSM base set: the points whose exponent is non-zero, and the variable
    (or coefficient) index each one multiplies."""

    bases: Optional[N.Bases]
    idx: Optional[N.DeviceArray]  # uint32 device indices, None when the set is the identity map
    count: int
    rows_bytes: int = 0  # fixed-base rows of the G1 bases (zk_bases_precompute), if built


@dataclass
class DeviceKey:
    """A proving key (types.py:26-41) resident on the device."""

    r1cs: R1CS
    vk: VerifyingKey
    beta_g1: tuple
    delta_g1: tuple
    a: Query
    b1: Query
    b2: Query
    l: Query
    h: Query
    mats: Tuple[tuple, tuple, tuple]  # device CSR (row_ptr, cols, coeffs Montgomery) of A, B, C
    exps: Dict[str, np.ndarray] = field(default_factory=dict)  # canonical exponents (kept on request)

    @property
    def n(self) -> int:
        return self.r1cs.n

    def device_bytes(self) -> int:
        qs = (self.a, self.b1, self.l, self.h)
        g1 = sum(q.count for q in qs) * 128 + sum(q.rows_bytes for q in qs)  # points + GLV images, rows
        g2 = self.b2.count * 256 + self.b2.rows_bytes
        return g1 + g2 + 4 * (self.a.count + self.b1.count + self.l.count)


def _upload_csr(ctx: N.Context, m: CSR):
    nnz = len(m.cols)
    ptr = ctx.to_device(m.row_ptr.astype(np.uint32))
    cols = ctx.to_device(m.cols.astype(np.uint32) if nnz else np.zeros(1, np.uint32))
    vals = ctx.to_device(m.vals if nnz else np.zeros((1, 4), np.uint64))
    if nnz:
        ctx.fr_to_mont(vals, vals, nnz)
    return ptr, cols, vals


def _download_fr(ctx: N.Context, d, n: int) -> np.ndarray:
    """Montgomery device vector -> canonical uint64[n, 4] (the device copy is left as is)."""
    tmp = ctx.alloc(max(1, n) * 32)
    if n:
        ctx.fr_from_mont(tmp, d, n)
    return tmp.download(n * 32).view("<u8").reshape(n, 4).astype(np.uint64)


def _points(ctx: N.Context, exps: np.ndarray, g2: bool) -> N.DeviceArray:
    """[e_i] G (canonical affine, device) for canonical exponents e_i (host limbs)."""
    n = exps.shape[0]
    dk = ctx.to_device(exps if n else np.zeros((1, 4), np.uint64))
    out = ctx.alloc(max(1, n) * (128 if g2 else 64))
    if n:
        if g2:
            ctx.g2_fixed_base_mul(G2_GEN, dk, n, out)
        else:
            ctx.g1_fixed_base_mul(G1_GEN, dk, n, out)
    return out


def _query(ctx: N.Context, exps: np.ndarray, g2: bool = False, identity: bool = False) -> Query:
    nz = np.nonzero(exps.any(axis=1))[0].astype(np.uint32)
    if identity and len(nz) == exps.shape[0]:
        idx = None
    else:
        identity = False
        idx = ctx.to_device(nz if len(nz) else np.zeros(1, np.uint32))
    pts = _points(ctx, exps[nz], g2)
    count = int(len(nz))
    bases = None
    if count:
        bases = ctx.bases_g2_from_device(pts, count) if g2 else ctx.bases_from_device(pts, count)
    return Query(bases, idx, count)


def _precompute(ctx: N.Context, q: Query, g2: bool = False) -> None:
    """Fixed-base rows for a query's bases (the reference's fixed_base_precompute policy for
    proving keys, runtime/warmup.py:125-150): every later MSM on them runs in fixed-base mode."""
    from .plugin import fixed_base_window

    if q.count:
        c = fixed_base_window(q.count)
        ctx.bases_precompute(q.bases, c)
        q.rows_bytes = -(-255 // c) * q.count * (128 if g2 else 64)


def setup(ctx: N.Context, r1cs: R1CS, td: Trapdoors, keep_exponents: bool = False,
          fixed_base: bool = True) -> DeviceKey:
    """The proving key of protocols/groth16/setup.py:25-121 for the trapdoors `td`. With
    fixed_base, the query bases (G1 and G2) also get their window-shifted rows (same proofs,
    faster MSMs)."""
    n, nv = r1cs.n, r1cs.n_vars
    log_n = n.bit_length() - 1
    t_tau = (pow(td.tau, n, FR_MODULUS) - 1) % FR_MODULUS
    if t_tau == 0:
        raise ValueError("tau lies in the evaluation domain")
    # L_j(tau) = iNTT(tau^0 .. tau^(n-1))_j
    pw = ctx.alloc(n * 32)
    ctx.fr_powers(pw, td.tau, n)
    lag = ctx.alloc(n * 32)
    ctx.ntt(MODE_COEFFS, lag, pw, n, log_n, omega_for_size(n))
    # column values u^A = A^T L, u^B = B^T L, and k = beta u^A + alpha u^B + u^C
    u = {}
    for name, m in (("a", r1cs.a), ("b", r1cs.b), ("c", r1cs.c)):
        t = _upload_csr(ctx, m.transpose(nv))
        out = ctx.alloc(nv * 32)
        ctx.fr_spmv(nv, t[0], t[1], t[2], lag, out)
        u[name] = out
    k = ctx.alloc(nv * 32)
    tmp = ctx.alloc(nv * 32)
    ctx.fr_scale(k, u["a"], td.beta, nv)
    ctx.fr_scale(tmp, u["b"], td.alpha, nv)
    ctx.fr_add(k, k, tmp, nv)
    ctx.fr_add(k, k, u["c"], nv)
    inv_g, inv_d = pow(td.gamma, FR_MODULUS - 2, FR_MODULUS), pow(td.delta, FR_MODULUS - 2, FR_MODULUS)
    ua = _download_fr(ctx, u["a"], nv)
    ub = _download_fr(ctx, u["b"], nv)
    # ic = k / gamma on the public ids, l_query = k / delta on the aux ids
    ctx.fr_scale(tmp, k, inv_g, nv)
    ic_exp = limbs_to_ints(_download_fr(ctx, tmp, nv)[np.asarray(r1cs.public_ids, dtype=np.int64)])
    ctx.fr_scale(tmp, k, inv_d, nv)
    l_exp = _download_fr(ctx, tmp, nv)[np.asarray(r1cs.aux_ids, dtype=np.int64)]
    # h_query[k] = tau^k (tau^n - 1) / delta, k < n - 1
    hs = ctx.alloc(n * 32)
    ctx.fr_scale(hs, pw, t_tau * inv_d % FR_MODULUS, n)
    h_exp = _download_fr(ctx, hs, n)[: n - 1]

    a_q = _query(ctx, ua)
    b1_q = _query(ctx, ub)
    b2_q = _query(ctx, ub, g2=True)
    l_q = _query(ctx, l_exp)
    # the l scalars are w[aux_ids[i]]: fold the aux map into the index list
    if l_q.count:
        nz = np.nonzero(l_exp.any(axis=1))[0]
        l_q.idx = ctx.to_device(np.asarray(r1cs.aux_ids, dtype=np.uint32)[nz])
    h_q = _query(ctx, h_exp, identity=True)

    vk = VerifyingKey(
        alpha_g1=N.host_g1_mul(G1_GEN, td.alpha),
        beta_g2=N.host_g2_mul(G2_GEN, td.beta),
        gamma_g2=N.host_g2_mul(G2_GEN, td.gamma),
        delta_g2=N.host_g2_mul(G2_GEN, td.delta),
        ic=[N.host_g1_mul(G1_GEN, e) for e in ic_exp],
    )
    key = DeviceKey(r1cs=r1cs, vk=vk, beta_g1=N.host_g1_mul(G1_GEN, td.beta),
                    delta_g1=N.host_g1_mul(G1_GEN, td.delta), a=a_q, b1=b1_q, b2=b2_q, l=l_q, h=h_q,
                    mats=(_upload_csr(ctx, r1cs.a), _upload_csr(ctx, r1cs.b), _upload_csr(ctx, r1cs.c)))
    if keep_exponents:
        key.exps = {"a": ua, "b": ub, "l": l_exp, "h": h_exp, "ic": ints_to_limbs(ic_exp)}
    if fixed_base:
        for q in (a_q, b1_q, l_q, h_q):
            _precompute(ctx, q)
        _precompute(ctx, b2_q, g2=True)
    ctx.sync()
    return key


def query_points(ctx: N.Context, key: DeviceKey) -> Dict[str, list]:
    """The full query lists of the key (a_query, b_query_g1, b_query_g2, l_query, h_query) as
    canonical affine ints, from the exponents kept by setup(..., keep_exponents=True); for
    comparisons with the reference's ProvingKey."""
    if not key.exps:
        raise ValueError("setup(..., keep_exponents=True) keeps the exponents")
    out = {}
    for name, e, g2 in (("a_query", key.exps["a"], False), ("b_query_g1", key.exps["b"], False),
                        ("b_query_g2", key.exps["b"], True), ("l_query", key.exps["l"], False),
                        ("h_query", key.exps["h"], False)):
        n = e.shape[0]
        if n == 0:
            out[name] = []
            continue
        raw = _points(ctx, e, g2).download(n * (128 if g2 else 64)).view("<u8").reshape(n, 16 if g2 else 8)
        pts = []
        for row in raw:
            v = limbs_to_ints(row.reshape(-1, 4))
            if not any(v):
                pts.append(None)
            else:
                pts.append(((v[0], v[1]), (v[2], v[3])) if g2 else (v[0], v[1]))
        out[name] = pts
    return out


# ------------------------------------------------------------------------------------ prover
@dataclass
class Request:
    key: DeviceKey
    witness: np.ndarray  # canonical uint64[n_vars, 4], ONE last (prove.py:49-53)
    r: int
    s: int


class PendingProofs:
    """Requests whose device work is enqueued (``Prover.submit``). ``done()`` asks whether the
    device has finished it; ``results()`` waits and returns, per request in order, its Proof
    or the exception that failed that request alone (an unsatisfied witness or a bad
    argument fails its own request, never the others of the batch).

    ``results()`` = ``finish_device()`` (on the thread that uses the context: collects the
    MSM values and releases the device buffers) + ``finish_host()`` (the proof assembly,
    host-only, any thread)."""

    def __init__(self, prover: "Prover", ctx: N.Context, live, errors, g1_job, g2_job, bad_host, fence,
                 buffers) -> None:
        self._prover, self._ctx = prover, ctx
        self._live, self._errors = live, errors
        self._g1_job, self._g2_job = g1_job, g2_job
        self._bad_host, self._fence, self._buffers = bad_host, fence, buffers
        self._g1 = self._g2 = self._bad = None
        self._device_done = False
        self._results: Optional[list] = None

    def __len__(self) -> int:
        return len(self._errors)

    def done(self) -> bool:
        return self._device_done or self._fence.done()

    def finish_device(self) -> None:
        if self._device_done:
            return
        try:
            self._fence.wait()
            self._g1 = Prover._collect(self._g1_job, 4 * len(self._live))
            self._g2 = Prover._collect(self._g2_job, len(self._live))
            if self._bad_host is not None:
                self._bad = self._bad_host.array[:8 * len(self._live)].view(np.uint64).copy()
        finally:
            for b in self._buffers:
                b.free()
            self._buffers = []
            self._fence.destroy()
            if self._bad_host is not None:
                self._prover._give_pinned(self._bad_host)
                self._bad_host = None
            self._device_done = True

    def finish_host(self) -> list:
        if self._results is not None:
            return self._results
        g1, g2, bad = self._g1, self._g2, self._bad
        out = list(self._errors)

        def one(i):
            q = self._live[i][0]
            if bad is not None and int(bad[i]) != 0:
                return ValueError("witness does not satisfy R1CS (non-zero remainder)")
            a_lin, b_lin_g1, l_acc, h_acc = g1[4 * i:4 * i + 4]
            try:
                return assemble(q.key, a_lin, b_lin_g1, g2[i], l_acc, h_acc, q.r, q.s)
            except Exception as e:  # noqa: BLE001 -- the request's own failure
                return e

        # host scalar multiplications release the GIL inside the library: assemble in parallel
        n = len(self._live)
        proofs = list(Prover._pool().map(one, range(n))) if n > 1 else [one(i) for i in range(n)]
        for (_, _, _, slot), pr in zip(self._live, proofs):
            out[slot] = pr
        self._results = out
        return out

    def results(self) -> list:
        self.finish_device()
        return self.finish_host()


def pin_witness(witness: np.ndarray) -> np.ndarray:
    """A page-locked copy of a witness (canonical uint64[n_vars, 4]): ``Prover.submit`` then
    uploads it without waiting for earlier device work."""
    return N.pinned_copy(np.ascontiguousarray(witness, dtype=np.uint64).reshape(-1, 4))


class Prover:
    """Groth16 proofs on the device, one at a time or a batch per call (prove / prove_batch of
    protocols/groth16/prove.py with the randomness passed in), or asynchronously (``submit``)."""

    def __init__(self, ctx: N.Context) -> None:
        import threading

        self.ctx = ctx
        self._pinned: List[N.PinnedBuffer] = []  # small page-locked buffers for reuse
        self._pinned_lock = threading.Lock()

    def _take_pinned(self, nbytes: int) -> N.PinnedBuffer:
        """A page-locked buffer of at least nbytes (allocating page-locked memory per batch can
        wait for the whole device, so buffers are kept and reused)."""
        with self._pinned_lock:
            for i, b in enumerate(self._pinned):
                if b.nbytes >= nbytes:
                    return self._pinned.pop(i)
        return N.PinnedBuffer(max(nbytes, 4096))

    def _give_pinned(self, buf: N.PinnedBuffer) -> None:
        with self._pinned_lock:
            self._pinned.append(buf)

    def prove(self, key: DeviceKey, witness: np.ndarray, r: int, s: int) -> Proof:
        return self.prove_batch([Request(key, witness, r, s)])[0]

    def prove_batch(self, reqs: Sequence[Request]) -> List[Proof]:
        """All proofs of ``reqs``; raises the first request's error (as the reference's
        prove_batch raises for an unsatisfied witness, qap.py:98-99)."""
        res = self.submit(reqs).results()
        for r in res:
            if isinstance(r, Exception):
                raise r
        return res

    def submit(self, reqs: Sequence[Request], ctx: Optional[N.Context] = None) -> PendingProofs:
        """Enqueue the device work of ``reqs`` on ``ctx`` (default: the prover's context) and
        return at once: R1CS rows A w, B w, C w, the satisfiability count (read back with the
        results, so that nothing here waits for the device), the QAP transforms, the MSM
        scalar gathers, and one asynchronous G1 and one G2 MSM batch. Witnesses made by
        ``pin_witness`` are uploaded without waiting; others with a blocking copy."""
        ctx = ctx or self.ctx
        live, errors, buffers = [], [None] * len(reqs), []
        for slot, q in enumerate(reqs):
            k = q.key
            w = q.witness
            pinned = (isinstance(w, N.PinnedArray) and w.flags.c_contiguous and w.dtype == np.uint64
                      and w.ndim == 2 and w.shape[1] == 4)
            if not pinned:
                w = np.ascontiguousarray(w, dtype=np.uint64).reshape(-1, 4)
            if w.shape[0] != k.r1cs.n_vars:
                errors[slot] = ValueError("witness length mismatch")
                continue
            n = k.n
            wd = ctx.alloc(w.shape[0] * 32)
            buffers.append(wd)
            if pinned:
                ctx.h2d_async(wd, w)
            else:
                wd.upload(w)
            ctx.fr_to_mont(wd, wd, w.shape[0])
            ev = [ctx.alloc(n * 32) for _ in range(3)]
            buffers.extend(ev)
            for mat, out in zip(k.mats, ev):
                ctx.fr_spmv(n, mat[0], mat[1], mat[2], wd, out)
            live.append((q, wd, ev, slot))
        if not live:
            return PendingProofs(self, ctx, [], errors, ([], None), ([], None), None, ctx.fence(), buffers)
        # the remainder of (A B - C) / (X^n - 1) is empty iff A B == C on the domain: one
        # counter per request, read back with the results
        bad_dev = ctx.alloc(8 * len(live))
        buffers.append(bad_dev)
        ctx.memset(bad_dev, 0)
        for i, (q, _, ev, _) in enumerate(live):
            ctx.fr_r1cs_check_async(ev[0], ev[1], ev[2], q.key.n, bad_dev.ptr + 8 * i)
        bad_host = self._take_pinned(8 * len(live))
        ctx.d2h_async(bad_host.array[:8 * len(live)], bad_dev)
        # H = coset_iNTT((A B - C)(5 w^i) / (5^n - 1)), every transform in place, batched
        jobs1, jobs2, jobs3 = [], [], []
        for q, _, ev, _ in live:
            n = q.key.n
            lg, om = n.bit_length() - 1, omega_for_size(n)
            for e in ev:
                jobs1.append((MODE_COEFFS, e, e, n, lg, om, 1))
                jobs2.append((MODE_COSET_EVALS, e, e, n, lg, om, COSET_SHIFT))
            jobs3.append((MODE_COSET_COEFFS, ev[0], ev[0], n, lg, om, COSET_SHIFT))
        ctx.ntt_batch(jobs1)
        ctx.ntt_batch(jobs2)
        for q, _, ev, _ in live:
            n = q.key.n
            zinv = pow((pow(COSET_SHIFT, n, FR_MODULUS) - 1) % FR_MODULUS, FR_MODULUS - 2, FR_MODULUS)
            ctx.fr_qap_quotient(ev[0], ev[0], ev[1], ev[2], n, zinv)
        ctx.ntt_batch(jobs3)
        # MSM scalars: w gathered by each resident base set's index list; h = ev[0][:n-1]
        g1_bases, g1_sc, g1_n, g2_bases, g2_sc, g2_n = [], [], [], [], [], []
        for q, wd, ev, _ in live:
            k = q.key
            sc = {}
            for name, qu in (("a", k.a), ("b", k.b1), ("l", k.l)):
                d = ctx.alloc(max(1, qu.count) * 32)
                buffers.append(d)
                if qu.count:
                    ctx.fr_gather(d, wd, qu.idx, qu.count)
                sc[name] = d
            for qu, d in ((k.a, sc["a"]), (k.b1, sc["b"]), (k.l, sc["l"]), (k.h, ev[0])):
                g1_bases.append(qu.bases)
                g1_sc.append(d)
                g1_n.append(qu.count)
            g2_bases.append(k.b2.bases)
            g2_sc.append(sc["b"])  # b_query_g2 and b_query_g1 share their non-zero pattern
            g2_n.append(k.b2.count)
        # both batches in flight: the G1 windows are combined on the host while the G2 MSMs run
        g1_job = self._submit(ctx, g1_bases, g1_sc, g1_n, g2=False)
        g2_job = self._submit(ctx, g2_bases, g2_sc, g2_n, g2=True)
        return PendingProofs(self, ctx, live, errors, g1_job, g2_job, bad_host, ctx.fence(), buffers)

    _executor = None

    @classmethod
    def _pool(cls):
        if cls._executor is None:
            import concurrent.futures
            import os

            cls._executor = concurrent.futures.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1))
        return cls._executor

    @staticmethod
    def _submit(ctx, bases, scalars, sizes, g2: bool):
        """Submit one asynchronous batched MSM over the non-empty instances."""
        sel = [i for i, m in enumerate(sizes) if m]
        if not sel:
            return sel, None
        return sel, ctx.msm_batch_submit([bases[i] for i in sel], [scalars[i] for i in sel],
                                         [sizes[i] for i in sel], g2=g2)

    @staticmethod
    def _collect(job, count: int):
        """Results of _submit in instance order (an empty instance is the identity)."""
        sel, batch = job
        out: List[Optional[tuple]] = [None] * count
        if batch is not None:
            try:
                for i, v in zip(sel, batch.wait()):
                    out[i] = v
            finally:
                batch.destroy()
        return out


def assemble(key: DeviceKey, a_lin, b_lin_g1, b_lin_g2, l_acc, h_acc, r: int, s: int) -> Proof:
    """prove.py:87-88 and :118-124."""
    vk = key.vk
    a = N.host_g1_add(vk.alpha_g1, N.host_g1_add(a_lin, N.host_g1_mul(key.delta_g1, r)))
    b = N.host_g2_add(vk.beta_g2, N.host_g2_add(b_lin_g2, N.host_g2_mul(vk.delta_g2, s)))
    sa = N.host_g1_mul(N.host_g1_add(vk.alpha_g1, a_lin), s)
    rb = N.host_g1_mul(N.host_g1_add(key.beta_g1, b_lin_g1), r)
    rs_delta = N.host_g1_mul(key.delta_g1, r * s % FR_MODULUS)
    c = N.host_g1_add(N.host_g1_add(l_acc, h_acc), N.host_g1_add(N.host_g1_add(sa, rb), rs_delta))
    return Proof(a=a, b=b, c=c)


__all__ = ["R1CS", "CSR", "diagonal_r1cs", "diagonal_witness", "Trapdoors", "VerifyingKey", "Proof", "DeviceKey",
           "setup", "query_points", "Request", "Prover", "PendingProofs", "pin_witness", "assemble", "omega_for_size",
           "int_to_limbs"]
