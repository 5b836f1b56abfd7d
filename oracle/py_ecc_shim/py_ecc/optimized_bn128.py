"""BN254 (alt_bn128) curve arithmetic and optimal-ate pairing — test-only stand-in.

ORACLE / TEST INFRASTRUCTURE. Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import this module.

It provides exactly the ``py_ecc.optimized_bn128`` surface that the reference uses:

* ``curve_order`` (crypto/field/fr.py:7), ``field_modulus``
* ``FQ`` with ``+ - * /``, ``==``, ``int()``, ``FQ(x)`` (runtime/metal/msm.py:37,63), ``FQ2``, ``FQ12``
  with ``one()``, ``*``, ``==`` (crypto/pairing/bn254.py:15-17)
* ``G1`` = (1, 2), ``G2``, ``Z1``, ``Z2`` (crypto/ecc/bn254.py:51-54)
* ``add``, ``double``, ``neg``, ``multiply``, ``normalize``, ``eq``, ``is_on_curve``
  (crypto/ecc/bn254.py:9-48, plonk/transcript.py:18)
* ``pairing(Q_G2, P_G1)`` (crypto/pairing/bn254.py:11)

Points are 3-tuples in Jacobian coordinates (x = X/Z^2, y = Y/Z^3); the point at
infinity has Z == 0 (runtime/metal/msm.py:18 tests ``p[2] == 0``).  ``normalize``
returns the affine pair; the point at infinity normalises to (0, 0).

Everything here is written from the curve's definition: y^2 = x^3 + 3 over
F_q, the sextic D-twist y^2 = x^3 + 3/(9+u) over F_q2 = F_q[u]/(u^2+1), the
tower-free field F_q12 = F_q[w]/(w^12 - 18 w^6 + 82) (w^6 = 9 + u), and the
optimal ate pairing with loop parameter 6x+2, x = 4965661367192848881.
"""

from __future__ import annotations

from typing import List, Sequence, Tuple, Union

field_modulus = 21888242871839275222246405745257275088696311157297823662689037894645226208583
curve_order = 21888242871839275222246405745257275088548364400416034343698204186575808495617

_Q = field_modulus
_R = curve_order


def _inv(a: int) -> int:
    a %= _Q
    if a == 0:
        return 0  # convention: inverse of zero is zero (normalize(inf) -> (0, 0))
    return pow(a, _Q - 2, _Q)


IntLike = Union[int, "FQ"]


class FQ:
    """Element of the BN254 base field F_q."""

    __slots__ = ("n",)
    field_modulus = _Q

    def __init__(self, val) -> None:
        if isinstance(val, FQ):
            self.n = val.n
        else:
            self.n = int(val) % _Q

    @staticmethod
    def _v(o) -> int:
        return o.n if isinstance(o, FQ) else int(o)

    def __add__(self, o):
        if isinstance(o, (FQ2, FQ12)):
            return o + self
        return FQ(self.n + FQ._v(o))

    __radd__ = __add__

    def __sub__(self, o):
        if isinstance(o, (FQ2, FQ12)):
            return (-o) + self
        return FQ(self.n - FQ._v(o))

    def __rsub__(self, o):
        return FQ(FQ._v(o) - self.n)

    def __mul__(self, o):
        if isinstance(o, (FQ2, FQ12)):
            return o * self
        return FQ(self.n * FQ._v(o))

    __rmul__ = __mul__

    def __truediv__(self, o):
        return FQ(self.n * _inv(FQ._v(o)))

    __div__ = __truediv__

    def __rtruediv__(self, o):
        return FQ(FQ._v(o) * _inv(self.n))

    def __pow__(self, e: int):
        return FQ(pow(self.n, int(e), _Q))

    def __neg__(self):
        return FQ(-self.n)

    def __eq__(self, o) -> bool:
        if isinstance(o, FQ):
            return self.n == o.n
        if isinstance(o, int):
            return self.n == o % _Q
        return NotImplemented

    def __ne__(self, o) -> bool:
        r = self.__eq__(o)
        return r if r is NotImplemented else not r

    def __hash__(self) -> int:
        return hash(("FQ", self.n))

    def __int__(self) -> int:
        return self.n

    def __index__(self) -> int:
        return self.n

    def __repr__(self) -> str:
        return repr(self.n)

    @classmethod
    def one(cls) -> "FQ":
        return cls(1)

    @classmethod
    def zero(cls) -> "FQ":
        return cls(0)


class FQ2:
    """Element c0 + c1*u of F_q2 = F_q[u]/(u^2 + 1)."""

    __slots__ = ("coeffs",)
    degree = 2

    def __init__(self, coeffs: Sequence) -> None:
        c0, c1 = coeffs
        self.coeffs = (int(c0) % _Q, int(c1) % _Q)

    def _o(self, o) -> Tuple[int, int]:
        if isinstance(o, FQ2):
            return o.coeffs
        if isinstance(o, FQ):
            return (o.n, 0)
        return (int(o) % _Q, 0)

    def __add__(self, o):
        a0, a1 = self.coeffs
        b0, b1 = self._o(o)
        return FQ2((a0 + b0, a1 + b1))

    __radd__ = __add__

    def __sub__(self, o):
        a0, a1 = self.coeffs
        b0, b1 = self._o(o)
        return FQ2((a0 - b0, a1 - b1))

    def __rsub__(self, o):
        return (-self) + o

    def __mul__(self, o):
        a0, a1 = self.coeffs
        if isinstance(o, FQ2):
            b0, b1 = o.coeffs
            return FQ2((a0 * b0 - a1 * b1, a0 * b1 + a1 * b0))
        k = o.n if isinstance(o, FQ) else int(o)
        return FQ2((a0 * k, a1 * k))

    __rmul__ = __mul__

    def inv(self) -> "FQ2":
        a0, a1 = self.coeffs
        d = _inv(a0 * a0 + a1 * a1)
        return FQ2((a0 * d, -a1 * d))

    def __truediv__(self, o):
        if isinstance(o, FQ2):
            return self * o.inv()
        return self * _inv(o.n if isinstance(o, FQ) else int(o))

    __div__ = __truediv__

    def __rtruediv__(self, o):
        return self.inv() * o

    def __pow__(self, e: int):
        e = int(e)
        result = FQ2.one()
        base = self
        while e > 0:
            if e & 1:
                result = result * base
            base = base * base
            e >>= 1
        return result

    def __neg__(self):
        a0, a1 = self.coeffs
        return FQ2((-a0, -a1))

    def conj(self) -> "FQ2":
        """The q-power Frobenius of F_q2 (u -> -u)."""
        a0, a1 = self.coeffs
        return FQ2((a0, -a1))

    def __eq__(self, o) -> bool:
        if isinstance(o, FQ2):
            return self.coeffs == o.coeffs
        if isinstance(o, (FQ, int)):
            return self.coeffs == self._o(o)
        return NotImplemented

    def __ne__(self, o) -> bool:
        r = self.__eq__(o)
        return r if r is NotImplemented else not r

    def __hash__(self) -> int:
        return hash(("FQ2",) + self.coeffs)

    def __repr__(self) -> str:
        return f"FQ2({list(self.coeffs)})"

    @classmethod
    def one(cls) -> "FQ2":
        return cls((1, 0))

    @classmethod
    def zero(cls) -> "FQ2":
        return cls((0, 0))


# F_q12 = F_q[w] / (w^12 - 18 w^6 + 82): w^12 = 18 w^6 - 82.
_FQ12_MOD = [82, 0, 0, 0, 0, 0, -18, 0, 0, 0, 0, 0]  # low coefficients of the monic modulus


class FQ12:
    """Element sum_i c_i w^i of F_q12 in the polynomial basis (w^6 = 9 + u)."""

    __slots__ = ("coeffs",)
    degree = 12

    def __init__(self, coeffs: Sequence) -> None:
        if len(coeffs) != 12:
            raise ValueError("FQ12 needs 12 coefficients")
        self.coeffs = tuple(int(c) % _Q for c in coeffs)

    @classmethod
    def one(cls) -> "FQ12":
        return cls([1] + [0] * 11)

    @classmethod
    def zero(cls) -> "FQ12":
        return cls([0] * 12)

    def __add__(self, o):
        if isinstance(o, FQ12):
            return FQ12([a + b for a, b in zip(self.coeffs, o.coeffs)])
        k = o.n if isinstance(o, FQ) else int(o)
        c = list(self.coeffs)
        c[0] += k
        return FQ12(c)

    __radd__ = __add__

    def __neg__(self):
        return FQ12([-a for a in self.coeffs])

    def __sub__(self, o):
        return self + (-o if isinstance(o, FQ12) else -(o.n if isinstance(o, FQ) else int(o)))

    def __rsub__(self, o):
        return (-self) + o

    def __mul__(self, o):
        if not isinstance(o, FQ12):
            k = o.n if isinstance(o, FQ) else int(o)
            return FQ12([a * k for a in self.coeffs])
        a = self.coeffs
        b = o.coeffs
        prod = [0] * 23
        for i in range(12):
            ai = a[i]
            if ai == 0:
                continue
            for j in range(12):
                prod[i + j] += ai * b[j]
        # reduce with w^12 = 18 w^6 - 82, from the top down
        for k in range(22, 11, -1):
            t = prod[k]
            if t:
                prod[k - 6] += 18 * t
                prod[k - 12] -= 82 * t
        return FQ12(prod[:12])

    __rmul__ = __mul__

    def __pow__(self, e: int):
        e = int(e)
        result = FQ12.one()
        base = self
        while e > 0:
            if e & 1:
                result = result * base
            base = base * base
            e >>= 1
        return result

    def inv(self) -> "FQ12":
        """Inverse modulo w^12 - 18 w^6 + 82 by the extended Euclidean algorithm over F_q[w]."""

        def trim(p: List[int]) -> List[int]:
            p = [c % _Q for c in p]
            while p and p[-1] == 0:
                p.pop()
            return p

        def divmod_poly(num: List[int], den: List[int]):
            num = list(num)
            quot = [0] * max(1, len(num) - len(den) + 1)
            inv_lead = _inv(den[-1])
            for i in range(len(num) - len(den), -1, -1):
                coef = num[i + len(den) - 1] * inv_lead % _Q
                quot[i] = coef
                if coef:
                    for j, d in enumerate(den):
                        num[i + j] = (num[i + j] - coef * d) % _Q
            return trim(quot), trim(num)

        def mul_poly(a: List[int], c: List[int]) -> List[int]:
            if not a or not c:
                return []
            out = [0] * (len(a) + len(c) - 1)
            for i, x in enumerate(a):
                for j, y in enumerate(c):
                    out[i + j] += x * y
            return trim(out)

        def sub_poly(a: List[int], c: List[int]) -> List[int]:
            n = max(len(a), len(c))
            return trim([(a[i] if i < len(a) else 0) - (c[i] if i < len(c) else 0) for i in range(n)])

        r0 = trim(list(_FQ12_MOD) + [1])
        r1 = trim(list(self.coeffs))
        if not r1:
            raise ZeroDivisionError("FQ12 inverse of zero")
        s0: List[int] = []
        s1: List[int] = [1]
        while r1:
            q, rem = divmod_poly(r0, r1)
            r0, r1 = r1, rem
            s0, s1 = s1, sub_poly(s0, mul_poly(q, s1))
        if len(r0) != 1:
            raise ZeroDivisionError("FQ12 element not invertible")
        k = _inv(r0[0])
        out = [(c * k) % _Q for c in s0] + [0] * 12
        return FQ12(out[:12])

    def __truediv__(self, o):
        if isinstance(o, FQ12):
            return self * o.inv()
        return self * _inv(o.n if isinstance(o, FQ) else int(o))

    __div__ = __truediv__

    def __eq__(self, o) -> bool:
        if isinstance(o, FQ12):
            return self.coeffs == o.coeffs
        return NotImplemented

    def __ne__(self, o) -> bool:
        r = self.__eq__(o)
        return r if r is NotImplemented else not r

    def __hash__(self) -> int:
        return hash(("FQ12",) + self.coeffs)

    def __repr__(self) -> str:
        return f"FQ12({list(self.coeffs)})"


# ---------------------------------------------------------------------------
# curve constants
# ---------------------------------------------------------------------------
b = FQ(3)
b2 = FQ2((3, 0)) / FQ2((9, 1))
G1 = (FQ(1), FQ(2), FQ(1))
G2 = (
    FQ2((10857046999023057135944570762232829481370756359578518086990519993285655852781,
         11559732032986387107991004021392285783925812861821192530917403151452391805634)),
    FQ2((8495653923123431417604973247489272438418190587263600148770280649306958101930,
         4082367875863433681332203403145435568316851327593401208105741076214120093531)),
    FQ2.one(),
)
Z1 = (FQ(1), FQ(1), FQ(0))
Z2 = (FQ2.one(), FQ2.one(), FQ2.zero())


def _zero_like(x):
    return FQ.zero() if isinstance(x, FQ) else FQ2.zero()


def _one_like(x):
    return FQ.one() if isinstance(x, FQ) else FQ2.one()


def is_inf(pt) -> bool:
    return pt[2] == 0


# -- G1 fast paths on plain ints (Jacobian, a = 0) ---------------------------

def _dbl_int(X: int, Y: int, Z: int):
    if Z == 0:
        return X, Y, Z
    A = X * X % _Q
    B = Y * Y % _Q
    C = B * B % _Q
    S = 4 * X * B % _Q
    M = 3 * A % _Q
    X3 = (M * M - 2 * S) % _Q
    Y3 = (M * (S - X3) - 8 * C) % _Q
    Z3 = 2 * Y * Z % _Q
    return X3, Y3, Z3


def _add_int(X1: int, Y1: int, Z1_: int, X2: int, Y2: int, Z2_: int):
    if Z1_ == 0:
        return X2, Y2, Z2_
    if Z2_ == 0:
        return X1, Y1, Z1_
    Z1Z1 = Z1_ * Z1_ % _Q
    Z2Z2 = Z2_ * Z2_ % _Q
    U1 = X1 * Z2Z2 % _Q
    U2 = X2 * Z1Z1 % _Q
    S1 = Y1 * Z2_ * Z2Z2 % _Q
    S2 = Y2 * Z1_ * Z1Z1 % _Q
    H = (U2 - U1) % _Q
    R = (S2 - S1) % _Q
    if H == 0:
        if R == 0:
            return _dbl_int(X1, Y1, Z1_)
        return 1, 1, 0
    HH = H * H % _Q
    HHH = H * HH % _Q
    V = U1 * HH % _Q
    X3 = (R * R - HHH - 2 * V) % _Q
    Y3 = (R * (V - X3) - S1 * HHH) % _Q
    Z3 = Z1_ * Z2_ * H % _Q
    return X3, Y3, Z3


def double(pt):
    x, y, z = pt
    if isinstance(x, FQ):
        X3, Y3, Z3 = _dbl_int(x.n, y.n, z.n)
        return (FQ(X3), FQ(Y3), FQ(Z3))
    if z == 0:
        return pt
    A = x * x
    B = y * y
    C = B * B
    S = x * B * 4
    M = A * 3
    X3 = M * M - S * 2
    Y3 = M * (S - X3) - C * 8
    Z3 = y * z * 2
    return (X3, Y3, Z3)


def add(p1, p2):
    x1, y1, z1 = p1
    x2, y2, z2 = p2
    if isinstance(x1, FQ):
        X3, Y3, Z3 = _add_int(x1.n, y1.n, z1.n, x2.n, y2.n, z2.n)
        return (FQ(X3), FQ(Y3), FQ(Z3))
    if z1 == 0:
        return p2
    if z2 == 0:
        return p1
    Z1Z1 = z1 * z1
    Z2Z2 = z2 * z2
    U1 = x1 * Z2Z2
    U2 = x2 * Z1Z1
    S1 = y1 * z2 * Z2Z2
    S2 = y2 * z1 * Z1Z1
    H = U2 - U1
    R = S2 - S1
    if H == 0:
        if R == 0:
            return double(p1)
        return (_one_like(x1), _one_like(x1), _zero_like(x1))
    HH = H * H
    HHH = H * HH
    V = U1 * HH
    X3 = R * R - HHH - V * 2
    Y3 = R * (V - X3) - S1 * HHH
    Z3 = z1 * z2 * H
    return (X3, Y3, Z3)


def neg(pt):
    x, y, z = pt
    return (x, -y, z)


def multiply(pt, n: int):
    n = int(n)
    if n < 0:
        return multiply(neg(pt), -n)
    x, y, z = pt
    if isinstance(x, FQ):
        X, Y, Z = x.n, y.n, z.n
        RX, RY, RZ = 1, 1, 0
        for bit in bin(n)[2:] if n else "":
            RX, RY, RZ = _dbl_int(RX, RY, RZ)
            if bit == "1":
                RX, RY, RZ = _add_int(RX, RY, RZ, X, Y, Z)
        return (FQ(RX), FQ(RY), FQ(RZ))
    result = (_one_like(x), _one_like(x), _zero_like(x))
    for bit in bin(n)[2:] if n else "":
        result = double(result)
        if bit == "1":
            result = add(result, pt)
    return result


def normalize(pt):
    x, y, z = pt
    if z == 0:
        return (_zero_like(x), _zero_like(x))
    if isinstance(x, FQ):
        zi = _inv(z.n)
        zi2 = zi * zi % _Q
        return (FQ(x.n * zi2), FQ(y.n * zi2 * zi))
    zi = 1 / z if isinstance(z, FQ2) else z.inv()
    zi2 = zi * zi
    return (x * zi2, y * zi2 * zi)


def eq(p1, p2) -> bool:
    x1, y1, z1 = p1
    x2, y2, z2 = p2
    if z1 == 0 or z2 == 0:
        return (z1 == 0) and (z2 == 0)
    z1z1 = z1 * z1
    z2z2 = z2 * z2
    return x1 * z2z2 == x2 * z1z1 and y1 * z2z2 * z2 == y2 * z1z1 * z1


def is_on_curve(pt, b_) -> bool:
    x, y, z = pt
    if z == 0:
        return True
    z2_ = z * z
    z6 = z2_ * z2_ * z2_
    return y * y == x * x * x + b_ * z6


# ---------------------------------------------------------------------------
# optimal ate pairing
# ---------------------------------------------------------------------------
ate_loop_count = 29793968203157093288  # 6x + 2 with x = 4965661367192848881

_XI = FQ2((9, 1))  # w^6
_FROB_G2_X = _XI ** ((_Q - 1) // 3)   # x-coordinate factor of the q-Frobenius on the twist
_FROB_G2_Y = _XI ** ((_Q - 1) // 2)   # y-coordinate factor


def _fq2_to_fq12_terms(c: FQ2, k: int, acc: List[int]) -> None:
    """acc += c * w^k for c = c0 + c1 u, using u = w^6 - 9."""
    c0, c1 = c.coeffs
    acc[k] += c0 - 9 * c1
    acc[k + 6] += c1


def _line(xt: FQ2, yt: FQ2, lam: FQ2, xp: int, yp: int) -> FQ12:
    """Line of slope lam*w through the untwisted image of (xt, yt), evaluated at (xp, yp).

    With x' = xt w^2, y' = yt w^3 and slope lam w:
    l = yp - lam xp w + (lam xt - yt) w^3.
    """
    acc = [0] * 12
    acc[0] += yp
    _fq2_to_fq12_terms(lam * (-xp), 1, acc)
    _fq2_to_fq12_terms(lam * xt - yt, 3, acc)
    return FQ12(acc)


def _vertical(xt: FQ2, xp: int) -> FQ12:
    acc = [0] * 12
    acc[0] += xp
    _fq2_to_fq12_terms(-xt, 2, acc)
    return FQ12(acc)


def _tw_add(T, Q, xp: int, yp: int):
    xt, yt = T
    xq, yq = Q
    if xt == xq:
        if yt == yq:
            lam = (xt * xt * 3) / (yt * 2)
        else:
            return None, _vertical(xt, xp)
    else:
        lam = (yq - yt) / (xq - xt)
    x3 = lam * lam - xt - xq
    y3 = lam * (xt - x3) - yt
    return (x3, y3), _line(xt, yt, lam, xp, yp)


_W_FROB: List[FQ12] = []


def _frobenius12(f: FQ12, power: int = 1) -> FQ12:
    """f^(q^power) via the precomputed images of w^i."""
    global _W_FROB
    if not _W_FROB:
        w = FQ12([0, 1] + [0] * 10)
        wq = w ** _Q
        cur = FQ12.one()
        for _ in range(12):
            _W_FROB.append(cur)
            cur = cur * wq
    out = f
    for _ in range(power):
        acc = [0] * 12
        for i, c in enumerate(out.coeffs):
            if c:
                for j, wj in enumerate(_W_FROB[i].coeffs):
                    acc[j] += c * wj
        out = FQ12(acc)
    return out


def _final_exponentiate(f: FQ12) -> FQ12:
    # easy part: f^((q^6 - 1)(q^2 + 1))
    f1 = _frobenius12(f, 6) * f.inv()
    f2 = _frobenius12(f1, 2) * f1
    # hard part: (q^4 - q^2 + 1) / r
    return f2 ** ((_Q ** 4 - _Q ** 2 + 1) // _R)


def miller_loop(Q, P) -> FQ12:
    xq, yq = Q
    xp, yp = P
    T = (xq, yq)
    f = FQ12.one()
    for bit in bin(ate_loop_count)[3:]:
        T, l = _tw_add(T, T, xp, yp)
        f = f * f * l
        if bit == "1":
            T, l = _tw_add(T, Q, xp, yp)
            f = f * l
    q1 = (xq.conj() * _FROB_G2_X, yq.conj() * _FROB_G2_Y)
    q2 = (q1[0].conj() * _FROB_G2_X, -(q1[1].conj() * _FROB_G2_Y))
    T, l = _tw_add(T, q1, xp, yp)
    f = f * l
    _, l = _tw_add(T, q2, xp, yp)
    f = f * l
    return f


def pairing(Q, P) -> FQ12:
    """Optimal ate pairing e(P, Q) for P in G1 and Q in G2 (argument order of py_ecc)."""
    if Q[2] == 0 or P[2] == 0:
        return FQ12.one()
    if not is_on_curve(Q, b2):
        raise ValueError("Q is not on the twist curve")
    if not is_on_curve(P, b):
        raise ValueError("P is not on the curve")
    qa = normalize(Q)
    pa = normalize(P)
    return _final_exponentiate(miller_loop(qa, (pa[0].n, pa[1].n)))


def final_exponentiate(f: FQ12) -> FQ12:
    return _final_exponentiate(f)
