"""Symmetry algebra restated from the reference (test infrastructure only).

Charges are plain ints (all symmetries on the hot path have Nq == 1).

References:
  U(1):  include/Xped/Symmetry/U1.hpp:95-226
  Z(N):  include/Xped/Symmetry/ZN.hpp:91-237
  SU(2): include/Xped/Symmetry/SU2.hpp:108-180, src/Symmetry/SU2.cpp:17-119
  defaults (coeff_FS, coeff_turn): include/Xped/Symmetry/SymBase.hpp:69-77
  phase(): include/Xped/Symmetry/functions.hpp:79-84
  CGC:   src/Symmetry/SU2.cpp:71-89 (3j symbol from GSL, SU2Wrappers.hpp:78-81)
"""
from __future__ import annotations

import math
from fractions import Fraction
from functools import lru_cache

import numpy as np


def phase(q: int) -> float:
    """(-1)^q with C++ int semantics (functions.hpp:79-84)."""
    return -1.0 if (int(q) % 2) else 1.0  # Python % gives the same parity as C++ for negatives


def _cdiv(a: int, b: int) -> int:
    """C++ integer division (truncation toward zero)."""
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b >= 0) else -q


class _Sym:
    name = "sym"
    ABELIAN = True
    FERMIONIC = False
    vacuum = 0
    kind_id = -1

    def conj(self, q):
        raise NotImplementedError

    def degeneracy(self, q):
        return 1

    def combine(self, ql, qr):
        raise NotImplementedError

    def triangle(self, q1, q2, q3):
        raise NotImplementedError

    def coeff_twist(self, q):
        return 1.0

    def coeff_FS(self, q):
        return 1.0

    def cgc(self, q1, q2, q3):
        """Symmetry::CGC for abelian symmetries: the single coefficient 1 of a
        one-dimensional vertex (U1.hpp / ZN.hpp CGC)."""
        return np.ones((1, 1, 1)) if self.triangle(q1, q2, q3) else np.zeros((1, 1, 1))

    def one_j(self, q):
        """Symmetry::one_j_tensor for abelian symmetries (U1.hpp:139-143, ZN.hpp:150-154): [[1]]."""
        return np.ones((1, 1))

    def __eq__(self, other):
        return type(self) is type(other) and self.__dict__ == other.__dict__

    def __hash__(self):
        return hash((type(self).__name__, tuple(sorted(self.__dict__.items()))))


class U1(_Sym):
    """U(1); ``fermionic`` selects the FChargeU1 kind (U1.hpp:50,130-134,174-182)."""

    def __init__(self, fermionic: bool = False):
        self.FERMIONIC = bool(fermionic)
        self.name = "fU1" if fermionic else "U1"
        self.kind_id = 1 if fermionic else 0

    def conj(self, q):
        return -q

    def combine(self, ql, qr):
        return [ql + qr]

    def triangle(self, q1, q2, q3):
        return q1 + q2 == q3

    def coeff_twist(self, q):
        if not self.FERMIONIC:
            return 1.0
        return -1.0 if (q % 2 != 0) else 1.0

    def coeff_turn(self, ql, qr, qf):
        return 1.0 if self.triangle(ql, qr, qf) else 0.0

    def coeff_6j(self, q1, q2, q3, q4, q5, q6):
        t = self.triangle
        if t(q1, q2, q3) and t(q1, q6, q5) and t(q2, q4, q6) and t(q3, q4, q5):
            return 1.0
        return 0.0

    def coeff_recouple(self, q1, q2, q3, Q, Q12, Q23):
        return self.coeff_6j(q1, q2, Q12, q3, Q, Q23)

    def coeff_swap(self, ql, qr, qf):
        sign = 1.0
        if self.FERMIONIC and (ql % 2 != 0) and (qr % 2 != 0):
            sign = -1.0
        return sign if self.triangle(ql, qr, qf) else 0.0


class ZN(_Sym):
    """Z(N); ``fermionic`` selects FChargeU1 parity (ZN.hpp:115-193)."""

    def __init__(self, N: int = 2, fermionic: bool = False):
        self.N = int(N)
        self.FERMIONIC = bool(fermionic)
        self.name = ("fZ%d" if fermionic else "Z%d") % N
        self.kind_id = 3 if fermionic else 2

    def conj(self, q):
        return (-q) % self.N

    def combine(self, ql, qr):
        return [(ql + qr) % self.N]

    def triangle(self, q1, q2, q3):
        return (q1 + q2) % self.N == q3

    def coeff_twist(self, q):
        if not self.FERMIONIC:
            return 1.0
        return -1.0 if (q % 2 != 0) else 1.0

    def coeff_turn(self, ql, qr, qf):
        return 1.0 if self.triangle(ql, qr, qf) else 0.0

    def coeff_6j(self, q1, q2, q3, q4, q5, q6):
        t = self.triangle
        if t(q1, q2, q3) and t(q1, q6, q5) and t(q2, q4, q6) and t(q3, q4, q5):
            return 1.0
        return 0.0

    def coeff_recouple(self, q1, q2, q3, Q, Q12, Q23):
        return self.coeff_6j(q1, q2, Q12, q3, Q, Q23)

    def coeff_swap(self, ql, qr, qf):
        sign = 1.0
        if self.FERMIONIC and (ql % 2 != 0) and (qr % 2 != 0):
            sign = -1.0
        return sign if self.triangle(ql, qr, qf) else 0.0


def _fact(n: int) -> int:
    return math.factorial(n)


@lru_cache(maxsize=None)
def wigner6j_twice(a2, b2, c2, d2, e2, f2) -> float:
    """Wigner 6j {a b c; d e f} from doubled spins by Racah's formula, in exact
    rational arithmetic (a published closed form; replaces GSL's
    gsl_sf_coupling_6j called at include/Xped/Symmetry/SU2Wrappers.hpp:73-76)."""

    def tri(x, y, z):
        if x < 0 or y < 0 or z < 0:
            return False
        if (x + y + z) % 2:
            return False
        return abs(x - y) <= z <= x + y

    if not (tri(a2, b2, c2) and tri(a2, e2, f2) and tri(d2, b2, f2) and tri(d2, e2, c2)):
        return 0.0

    def delta_sq(x, y, z):  # Delta^2 as a Fraction
        return Fraction(_fact((x + y - z) // 2) * _fact((x - y + z) // 2) * _fact((-x + y + z) // 2),
                        _fact((x + y + z) // 2 + 1))

    pref_sq = delta_sq(a2, b2, c2) * delta_sq(a2, e2, f2) * delta_sq(d2, b2, f2) * delta_sq(d2, e2, c2)
    s1 = (a2 + b2 + c2) // 2
    s2 = (a2 + e2 + f2) // 2
    s3 = (d2 + b2 + f2) // 2
    s4 = (d2 + e2 + c2) // 2
    p1 = (a2 + b2 + d2 + e2) // 2
    p2 = (a2 + c2 + d2 + f2) // 2
    p3 = (b2 + c2 + e2 + f2) // 2
    tmin = max(s1, s2, s3, s4)
    tmax = min(p1, p2, p3)
    total = Fraction(0)
    for t in range(tmin, tmax + 1):
        num = (-1) ** t * _fact(t + 1)
        den = (_fact(t - s1) * _fact(t - s2) * _fact(t - s3) * _fact(t - s4)
               * _fact(p1 - t) * _fact(p2 - t) * _fact(p3 - t))
        total += Fraction(num, den)
    # value = sqrt(pref_sq) * total; keep the sign of total
    val = math.sqrt(pref_sq.numerator) / math.sqrt(pref_sq.denominator) * float(total)
    return val


@lru_cache(maxsize=None)
def wigner3j_twice(a2, b2, c2, ma2, mb2, mc2) -> float:
    """Wigner 3j (a b c; ma mb mc) from doubled spins and projections by Racah's
    closed form, in exact rational arithmetic (a published formula; replaces
    GSL's gsl_sf_coupling_3j called at include/Xped/Symmetry/SU2Wrappers.hpp:78-81).
    Zero unless ma + mb + mc = 0, |m| <= j with j - m integral and the triangle rule holds."""
    if ma2 + mb2 + mc2 != 0:
        return 0.0
    for j2, m2 in ((a2, ma2), (b2, mb2), (c2, mc2)):
        if j2 < 0 or abs(m2) > j2 or (j2 - m2) % 2:
            return 0.0
    if (a2 + b2 + c2) % 2 or not abs(a2 - b2) <= c2 <= a2 + b2:
        return 0.0
    f = _fact
    # integer arguments (all sums below are even before halving)
    jab_c, jac_b, jbc_a, jabc = (a2 + b2 - c2) // 2, (a2 - b2 + c2) // 2, (-a2 + b2 + c2) // 2, (a2 + b2 + c2) // 2
    num_sq = Fraction(f(jab_c) * f(jac_b) * f(jbc_a), f(jabc + 1))
    num_sq *= (f((a2 + ma2) // 2) * f((a2 - ma2) // 2) * f((b2 + mb2) // 2) * f((b2 - mb2) // 2)
               * f((c2 + mc2) // 2) * f((c2 - mc2) // 2))
    # summation bounds: every factorial argument non-negative
    t1 = (c2 - b2 + ma2) // 2      # j3 - j2 + m1
    t2 = (c2 - a2 - mb2) // 2      # j3 - j1 - m2
    t3 = jab_c                     # j1 + j2 - j3
    t4 = (a2 - ma2) // 2           # j1 - m1
    t5 = (b2 + mb2) // 2           # j2 + m2
    kmin = max(0, -t1, -t2)
    kmax = min(t3, t4, t5)
    total = Fraction(0)
    for k in range(kmin, kmax + 1):
        total += Fraction((-1) ** k, f(k) * f(t1 + k) * f(t2 + k) * f(t3 - k) * f(t4 - k) * f(t5 - k))
    if total == 0:
        return 0.0
    sign = -1.0 if ((a2 - b2 - mc2) // 2) % 2 else 1.0   # (-1)^(j1 - j2 - m3)
    return sign * math.sqrt(num_sq.numerator) / math.sqrt(num_sq.denominator) * float(total)


class SU2(_Sym):
    """SU(2) with q = 2j+1 (SU2.hpp:108-180, SU2.cpp:17-119).  Non-fermionic
    (SpinSU2 kind)."""

    ABELIAN = False
    vacuum = 1

    def __init__(self):
        self.name = "SU2"
        self.kind_id = 4

    def conj(self, q):
        return q

    def degeneracy(self, q):
        return q

    def combine(self, ql, qr):
        qmin = abs(ql - qr) + 1
        qmax = abs(ql + qr) - 1
        return list(range(qmin, qmax + 1, 2))

    def triangle(self, q1, q2, q3):
        # SU2.cpp:114-119 (no parity check, as in the reference)
        return (q3 - 1 >= abs(q1 - q2)) and (q3 - 1 <= q1 + q2 - 2)

    def coeff_FS(self, q):
        return -1.0 if q % 2 == 0 else 1.0

    def coeff_swap(self, ql, qr, qf):
        if not self.triangle(ql, qr, qf):
            return 0.0
        return phase(_cdiv(ql + qr - qf - 1, 2))

    def coeff_turn(self, ql, qr, qf):
        if not self.triangle(ql, qr, qf):
            return 0.0
        return self.coeff_swap(ql, qr, qf) * math.sqrt(float(qf) / float(ql))

    def coeff_6j(self, q1, q2, q3, q4, q5, q6):
        return wigner6j_twice(q1 - 1, q2 - 1, q3 - 1, q4 - 1, q5 - 1, q6 - 1)

    def one_j(self, q):
        """SU2::one_j_tensor (src/Symmetry/SU2.cpp:42-61): entry (i, j) = (-1)^i where the
        projections of i and j are opposite, 0 elsewhere."""
        out = np.zeros((q, q))
        for i in range(q):
            out[i, q - 1 - i] = phase(i)
        return out

    def cgc(self, q1, q2, q3):
        """SU2::CGC (src/Symmetry/SU2.cpp:71-89): the Clebsch-Gordan tensor of one
        vertex, index i of an irrep q standing for the projection 2m = (q - 1) - 2i
        (largest m first); value 3j(q1 q2 q3; m1 m2 -m3) (-1)^((q1 - q2 + 2 m3) / 2) sqrt(q3)."""
        out = np.zeros((q1, q2, q3))
        for i1 in range(q1):
            m1 = (q1 - 1) - 2 * i1
            for i2 in range(q2):
                m2 = (q2 - 1) - 2 * i2
                for i3 in range(q3):
                    m3 = (q3 - 1) - 2 * i3
                    w = wigner3j_twice(q1 - 1, q2 - 1, q3 - 1, m1, m2, -m3)
                    if w != 0.0:
                        out[i1, i2, i3] = w * phase(_cdiv(q1 - q2 + m3, 2)) * math.sqrt(q3)
        return out

    def coeff_recouple(self, q1, q2, q3, Q, Q12, Q23):
        # sqrt(Q12*Q23) * phase((q1+q2+q3+Q)/2.) * 6j(q1,q2,Q12,q3,Q,Q23)   (SU2.hpp:164-167)
        ph = phase(int((q1 + q2 + q3 + Q) / 2.0))
        return math.sqrt(Q12 * Q23) * ph * self.coeff_6j(q1, q2, Q12, q3, Q, Q23)


def make_symmetry(name: str):
    name = name.lower()
    if name == "u1":
        return U1(False)
    if name in ("fu1", "u1f"):
        return U1(True)
    if name == "z2":
        return ZN(2, False)
    if name in ("fz2", "z2f"):
        return ZN(2, True)
    if name == "su2":
        return SU2()
    raise ValueError(name)
