"""Three- and four-body invariants of the spherical expansion (l3max / l4max columns).

TEST INFRASTRUCTURE ONLY (the oracle).  The reference evaluates these columns from
tables (calSphL3 / calSphL4, basis_SphericalUtil.hpp:395-467, tables in
basis_SphericalUtil0.hpp:10-500); here they are generated from their definitions, which
were identified against the reference's compiled output (every column agrees to ~1e-15):

    L3(l1 l2 l3)    = sum_{m1+m2+m3=0} (l1 l2 l3; m1 m2 m3) a_{l1 m1} a_{l2 m2} a_{l3 m3}
    L4(l1 l2 l3 l4) = sum_L (-1)^(l1+l2+L) / (2L+1) sum_M X12_{LM} conj(X34_{LM}),
                      X12_{LM} = sum <l1 m1 l2 m2 | L M> a_{l1 m1} a_{l2 m2}

with a the complex-basis coefficients of the real expansion A (real harmonics with the
Condon-Shortley phase: Y_{l,m>0} = sqrt2 (-1)^m Re Y^C_{lm}, Y_{l,-m} = sqrt2 (-1)^m Im Y^C_{lm}):
    a_{l,0} = A_{l,0},  a_{l,m} = (-1)^m (A_{l,m} + i A_{l,-m}) / sqrt2,  a_{l,-m} = (A_{l,m} - i A_{l,-m}) / sqrt2.
Each column becomes a polynomial in A: a list of (indices into A[l^2 + l + m], coefficient)
with index tuples sorted ascending and repeated products folded together.

Column order (an interface: the descriptor layout), per channel after the lmax+1
power-spectrum columns:
    l3max 2: 222 112 | 3: 233 123 | 4: 444 224 334 244 134 | 5: 255 455 235 145 345 |
    6: 666 336 446 556 266 466 246 156 356
    l4max 1: 1111 | 2: 2222 1122 | 3: 3333 1133 2233 1113 1333 1223
"""
from __future__ import annotations

import itertools
from fractions import Fraction
from functools import lru_cache
from math import factorial, sqrt
from typing import Dict, List, Tuple

L3_COMBOS = [[], [], [(2, 2, 2), (1, 1, 2)], [(2, 3, 3), (1, 2, 3)],
             [(4, 4, 4), (2, 2, 4), (3, 3, 4), (2, 4, 4), (1, 3, 4)],
             [(2, 5, 5), (4, 5, 5), (2, 3, 5), (1, 4, 5), (3, 4, 5)],
             [(6, 6, 6), (3, 3, 6), (4, 4, 6), (5, 5, 6), (2, 6, 6), (4, 6, 6), (2, 4, 6), (1, 5, 6), (3, 5, 6)]]
L4_COMBOS = [[], [(1, 1, 1, 1)], [(2, 2, 2, 2), (1, 1, 2, 2)],
             [(3, 3, 3, 3), (1, 1, 3, 3), (2, 2, 3, 3), (1, 1, 1, 3), (1, 3, 3, 3), (1, 2, 2, 3)]]


def l3_columns(l3max: int):
    return [c for l in range(l3max + 1) for c in L3_COMBOS[l]]


def l4_columns(l4max: int):
    return [c for l in range(l4max + 1) for c in L4_COMBOS[l]]


@lru_cache(None)
def wigner3j(j1, j2, j3, m1, m2, m3) -> float:
    """Racah's formula with exact integer arithmetic."""
    if m1 + m2 + m3 != 0 or not (abs(j1 - j2) <= j3 <= j1 + j2):
        return 0.0
    if abs(m1) > j1 or abs(m2) > j2 or abs(m3) > j3:
        return 0.0
    tri = Fraction(factorial(j1 + j2 - j3) * factorial(j1 - j2 + j3) * factorial(-j1 + j2 + j3),
                   factorial(j1 + j2 + j3 + 1))
    pre = tri * factorial(j1 + m1) * factorial(j1 - m1) * factorial(j2 + m2) * factorial(j2 - m2) * \
        factorial(j3 + m3) * factorial(j3 - m3)
    s = Fraction(0)
    for k in range(0, j1 + j2 + j3 + 1):
        den = [k, j3 - j2 + k + m1, j3 - j1 + k - m2, j1 + j2 - j3 - k, j1 - k - m1, j2 - k + m2]
        if min(den) < 0:
            continue
        d = 1
        for x in den:
            d *= factorial(x)
        s += Fraction((-1) ** k, d)
    sign = (-1) ** (j1 - j2 - m3)
    return sign * float(s) * sqrt(float(pre))


def clebsch(j1, m1, j2, m2, J, M) -> float:
    return (-1) ** (j1 - j2 + M) * sqrt(2 * J + 1) * wigner3j(j1, j2, J, m1, m2, -M)


def _V(l: int) -> Dict[int, List[Tuple[int, complex]]]:
    """a_{l mu} = sum_m V[mu] (m, v) A_{l m}."""
    r2 = 1.0 / sqrt(2.0)
    V = {0: [(0, 1.0 + 0j)]}
    for m in range(1, l + 1):
        V[m] = [(m, (-1) ** m * r2 + 0j), (-m, 1j * (-1) ** m * r2)]
        V[-m] = [(m, r2 + 0j), (-m, -1j * r2)]
    return V


def _fold(terms: Dict[Tuple[int, ...], complex]) -> List[Tuple[Tuple[int, ...], float]]:
    out: Dict[Tuple[int, ...], float] = {}
    for idx, c in terms.items():
        key = tuple(sorted(idx))
        out[key] = out.get(key, 0.0) + c.real
    return sorted(((k, v) for k, v in out.items() if abs(v) > 1e-13), key=lambda kv: kv[0])


def _lm(l, m):
    return l * l + l + m


@lru_cache(None)
def l3_terms(l1, l2, l3):
    V1, V2, V3 = _V(l1), _V(l2), _V(l3)
    acc: Dict[Tuple[int, ...], complex] = {}
    for mu1 in range(-l1, l1 + 1):
        for mu2 in range(-l2, l2 + 1):
            mu3 = -mu1 - mu2
            if abs(mu3) > l3:
                continue
            w = wigner3j(l1, l2, l3, mu1, mu2, mu3)
            if w == 0.0:
                continue
            for (a, va), (b, vb), (c, vc) in itertools.product(V1[mu1], V2[mu2], V3[mu3]):
                k = (_lm(l1, a), _lm(l2, b), _lm(l3, c))
                acc[k] = acc.get(k, 0) + w * va * vb * vc
    return _fold(acc)


@lru_cache(None)
def l4_terms(l1, l2, l3, l4):
    V1, V2, V3, V4 = _V(l1), _V(l2), _V(l3), _V(l4)
    acc: Dict[Tuple[int, ...], complex] = {}
    for L in range(abs(l1 - l2), l1 + l2 + 1):
        if not abs(l3 - l4) <= L <= l3 + l4:
            continue
        wL = (-1) ** (l1 + l2 + L) / (2 * L + 1)
        for M in range(-L, L + 1):
            left, right = {}, {}
            for mu1 in range(-l1, l1 + 1):
                mu2 = M - mu1
                if abs(mu2) > l2:
                    continue
                c = clebsch(l1, mu1, l2, mu2, L, M)
                if c == 0.0:
                    continue
                for (a, va), (b, vb) in itertools.product(V1[mu1], V2[mu2]):
                    k = (_lm(l1, a), _lm(l2, b))
                    left[k] = left.get(k, 0) + c * va * vb
            for mu3 in range(-l3, l3 + 1):
                mu4 = M - mu3
                if abs(mu4) > l4:
                    continue
                c = clebsch(l3, mu3, l4, mu4, L, M)
                if c == 0.0:
                    continue
                for (a, va), (b, vb) in itertools.product(V3[mu3], V4[mu4]):
                    k = (_lm(l3, a), _lm(l4, b))
                    right[k] = right.get(k, 0) + c * (va * vb).conjugate()
            for kl, vl in left.items():
                for kr, vr in right.items():
                    k = kl + kr
                    acc[k] = acc.get(k, 0) + wL * vl * vr
    return _fold(acc)


def column_terms(l3max: int, l4max: int):
    """Term lists of every invariant column, in descriptor order."""
    return [l3_terms(*c) for c in l3_columns(l3max)] + [l4_terms(*c) for c in l4_columns(l4max)]
