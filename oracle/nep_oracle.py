"""NEP descriptors and per-atom energies, restated in numpy (oracle).

TEST INFRASTRUCTURE ONLY.  FP64 restatement of the reference's per-atom NEP arithmetic
(nep_core.hpp, expanded for one model by NEP.java) for potential models nep3 / nep4 /
nep5 without ZBL or type-wise cutoffs, written in the quantities of the NNAP pipeline:

  radial functions   x = 2 (r/rc - 1)^2 - 1,  fc = (cos(pi r/rc) + 1) / 2,
                     f_k = (T_k(x) + 1) / 2 * fc                      (find_fn, find_fc)
  channel functions  g_n = sum_k c[(n (b+1) + k) T^2 + t_i T + t_j] f_k
                     (angular coefficients start after the radial ones, NUMC_R)
  radial columns     q_n = sum_j g_n(r_ij)                            (n = 0 .. n_max_R)
  expansion          A[n][lm] = sum_j g_n(r_ij) Y_lm(r_ij)            (r_ij < rc_A)
  angular columns    q[(l-1)(n_max_A+1) + n] = sum_m A[n][lm]^2        (l = 1 .. l_max)
  4-body column      L3(2 2 2)(A[n])   when num_L >= l_max + 1
  5-body column      L4(1 1 1 1)(A[n]) when num_L >= l_max + 2
                     (num_L = l_max + [l_max_4body == 2] + [l_max_5body == 1], so a file with
                     the 5-body flag alone gets the 4-body column, as the reference computes)
  network            E_i = sum_h w1[h] tanh(sum_d w0[h][d] q_d s_d - b0[h]) - b1
                     (nep5 also subtracts the species' own output bias)

with Y the orthonormal real spherical harmonics (Condon-Shortley phase) and L3 / L4 the
Wigner-3j / Clebsch-Gordan invariants of oracle/bispectrum.py.  The NEP routines named in
parentheses (find_fn, find_fc, find_q, find_q_with_4body, find_q_with_5body,
apply_ann_one_layer in nep_core.hpp) state the same quantities with GPUMD's own
unnormalised polynomial forms; tests/test_oracle_nep.py pins this restatement to the
compiled reference's outputs stored in tests/golden/nep_*.npz.
"""
from __future__ import annotations

import math

import numpy as np

from . import bispectrum as BS
from .nep_model import NEPModel


def radial_functions(r: np.ndarray, rc: float, bsize: int) -> np.ndarray:
    """f_k(r), k = 0 .. bsize, shape [bsize + 1, len(r)]."""
    x = 2.0 * (r / rc - 1.0) ** 2 - 1.0
    fc = 0.5 * np.cos(np.pi * r / rc) + 0.5
    t = [np.ones_like(x), x]
    for _ in range(2, bsize + 1):
        t.append(2.0 * x * t[-1] - t[-2])
    return np.array([0.5 * (tk + 1.0) * fc for tk in t[:bsize + 1]])


def real_sph(L: int, d: np.ndarray) -> np.ndarray:
    """Orthonormal real spherical harmonics Y[l^2 + l + m] of the directions d [n, 3]."""
    r = np.linalg.norm(d, axis=1)
    ct = d[:, 2] / r
    st = np.sqrt(np.maximum(0.0, 1.0 - ct * ct))
    phi = np.arctan2(d[:, 1], d[:, 0])
    n = len(r)
    # associated Legendre P_l^m(cos theta) with the Condon-Shortley phase
    P = np.zeros((L + 1, L + 1, n))
    P[0, 0] = 1.0
    for m in range(1, L + 1):
        P[m, m] = -(2 * m - 1) * st * P[m - 1, m - 1]
    for m in range(0, L):
        P[m + 1, m] = (2 * m + 1) * ct * P[m, m]
    for m in range(0, L + 1):
        for l in range(m + 2, L + 1):
            P[l, m] = ((2 * l - 1) * ct * P[l - 1, m] - (l + m - 1) * P[l - 2, m]) / (l - m)
    Y = np.zeros(((L + 1) ** 2, n))
    for l in range(L + 1):
        for m in range(0, l + 1):
            N = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - m) / math.factorial(l + m))
            if m == 0:
                Y[l * l + l] = N * P[l, 0]
            else:
                Y[l * l + l + m] = math.sqrt(2.0) * N * P[l, m] * np.cos(m * phi)
                Y[l * l + l - m] = math.sqrt(2.0) * N * P[l, m] * np.sin(m * phi)
    return Y


def _channels(m: NEPModel, r: np.ndarray, ti: int, tj: np.ndarray, angular: bool) -> np.ndarray:
    """g_n(r_j) of centre species ti and neighbour species tj [len(r)], shape [n_max + 1, len(r)]."""
    T = m.ntypes
    if angular:
        rc, nmax, b, off = m.rc_angular, m.n_max_angular, m.basis_size_angular, m.num_c_radial
    else:
        rc, nmax, b, off = m.rc_radial, m.n_max_radial, m.basis_size_radial, 0
    if m.typewise_descriptors:   # each pair's own cutoff; pairs beyond it add nothing
        rc = m.pair_cutoff(rc, m.typewise[1 if angular else 0], ti, np.asarray(tj))
        f = radial_functions(r, rc, b) * (r < rc)
    else:
        f = radial_functions(r, rc, b)                                    # [b+1, nj]
    nk = (np.arange(nmax + 1)[:, None] * (b + 1) + np.arange(b + 1)[None, :]) * T * T
    C = m.c[off + nk[None, :, :] + ti * T + np.asarray(tj)[:, None, None]]  # [nj, nmax+1, b+1]
    return np.einsum("jnk,kj->nj", C, f)


def descriptors(m: NEPModel, types0: np.ndarray, nl) -> np.ndarray:
    """Unscaled descriptor vectors q [n, dim] over the caller's full neighbour list."""
    n = len(types0)
    L, nA = m.l_max, m.n_max_angular
    q = np.zeros((n, m.dim))
    # the reference keys both terms on the column count alone (find_q, nep_core.hpp:943-955):
    # num_L >= l_max + 1 gives the 4-body column, num_L >= l_max + 2 the 5-body column
    t222 = BS.l3_terms(2, 2, 2) if m.num_L >= L + 1 else []
    t1111 = BS.l4_terms(1, 1, 1, 1) if m.num_L >= L + 2 else []
    Lx = max(L, 2 if t222 else 0, 1 if t1111 else 0)
    for i in range(n):
        o0, o1 = nl.offsets[i], nl.offsets[i + 1]
        d = np.asarray(nl.dx[o0:o1], dtype=np.float64)
        tj = types0[nl.j[o0:o1]]
        r = np.linalg.norm(d, axis=1)
        sel = r < m.rc_radial
        q[i, :m.n_max_radial + 1] = _channels(m, r[sel], types0[i], tj[sel], False).sum(axis=1)
        sel = r < m.rc_angular
        A = np.zeros((nA + 1, (Lx + 1) ** 2))
        if sel.any():
            A = _channels(m, r[sel], types0[i], tj[sel], True) @ real_sph(Lx, d[sel]).T
        off = m.n_max_radial + 1
        for l in range(1, L + 1):
            for nn in range(nA + 1):
                q[i, off + (l - 1) * (nA + 1) + nn] = np.sum(A[nn, l * l:(l + 1) ** 2] ** 2)
        off += L * (nA + 1)
        for terms in (t222, t1111):
            if not terms:
                continue
            for nn in range(nA + 1):
                q[i, off + nn] = sum(cf * np.prod([A[nn, j] for j in idx]) for idx, cf in terms)
            off += nA + 1
    return q


# Universal ZBL screening function (Ziegler, Biersack and Littmark): phi(x) = sum a_k exp(-b_k x)
ZBL_UNIVERSAL = ((0.18175, 3.1998), (0.50986, 0.94229), (0.28022, 0.4029), (0.02817, 0.20162))
K_COULOMB = 14.399645   # e^2 / (4 pi eps0) in eV A
ZBL_MAX_R = 2.5         # pairs at or beyond this distance carry no ZBL term (find_force_ZBL)


def zbl_pair_energy(m: NEPModel, ti: int, tj: int, r: float) -> float:
    """The ZBL energy of one pair (find_force_ZBL, nep_core.hpp:1321-1386): the screened
    Coulomb repulsion Z_i Z_j k / r phi(r / a), 1/a = 2.134563 (Z_i^0.23 + Z_j^0.23), times a
    cosine switch from 1 at rc_inner to 0 at rc_outer.  Fixed form: the universal phi and the
    file's two radii; flexible form: per species pair [rc_inner, rc_outer, a1, b1, .., a4, b4]."""
    if r >= ZBL_MAX_R:
        return 0.0
    zi, zj = m.atomic_numbers0[ti] + 1, m.atomic_numbers0[tj] + 1
    a_inv = (zi ** 0.23 + zj ** 0.23) * 2.134563   # 1 / a in 1/A
    x = r * a_inv
    if m.zbl_flexible:
        t1, t2 = min(ti, tj), max(ti, tj)
        k = t1 * m.ntypes - t1 * (t1 - 1) // 2 + (t2 - t1)
        p = m.zbl_para[10 * k:10 * k + 10]
        rin, rout, coefs = p[0], p[1], [(p[2 + 2 * q], p[3 + 2 * q]) for q in range(4)]
    else:
        rin, rout, coefs = m.zbl_rc_inner, m.zbl_rc_outer, ZBL_UNIVERSAL
        if m.typewise_zbl:   # rc_outer shrunk to the pair's covalent size, rc_inner its half
            rout = float(m.pair_cutoff(rout, m.typewise[2], ti, tj))
            rin = 0.5 * rout
    phi = sum(a * np.exp(-b * x) for a, b in coefs)
    if r < rin:
        fc = 1.0
    elif r < rout:
        fc = 0.5 * np.cos(np.pi / (rout - rin) * (r - rin)) + 0.5
    else:
        fc = 0.0
    return K_COULOMB * zi * zj * phi / r * fc


def energies(m: NEPModel, types0: np.ndarray, nl) -> np.ndarray:
    q = descriptors(m, types0, nl) * m.q_scaler[None, :]
    e = np.zeros(len(types0))
    for i, t in enumerate(types0):
        w0, b0, w1, extra = m.ann(int(t))
        e[i] = float(w1 @ np.tanh(w0 @ q[i] - b0)) - m.b1 - extra
    if m.zbl:  # each atom holds half of each of its pairs' ZBL energies
        r = np.linalg.norm(np.asarray(nl.dx, dtype=np.float64), axis=1)
        owner = np.repeat(np.arange(len(types0)), np.diff(nl.offsets))
        for q in np.nonzero(r < ZBL_MAX_R)[0]:
            e[owner[q]] += 0.5 * zbl_pair_energy(m, int(types0[owner[q]]), int(types0[nl.j[q]]), float(r[q]))
    return e
