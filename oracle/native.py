"""ctypes bindings to the FP64 oracle (``nnap_oracle.cpp``) and to the reference driver.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from . import bispectrum, build
from .model import PackedModel

_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        _LIB = C.CDLL(build.build_oracle())
        _LIB.oracle_neighbors.restype = C.c_long
        _LIB.oracle_neighbors_brute.restype = C.c_long
    return _LIB


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


BOX_ORTHO, BOX_LMP, BOX_PRISM = 0, 1, 2


def pack(model: PackedModel):
    """Flatten a model into (spec int32, rcuts float64, params float64) for oracle_compute."""
    spec, rcuts, blocks = [], [], []
    off = 0

    def add(arr):
        nonlocal off
        o = off
        blocks.append(np.asarray(arr, dtype=np.float64))
        off += blocks[-1].size
        return o

    for t in range(model.ntypes):
        b, nn = model.basis[t], model.nn[t]
        sub_entries = []
        fp_off = 0
        for sb in b.subs:
            po = add(sb.param)
            if sb.kind == "spherical_chebyshev":
                cols = bispectrum.column_terms(sb.l3max, sb.l4max)
                tab = []
                for terms in cols:
                    tab.append(len(terms))
                    for idx, coef in terms:
                        tab += [len(idx)] + list(idx) + [-1] * (4 - len(idx)) + [coef]
                io = add(np.asarray(tab, dtype=np.float64)) if tab else 0
                L = max(sb.lmax, sb.l3max, sb.l4max)
                sub_entries += [1, sb.nmax, L, sb.size_np, po, fp_off, sb.lmax + 1, len(cols), io]
            else:
                sub_entries += [0, sb.nmax, 0, sb.size_np, po, fp_off, 1, 0, 0]
            rcuts.append(sb.rcut)
            fp_off += sb.size
        nn_off = add(nn.cparam)
        norm_off = add(model.norm[t])
        mirror = b.src if b.kind == "mirror" else 0
        spec += [len(b.subs), b.size, mirror, len(nn.hidden_dims)] + list(nn.hidden_dims) + [nn_off, norm_off] + \
            sub_entries
    return (np.asarray(spec, dtype=np.int32), np.asarray(rcuts, dtype=np.float64),
            np.concatenate(blocks) if blocks else np.zeros(0))


def wrap(x, box_kind: int, box) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    box = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
    out = np.empty_like(x)
    lib().oracle_wrap(len(x), _p(x, C.c_double), box_kind, _p(box, C.c_double), _p(out, C.c_double))
    return out


class NeighborList:
    """CSR neighbour list: offsets[n+1], j, image (n_pairs x 3), dx (n_pairs x 3)."""

    def __init__(self, offsets, j, img, dx):
        self.offsets, self.j, self.img, self.dx = offsets, j, img, dx

    @property
    def counts(self):
        return np.diff(self.offsets)

    def as_set(self, i_filter=None):
        out = set()
        n = len(self.offsets) - 1
        for i in range(n):
            for k in range(self.offsets[i], self.offsets[i + 1]):
                out.add((i, int(self.j[k]), int(self.img[k, 0]), int(self.img[k, 1]), int(self.img[k, 2])))
        return out


def neighbors(xw, box_kind: int, box, rcut: float, brute: bool = False) -> NeighborList:
    xw = np.ascontiguousarray(xw, dtype=np.float64)
    box = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
    n = len(xw)
    counts = np.zeros(n, dtype=np.int32)
    L = lib()
    if brute:
        total = L.oracle_neighbors_brute(n, _p(xw, C.c_double), box_kind, _p(box, C.c_double), C.c_double(rcut),
                                         _p(counts, C.c_int), C.c_long(0), None, None)
    else:
        total = L.oracle_neighbors(n, _p(xw, C.c_double), box_kind, _p(box, C.c_double), C.c_double(rcut),
                                   _p(counts, C.c_int), C.c_long(0), None, None, None)
    j = np.zeros(max(total, 1), dtype=np.int32)
    img = np.zeros((max(total, 1), 3), dtype=np.int32)
    dx = np.zeros((max(total, 1), 3), dtype=np.float64)
    if brute:
        r = L.oracle_neighbors_brute(n, _p(xw, C.c_double), box_kind, _p(box, C.c_double), C.c_double(rcut),
                                     _p(counts, C.c_int), C.c_long(total), _p(j, C.c_int), _p(img, C.c_int))
    else:
        r = L.oracle_neighbors(n, _p(xw, C.c_double), box_kind, _p(box, C.c_double), C.c_double(rcut),
                               _p(counts, C.c_int), C.c_long(total), _p(j, C.c_int), _p(img, C.c_int),
                               _p(dx, C.c_double))
    if r != total:
        raise RuntimeError("neighbour enumeration changed between passes")
    off = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=off[1:])
    return NeighborList(off, j[:total], img[:total], dx[:total])


def compute(model: PackedModel, x, types, box_kind: int, box, want_fp: bool = False, want_pair: bool = False,
            nl: Optional[NeighborList] = None, n_eval: Optional[int] = None):
    """Full structure evaluation: wrap -> neighbour list -> per-atom arithmetic -> scatter.

    ``n_eval`` restricts the per-atom evaluation to the first ``n_eval`` atoms (timing samples)."""
    types = np.ascontiguousarray(types, dtype=np.int32)
    n = len(types)
    xw = wrap(x, box_kind, box)
    if nl is None:
        nl = neighbors(xw, box_kind, box, model.rcut_max)
    spec, rcuts, params = pack(model)
    e = np.zeros(n)
    f = np.zeros((n, 3))
    v = np.zeros((n, 9))
    Dmax = max(b.size for b in model.basis)
    fp = np.zeros((n, Dmax)) if want_fp else None
    pg = np.zeros((max(len(nl.j), 1), 3)) if want_pair else None
    code = lib().oracle_compute(model.ntypes, _p(spec, C.c_int), _p(rcuts, C.c_double), _p(params, C.c_double),
                                n, n if n_eval is None else int(n_eval), _p(types, C.c_int),
                                _p(nl.offsets, C.c_long), _p(nl.j, C.c_int),
                                _p(nl.dx, C.c_double), _p(e, C.c_double), _p(f, C.c_double), _p(v, C.c_double),
                                _p(fp, C.c_double) if want_fp else None, Dmax,
                                _p(pg, C.c_double) if want_pair else None)
    if code != 0:
        raise ValueError("oracle_compute failed with code %d" % code)
    out = {"energies": e, "energy": float(e.sum()), "forces": f, "virials": v, "virial": v.sum(axis=0),
           "xw": xw, "nl": nl}
    if want_fp:
        out["fp"] = fp
    if want_pair:
        out["pair_g"] = pg[:len(nl.j)]
    return out


# ------------------------------------------------------------------ reference driver
class RefLib:
    """The reference's own per-atom arithmetic for one model shape (see oracle/build.py)."""

    def __init__(self, model: PackedModel, fast: bool = False):
        key = build.expand_ref(model)
        libs = build.build_ref(key)
        path = libs.get("fast" if fast else "exact")
        if not path or not os.path.exists(path):
            raise FileNotFoundError("reference sources for shape %s are not expanded" % key)
        self.lib = C.CDLL(path)
        self.model = model
        T = model.ntypes
        self._keep = []
        hp = (C.POINTER(C.c_double) * T)()
        fpp = (C.POINTER(C.c_double) * T)()
        nnp = (C.POINTER(C.c_double) * T)()
        nrm = (C.POINTER(C.c_double) * T)()
        for t in range(T):
            for arr, tab in ((model.basis[t].hparam, hp), (model.basis[t].param, fpp),
                             (model.nn[t].cparam, nnp), (model.norm[t], nrm)):
                a = np.ascontiguousarray(arr, dtype=np.float64).copy()
                if a.size == 0:
                    a = np.zeros(1)
                self._keep.append(a)
                tab[t] = _p(a, C.c_double)
        self.hp, self.fpp, self.nnp, self.nrm = hp, fpp, nnp, nrm
        per, const = 0, 0
        for b in model.basis:
            p, c = 0, 0
            for sb in b.subs:
                K = (max(sb.lmax, sb.l3max, sb.l4max) + 1) ** 2 if sb.kind == "spherical_chebyshev" else 0
                p += 1 + sb.nmax + 1 + sb.size_np + K
                c += sb.size_np * K
            per, const = max(per, p), max(const, c)
        self.cache_per, self.cache_const = per, const + 16

    def compute(self, types, nl: NeighborList, nthreads: int = 1, n_eval: Optional[int] = None):
        types = np.ascontiguousarray(types, dtype=np.int32)
        n = len(types)
        e = np.zeros(n)
        f = np.zeros((n, 3))
        v = np.zeros((n, 9))
        dx = np.ascontiguousarray(nl.dx, dtype=np.float64)
        code = self.lib.ref_compute(self.model.ntypes, self.hp, self.fpp, self.nnp, self.nrm, n,
                                    n if n_eval is None else int(n_eval), _p(types, C.c_int),
                                    _p(nl.offsets, C.c_long), _p(nl.j, C.c_int), _p(dx, C.c_double),
                                    C.c_long(self.cache_per), C.c_long(self.cache_const), nthreads,
                                    _p(e, C.c_double), _p(f, C.c_double), _p(v, C.c_double))
        if code != 0:
            raise RuntimeError("reference per-atom function returned %d" % code)
        return {"energies": e, "energy": float(e.sum()), "forces": f, "virials": v, "virial": v.sum(axis=0)}

    def train_grad(self, types, nl: NeighborList, bgrad_e=None, bgrad_f=None, bgrad_w=None, nthreads: int = 1):
        """Parameter gradients of L = bE.E + bF.F + bW.W through the reference's training pair
        (ref_train_grad in ref_driver.cpp); returns per-species lists ``grad_fp`` and ``grad_nn``
        in the reference's C-level parameter layouts."""
        m = self.model
        T = m.ntypes
        types = np.ascontiguousarray(types, dtype=np.int32)
        n = len(types)
        fp_size = np.array([m.basis[t].param.size for t in range(T)], dtype=np.int64)
        nn_size = np.array([m.nn[t].cparam.size for t in range(T)], dtype=np.int64)
        per, const = 0, 0
        for t in range(T):
            p, c = 0, 0
            for sb in m.basis[t].subs:
                K = (max(sb.lmax, sb.l3max, sb.l4max) + 1) ** 2 if sb.kind == "spherical_chebyshev" else 1
                p += 2 + 2 * (sb.nmax + 1) + 2 * sb.size_np + 3 * K
                c += 3 * sb.size_np * K
            nnw = m.nn[t].input_dim + sum(m.nn[t].hidden_dims)
            per, const = max(per, p), max(const, c + 4 * nnw)
        const += 64
        be = None if bgrad_e is None else np.ascontiguousarray(bgrad_e, dtype=np.float64).reshape(n)
        bf = None if bgrad_f is None else np.ascontiguousarray(bgrad_f, dtype=np.float64).reshape(n, 3)
        bw = None if bgrad_w is None else np.ascontiguousarray(bgrad_w, dtype=np.float64).reshape(9)
        gfp = np.zeros(max(int(fp_size.sum()), 1))
        gnn = np.zeros(max(int(nn_size.sum()), 1))
        dx = np.ascontiguousarray(nl.dx, dtype=np.float64)
        nul = C.POINTER(C.c_double)()
        code = self.lib.ref_train_grad(T, self.hp, self.fpp, self.nnp, self.nrm, n, _p(types, C.c_int),
                                       _p(nl.offsets, C.c_long), _p(nl.j, C.c_int), _p(dx, C.c_double),
                                       C.c_long(per), C.c_long(const), nthreads,
                                       nul if be is None else _p(be, C.c_double),
                                       nul if bf is None else _p(bf, C.c_double),
                                       nul if bw is None else _p(bw, C.c_double),
                                       _p(fp_size, C.c_long), _p(nn_size, C.c_long),
                                       _p(gfp, C.c_double), _p(gnn, C.c_double))
        if code != 0:
            raise RuntimeError("reference training functions returned %d" % code)
        of = np.concatenate([[0], np.cumsum(fp_size)])
        on = np.concatenate([[0], np.cumsum(nn_size)])
        return {"grad_fp": [gfp[of[t]:of[t + 1]].copy() for t in range(T)],
                "grad_nn": [gnn[on[t]:on[t + 1]].copy() for t in range(T)]}

    def fp(self, types, nl: NeighborList):
        types = np.ascontiguousarray(types, dtype=np.int32)
        n = len(types)
        D = max(b.size for b in self.model.basis)
        out = np.zeros((n, D))
        dx = np.ascontiguousarray(nl.dx, dtype=np.float64)
        code = self.lib.ref_fp(self.hp, self.fpp, n, _p(types, C.c_int), _p(nl.offsets, C.c_long), _p(nl.j, C.c_int),
                               _p(dx, C.c_double), _p(out, C.c_double), D)
        if code != 0:
            raise RuntimeError("reference calFp returned %d" % code)
        return out
