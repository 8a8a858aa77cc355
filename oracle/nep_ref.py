"""The reference's NEP arithmetic for one model, compiled here (oracle).

TEST INFRASTRUCTURE ONLY.  The model's shape expands the reference's NEP sources
(``src/nep/resources/assets/nep/src``, read from the reference checkout at build time;
nothing is committed) with oracle/nepgen.py into oracle/_ref/nep_<key>/src, which is
compiled with oracle/nep_driver.cpp into libnepref.so (g++ -O2, no fast-math: the oracle
values) or libnepref_fast.so (-O3 -ffast-math: the CPU baseline).  An expansion made where a
reference checkout exists is compiled wherever the repository is copied.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import subprocess
from typing import Optional

import numpy as np

from . import nepgen
from .build import REF_OUT, reference_root
from .nep_model import NEPModel

HERE = os.path.dirname(os.path.abspath(__file__))


def nep_src_dir() -> str:
    return os.path.join(reference_root(), "src", "nep", "resources", "assets", "nep", "src")


def shape_key(m: NEPModel) -> str:
    blob = json.dumps({k: str(v) for k, v in nepgen.gen_map(m).items()}, sort_keys=True)
    return "nep" + hashlib.sha1(blob.encode()).hexdigest()[:12]


def expand(m: NEPModel) -> str:
    """Expand the reference's NEP sources for the model's shape (needs a reference checkout,
    unless an earlier expansion is present); returns the source directory."""
    src = os.path.join(REF_OUT, shape_key(m), "src")
    if not os.path.exists(os.path.join(src, "nep_interface.cpp")):
        sd = nep_src_dir()
        if not os.path.isdir(sd):
            raise FileNotFoundError("reference NEP sources are not available")
        nepgen.expand(sd, src, m)
    return src


def build(m: NEPModel, fast: bool = False) -> str:
    """Compile the expanded sources: exact (-O2, no contraction; oracle values) or fast
    (-O3 -ffast-math, the reference's default JIT optimisation without -march=native; the
    CPU baseline)."""
    src = expand(m)
    d = os.path.dirname(src)
    out = os.path.join(d, "libnepref_fast.so" if fast else "libnepref.so")
    drv = os.path.join(HERE, "nep_driver.cpp")
    deps = [os.path.join(src, "nep_interface.cpp"), os.path.join(src, "nep_core.hpp"), drv]
    if not os.path.exists(out) or any(os.path.getmtime(p) > os.path.getmtime(out) for p in deps):
        opt = ["-O3", "-ffast-math"] if fast else ["-O2", "-ffp-contract=off"]
        cmd = ["g++", "-std=c++14"] + opt + ["-fPIC", "-shared", "-w", "-pthread", "-I", src,
               os.path.join(src, "nep_interface.cpp"), drv, "-o", out]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("building the reference NEP failed:\n" + r.stderr[-3000:])
    return out


class RefNEP:
    def __init__(self, m: NEPModel, fast: bool = False):
        self.m = m
        self.lib = C.CDLL(build(m, fast))
        T = m.ntypes
        self._keep = []
        dp = C.POINTER(C.c_double)

        def arr(a):
            a = np.ascontiguousarray(a, dtype=np.float64).copy()
            self._keep.append(a)
            return a.ctypes.data_as(dp)
        self.w0 = (dp * T)()
        self.b0 = (dp * T)()
        self.w1 = (dp * T)()
        for t in range(T):
            w0, b0, w1, extra = m.ann(t)
            self.w0[t] = arr(w0.reshape(-1))
            self.b0[t] = arr(b0)
            self.w1[t] = arr(np.concatenate([w1, [extra]]) if m.version == 5 else w1)
        self.b1 = arr(np.array([m.b1]))
        self.c = arr(m.c)
        self.qs = arr(m.q_scaler)
        self.zp = arr(m.zbl_para if len(m.zbl_para) else np.zeros(1))
        self.an = np.ascontiguousarray(m.atomic_numbers0, dtype=np.int32)

    def compute(self, types0, nl, nthreads: int = 1, n_eval: Optional[int] = None):
        types0 = np.ascontiguousarray(types0, dtype=np.int32)
        n = len(types0)
        n_eval = n if n_eval is None else int(n_eval)
        e, f, v = np.zeros(n), np.zeros((n, 3)), np.zeros((n, 9))
        dx = np.ascontiguousarray(nl.dx, dtype=np.float64)
        ip, lp, dp = C.POINTER(C.c_int), C.POINTER(C.c_long), C.POINTER(C.c_double)
        code = self.lib.nep_ref_compute(self.m.ntypes, self.an.ctypes.data_as(ip), self.zp, self.qs, self.w0, self.b0,
                                        self.w1, self.b1, self.c, self.m.dim, (self.m.n_max_angular + 1) * 80, n, n_eval,
                                        int(nthreads), types0.ctypes.data_as(ip), nl.offsets.ctypes.data_as(lp),
                                        nl.j.ctypes.data_as(ip), dx.ctypes.data_as(dp), e.ctypes.data_as(dp),
                                        f.ctypes.data_as(dp), v.ctypes.data_as(dp))
        if code:
            raise RuntimeError("reference NEP returned %d" % code)
        return {"energies": e, "energy": float(e.sum()), "forces": f, "virials": v, "virial": v.sum(axis=0)}
