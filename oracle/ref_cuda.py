"""The reference's own CUDA path for NNAP, compiled here (baseline only).

TEST INFRASTRUCTURE ONLY.  The reference's LAMMPS GPU kernels (nnap_interface_cuda.cu:
initLammpsNeiKernel, computeLammpsKernel, collectLammpsResultsKernel; one thread per
atom, FP32) are expanded by oracle/nnapgen.py with the picks NNAPGEN.initEngineCuda makes
(NNAPGEN.java:143-167: [ARCH] cuda, [PRECISION] single, block size 256) into
oracle/_ref/<key>_cuda/src, and compiled with nvcc for sm_103a at -O3 (the CMake Release
default of the reference's JIT) into libnnapref_cuda.so.  Only the reference's own
sources are compiled; nothing of this repository's kernels is on that path.

RefCudaNNAP does what NNAP does for a CUDA model (NNAP.java:311-397: per-species FP32
parameter blocks on the device behind device pointer tables, cutoffs squared and merge
order per species) and what NNAP.computeLammpsCuda does per call (NNAP.java:948-1030):
jse_nnap_lammps2cuda, jse_nnap_computeLammpsCuda, jse_nnap_cuda2lammps on LAMMPS-form
inputs (local atoms then ghosts, full neighbour lists).  Device memory comes from torch.
Models with one sub-basis per species only (the merge order of a merged basis is not
restated).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from . import build as OB
from . import nnapgen as NG
from .model import PackedModel

HERE = os.path.dirname(os.path.abspath(__file__))
BLOCK = 256  # NNAP.Conf.CUDA_BLOCKSIZE default (NNAP.java:51)


def gen_map_cuda(model: PackedModel):
    g = NG.gen_map(model)
    g["[ARCH]"] = "cuda"
    g["[PRECISION]"] = "single"
    g["NNAPGEN_CUDA_BLOCKSIZE"] = BLOCK
    return g


def expand(model: PackedModel) -> str:
    """Expand the reference's sources for the model (needs a reference checkout unless an
    earlier expansion is present); returns the source directory."""
    src = os.path.join(OB.REF_OUT, OB.shape_key(model) + "_cuda", "src")
    if not os.path.exists(os.path.join(src, "nnap_interface_cuda.cu")):
        rd = OB.reference_src_dir()
        if not os.path.isdir(rd):
            raise FileNotFoundError("reference NNAP sources are not available")
        os.makedirs(src, exist_ok=True)
        g = gen_map_cuda(model)
        for name in NG.HEADERS + ["nnap_interface_cuda.cu"]:
            with open(os.path.join(rd, name)) as f:
                lines = f.read().split("\n")
            with open(os.path.join(src, name), "w") as f:
                f.write("\n".join(NG.process(lines, g)))
    return src


def build(model: PackedModel) -> str:
    src = expand(model)
    out = os.path.join(os.path.dirname(src), "libnnapref_cuda.so")
    cu = os.path.join(src, "nnap_interface_cuda.cu")
    deps = [cu] + [os.path.join(src, h) for h in NG.HEADERS]
    if not os.path.exists(out) or any(os.path.getmtime(p) > os.path.getmtime(out) for p in deps):
        nvcc = os.environ.get("NVCC") or "nvcc"
        cmd = [nvcc, "-O3", "-std=c++14", "-gencode", "arch=compute_103a,code=sm_103a", "-Xcompiler", "-fPIC",
               "-shared", "-w", "-I", src, cu, "-o", out]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("building the reference CUDA path failed:\n" + r.stderr[-3000:])
    return out


def lammps_arrays(x_all, types_all, inum: int, lists):
    """LAMMPS-form inputs as the reference's host functions read them: x rows, types,
    ilist = 0..inum-1, numneigh and firstneigh per local atom."""
    x_all = np.ascontiguousarray(x_all, dtype=np.float64).reshape(-1, 3)
    types_all = np.ascontiguousarray(types_all, dtype=np.int32)
    rows = [np.ascontiguousarray(l, dtype=np.int32) for l in lists[:inum]]
    return x_all, types_all, rows


class LammpsRef:
    """LAMMPS-side plumbing of a reference CUDA path: the host arrays LAMMPS holds (row
    pointers), the device buffers NNAP / NEP keep, and the reference's own lammps2cuda /
    cuda2lammps host functions (``<prefix>lammps2cuda``, ``<prefix>cuda2lammps``).
    Subclasses add their parameter tables, their work buffers and ``compute``."""
    prefix = ""

    def _bind_io(self):
        P, I = C.c_void_p, C.c_int
        getattr(self.lib, self.prefix + "lammps2cuda").argtypes = [I, I, I, I] + [P] * 12
        getattr(self.lib, self.prefix + "cuda2lammps").argtypes = [I] * 7 + [P] * 12

    def _work_buffers(self, nb: int, inum: int, nall: int) -> dict:
        return {}

    def setup(self, x_all, types_all, inum: int, lists, cvflag_atom: bool = False):
        """Size every buffer for one LAMMPS-form configuration (NNAP.java:953-992,
        NEP.java:262-311)."""
        torch = self.torch
        x, t, rows = lammps_arrays(x_all, types_all, inum, lists)
        if t.min() < 1 or t.max() > self.T:
            raise ValueError("species outside 1..ntypes")
        nall = len(x)
        self.inum, self.nall = inum, nall
        self.maxn = max(1, max((len(r) for r in rows), default=1))
        if any(((r < 0) | (r >= nall)).any() for r in rows):
            raise ValueError("neighbour index outside the local + ghost atoms")
        self.cv = bool(cvflag_atom)
        # host side: row pointers, as LAMMPS holds them
        self.h_x = x
        self.h_xrows = (C.c_void_p * nall)(*[x[i:].ctypes.data for i in range(nall)])
        self.h_type = t
        self.h_ilist = np.arange(inum, dtype=np.int32)
        self.h_num = np.array([len(r) for r in rows], dtype=np.int32)
        self.h_rows = rows
        self.h_first = (C.c_void_p * inum)(*[r.ctypes.data if len(r) else 0 for r in rows])
        self.h_flt = np.zeros(max(9 * nall, 6 * inum, 1), dtype=np.float32)
        self.h_int = np.zeros(max(inum * self.maxn, inum, 1), dtype=np.int32)
        self.h_f = np.zeros((nall, 3))
        self.h_frows = (C.c_void_p * nall)(*[self.h_f[i:].ctypes.data for i in range(nall)])
        self.h_eng = np.zeros(1)
        self.h_eatom = np.zeros(nall)
        self.h_vir = np.zeros(6)
        self.h_cv = np.zeros((nall, 9))
        self.h_cvrows = (C.c_void_p * nall)(*[self.h_cv[i:].ctypes.data for i in range(nall)])
        d = self.dev
        f32, i32 = torch.float32, torch.int32
        nb = inum * self.maxn
        self.d = {
            "x": torch.zeros(3 * nall, dtype=f32, device=d), "type": torch.zeros(nall, dtype=i32, device=d),
            "ilist": torch.zeros(inum, dtype=i32, device=d), "num": torch.zeros(inum, dtype=i32, device=d),
            "first": torch.zeros(nb, dtype=i32, device=d), "f": torch.zeros(3 * nall, dtype=f32, device=d),
            "eatom0": torch.zeros(inum, dtype=f32, device=d), "vatom0": torch.zeros(6 * inum, dtype=f32, device=d),
            "vatom1": torch.zeros((9 if self.cv else 6) * nall, dtype=f32, device=d),
        }
        self.d.update(self._work_buffers(nb, inum, nall))
        torch.cuda.synchronize(d)

    def to_device(self, nlflag: bool = True):
        """<prefix>lammps2cuda: positions and types (and the lists when nlflag)."""
        D = self.d
        code = getattr(self.lib, self.prefix + "lammps2cuda")(
            self.inum, self.nall, 1 if nlflag else 0, self.maxn, C.cast(self.h_xrows, C.c_void_p),
            self.h_type.ctypes.data, self.h_ilist.ctypes.data, self.h_num.ctypes.data,
            C.cast(self.h_first, C.c_void_p), self.h_flt.ctypes.data, self.h_int.ctypes.data, D["x"].data_ptr(),
            D["type"].data_ptr(), D["ilist"].data_ptr(), D["num"].data_ptr(), D["first"].data_ptr())
        if code:
            raise RuntimeError(self.prefix + "lammps2cuda returned %d" % code)

    def to_host(self, eflag: bool = True, vflag: bool = True, eflag_atom: bool = True) -> dict:
        """<prefix>cuda2lammps into fresh accumulators."""
        D = self.d
        self.h_f[:] = 0.0
        self.h_eng[:] = 0.0
        self.h_eatom[:] = 0.0
        self.h_vir[:] = 0.0
        self.h_cv[:] = 0.0
        code = getattr(self.lib, self.prefix + "cuda2lammps")(
            self.inum, self.nall, int(eflag), int(vflag), int(eflag_atom), 0, int(self.cv),
            C.cast(self.h_frows, C.c_void_p), self.h_eng.ctypes.data, self.h_eatom.ctypes.data,
            self.h_vir.ctypes.data, None, C.cast(self.h_cvrows, C.c_void_p), self.h_flt.ctypes.data,
            self.h_ilist.ctypes.data, D["f"].data_ptr(), D["eatom0"].data_ptr(), D["vatom0"].data_ptr(),
            D["vatom1"].data_ptr())
        if code:
            raise RuntimeError(self.prefix + "cuda2lammps returned %d" % code)
        return {"forces": self.h_f.copy(), "eng": float(self.h_eng[0]), "eatom": self.h_eatom.copy(),
                "virial": self.h_vir.copy(), "cvatom": self.h_cv.copy() if self.cv else None}

    def step(self) -> dict:
        """One LAMMPS step as the reference runs it (lists sent every call)."""
        self.to_device(True)
        self.compute()
        return self.to_host()


class RefCudaNNAP(LammpsRef):
    """The reference's CUDA NNAP for one model on one device (FP32, one thread per atom)."""
    prefix = "jse_nnap_"

    def __init__(self, model, device: int = 0):
        import torch
        from . import model as OM
        pm = model if isinstance(model, PackedModel) else OM.load(model)
        if any(len(b.subs) != 1 for b in pm.basis):
            raise ValueError("models with one sub-basis per species only")
        self.pm = pm
        self.lib = C.CDLL(build(pm))
        self.dev = torch.device("cuda", device)
        self.torch = torch
        T = pm.ntypes
        self.T = T
        self._keep = []

        def dev_f32(a):
            a = np.ascontiguousarray(a, dtype=np.float32).reshape(-1)
            if a.size == 0:
                a = np.zeros(1, dtype=np.float32)
            t = torch.from_numpy(a.copy()).to(self.dev)
            self._keep.append(t)
            return t

        def table(tensors):
            t = torch.tensor([x.data_ptr() for x in tensors], dtype=torch.int64, device=self.dev)
            self._keep.append(t)
            return t
        self.hp = table([dev_f32(pm.basis[t].hparam) for t in range(T)])
        self.fpp = table([dev_f32(pm.basis[t].param) for t in range(T)])
        self.nnp = table([dev_f32(pm.nn[t].cparam) for t in range(T)])
        self.nrm = table([dev_f32(pm.norm[t]) for t in range(T)])
        self.nmerges = torch.ones(T, dtype=torch.int32, device=self.dev)
        cut = [dev_f32(np.array([pm.basis[t].subs[0].rcut ** 2])) for t in range(T)]
        self.cutsq = table(cut)
        ms = []
        for _ in range(T):
            m = torch.zeros(1, dtype=torch.int32, device=self.dev)
            self._keep.append(m)
            ms.append(m)
        self.merge_sorted = table(ms)
        self.type_map = torch.arange(T + 1, dtype=torch.int32, device=self.dev)
        L = self.lib
        P, I = C.c_void_p, C.c_int
        L.jse_nnap_computeLammpsCuda.argtypes = [I] * 7 + [P] * 27
        self._bind_io()

    def _work_buffers(self, nb: int, inum: int, nall: int) -> dict:
        torch, d = self.torch, self.dev
        f32, i32 = torch.float32, torch.int32
        return {"nldx": torch.zeros(nb, dtype=f32, device=d), "nldy": torch.zeros(nb, dtype=f32, device=d),
                "nldz": torch.zeros(nb, dtype=f32, device=d), "nltype": torch.zeros(nb, dtype=i32, device=d),
                "nlidx": torch.zeros(nb, dtype=i32, device=d), "neinum": torch.zeros(2 * inum, dtype=i32, device=d),
                "ctype": torch.zeros(inum, dtype=i32, device=d), "gdx": torch.zeros(nb, dtype=f32, device=d),
                "gdy": torch.zeros(nb, dtype=f32, device=d), "gdz": torch.zeros(nb, dtype=f32, device=d)}

    def compute(self, eflag: bool = True, vflag: bool = True, eflag_atom: bool = True):
        """jse_nnap_computeLammpsCuda (three kernels, then cudaDeviceSynchronize)."""
        D = self.d
        code = self.lib.jse_nnap_computeLammpsCuda(
            self.inum, self.nall, int(eflag), int(vflag), int(eflag_atom), 0, int(self.cv),
            D["x"].data_ptr(), D["type"].data_ptr(), D["ilist"].data_ptr(), self.nmerges.data_ptr(),
            self.merge_sorted.data_ptr(), self.cutsq.data_ptr(), D["num"].data_ptr(), D["first"].data_ptr(),
            self.type_map.data_ptr(), self.hp.data_ptr(), self.fpp.data_ptr(), self.nnp.data_ptr(),
            self.nrm.data_ptr(), D["f"].data_ptr(), D["eatom0"].data_ptr(), D["vatom0"].data_ptr(),
            D["vatom1"].data_ptr(), D["nldx"].data_ptr(), D["nldy"].data_ptr(), D["nldz"].data_ptr(),
            D["nltype"].data_ptr(), D["nlidx"].data_ptr(), D["neinum"].data_ptr(), D["ctype"].data_ptr(),
            D["gdx"].data_ptr(), D["gdy"].data_ptr(), D["gdz"].data_ptr())
        if code:
            raise RuntimeError("jse_nnap_computeLammpsCuda returned %d" % code)
