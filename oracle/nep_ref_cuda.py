"""The reference's own CUDA path for NEP, compiled here (baseline only).

TEST INFRASTRUCTURE ONLY.  The reference's LAMMPS GPU kernels for NEP
(nep_interface_cuda.cu: initLammpsNeiKernel, computeLammpsKernel with GPUMD's
find_descriptor / find_force_radial / find_force_angular, collectLammpsResultsKernel; one
thread per atom, FP32) are expanded by oracle/nepgen.py with the picks NEP makes for a
CUDA model (NEP.java:594-600: [ARCH] cuda, [PRECISION] single, block size 256) into
oracle/_ref/nep_<key>_cuda/src and compiled with nvcc for sm_103a at -O3 into
libnepref_cuda.so.  RefCudaNEP uploads the model as NEP does for CUDA (ParaMB / ANN
parse2cuda: q_scaler, per-species network pointer tables, b1, the descriptor
coefficients) and runs jse_nep_lammps2cuda / jse_nep_computeLammpsCuda /
jse_nep_cuda2lammps per step like NEP.computeLammpsCuda (NEP.java:262-348).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from . import nepgen
from .build import REF_OUT
from .nep_model import NEPModel
from .nep_ref import nep_src_dir, shape_key
from .ref_cuda import LammpsRef

BLOCK = 256       # NEP.Conf.CUDA_BLOCKSIZE default (NEP.java:59)
NUM_OF_ABC = 80   # nep_core.hpp: angular components kept per channel (L_max = 8)
NUM_ELEMENTS = 94


def expand(m: NEPModel) -> str:
    src = os.path.join(REF_OUT, shape_key(m) + "_cuda", "src")
    if not os.path.exists(os.path.join(src, "nep_interface_cuda.cu")):
        sd = nep_src_dir()
        if not os.path.isdir(sd):
            raise FileNotFoundError("reference NEP sources are not available")
        g = nepgen.gen_map(m)
        g["[ARCH]"] = "cuda"
        g["[PRECISION]"] = "single"
        g["NEPGEN_CUDA_BLOCKSIZE"] = BLOCK
        os.makedirs(src, exist_ok=True)
        for name in ("nep_core.hpp", "nep_interface_cuda.cu"):
            with open(os.path.join(sd, name)) as f:
                lines = f.read().split("\n")
            with open(os.path.join(src, name), "w") as f:
                f.write("\n".join(nepgen.process(lines, g)))
    return src


def build(m: NEPModel) -> str:
    src = expand(m)
    out = os.path.join(os.path.dirname(src), "libnepref_cuda.so")
    cu = os.path.join(src, "nep_interface_cuda.cu")
    deps = [cu, os.path.join(src, "nep_core.hpp")]
    if not os.path.exists(out) or any(os.path.getmtime(p) > os.path.getmtime(out) for p in deps):
        nvcc = os.environ.get("NVCC") or "nvcc"
        cmd = [nvcc, "-O3", "-std=c++14", "-gencode", "arch=compute_103a,code=sm_103a", "-Xcompiler", "-fPIC",
               "-shared", "-w", "-I", src, cu, "-o", out]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("building the reference NEP CUDA path failed:\n" + r.stderr[-3000:])
    return out


class RefCudaNEP(LammpsRef):
    """The reference's CUDA NEP for one model on one device (FP32, one thread per atom)."""
    prefix = "jse_nep_"

    def __init__(self, m: NEPModel, device: int = 0):
        import torch
        self.m = m
        self.lib = C.CDLL(build(m))
        self.torch = torch
        self.dev = torch.device("cuda", device)
        self.T = m.ntypes
        self._keep = []

        def dev(a, dtype):
            t = torch.from_numpy(np.ascontiguousarray(a, dtype=dtype).reshape(-1).copy()).to(self.dev)
            self._keep.append(t)
            return t

        def table(ts):
            t = torch.tensor([x.data_ptr() for x in ts], dtype=torch.int64, device=self.dev)
            self._keep.append(t)
            return t
        qs = np.zeros(max(140, m.dim), dtype=np.float32)
        qs[:m.dim] = m.q_scaler
        self.q_scaler = dev(qs, np.float32)
        an = np.zeros(NUM_ELEMENTS)
        an[:m.ntypes] = m.atomic_numbers0
        self.atomic_numbers = dev(an, np.int32)
        w0, b0, w1 = [], [], []
        for t in range(m.ntypes):
            a, b, c, extra = m.ann(t)
            w0.append(dev(a, np.float32))
            b0.append(dev(b, np.float32))
            w1.append(dev(np.concatenate([c, [extra]]) if m.version == 5 else c, np.float32))
        self.w0, self.b0, self.w1 = table(w0), table(b0), table(w1)
        self.b1 = dev(np.array([m.b1]), np.float32)
        self.c = dev(m.c, np.float32)
        self.type_map = dev(np.arange(-1, m.ntypes), np.int32)   # LAMMPS type t -> NEP type t - 1
        self.cutsq = max(m.rc_radial, m.rc_angular) ** 2
        P, I = C.c_void_p, C.c_int
        self.lib.jse_nep_computeLammpsCuda.argtypes = [I] * 7 + [P] * 5 + [C.c_double] + [P] * 29
        self._bind_io()

    def _work_buffers(self, nb: int, inum: int, nall: int) -> dict:
        torch, d = self.torch, self.dev
        f32, i32 = torch.float32, torch.int32
        m = self.m
        return {"nldx": torch.zeros(nb, dtype=f32, device=d), "nldy": torch.zeros(nb, dtype=f32, device=d),
                "nldz": torch.zeros(nb, dtype=f32, device=d), "nltype": torch.zeros(nb, dtype=i32, device=d),
                "nlidx": torch.zeros(nb, dtype=i32, device=d), "neinum": torch.zeros(inum, dtype=i32, device=d),
                "ctype": torch.zeros(inum, dtype=i32, device=d), "nlfx": torch.zeros(nb, dtype=f32, device=d),
                "nlfy": torch.zeros(nb, dtype=f32, device=d), "nlfz": torch.zeros(nb, dtype=f32, device=d),
                "fp": torch.zeros(inum * m.dim, dtype=f32, device=d),
                "sum_fxyz": torch.zeros(inum * (m.n_max_angular + 1) * NUM_OF_ABC, dtype=f32, device=d)}

    def compute(self, eflag: bool = True, vflag: bool = True, eflag_atom: bool = True):
        """jse_nep_computeLammpsCuda (three kernels, then cudaDeviceSynchronize)."""
        D = self.d
        code = self.lib.jse_nep_computeLammpsCuda(
            self.inum, self.nall, int(eflag), int(vflag), int(eflag_atom), 0, int(self.cv),
            D["x"].data_ptr(), D["type"].data_ptr(), D["ilist"].data_ptr(), D["num"].data_ptr(), D["first"].data_ptr(),
            self.cutsq, self.type_map.data_ptr(), self.atomic_numbers.data_ptr(), self.q_scaler.data_ptr(),
            self.w0.data_ptr(), self.b0.data_ptr(), self.w1.data_ptr(), self.b1.data_ptr(), self.c.data_ptr(),
            None, None, None, None, None,
            D["f"].data_ptr(), D["eatom0"].data_ptr(), D["vatom0"].data_ptr(), D["vatom1"].data_ptr(),
            D["nldx"].data_ptr(), D["nldy"].data_ptr(), D["nldz"].data_ptr(), D["nltype"].data_ptr(),
            D["nlidx"].data_ptr(), D["neinum"].data_ptr(), D["ctype"].data_ptr(),
            D["nlfx"].data_ptr(), D["nlfy"].data_ptr(), D["nlfz"].data_ptr(), D["fp"].data_ptr(),
            D["sum_fxyz"].data_ptr())
        if code:
            raise RuntimeError("jse_nep_computeLammpsCuda returned %d" % code)
