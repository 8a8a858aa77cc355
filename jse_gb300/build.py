"""Build the CUDA library ``jse_gb300/libnnap_gb300.so`` for sm_103a with nvcc.

Translation units are compiled in parallel into ``jse_gb300/_build`` and linked with
the CUDA runtime.  Host code is compiled without floating-point contraction so the
box arithmetic rounds exactly like the reference's Java doubles.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libnnap_gb300.so")
BUILD = os.path.join(HERE, "_build")
SOURCES = ["nnap_api.cu", "nnap_server.cu", "nnap_lammps.cu", "k_struct.cu", "k_resident.cu", "k_lammps.cu",
           "k_desc.cu", "k_desc_gen.cu", "k_net.cu", "k_zbl.cu", "k_net_tc.cu", "nnap_noalloc.cu", "k_train.cu", "nnap_train.cu",
           "model.cpp", "nep_model.cpp", "invariants.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _flags(verbose_ptxas: bool):
    f = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr",
         "-I", os.path.join(HERE, "..", "include")] + ARCH
    if verbose_ptxas:
        f += ["-Xptxas", "-v"]
    return f


def _stale(obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose_ptxas: bool = False, jobs: int = 0) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "nnap_gb300.h"))
    cmds, objs = [], []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmds.append([nvcc(), "-c", src, "-o", obj] + _flags(verbose_ptxas))

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(cmd), r.stderr[-6000:]))
        return r.stderr

    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        logs = list(ex.map(run, cmds))
    if verbose_ptxas:
        for lg in logs:
            sys.stderr.write(lg)
    if cmds or not os.path.exists(OUT):
        r = subprocess.run([nvcc(), "-shared", "-o", OUT] + objs + ARCH + ["-lcudart"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s" % r.stderr[-4000:])
    return OUT


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv)
    print(OUT)
