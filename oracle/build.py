"""Build recipes for the CPU oracle and for the reference's own per-atom arithmetic.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

* ``build_oracle()``  compiles ``nnap_oracle.cpp`` (FP64, no fast-math, no FMA contraction)
  into ``oracle/liboracle.so``.
* ``expand_ref(model)`` expands the reference's headers for one model shape from a
  reference checkout (``$JSE_REFERENCE``, else a ``reference`` folder beside the repository) into
  ``oracle/_ref/<shape>/src`` with :mod:`oracle.nnapgen`.  This needs the checkout and
  therefore only runs where it exists; the expanded sources travel with the tree.
* ``build_ref(shape)`` compiles an expanded shape with ``ref_driver.cpp`` into
  ``oracle/_ref/<shape>/libnnapref.so`` (FP64, ``-O2``, no fast-math: parity values) and
  ``libnnapref_fast.so`` (``-O3 -ffast-math``: the reference's default JIT optimisation
  level ``OPTIM_BASE`` from ``CMakeLists.txt:44-52`` without the host-specific
  ``-march=native -mfma``, so it also builds on aarch64).
"""
from __future__ import annotations

import glob
import hashlib
import json
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")


def reference_root() -> str:
    """The reference checkout: ``$JSE_REFERENCE``, else a ``reference`` folder beside this
    repository."""
    return os.environ.get("JSE_REFERENCE",
                          os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))


def reference_src_dir() -> str:
    root = reference_root()
    return os.path.join(root, "src", "nnap", "resources", "assets", "nnap", "src")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), r.stderr[-4000:]))


def _stale(out: str, srcs) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "nnap_oracle.cpp")
    out = os.path.join(HERE, "liboracle.so")
    if force or _stale(out, [src]):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", src, "-o", out])
    return out


def shape_key(model) -> str:
    from .nnapgen import gen_map
    g = gen_map(model)
    blob = json.dumps({k: v for k, v in g.items()}, sort_keys=True, default=str)
    return "m" + hashlib.sha1(blob.encode()).hexdigest()[:12]


def expand_ref(model) -> str:
    """Expand the reference headers for ``model``'s shape; returns the shape key."""
    from .nnapgen import expand, gen_map
    key = shape_key(model)
    out = os.path.join(REF_OUT, key, "src")
    src = reference_src_dir()
    if os.path.isdir(src):
        if not os.path.exists(os.path.join(out, "nnap_interface.cpp")):
            expand(src, out, gen_map(model))
    return key


def build_ref(key: str, force: bool = False) -> dict:
    """Compile an expanded shape; returns {'exact': path, 'fast': path} (missing when unexpanded)."""
    d = os.path.join(REF_OUT, key)
    src = os.path.join(d, "src", "nnap_interface.cpp")
    drv = os.path.join(HERE, "ref_driver.cpp")
    outs = {}
    if not os.path.exists(src):
        return outs
    deps = [src, drv] + glob.glob(os.path.join(d, "src", "*.hpp"))
    jobs = []
    for name, flags in (("exact", ["-O2", "-ffp-contract=off"]), ("fast", ["-O3", "-ffast-math"])):
        out = os.path.join(d, "libnnapref.so" if name == "exact" else "libnnapref_fast.so")
        outs[name] = out
        if force or _stale(out, deps):
            jobs.append(["g++", "-std=c++14", "-fPIC", "-shared", "-pthread", "-w"] + flags +
                        ["-I", os.path.join(d, "src"), src, drv, "-o", out])
    with ThreadPoolExecutor(max_workers=4) as ex:
        list(ex.map(_run, jobs))
    return outs


def build_all_ref() -> None:
    """Compile every expanded shape present under ``oracle/_ref``."""
    keys = [os.path.basename(os.path.dirname(p)) for p in glob.glob(os.path.join(REF_OUT, "*", "src"))]
    with ThreadPoolExecutor(max_workers=4) as ex:
        list(ex.map(build_ref, keys))
