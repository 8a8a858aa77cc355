"""Golden fixtures of model shapes beyond the benchmark configurations (``shapes/*.npz``).

The model format allows any nmax <= 20 (WTypeBasis.java:56), lmax <= 12
(SphericalChebyshev.java:32), any number of species and weight type, and any hidden
widths (FeedForward.java:131-221); the reference compiles a kernel per model
(NNAPGEN.java:120-168).  These cases sweep those dimensions, including the reference's
default model (a spherical Chebyshev basis with no keys but its type: nmax 5, lmax 6,
rcut 6, hidden [32, 32]), radial nmax 0 / 3 / 20, lmax 0 / 1 / 12, five species with
every weight type, one species with fused weights, networks of one and of three hidden
layers and of widths that are not multiples of 16, and a 252-column descriptor.  Each
fixture holds the model JSON, the structure, the neighbour set and the FP64 energies,
forces, per-atom virials and descriptors of the reference's own arithmetic (expanded
and compiled by oracle/build.py without fast-math, driven over the oracle's neighbour
list), like make_golden.py.  NEP cases of shapes beyond GPUMD's defaults hold the
reference NEP arithmetic's outputs, like make_golden_nep.py.

Run from the repository root with a reference checkout available:

    python -m tests.golden.make_golden_shapes [case ...]
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from jse_gb300 import workloads as W  # noqa: E402
from oracle import model as OM, native as ON  # noqa: E402
from oracle import nep_model as NM, nep_ref as NR  # noqa: E402
from tests.golden.make_golden import _model, _normalised, _sph  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "shapes")

SYM5 = ["A", "B", "C", "D", "E"]


def _liquid(n, T, seed, tilt=None, rho=0.06):
    return W.random_liquid(n, rho, [1.0 / T] * T, 2.0, seed, tilt=tilt)


def cases():
    rng = np.random.default_rng(777)
    out = {}
    s1 = _liquid(90, 1, 51, tilt=0.1)
    s2 = _liquid(110, 2, 52)
    s3 = _liquid(120, 3, 53, tilt=0.08)
    s5 = _liquid(150, 5, 54)
    # the reference's default model: basis keys all defaulted, hidden_dims defaulted
    for name, syms, s in (("default_model_t1", ["A"], s1), ("default_model_t2", ["A", "B"], s2)):
        m = _model(syms, {"type": "spherical_chebyshev"}, [32, 32], 61)
        for mm in m["models"]:
            del mm["nn"]["hidden_dims"]
        out[name] = (_normalised(m, s), s)
    # radial bases: nmax 0, 3 (five species, exfull) and 20
    out["radial_nmax0"] = (_normalised(_model(["A", "B"], {"type": "chebyshev", "nmax": 0, "rcut": 5.0}, [16, 16], 62), s2), s2)
    out["radial_nmax3_t5_exfull"] = (_normalised(_model(SYM5, {"type": "chebyshev", "nmax": 3, "rcut": 5.5,
                                                               "wtype": "exfull"}, [16, 16], 63), s5), s5)
    out["radial_nmax20"] = (_normalised(_model(["A", "B"], {"type": "chebyshev", "nmax": 20, "rcut": 6.0}, [24, 16], 64), s2), s2)
    # spherical bases: lmax 0, 1 and 12
    out["sph_lmax0"] = (_normalised(_model(["A", "B"], _sph(5, 0, 5.5), [16, 16], 65), s2), s2)
    out["sph_lmax1_t3_full"] = (_normalised(_model(["A", "B", "C"], _sph(3, 1, 5.5, "full"), [16, 16], 66), s3), s3)
    out["sph_lmax12"] = (_normalised(_model(["A", "B"], _sph(4, 12, 5.0), [16, 16], 67), s2), s2)
    # five species with every weight type (nmax 3, lmax 3)
    for wt in ("default", "none", "full", "exfull"):
        out["t5_" + wt] = (_normalised(_model(SYM5, _sph(3, 3, 5.0, wt), [16, 16], 70), s5), s5)
    fw5 = rng.uniform(-1, 1, 5 * 2).tolist()
    out["t5_fuse"] = (_normalised(_model(SYM5, _sph(3, 3, 5.0, "fuse", fuse_size=2, fuse_weight=fw5), [16, 16], 71), s5), s5)
    out["t5_exfuse"] = (_normalised(_model(SYM5, _sph(3, 3, 5.0, "exfuse", fuse_size=2, fuse_weight=fw5), [16, 16], 72), s5), s5)
    rw5 = rng.uniform(-1, 1, 6 * 5 * 4).tolist()
    out["t5_rfuse"] = (_normalised(_model(SYM5, _sph(3, 3, 5.0, "rfuse", rfuse_size=6, rfuse_weight=rw5), [16, 16], 73), s5), s5)
    # one species: fused weights and exfull
    fw1 = rng.uniform(-1, 1, 3).tolist()
    out["t1_fuse"] = (_normalised(_model(["A"], _sph(4, 3, 5.5, "fuse", fuse_size=3, fuse_weight=fw1), [16, 16], 74), s1), s1)
    out["t1_exfull"] = (_normalised(_model(["A"], _sph(4, 3, 5.5, "exfull"), [16, 16], 75), s1), s1)
    # networks: one hidden layer of 20, three layers 48 / 24 / 12, two layers of 100
    out["hidden_20"] = (_normalised(_model(["A", "B"], _sph(4, 4, 5.5), [20], 76), s2), s2)
    out["hidden_48_24_12"] = (_normalised(_model(["A"], {"type": "chebyshev", "nmax": 10, "rcut": 6.0},
                                                 [48, 24, 12], 77), s1), s1)
    out["hidden_100_100"] = (_normalised(_model(["A", "B", "C"], W.C2_BASIS, [100, 100], 78), s3), s3)
    # 252 descriptor columns: the liquid's basis with the exfull weight type
    out["exfull_d252"] = (_normalised(_model(["A", "B", "C"], dict(W.C2_BASIS, wtype="exfull"), [64, 64], 79), s3), s3)
    return out


NEP_CASES = {
    # (symbols, version, cutoffs, n_max, basis_size, l_max, neurons, atoms)
    "nep_small": (["Si", "O"], 4, (5.0, 4.0), (3, 3), (5, 5), (4, 2, 1), 6, 120),
    "nep_large": (["Ga", "N", "O"], 5, (5.5, 4.5), (8, 6), (12, 10), (6, 2, 0), 24, 150),
}


def make_nnap(name, model, s):
    pm = OM.load(model)
    o = ON.compute(pm, s.x, s.types, s.box_kind, s.box)
    nl = o["nl"]
    ref = ON.RefLib(pm)
    r = ref.compute(s.types, nl)
    fp = ref.fp(s.types, nl)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), model_json=np.array(json.dumps(model)), x=s.x,
                        types=s.types, box=s.box, box_kind=np.array(s.box_kind), xw=o["xw"], nl_offsets=nl.offsets,
                        nl_j=nl.j, nl_img=nl.img, energies=r["energies"], forces=r["forces"], virials=r["virials"],
                        fp=fp)
    D = [b.size for b in pm.basis]
    print("%-24s n=%4d pairs=%6d D=%s E=%.10f" % (name, len(s.types), len(nl.j), D, r["energy"]))


def make_nep(name):
    symbols, version, rc, n_max, basis, l_max, neurons, n = NEP_CASES[name]
    seed = 2000 + sum(map(ord, name))
    text = NM.write(symbols, version=version, rc=rc, n_max=n_max, basis=basis, l_max=l_max, neurons=neurons,
                    seed=seed)
    m = NM.load(text)
    s = W.random_liquid(n, 0.06, [1.0 / len(symbols)] * len(symbols), 2.0, seed)
    xw = ON.wrap(s.x, s.box_kind, s.box)
    nl = ON.neighbors(xw, s.box_kind, s.box, max(m.rc_radial, m.rc_angular))
    o = NR.RefNEP(m).compute(s.types - 1, nl)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), nep=np.array(text), x=s.x, types=s.types,
                        box=np.asarray(s.box, dtype=np.float64).reshape(9), box_kind=np.int32(s.box_kind),
                        energies=o["energies"], forces=o["forces"], virials=o["virials"])
    print("%-24s n=%4d E=%.6f" % (name, len(s.types), o["energy"]))


def main():
    os.makedirs(OUT, exist_ok=True)
    only = set(sys.argv[1:])
    for name, (model, s) in cases().items():
        if not only or name in only:
            make_nnap(name, model, s)
    for name in NEP_CASES:
        if not only or name in only:
            make_nep(name)


if __name__ == "__main__":
    main()
