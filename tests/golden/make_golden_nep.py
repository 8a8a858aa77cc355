"""Generate the NEP golden fixtures (tests/golden/nep_*.npz) from the reference's own arithmetic.

Run from the repository root, where a reference checkout is available
(``$JSE_REFERENCE``, else a ``reference`` folder beside the repository):

    python -m tests.golden.make_golden_nep

For every case the reference's NEP sources are expanded for the model
(``oracle/nepgen.py``) and compiled without fast-math (``oracle/nep_ref.py``); the
reference's per-atom ``jse_nep_calEnergyForce`` then runs over the neighbour list of the
oracle's restatement of ``NeighborListGetter`` and ``oracle/nep_driver.cpp`` scatters
energies, forces and per-atom virials like ``NEP.calEnergyForceVirial``.

Each ``nep_<case>.npz`` holds the nep.txt text of a seeded random model, the structure
(1-based species, as the potential's callers pass them) and the reference's FP64 outputs.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from jse_gb300 import workloads as W  # noqa: E402
from oracle import native as ON, nep_model as NM, nep_ref as NR  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))

# name: (symbols, version, rc (R, A), n_max, basis, l_max (3-, 4-, 5-body), neurons, structure
#        (kind, atoms, tilt[, minimum separation]) [, ZBL: (rc_inner, rc_outer) or "flexible"
#        [, type-wise cutoff factors (radial, angular, ZBL)]])
CASES = {
    "nep4_binary": (["Si", "O"], 4, (5.0, 4.0), (4, 4), (8, 8), (4, 2, 1), 16, ("liquid", 150, 0.1)),
    "nep3_single": (["C"], 3, (4.5, 4.5), (4, 4), (8, 8), (4, 0, 0), 8, ("liquid", 90, None)),
    "nep5_ternary": (["A", "B", "C"], 5, (5.5, 4.2), (4, 4), (8, 8), (4, 2, 0), 12, ("liquid", 200, 0.05)),
    "nep4_wide": (["Ga", "N"], 4, (5.2, 4.6), (6, 6), (8, 8), (4, 2, 1), 20, ("liquid", 120, None)),
    "nep4_5body": (["Li", "P", "S"], 4, (6.0, 4.0), (4, 4), (8, 8), (4, 0, 1), 10, ("liquid", 160, 0.08)),
    # ZBL: the fixed universal form with its two radii, and the flexible per-pair form; a 1.3 A
    # minimum separation puts pairs inside rc_inner as well as in the switching range
    "nep4_zbl": (["Si", "O"], 4, (5.0, 4.0), (4, 4), (8, 8), (4, 2, 1), 12, ("liquid", 150, 0.1, 1.3),
                 (1.6, 2.3)),
    "nep3_zbl_flex": (["W", "Be"], 3, (5.0, 4.0), (4, 4), (8, 8), (4, 2, 0), 8, ("liquid", 120, None, 1.3),
                      "flexible"),
    # type-wise cutoffs: Si-Si, Si-O and O-O pairs each get their own radial and angular
    # cutoffs inside the global ones; the second case also shrinks the fixed ZBL radii per pair
    "nep4_typewise": (["Si", "O"], 4, (6.0, 5.0), (4, 4), (8, 8), (4, 2, 1), 12, ("liquid", 160, 0.07),
                      None, (2.0, 1.6, 0.0)),
    "nep5_typewise_zbl": (["Ga", "N", "O"], 5, (6.0, 4.5), (4, 4), (8, 8), (4, 2, 0), 10,
                          ("liquid", 150, None, 1.3), (1.0, 2.2), (1.9, 1.5, 0.7)),
}


def structure(spec, T, seed):
    kind, n, tilt = spec[:3]
    rmin = spec[3] if len(spec) > 3 else 2.0
    return W.random_liquid(n, 0.06, [1.0 / T] * T, rmin, seed, tilt=tilt)


def make(name):
    symbols, version, rc, n_max, basis, l_max, neurons, spec = CASES[name][:8]
    zbl = CASES[name][8] if len(CASES[name]) > 8 else None
    typewise = CASES[name][9] if len(CASES[name]) > 9 else None
    seed = 1000 + sum(map(ord, name))
    text = NM.write(symbols, version=version, rc=rc, n_max=n_max, basis=basis, l_max=l_max, neurons=neurons,
                    seed=seed, zbl=zbl, typewise=typewise)
    m = NM.load(text)
    s = structure(spec, len(symbols), seed)
    xw = ON.wrap(s.x, s.box_kind, s.box)
    nl = ON.neighbors(xw, s.box_kind, s.box, max(m.rc_radial, m.rc_angular))
    out = NR.RefNEP(m).compute(s.types - 1, nl)
    np.savez_compressed(os.path.join(HERE, "nep_%s.npz" % name), nep=np.array(text), x=s.x, types=s.types,
                        box=np.asarray(s.box, dtype=np.float64).reshape(9), box_kind=np.int32(s.box_kind),
                        energies=out["energies"], forces=out["forces"], virials=out["virials"])
    print("%-14s n=%d  E=%.6f  |F|max=%.3f" % (name, len(s.types), out["energy"], np.abs(out["forces"]).max()))


if __name__ == "__main__":
    for k in (sys.argv[1:] or CASES):
        make(k)
