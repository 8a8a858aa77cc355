"""Descriptor normalisation of the benchmark models (``bench_norm.json`` in this folder).

A trained NNAP model carries ``norm_mu`` / ``norm_sigma``: per species, the mean and the
standard deviation (+ 1e-3) of its descriptor columns over the training structures.  The
benchmark's seeded models get theirs from the FP64 oracle's descriptors of one seeded
structure of their workload, so that both benchmark arms (this build and the reference's
CPU arithmetic) evaluate exactly the same model file:

  c1  the 4000-atom perturbed FCC lattice;
  c2  the 32000-atom ternary liquid (also used for the batch and serving workloads,
      whose model is the liquid's);
  c3  a 32768-atom sample of the binary glass generator (the 1048576-atom glass has the
      same statistics).

Run from the repository root after any change of the structure generator:

    python -m tests.golden.make_bench_norm
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

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "bench_norm.json")


def stats(cfg: str, s) -> dict:
    pm = OM.load(W.model_for(cfg))
    fp = ON.compute(pm, s.x, s.types, s.box_kind, s.box, want_fp=True)["fp"]
    mu, sg = [], []
    for t in range(pm.ntypes):
        sel = fp[s.types == t + 1, :pm.basis[t].size]
        mu.append([float(v) for v in sel.mean(0)])
        sg.append([float(v) for v in sel.std(0) + 1e-3])
    return {"mu": mu, "sigma": sg, "structure": "%d atoms" % s.natoms}


def main():
    out = {"c1": stats("c1", W.c1_structure()), "c2": stats("c2", W.c2_structure()),
           "c3": stats("c3", W.c3_structure(32768))}
    with open(OUT, "w") as f:
        json.dump(out, f, indent=0)
    print(OUT)


if __name__ == "__main__":
    main()
