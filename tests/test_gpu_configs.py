"""The benchmark configurations at their stated sizes against the reference's FP64 arithmetic.

* the 32000-atom ternary liquid (spherical Chebyshev nmax 8 lmax 6, 126 -> 64 -> 64 -> 1),
  plain FP32 and mixed precision;
* the 1048576-atom binary glass in a LAMMPS triclinic box (nmax 8 lmax 4, 90 -> 64 -> 64 -> 1),
  mixed precision;
* every structure of the 1024-structure mixed-size batch (32 to 2048 atoms, half triclinic,
  the liquid's model) evaluated by one batched call, mixed precision.

Each uses the benchmark's own model (normalisation from tests/golden/bench_norm.json).
The expected values come from the reference's own per-atom arithmetic (its NNAP headers
expanded and compiled without fast-math into oracle/_ref, run on all host threads over
the oracle's neighbour list), or from the FP64 oracle where that build is absent.

Targets of the mixed-precision path: bit-exact neighbour sets (every (i, j, image) triple); force
RMSE <= 1e-3 eV/A; |E - E_ref| / N <= 1e-5 eV/atom (per structure for the batch); max
|dE_i| <= 1e-4 eV; virials within 1e-3 relative.
"""
import os

import numpy as np
import pytest

import bench
from jse_gb300 import workloads as W
from oracle import model as OM, native as ON

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def _keys(offsets, j, img):
    """One int64 per pair: atom i, neighbour j (20 bits each) and the image (8 bits a component)."""
    offsets = np.asarray(offsets, dtype=np.int64)
    i = np.repeat(np.arange(len(offsets) - 1, dtype=np.int64), np.diff(offsets))
    im = np.asarray(img, dtype=np.int64).reshape(-1, 3) + 128
    k = (i << 44) | (np.asarray(j, dtype=np.int64) << 24) | (im[:, 0] << 16) | (im[:, 1] << 8) | im[:, 2]
    return np.sort(k)


class _Ref:
    """Reference outputs of a model over neighbour lists (the reference's exact build when
    present, else the FP64 oracle)."""

    def __init__(self, model):
        self.pm = OM.load(model)
        try:
            self.lib = ON.RefLib(self.pm)
        except (FileNotFoundError, OSError, RuntimeError):
            self.lib = None

    def compute(self, s, nl):
        if self.lib is not None:
            return self.lib.compute(s.types, nl, nthreads=THREADS)
        return ON.compute(self.pm, s.x, s.types, s.box_kind, s.box, nl=nl)


def _check(o, r, n, label):
    f_rmse = float(np.sqrt(((o["forces"] - r["forces"]) ** 2).mean()))
    e_err = abs(o["energy"] - r["energy"]) / n
    e_max = float(np.abs(o["energies"] - r["energies"]).max())
    print("%s: force RMSE %.2e eV/A, |dE|/N %.2e eV/atom, max |dE_i| %.2e eV" % (label, f_rmse, e_err, e_max))
    assert f_rmse <= 1e-3, label
    assert e_err <= 1e-5, label
    assert e_max <= 1e-4, label
    np.testing.assert_allclose(o["virial"], r["virial"], rtol=1e-3, atol=1e-3 * max(1.0, np.abs(r["virial"]).max()))


def _single(cfg, s, precisions):
    from jse_gb300.nnap import NNAP
    model = bench.bench_model(cfg)
    ref = _Ref(model)
    nl = ON.neighbors(ON.wrap(s.x, s.box_kind, s.box), s.box_kind, s.box, ref.pm.rcut_max)
    r = ref.compute(s, nl)
    r["energy"] = float(r["energies"].sum())
    for precision in precisions:
        with NNAP(model, precision=precision) as p:
            if precision == precisions[0]:
                off, j, img = p.neighborList(s)
                assert np.array_equal(np.diff(off), nl.counts)
                assert np.array_equal(_keys(off, j, img), _keys(nl.offsets, nl.j, nl.img))
            o = p.calEnergyForceVirials(s, per_atom_virial=False)
        _check(o, r, s.natoms, "%s %d atoms %s" % (cfg, s.natoms, precision))


def test_liquid_32000_atoms():
    _single("c2", W.c2_structure(), ["fp32", "mixed"])


def test_glass_1048576_atoms():
    s = W.c3_structure()
    assert s.natoms == 1048576 and s.box_kind == W.BOX_LMP
    _single("c3", s, ["mixed"])


def test_batch_1024_structures():
    """One batched mixed-precision call over the whole batch; every structure against the
    reference (energy per structure, forces per atom) and its neighbour set bit-exact."""
    from jse_gb300.nnap import NNAP
    structs = W.c4_structures()
    assert len(structs) == 1024
    model = bench.bench_model("c4")
    ref = _Ref(model)
    nls = [ON.neighbors(ON.wrap(s.x, s.box_kind, s.box), s.box_kind, s.box, ref.pm.rcut_max) for s in structs]
    # the reference over the concatenated structures (independent atoms; indices shifted)
    smp = bench._RefSample(structs, ref.pm.rcut_max, 1 << 30)
    assert smp.nstruct == 1024
    cat = W.Structure(np.concatenate([s.x for s in structs]), smp.types, np.eye(3), 0)
    rr = ref.compute(cat, smp.nl)
    with NNAP(model, precision="mixed") as p:
        out = p.calEnergyForceVirialsBatch(structs, per_atom_virial=False)
        a0 = 0
        for k, (s, nl, o) in enumerate(zip(structs, nls, out)):
            n = s.natoms
            off, j, img = p.neighborList(s)
            assert np.array_equal(_keys(off, j, img), _keys(nl.offsets, nl.j, nl.img)), k
            r = {"energies": rr["energies"][a0:a0 + n], "forces": rr["forces"][a0:a0 + n],
                 "virial": rr["virials"][a0:a0 + n].sum(0)}
            r["energy"] = float(r["energies"].sum())
            _check(o, r, n, "batch structure %d (%d atoms, box kind %d)" % (k, n, s.box_kind))
            a0 += n
