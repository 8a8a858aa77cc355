"""Compact rows for a spherical sub-basis with a short cutoff.

When a spherical sub-basis after the first runs on the channel-space kernels and its
cutoff is at most 0.85 of the neighbour cutoff (a merged NNAP basis, or NEP's angular
cutoff), one extra kernel copies each row's entries within that cutoff into a compact row
and the spherical kernels scan those.  Results must equal the FP64 oracle like any other
model, through the single, batched and LAMMPS-style entry points.
"""
import numpy as np
import pytest

from jse_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _model(rc_sph):
    from tests.golden.make_golden import _model as make, _sph
    rng = np.random.default_rng(77)
    rw = rng.uniform(-1, 1, 5 * 8).tolist()
    basis = {"type": "merge", "basis": [{"type": "chebyshev", "nmax": 5, "rcut": 6.0},
                                        _sph(3, 3, rc_sph, "rfuse", rfuse_size=5, rfuse_weight=rw, rfuse_scale=0.4)]}
    return make(["A", "B"], basis, [8, 8], 41)


def test_subrows_match_oracle_and_add_one_launch():
    from jse_gb300.nnap import NNAP
    from oracle import model as OM, native as ON
    s = W.random_liquid(400, 0.06, [0.5, 0.5], 2.0, 42, tilt=0.1)
    launches = []
    for rc in (4.5, 6.0):
        model = _model(rc)
        with NNAP(model) as p:
            o = p.calEnergyForceVirials(s)
            launches.append(p.lastLaunchCount())
        r = ON.compute(OM.load(model), s.x, s.types, s.box_kind, s.box)
        assert np.max(np.abs(o["energies"] - r["energies"])) <= 1e-5
        assert np.max(np.abs(o["forces"] - r["forces"])) <= 1e-4
        assert np.max(np.abs(o["virials"] - r["virials"])) <= 1e-3
    assert launches[0] == launches[1] + 1   # the compact-row kernel


def test_subrows_batch_and_lammps_agree():
    from jse_gb300.nnap import NNAP
    from tests.test_gpu_lammps import _lammps_form, _reverse
    structs = [W.random_liquid(n, 0.06, [0.5, 0.5], 2.0, 60 + n, tilt=0.1 if n % 2 else None) for n in (90, 333, 800)]
    with NNAP(_model(4.5)) as p:
        batch = p.calEnergyForceVirialsBatch(structs)
        for s, b in zip(structs, batch):
            r = p.calEnergyForceVirials(s)
            assert abs(b["energy"] - r["energy"]) / s.natoms <= 1e-5
            assert np.max(np.abs(b["forces"] - r["forces"])) <= 1e-4
        s = structs[1]
        x, types, lists, owner, xw = _lammps_form(s, p.rcutMax() + 0.4)
        n = s.natoms
        out = p.computeLammps(np.arange(n), lists, x, types)
        ref = p.calEnergyForceVirials(W.Structure(xw, s.types, s.box, s.box_kind))
        assert np.max(np.abs(out["eatom"][:n] - ref["energies"])) <= 1e-5
        assert np.max(np.abs(_reverse(out["forces"], n, owner) - ref["forces"])) <= 1e-4
