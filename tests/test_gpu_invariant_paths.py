"""Invariant (l3max / l4max) columns through every evaluation entry point.

The golden fixtures pin nnap_compute for models with three- and four-body invariant
columns.  Here the same model runs through the other entry points, which share the
descriptor pipeline but not its callers: the batched call, the LAMMPS-style boundary
(full lists with ghosts) and the serving loop (resident Verlet rows).  Each must agree
with nnap_compute on the same structure.
"""
import json
import os

import numpy as np
import pytest

from jse_gb300 import workloads as W
from tests.conftest import GOLDEN_DIR, Case

pytestmark = pytest.mark.gpu

E_TOL = 1e-5   # eV per atom (the path's energy target)
F_TOL = 1e-4   # eV/A


@pytest.fixture(scope="module", params=["sph_bispectrum", "sph_bispectrum_high"])
def model(request):
    return Case(os.path.join(GOLDEN_DIR, request.param + ".npz")).model


def _structs(model):
    T = len(model["models"])
    fr = [1.0 / T] * T
    return [W.random_liquid(n, 0.06, fr, 2.0, 300 + n, tilt=0.1 if n % 2 else None) for n in (150, 601, 1200)]


def test_batch_equals_single(model):
    from jse_gb300.nnap import NNAP
    structs = _structs(model)
    with NNAP(json.dumps(model)) as p:
        batch = p.calEnergyForceVirialsBatch(structs)
        for s, b in zip(structs, batch):
            r = p.calEnergyForceVirials(s)
            assert abs(b["energy"] - r["energy"]) / s.natoms <= E_TOL
            assert np.max(np.abs(b["forces"] - r["forces"])) <= F_TOL


def test_lammps_form_equals_periodic(model):
    from jse_gb300.nnap import NNAP
    from tests.test_gpu_lammps import _lammps_form, _reverse
    s = _structs(model)[1]
    with NNAP(json.dumps(model)) as p:
        x, types, lists, owner, xw = _lammps_form(s, p.rcutMax() + 0.4)
        n = s.natoms
        out = p.computeLammps(np.arange(n), lists, x, types)
        ref = p.calEnergyForceVirials(W.Structure(xw, s.types, s.box, s.box_kind))
    assert np.max(np.abs(out["eatom"][:n] - ref["energies"])) <= E_TOL
    f = _reverse(out["forces"], n, owner)
    assert np.max(np.abs(f - ref["forces"])) <= F_TOL


def test_server_equals_compute(model):
    from jse_gb300.nnap import NNAP
    from jse_gb300.serve import NNAPServer
    s = _structs(model)[2]
    rng = np.random.default_rng(8)
    ref = NNAP(json.dumps(model))
    with NNAP(json.dumps(model)) as p, NNAPServer(p, skin=0.5, memory_budget=4e9) as srv:
        slot = srv.admit(s)
        x = s.x.copy()
        for k in range(3):
            if k:
                x = x + rng.normal(0.0, 0.02, size=x.shape)
            out = srv.step([slot], [x], energies=True)
            r = ref.calEnergyForceVirials(W.Structure(x, s.types, s.box, s.box_kind), per_atom_virial=False)
            assert abs(out["energy"][0] - r["energy"]) / s.natoms <= E_TOL
            assert np.max(np.abs(out["forces"] - r["forces"])) <= F_TOL
    ref.close()
