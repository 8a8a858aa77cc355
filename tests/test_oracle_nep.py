"""The NEP oracle against the reference's own outputs (CPU).

tests/golden/nep_*.npz hold FP64 energies, forces and per-atom virials of the reference's
compiled NEP arithmetic (tests/golden/make_golden_nep.py).  The numpy restatement
(oracle/nep_oracle.py) must reproduce the energies; its energy gradient, taken by central
differences, must reproduce the reference's forces, which pins the force sign convention
the GPU path follows.
"""
import glob
import os

import numpy as np
import pytest

from oracle import native as ON, nep_model as NM, nep_oracle as NO
from tests.conftest import GOLDEN_DIR

CASES = sorted(glob.glob(os.path.join(GOLDEN_DIR, "nep_*.npz")))


def _load(path):
    z = np.load(path)
    return NM.load(str(z["nep"])), z


def _nl(m, x, z):
    xw = ON.wrap(x, int(z["box_kind"]), z["box"])
    return ON.neighbors(xw, int(z["box_kind"]), z["box"], max(m.rc_radial, m.rc_angular))


def test_fixtures_present():
    assert len(CASES) >= 4


@pytest.mark.parametrize("path", CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_energies_match_reference(path):
    m, z = _load(path)
    e = NO.energies(m, z["types"] - 1, _nl(m, z["x"], z))
    assert np.max(np.abs(e - z["energies"])) <= 1e-11


FD_CASES = [os.path.join(GOLDEN_DIR, "nep_%s.npz" % k) for k in ("nep3_single", "nep4_binary", "nep4_zbl",
                                                                   "nep5_typewise_zbl")]


@pytest.mark.parametrize("path", FD_CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_forces_are_minus_energy_gradient(path):
    m, z = _load(path)
    t0 = z["types"] - 1
    h = 1e-5
    for atom, ax in ((0, 0), (7, 2), (len(t0) - 1, 1)):
        e = []
        for s in (1.0, -1.0):
            x = z["x"].copy()
            x[atom, ax] += s * h
            e.append(NO.energies(m, t0, _nl(m, x, z)).sum())
        f = z["forces"][atom, ax]
        assert abs(-(e[0] - e[1]) / (2 * h) - f) <= 2e-7 * max(1.0, abs(f))


@pytest.mark.parametrize("path", CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_reference_force_and_virial_invariants(path):
    _, z = _load(path)
    f, v = z["forces"], z["virials"].sum(axis=0)
    assert np.max(np.abs(f.sum(axis=0))) <= 1e-10                    # momentum
    assert np.max(np.abs(v[[3, 4, 5]] - v[[6, 7, 8]])) <= 1e-9       # rotation: symmetric virial


@pytest.mark.parametrize("path", CASES[:1], ids=lambda p: os.path.basename(p)[:-4])
def test_reference_reproduces_fixture(path):
    from oracle import nep_ref as NR
    if not os.path.isdir(NR.nep_src_dir()):
        pytest.skip("reference NEP sources not available")
    m, z = _load(path)
    out = NR.RefNEP(m).compute(z["types"] - 1, _nl(m, z["x"], z))
    assert np.array_equal(out["energies"], z["energies"])
    assert np.max(np.abs(out["forces"] - z["forces"])) <= 1e-13


def test_loader_round_trip_and_rejections():
    text = NM.write(["A", "B"], version=5, l_max=(4, 2, 0), neurons=4, seed=3)
    m = NM.load(text)
    assert (m.version, m.ntypes, m.num_L, m.dim) == (5, 2, 5, 5 + 25)
    assert len(m.params) == m.num_para_ann + m.num_para_descriptor and len(m.q_scaler) == m.dim
    lines = text.splitlines()
    with pytest.raises(ValueError):
        NM.load("\n".join(["nep4_zbl 2 A B"] + lines[1:]))
    with pytest.raises(ValueError):
        NM.load("\n".join(lines[:1] + ["cutoff 5 4 100 100 1 1"] + lines[2:]))
    assert NM.load("\n".join(lines[:1] + ["cutoff 5 4 100 100 2 1.5 0"] + lines[2:])).typewise == (2.0, 1.5, 0.0)
    with pytest.raises(ValueError):
        NM.load("\n".join(lines[:-1]))


def test_typewise_cutoffs_change_the_energies():
    """The type-wise fixture's pair cutoffs sit inside the global ones: evaluating the same
    model with the factors removed gives other energies, so the fixture pins them."""
    m, z = _load(os.path.join(GOLDEN_DIR, "nep_nep5_typewise_zbl.npz"))
    nl = _nl(m, z["x"], z)
    e_tw = NO.energies(m, z["types"] - 1, nl)
    m.typewise = (0.0, 0.0, 0.0)
    assert np.max(np.abs(NO.energies(m, z["types"] - 1, nl) - e_tw)) > 1e-3
