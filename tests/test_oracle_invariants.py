"""Analytic invariants of the oracle (FP64): F = -dE/dx, sum F = 0, translation and
rotation invariance, virial = -dE/d(strain), and per-atom virials summing to the total."""
import numpy as np
import pytest

from jse_gb300 import workloads as W
from oracle import model as OM, native as ON


def _sph_model(T=2):
    basis = {"type": "spherical_chebyshev", "nmax": 4, "lmax": 4, "rcut": 4.8}
    return OM.load(W.write_model(["A", "B", "C"][:T], basis, [12, 12], 5, norm_sigma_eng=0.3))


def _structure(seed=3, tilt=0.1):
    return W.random_liquid(48, 0.058, [0.5, 0.5], 2.0, seed, tilt=tilt)


def _energy(pm, x, s, box=None):
    return ON.compute(pm, x, s.types, s.box_kind, s.box if box is None else box)["energy"]


def test_forces_are_negative_energy_gradient():
    pm, s = _sph_model(), _structure()
    o = ON.compute(pm, s.x, s.types, s.box_kind, s.box)
    h = 1e-5
    rng = np.random.default_rng(0)
    for a in rng.choice(len(s.types), 5, replace=False):
        for d in range(3):
            xp, xm = s.x.copy(), s.x.copy()
            xp[a, d] += h
            xm[a, d] -= h
            fd = -(_energy(pm, xp, s) - _energy(pm, xm, s)) / (2 * h)
            assert abs(fd - o["forces"][a, d]) < 1e-6 * max(1.0, abs(fd)), (a, d, fd, o["forces"][a, d])


def test_forces_sum_to_zero_and_virials_sum_to_total():
    pm, s = _sph_model(), _structure()
    o = ON.compute(pm, s.x, s.types, s.box_kind, s.box)
    assert np.abs(o["forces"].sum(0)).max() < 1e-10
    np.testing.assert_allclose(o["virials"].sum(0), o["virial"], rtol=1e-12, atol=1e-12)


def test_translation_and_rotation_invariance():
    pm = _sph_model()
    s = _structure(tilt=None)
    o = ON.compute(pm, s.x, s.types, s.box_kind, s.box)
    t = ON.compute(pm, s.x + np.array([0.37, -1.2, 2.9]), s.types, s.box_kind, s.box)
    assert abs(o["energy"] - t["energy"]) < 1e-9
    np.testing.assert_allclose(t["forces"], o["forces"], atol=1e-9)
    # rigid rotation of structure and box together (general prism box)
    th = 0.3
    R = np.array([[np.cos(th), -np.sin(th), 0], [np.sin(th), np.cos(th), 0], [0, 0, 1]]) @ \
        np.array([[1, 0, 0], [0, np.cos(0.2), -np.sin(0.2)], [0, np.sin(0.2), np.cos(0.2)]])
    r = ON.compute(pm, s.x @ R.T, s.types, ON.BOX_PRISM, s.box @ R.T)
    assert abs(o["energy"] - r["energy"]) < 1e-9
    np.testing.assert_allclose(r["forces"], o["forces"] @ R.T, atol=1e-9)


def test_virial_is_strain_derivative():
    """Under x -> (I + eps) x every pair displacement becomes dx + eps dx, so
    dE/d eps_ab = -sum(dx_b g_a): the virial component with displacement index b and
    gradient index a (components ordered xx, yy, zz, xy, xz, yz, yx, zx, zy)."""
    pm, s = _sph_model(), _structure()
    o = ON.compute(pm, s.x, s.types, s.box_kind, s.box)
    h = 1e-6
    component = {(0, 0): 0, (1, 1): 1, (2, 2): 2, (0, 1): 6, (0, 2): 7, (1, 2): 8, (1, 0): 3, (2, 0): 4, (2, 1): 5}
    for (a, b), k in component.items():
        E = []
        for sgn in (1, -1):
            F = np.eye(3)
            F[a, b] += sgn * h
            E.append(ON.compute(pm, s.x @ F.T, s.types, ON.BOX_PRISM, s.box @ F.T)["energy"])
        dE = (E[0] - E[1]) / (2 * h)
        assert abs(dE + o["virial"][k]) < 1e-5 * max(1.0, abs(dE)), (a, b, dE, o["virial"][k])
