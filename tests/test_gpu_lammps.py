"""LAMMPS-style boundary (nnap_compute_lammps) against the periodic entry point.

A periodic structure is turned into LAMMPS's form:
* local atoms are the structure's atoms at their wrapped positions;
* one ghost atom stands for every periodic image that some local atom sees within
  rc + 0.4 A, an extra skin that the call must filter away;
* full lists point at local atoms or ghosts, with LAMMPS special-bond bits set on some
  entries.
After LAMMPS's reverse communication (ghost forces and per-atom virials added to their
owners), the results must equal nnap_compute's: per-atom energies, forces, the global
virial and the per-atom virials.  They differ only by FP32 rounding: displacements come
from other coordinates and rows are summed in another order (tolerances below).  Two
calls give identical results.
"""
import numpy as np
import pytest

from jse_gb300 import workloads as W
from oracle import native as ON

pytestmark = pytest.mark.gpu

E_TOL = 1e-5   # eV per atom: two FP32 descriptor sums in different orders (the path's energy target)
F_TOL = 1e-4   # eV/A, largest component
V_TOL = 1e-4   # eV, largest per-atom virial component


def _lammps_form(s, rlist):
    xw = ON.wrap(s.x, s.box_kind, s.box)
    nl = ON.neighbors(xw, s.box_kind, s.box, rlist)
    n = s.natoms
    box = np.asarray(s.box, dtype=np.float64).reshape(3, 3)
    ghost_of, gx, owner = {}, [], []
    lists = []
    for i in range(n):
        row = []
        for k in range(nl.offsets[i], nl.offsets[i + 1]):
            j, img = int(nl.j[k]), tuple(int(v) for v in nl.img[k])
            if img == (0, 0, 0):
                row.append(j)
                continue
            key = (j, img)
            if key not in ghost_of:
                ghost_of[key] = n + len(gx)
                gx.append(xw[j] + np.asarray(img, dtype=np.float64) @ box)
                owner.append(j)
            row.append(ghost_of[key])
        lists.append(np.asarray(row, dtype=np.int64))
    x = np.concatenate([xw, np.asarray(gx).reshape(-1, 3)])
    types = np.concatenate([s.types, s.types[np.asarray(owner, dtype=np.int64)]]).astype(np.int32)
    return x, types, lists, np.asarray(owner, dtype=np.int64), xw


def _reverse(values, n, owner):
    out = values[:n].copy()
    np.add.at(out, owner, values[n:])
    return out


@pytest.mark.parametrize("tilt", [None, 0.1])
def test_lammps_form_equals_periodic_evaluation(tilt):
    from jse_gb300.nnap import NNAP
    s = W.random_liquid(1500, 0.060, [0.46, 0.46, 0.08], 2.0, 71 if tilt is None else 72, tilt=tilt)
    model = W.model_for("c2")
    with NNAP(model, precision="mixed") as p:
        rc = p.rcutMax()
        x, types, lists, owner, xw = _lammps_form(s, rc + 0.4)
        n = s.natoms
        marked = [l.astype(np.int64) | (np.int64(1) << 30) * (np.arange(len(l)) % 3 == 0) for l in lists]
        marked = [np.asarray(m, dtype=np.int64).astype(np.uint32).view(np.int32) for m in marked]
        out = p.computeLammps(np.arange(n), marked, x, types, type_map=[0, 1, 2, 3])
        again = p.computeLammps(np.arange(n), lists, x, types)
        ref = p.calEnergyForceVirials(W.Structure(xw, s.types, s.box, s.box_kind))
    assert np.array_equal(out["forces"], again["forces"]) and out["eng"] == again["eng"]
    assert np.allclose(out["eatom"][n:], 0.0)
    assert np.max(np.abs(out["eatom"][:n] - ref["energies"])) <= E_TOL
    assert abs(out["eng"] - ref["energy"]) / n <= E_TOL
    f = _reverse(out["forces"], n, owner)
    assert np.max(np.abs(f - ref["forces"])) <= F_TOL
    assert np.max(np.abs(out["virial"] - ref["virial"][:6])) <= V_TOL * n ** 0.5
    cv = _reverse(out["cvatom"], n, owner)
    assert np.max(np.abs(cv - ref["virials"])) <= V_TOL
    assert np.max(np.abs(_reverse(out["vatom"], n, owner))) == 0.0  # vflag_atom was off


def test_lammps_rejects_bad_indices():
    from jse_gb300.nnap import NNAP, NNAPError
    s = W.random_liquid(200, 0.060, [0.46, 0.46, 0.08], 2.0, 73)
    with NNAP(W.model_for("c2"), precision="mixed") as p:
        lists = [np.array([1, 2], dtype=np.int32)] + [np.zeros(0, dtype=np.int32)] * (s.natoms - 1)
        lists[0][1] = s.natoms + 5  # beyond nall
        with pytest.raises(NNAPError):
            p.computeLammps(np.arange(s.natoms), lists, s.x, s.types)
        with pytest.raises(NNAPError):
            p.computeLammps(np.array([0, 0]), lists, s.x, s.types)  # duplicate ilist entry


def test_lammps_large_list_global_virial_only():
    """A list of more than 2^18 entries (the host copy runs on several threads) with only
    the global virial requested (summed on the device)."""
    from jse_gb300.nnap import NNAP
    s = W.random_liquid(6000, 0.060, [0.46, 0.46, 0.08], 2.0, 74, tilt=0.1)
    model = W.model_for("c2")
    with NNAP(model, precision="mixed") as p:
        x, types, lists, owner, xw = _lammps_form(s, p.rcutMax() + 0.4)
        n = s.natoms
        assert sum(len(l) for l in lists) > (1 << 18)
        out = p.computeLammps(np.arange(n), lists, x, types, cvflag_atom=False)
        full = p.computeLammps(np.arange(n), lists, x, types, cvflag_atom=True)
        ref = p.calEnergyForceVirials(W.Structure(xw, s.types, s.box, s.box_kind))
    assert np.array_equal(out["forces"], full["forces"]) and out["eng"] == full["eng"]
    assert np.max(np.abs(out["virial"] - full["virial"])) <= 1e-9 * max(1.0, np.abs(full["virial"]).max())
    assert np.max(np.abs(out["virial"] - ref["virial"][:6])) <= V_TOL * n ** 0.5
    assert np.max(np.abs(_reverse(out["forces"], n, owner) - ref["forces"])) <= F_TOL


def test_lammps_list_reuse_equals_resend():
    """nlflag = 0 (the list of the previous call, new positions) gives exactly what sending
    the same list again gives; without a previous list, or with another inum, it is refused."""
    from jse_gb300.nnap import NNAP, NNAPError
    s = W.random_liquid(1500, 0.060, [0.46, 0.46, 0.08], 2.0, 75)
    rng = np.random.default_rng(3)
    with NNAP(W.model_for("c2"), precision="mixed") as p:
        x, types, lists, owner, xw = _lammps_form(s, p.rcutMax() + 0.4)
        n = s.natoms
        with pytest.raises(NNAPError):
            p.computeLammps(np.arange(n), lists, x, types, nlflag=False)
        p.computeLammps(np.arange(n), lists, x, types)
        x2 = x + rng.normal(0.0, 0.02, size=x.shape)
        sent = p.computeLammps(np.arange(n), lists, x2, types)
        reused = p.computeLammps(np.arange(n), lists, x2, types, nlflag=False)
        assert np.array_equal(sent["forces"], reused["forces"]) and sent["eng"] == reused["eng"]
        assert np.array_equal(sent["cvatom"], reused["cvatom"])
        with pytest.raises(NNAPError):
            p.computeLammps(np.arange(n - 1), lists, x2, types, nlflag=False)
        again = p.computeLammps(np.arange(n), lists, x2, types, nlflag=False)  # a refusal keeps the list
        assert np.array_equal(sent["forces"], again["forces"])
