"""Workload-scale checks on the GPU against the FP64 oracle.

Accuracy targets (both precisions): force RMSE <= 1e-3 eV/A, |E - E_ref| / N <= 1e-5 eV/atom,
bit-exact neighbour sets.  Size-independent properties at the full workload size:
sum of forces ~ 0, per-atom virials summing to the total, determinism, and batch
results equal to single-structure results.
"""
import numpy as np
import pytest

from jse_gb300 import workloads as W
from oracle import model as OM, native as ON

pytestmark = pytest.mark.gpu


def _normalised(cfg, s):
    pm = OM.load(W.model_for(cfg))
    fp = ON.compute(pm, s.x, s.types, s.box_kind, s.box, want_fp=True)["fp"]
    T = pm.ntypes
    mu = [fp[s.types == t + 1, :pm.basis[t].size].mean(0) for t in range(T)]
    sg = [fp[s.types == t + 1, :pm.basis[t].size].std(0) + 1e-3 for t in range(T)]
    return W.model_for(cfg, norm_mu=mu, norm_sigma=sg)


CASES = {
    "liquid": ("c2", lambda: W.random_liquid(4000, 0.060, [0.46, 0.46, 0.08], 2.0, 31)),
    "fcc": ("c1", lambda: W.c1_structure()),
    "glass_tri": ("c3", lambda: W.random_liquid(6000, 0.058, [0.64, 0.36], 2.1, 32, tilt=0.1)),
}


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    cfg, mk = CASES[request.param]
    s = mk()
    model = _normalised(cfg, s)
    ref = ON.compute(OM.load(model), s.x, s.types, s.box_kind, s.box)
    return request.param, s, model, ref


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_accuracy_targets(case, precision):
    from jse_gb300.nnap import NNAP
    name, s, model, ref = case
    with NNAP(model, precision=precision) as p:
        o = p.calEnergyForceVirials(s)
    n = len(s.types)
    f_rmse = float(np.sqrt(((o["forces"] - ref["forces"]) ** 2).mean()))
    e_err = abs(o["energy"] - ref["energy"]) / n
    e_max = float(np.abs(o["energies"] - ref["energies"]).max())
    print("%s %s: force RMSE %.2e eV/A, |dE|/N %.2e eV/atom, max |dE_i| %.2e" % (name, precision, f_rmse, e_err, e_max))
    assert f_rmse <= 1e-3
    assert e_err <= 1e-5
    assert e_max <= 1e-4
    np.testing.assert_allclose(o["virial"], ref["virial"], rtol=1e-3, atol=1e-3 * max(1.0, np.abs(ref["virial"]).max()))


def test_neighbor_set_bit_exact(case):
    from jse_gb300.nnap import NNAP
    name, s, model, ref = case
    with NNAP(model) as p:
        off, j, img = p.neighborList(s)
    nl = ref["nl"]
    assert np.array_equal(off, nl.offsets)
    got = set(zip(np.repeat(np.arange(len(s.types)), np.diff(off)), j, *img.T))
    want = set(zip(np.repeat(np.arange(len(s.types)), np.diff(nl.offsets)), nl.j, *nl.img.T))
    assert got == want


def test_full_liquid_invariants_and_determinism():
    from jse_gb300.nnap import NNAP
    s = W.c2_structure()
    with NNAP(W.model_for("c2"), precision="mixed") as p:
        a = p.calEnergyForceVirials(s)
        b = p.calEnergyForceVirials(s)
    for k in ("energies", "forces", "virials", "virial"):
        assert np.array_equal(a[k], b[k]), k
    fscale = np.abs(a["forces"]).max()
    assert np.abs(a["forces"].sum(0)).max() <= 1e-6 * fscale * len(s.types) ** 0.5
    np.testing.assert_allclose(a["virials"].sum(0), a["virial"], rtol=1e-12, atol=1e-9)


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_batch_equals_single(precision):
    from jse_gb300.nnap import NNAP
    structs = W.c4_structures(count=12, seed=9)
    with NNAP(W.model_for("c2"), precision=precision) as p:
        batch = p.calEnergyForceVirialsBatch(structs, per_atom_virial=True)
        for s, b in zip(structs, batch):
            o = p.calEnergyForceVirials(s)
            assert np.array_equal(o["forces"], b["forces"])
            assert np.array_equal(o["energies"], b["energies"])
            assert np.array_equal(o["virials"], b["virials"])
            np.testing.assert_allclose(o["energy"], b["energy"], rtol=1e-13)
            np.testing.assert_allclose(o["virial"], b["virial"], rtol=1e-12, atol=1e-12)


def test_graph_replay_across_layout_changes():
    """Alternating layouts on one handle: each call re-plans or replays the captured
    launch sequence; results equal those of a fresh handle."""
    from jse_gb300.nnap import NNAP
    a = W.random_liquid(300, 0.06, [0.46, 0.46, 0.08], 2.0, 41)
    b = W.random_liquid(500, 0.06, [0.46, 0.46, 0.08], 2.0, 42, tilt=0.1)
    model = W.model_for("c2")
    with NNAP(model, precision="mixed") as p:
        ra = p.calEnergyForceVirials(a)
        rb = p.calEnergyForceVirials(b)
    with NNAP(model, precision="mixed") as p:
        for _ in range(3):
            for s, r in ((a, ra), (a, ra), (b, rb), (b, rb), (b, rb)):
                o = p.calEnergyForceVirials(s)
                assert np.array_equal(o["forces"], r["forces"])
                assert o["energy"] == r["energy"]


def test_autotuned_shapes_give_the_same_results():
    """Launch shapes chosen by the autotuner change no neighbour row and no per-atom
    arithmetic order except the network's energy split (<= 1e-9 eV/atom apart)."""
    from jse_gb300.nnap import NNAP
    s = W.random_liquid(3000, 0.060, [0.46, 0.46, 0.08], 2.0, 61, tilt=0.1)
    model = W.model_for("c2")
    with NNAP(model, precision="mixed") as p:
        ref = p.calEnergyForceVirials(s, per_atom_virial=False)
        assert p.tuning(s.natoms)["tuned"] is False
        p.setAutotune(True)
        got = p.calEnergyForceVirials(s, per_atom_virial=False)
        t = p.tuning(s.natoms)
        assert t["tuned"] is True
        assert t["desc_fwd_warps"] in (2, 4, 8) and t["gather_block"] in (64, 128, 256) and t["net_split"] in (2, 4)
        again = p.calEnergyForceVirials(s, per_atom_virial=False)
        p.setTuning(100000, {"desc_fwd_warps": 8, "desc_bwd_warps": 2, "nb_warps": 8, "gather_block": 64,
                             "net_split": 2})
        assert p.tuning(120000)["tuned"] is True and p.tuning(120000)["nb_warps"] == 8
    n = s.natoms
    assert abs(got["energy"] - ref["energy"]) / n <= 1e-9
    assert np.max(np.abs(got["forces"] - ref["forces"])) <= 1e-6
    assert np.array_equal(got["forces"], again["forces"])
