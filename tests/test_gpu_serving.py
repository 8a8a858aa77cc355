"""Serving path: resident neighbour rows, continuous batching, admission by budget.

Checks, against the one-shot entry points of a second handle on the same model:
* the neighbour set a step uses is the full search's set, bit for bit (same j, same
  image), on steps that rebuild and on steps that only filter, with atoms crossing the
  periodic boundary between rebuilds;
* energies and forces agree with nnap_compute (tolerances below; only the summation
  order inside a row differs);
* a request gives the same results alone and mixed with other requests arriving while
  it runs (exactly: every result depends only on its own structure);
* admission stops at the memory budget and resumes after a release.
"""
import numpy as np
import pytest

from jse_gb300 import workloads as W

pytestmark = pytest.mark.gpu

E_TOL = 1e-6   # eV/atom, server vs nnap_compute on the same positions
F_TOL = 1e-4   # eV/A, largest force component difference


def _pairs(off, j, img):
    i = np.repeat(np.arange(len(off) - 1), np.diff(off))
    return np.unique(np.stack([i, j, img[:, 0], img[:, 1], img[:, 2]], 1), axis=0)


@pytest.fixture(scope="module")
def model():
    return W.model_for("c2")


def test_neighbour_sets_bit_exact_across_moves(model):
    from jse_gb300.nnap import NNAP
    from jse_gb300.serve import NNAPServer
    s = W.random_liquid(3000, 0.060, [0.46, 0.46, 0.08], 2.0, 81, tilt=0.1)
    rng = np.random.default_rng(5)
    ref = NNAP(model, precision="mixed")
    with NNAP(model, precision="mixed") as p, NNAPServer(p, skin=0.5, memory_budget=8e9) as srv:
        slot = srv.admit(s)
        x = s.x.copy()
        rebuilds = []
        for k in range(8):
            if k:
                x = x + rng.normal(0.0, 0.03, size=x.shape)  # largest move ~0.14 A a step: rebuild every few steps
            out = srv.step([slot], [x], energies=True)
            rebuilds.append(srv.stats()["rebuilds"])
            st = W.Structure(x, s.types, s.box, s.box_kind)
            got = _pairs(*srv.neighborList(slot))
            want = _pairs(*ref.neighborList(st))
            assert got.shape == want.shape and np.array_equal(got, want), "step %d" % k
            r = ref.calEnergyForceVirials(st, per_atom_virial=False)
            assert abs(out["energy"][0] - r["energy"]) / s.natoms <= E_TOL
            assert np.max(np.abs(out["forces"] - r["forces"])) <= F_TOL
        # both kinds of step ran: some rebuilt, some only filtered
        inc = np.diff([0] + rebuilds)
        assert inc.max() == 1 and inc.min() == 0
    ref.close()


def test_wrapped_and_unwrapped_callers_agree(model):
    """Atoms handed over outside the box (whole box vectors away) give the same answer."""
    from jse_gb300.nnap import NNAP
    from jse_gb300.serve import NNAPServer
    s = W.random_liquid(1500, 0.060, [0.46, 0.46, 0.08], 2.0, 82, tilt=0.1)
    rng = np.random.default_rng(6)
    shift = rng.integers(-2, 3, size=(s.natoms, 3)) @ s.box
    with NNAP(model, precision="mixed") as p, NNAPServer(p, skin=0.5, memory_budget=8e9) as srv:
        a = srv.admit(s)
        b = srv.admit(s)
        x = s.x.copy()
        for k in range(3):
            if k:
                x = x + rng.normal(0.0, 0.02, size=x.shape)
            out = srv.step([a, b], [x, x + shift], energies=True)
            n = s.natoms
            assert abs(out["energy"][0] - out["energy"][1]) / n <= E_TOL
            assert np.max(np.abs(out["forces"][:n] - out["forces"][n:])) <= F_TOL


def test_same_results_alone_and_in_the_mix(model):
    from jse_gb300.nnap import NNAP
    from jse_gb300.serve import GaussianMoves, NNAPServer, Request, RequestLoop, poisson_requests
    pool = [W.random_liquid(n, 0.060, [0.46, 0.46, 0.08], 2.0, 90 + k) for k, n in enumerate([60, 250, 700, 1800])]
    target = W.random_liquid(900, 0.060, [0.46, 0.46, 0.08], 2.0, 99, tilt=0.1)
    moves = GaussianMoves(sigma=0.01, seed=3)

    def run(reqs):
        with NNAP(model, precision="mixed") as p, NNAPServer(p, skin=0.5, memory_budget=8e9) as srv:
            RequestLoop(srv, reqs, moves=moves, keep_results=True).run()
        return reqs

    alone = run([Request(1000, target, 12, 0.0)])[0]
    others = poisson_requests(pool, 30, rate=400.0, nsteps=12, seed=4)
    mixed = run(others + [Request(1000, target, 12, 0.01)])
    mine = [r for r in mixed if r.rid == 1000][0]
    assert mine.done == alone.done == 12
    for k in range(12):
        assert abs(mine.energies[k] - alone.energies[k]) <= 1e-10
        assert np.max(np.abs(mine.forces[k] - alone.forces[k])) <= 1e-10
    # the target really ran alongside others: some step held more than one request
    assert any(r.t_admit < mine.t_done and r.t_done > mine.t_admit for r in mixed if r.rid != 1000)


def test_admission_stops_at_the_budget(model):
    from jse_gb300.nnap import NNAP, NNAPError, NNAP_ERR_CAPACITY
    from jse_gb300.serve import NNAPServer
    s = W.random_liquid(2000, 0.060, [0.46, 0.46, 0.08], 2.0, 83)
    with NNAP(model, precision="mixed") as p:
        with NNAPServer(p, skin=0.5, memory_budget=80e6, max_structs=64) as srv:
            slots = []
            while True:
                k = srv.admit(s)
                if k is None:
                    break
                slots.append(k)
                assert len(slots) < 64
            # the budget, not the 64-slot cap, refused the next admission
            st = srv.stats()
            assert 1 <= len(slots) < 64 and st["resident_bytes"] + st["work_bytes"] <= 80e6
            srv.step(slots, [s.x] * len(slots))
            srv.release(slots[0])
            assert srv.admit(s) is not None
        with NNAPServer(p, skin=0.5, memory_budget=1e6) as srv:
            with pytest.raises(NNAPError) as e:
                srv.admit(s)
            assert e.value.status == NNAP_ERR_CAPACITY


def test_submit_collect_equals_step(model):
    """The two-phase step gives the one-call step's results bitwise; the positions are staged
    (changing them after submit changes nothing); one step is in flight at a time, a slot of
    it cannot be released before the collect, and admissions may happen meanwhile."""
    from jse_gb300.nnap import NNAP, NNAPError, NNAP_ERR_ARG, NNAP_ERR_BUSY
    from jse_gb300.serve import NNAPServer
    structs = [W.random_liquid(n, 0.060, [0.46, 0.46, 0.08], 2.0, 84 + n, tilt=0.1) for n in (300, 800, 1500)]
    rng = np.random.default_rng(7)
    with NNAP(model, precision="mixed") as p, NNAPServer(p, skin=0.5, memory_budget=8e9) as a, \
            NNAP(model, precision="mixed") as q, NNAPServer(q, skin=0.5, memory_budget=8e9) as b:
        sa = [a.admit(s) for s in structs]
        sb = [b.admit(s) for s in structs]
        xs = [np.array(s.x, copy=True) for s in structs]
        for k in range(4):
            if k:
                xs = [x + rng.normal(0.0, 0.02, size=x.shape) for x in xs]
            ref = a.step(sa, xs, energies=True, per_atom_virial=True)
            work = [np.array(x, copy=True) for x in xs]
            b.submit(sb, work, energies=True, per_atom_virial=True)
            for w in work:
                w += 5.0  # staged: no effect on the step in flight
            with pytest.raises(NNAPError) as e:
                b.submit(sb, work)
            assert e.value.status == NNAP_ERR_BUSY
            with pytest.raises(NNAPError) as e:
                b.release(sb[0])
            assert e.value.status == NNAP_ERR_ARG
            extra = b.admit(structs[0])  # admission while the step runs
            got = b.collect()
            b.release(extra)
            for key in ("energy", "virial", "forces", "energies", "virials"):
                assert np.array_equal(ref[key], got[key]), (k, key)
