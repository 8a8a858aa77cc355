"""NEP potentials on the GPU against the reference's own outputs.

tests/golden/nep_*.npz hold nep.txt models (nep3 / nep4 / nep5; one to three species;
with and without the 4- and 5-body columns) and the FP64 energies, forces and per-atom
virials of the reference's compiled NEP arithmetic on the same structures
(tests/golden/make_golden_nep.py).  The GPU path evaluates them through nnap_create_nep
with FP32 descriptors and network.

Tolerances: |dE_i| <= 1e-5 eV per atom (the path's energy target) on every fixture, close
ZBL contacts included (the ZBL pair terms run in FP64 on displacements carried to ~48
bits), max |dF| <= 1e-3 eV/A and force RMSE <= 1e-4 eV/A, per-atom virials within 2e-3 eV.
The energy per atom stays within 1e-5 eV.
"""
import glob
import os

import numpy as np
import pytest

from jse_gb300 import workloads as W
from tests.conftest import GOLDEN_DIR

pytestmark = pytest.mark.gpu

CASES = sorted(glob.glob(os.path.join(GOLDEN_DIR, "nep_*.npz")))
BINARY = os.path.join(GOLDEN_DIR, "nep_nep4_binary.npz")   # two species, 4- and 5-body terms
E_TOL, F_MAX, F_RMS, V_TOL = 1e-5, 1e-3, 1e-4, 2e-3


def _case(path):
    z = np.load(path)
    s = W.Structure(z["x"], z["types"], z["box"].reshape(3, 3), int(z["box_kind"]))
    return str(z["nep"]), s, z


@pytest.mark.parametrize("path", CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_nep_matches_reference(path):
    from jse_gb300.nep import NEP
    text, s, z = _case(path)
    with NEP(text) as p:
        out = p.calEnergyForceVirials(s)
    de = np.max(np.abs(out["energies"] - z["energies"]))
    print("%s: max |dE_i| %.2e eV, max |dF| %.2e eV/A" % (os.path.basename(path)[:-4], de,
                                                          np.max(np.abs(out["forces"] - z["forces"]))))
    assert de <= E_TOL
    df = out["forces"] - z["forces"]
    assert np.max(np.abs(df)) <= F_MAX
    assert np.sqrt(np.mean(df ** 2)) <= F_RMS
    assert np.max(np.abs(out["virials"] - z["virials"])) <= V_TOL
    assert abs(out["energy"] - z["energies"].sum()) / len(z["energies"]) <= E_TOL


def test_nep_mixed_handle_is_fp32():
    from jse_gb300.nep import NEP
    text, s, _ = _case(CASES[0])
    with NEP(text) as a, NEP(text, precision="mixed") as b:
        ra, rb = a.calEnergyForceVirials(s), b.calEnergyForceVirials(s)
    assert np.array_equal(ra["forces"], rb["forces"]) and ra["energy"] == rb["energy"]


def test_nep_file_path_and_symbols(tmp_path):
    from jse_gb300.nep import NEP
    text, s, z = _case(CASES[0])
    f = tmp_path / "nep.txt"
    f.write_text(text)
    with NEP(str(f)) as p:
        syms = text.split("\n", 1)[0].split()[2:]
        assert p.ntypes() == len(syms)
        assert [p.symbol(t + 1) for t in range(len(syms))] == syms
        assert abs(p.calEnergyForceVirials(s)["energy"] - z["energies"].sum()) / s.natoms <= E_TOL


def _structs(T):
    fr = [1.0 / T] * T
    return [W.random_liquid(n, 0.06, fr, 2.0, 500 + n, tilt=0.1 if n % 2 else None) for n in (150, 601, 1200)]


def test_nep_batch_lammps_server_agree():
    from jse_gb300.nep import NEP
    from jse_gb300.serve import NNAPServer
    from tests.test_gpu_lammps import _lammps_form, _reverse
    text, _, _ = _case(BINARY)
    T = int(text.split()[1])
    structs = _structs(T)
    with NEP(text) as p:
        batch = p.calEnergyForceVirialsBatch(structs)
        singles = [p.calEnergyForceVirials(s) for s in structs]
        for s, b, r in zip(structs, batch, singles):
            assert abs(b["energy"] - r["energy"]) / s.natoms <= E_TOL
            assert np.max(np.abs(b["forces"] - r["forces"])) <= 1e-4
        s = structs[1]
        x, types, lists, owner, xw = _lammps_form(s, p.rcutMax() + 0.4)
        n = s.natoms
        out = p.computeLammps(np.arange(n), lists, x, types)
        ref = p.calEnergyForceVirials(W.Structure(xw, s.types, s.box, s.box_kind))
        assert np.max(np.abs(out["eatom"][:n] - ref["energies"])) <= E_TOL
        assert np.max(np.abs(_reverse(out["forces"], n, owner) - ref["forces"])) <= 1e-4
    with NEP(text) as p, NNAPServer(p, skin=0.5, memory_budget=4e9) as srv:
        s = structs[2]
        slot = srv.admit(s)
        out = srv.step([slot], [s.x], energies=True)
        assert abs(out["energy"][0] - singles[2]["energy"]) / s.natoms <= E_TOL
        assert np.max(np.abs(out["forces"] - singles[2]["forces"])) <= 1e-4


def test_nep_training_is_rejected():
    from jse_gb300.nep import NEP
    from jse_gb300.nnap import NNAPError
    text, s, _ = _case(CASES[0])
    with NEP(text) as p:
        with pytest.raises(NNAPError):
            p.backwardEnergyForceBatch([s], np.ones(s.natoms), np.zeros((s.natoms, 3)), np.zeros((1, 9)))


def test_reference_cuda_nep_matches():
    """The reference's own CUDA NEP (nep_interface_cuda.cu, oracle/nep_ref_cuda.py) on the
    LAMMPS form of a fixture structure: it and this build's LAMMPS boundary both agree with
    the reference's FP64 CPU outputs."""
    from jse_gb300.nep import NEP
    from oracle import nep_model as NM, nep_ref_cuda as NRC
    text, s, z = _case(BINARY)
    try:
        ref = NRC.RefCudaNEP(NM.load(text))
    except (FileNotFoundError, RuntimeError) as e:
        pytest.skip(str(e))
    with NEP(text) as p:
        off, j, img = p.neighborList(s)
        x, t, lists, owner = W.lammps_form(s, off, j, img)
        n = s.natoms
        ours = p.computeLammps(np.arange(n), lists, x, t, cvflag_atom=False)
    ref.setup(x, t, n, lists)
    r = ref.step()

    def rev(v):
        out = v[:n].copy()
        np.add.at(out, owner, v[n:])
        return out
    assert np.max(np.abs(r["eatom"][:n] - z["energies"])) <= 1e-4
    assert np.max(np.abs(rev(r["forces"]) - z["forces"])) <= 2e-3
    assert np.max(np.abs(ours["eatom"][:n] - z["energies"])) <= E_TOL
    assert np.max(np.abs(rev(ours["forces"]) - z["forces"])) <= F_MAX
