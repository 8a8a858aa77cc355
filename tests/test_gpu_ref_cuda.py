"""The reference's own CUDA kernels (nnap_interface_cuda.cu) beside this build's.

oracle/ref_cuda.py compiles the reference's LAMMPS GPU path for a model and drives it
through its own host functions (jse_nnap_lammps2cuda, jse_nnap_computeLammpsCuda,
jse_nnap_cuda2lammps) on LAMMPS-form inputs.  Both FP32 paths must agree with each other
and with the FP64 oracle on the same structure; this pins the baseline the benchmark times.
"""
import numpy as np
import pytest

from jse_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _reverse(values, n, owner):
    out = values[:n].copy()
    np.add.at(out, owner, values[n:])
    return out


@pytest.mark.parametrize("tilt", [None, 0.1])
def test_reference_cuda_matches_this_build(tilt):
    from jse_gb300.nnap import NNAP
    from oracle import model as OM, native as ON, ref_cuda as RC
    model = W.model_for("c2")
    try:
        ref = RC.RefCudaNNAP(model)
    except FileNotFoundError as e:
        pytest.skip(str(e))
    s = W.random_liquid(1200, 0.060, [0.46, 0.46, 0.08], 2.0, 81, tilt=tilt)
    with NNAP(model) as p:
        off, j, img = p.neighborList(s)
        x, t, lists, owner = W.lammps_form(s, off, j, img)
        n = s.natoms
        ours = p.computeLammps(np.arange(n), lists, x, t)
    ref.setup(x, t, n, lists)
    r = ref.step()
    o = ON.compute(OM.load(model), s.x, s.types, s.box_kind, s.box)
    f_ref = _reverse(r["forces"], n, owner)
    f_ours = _reverse(ours["forces"], n, owner)
    assert np.max(np.abs(r["eatom"][:n] - o["energies"])) <= 1e-4
    assert np.max(np.abs(ours["eatom"][:n] - o["energies"])) <= 1e-5
    assert np.max(np.abs(f_ref - o["forces"])) <= 2e-3
    assert np.max(np.abs(f_ours - o["forces"])) <= 1e-4
    assert abs(r["eng"] - o["energy"]) / n <= 1e-5
    assert np.max(np.abs(r["virial"] - ours["virial"])) <= 1e-2 * max(1.0, np.abs(ours["virial"]).max())
