"""Every model shape of the sweep (tests/golden/shapes) on the GPU, through the C ABI, in
both precisions, against the reference's own FP64 outputs.

Shapes without a specialised descriptor kernel run the any-shape kernels (runtime channel
and radial-function counts); networks of any depth and width run on the tensor cores in
mixed precision (widths padded to 16).  No shape of the sweep is refused.

Tolerances as tests/test_gpu_parity.py: neighbour sets bit-exact; |dE_i| <= 2e-5 (FP32)
or 5e-5 (mixed) of the energy scale and the energy per atom within 1e-5 eV; forces and per-atom virials max |d| <= 1e-3 and RMS <= 2e-4 of their
scale; descriptors within 1e-4 of each column's scale.  NEP shapes as tests/test_gpu_nep.py.
"""
import os

import numpy as np
import pytest

from jse_gb300 import workloads as W
from tests.shapes_common import NEP_SHAPES, NNAP_SHAPES, ShapeCase

pytestmark = pytest.mark.gpu


class _S:
    def __init__(self, c):
        self.x, self.types, self.box, self.box_kind = c.x, c.types, c.box, c.box_kind


def _close(got, ref, tol_max, tol_rms):
    scale = max(1e-2, float(np.abs(ref).max()) if ref.size else 1.0)
    d = np.abs(got - ref)
    assert d.max() <= tol_max * scale, (d.max(), scale)
    assert np.sqrt((d ** 2).mean()) <= tol_rms * scale


def _ids(paths):
    return [os.path.basename(p)[:-4] for p in paths]


@pytest.fixture(params=NNAP_SHAPES, ids=_ids(NNAP_SHAPES))
def shape(request):
    return ShapeCase(request.param)


def test_neighbor_sets(shape):
    from jse_gb300.nnap import NNAP
    with NNAP(shape.model_json) as p:
        off, j, img = p.neighborList(_S(shape))
    got = set()
    for i in range(len(shape.types)):
        for k in range(off[i], off[i + 1]):
            got.add((i, int(j[k])) + tuple(int(v) for v in img[k]))
    assert got == shape.nl_set()


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_energy_force_virial(shape, precision):
    from jse_gb300.nnap import NNAP
    with NNAP(shape.model_json, precision=precision) as p:
        o = p.calEnergyForceVirials(_S(shape))
        again = p.calEnergyForceVirials(_S(shape))
    escale = max(1.0, float(np.abs(shape.energies).max()))
    assert np.abs(o["energies"] - shape.energies).max() <= (2e-5 if precision == "fp32" else 5e-5) * escale
    assert abs(o["energy"] - shape.energies.sum()) / len(shape.types) <= 1e-5
    _close(o["forces"], shape.forces, 1e-3, 2e-4)
    _close(o["virials"], shape.virials, 1e-3, 2e-4)
    for k in ("energies", "forces", "virials"):
        assert np.array_equal(o[k], again[k]), k


def test_descriptors(shape):
    from jse_gb300.nnap import NNAP
    with NNAP(shape.model_json) as p:
        fp = p.calFp(_S(shape))
    D = shape.fp.shape[1]
    scale = np.maximum(np.abs(shape.fp).max(0), 1e-6)
    assert (np.abs(fp[:, :D] - shape.fp) / scale).max() <= 1e-4


@pytest.mark.parametrize("name", ["default_model_t2", "exfull_d252", "sph_lmax12"])
def test_batch_equals_single(name):
    """A batch of three structures of an any-shape model (graph capture and replay of the
    any-shape kernels included) gives each structure's single-call results bitwise."""
    from jse_gb300.nnap import NNAP
    c = ShapeCase([p for p in NNAP_SHAPES if p.endswith(name + ".npz")][0])
    T = len(c.model["models"])
    structs = [W.random_liquid(n, 0.06, [1.0 / T] * T, 2.0, 90 + n, tilt=0.1 if n % 2 else None)
               for n in (40, 77, 130)]
    with NNAP(c.model_json, precision="mixed") as p:
        for _ in range(3):  # eager, captured, replayed
            batch = p.calEnergyForceVirialsBatch(structs, per_atom_virial=True)
        for s, b in zip(structs, batch):
            o = p.calEnergyForceVirials(s)
            assert np.array_equal(o["forces"], b["forces"])
            assert np.array_equal(o["energies"], b["energies"])


@pytest.mark.parametrize("path", NEP_SHAPES, ids=_ids(NEP_SHAPES))
def test_nep_shapes(path):
    from jse_gb300.nep import NEP
    z = np.load(path)
    s = W.Structure(z["x"], z["types"], z["box"].reshape(3, 3), int(z["box_kind"]))
    with NEP(str(z["nep"])) as p:
        out = p.calEnergyForceVirials(s)
    assert np.max(np.abs(out["energies"] - z["energies"])) <= 1e-5
    df = out["forces"] - z["forces"]
    assert np.max(np.abs(df)) <= 1e-3
    assert np.sqrt(np.mean(df ** 2)) <= 1e-4
    assert np.max(np.abs(out["virials"] - z["virials"])) <= 2e-3


def test_yaml_model_evaluates_like_json(tmp_path):
    """A model file written as YAML (NNAP.java:407-411) gives the JSON model's results bitwise."""
    from jse_gb300.nnap import NNAP
    from tests.yaml_emit import dump
    c = ShapeCase([p for p in NNAP_SHAPES if p.endswith("default_model_t2.npz")][0])
    path = tmp_path / "model.yml"
    path.write_text(dump(c.model))
    for precision in ("fp32", "mixed"):
        with NNAP(c.model_json, precision=precision) as a, NNAP(str(path), precision=precision) as b:
            ra, rb = a.calEnergyForceVirials(_S(c)), b.calEnergyForceVirials(_S(c))
        for k in ("energies", "forces", "virials"):
            assert np.array_equal(ra[k], rb[k]), (precision, k)
