"""GPU path (through the C ABI) against the golden vectors of the reference's arithmetic.

Tolerances (plain FP32 path; descriptors and network in FP32, displacements and all
reductions in FP64; the mixed path's own energy bounds are given in its test):
  * neighbour sets: bit-exact, (i, j, image) per pair;
  * energies: |dE_i| <= 2e-5 * max(1, max|E|);
  * forces and per-atom virials: max |d| <= 1e-3 * max(1e-2, max|ref|) and
    RMS |d| <= 2e-4 * max(1e-2, max|ref|);
  * descriptors: relative 1e-4 of each column's scale.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _nnap(model_json, precision="fp32"):
    from jse_gb300.nnap import NNAP
    return NNAP(model_json, precision=precision)


class _S:
    def __init__(self, c):
        self.x, self.types, self.box, self.box_kind = c.x, c.types, c.box, c.box_kind


def _close(got, ref, tol_max, tol_rms):
    scale = max(1e-2, float(np.abs(ref).max()) if ref.size else 1.0)
    d = np.abs(got - ref)
    assert d.max() <= tol_max * scale, (d.max(), scale)
    assert np.sqrt((d ** 2).mean()) <= tol_rms * scale


def test_neighbor_sets_bit_exact(golden):
    with _nnap(golden.model_json) as p:
        off, j, img = p.neighborList(_S(golden))
    got = set()
    for i in range(len(golden.types)):
        for k in range(off[i], off[i + 1]):
            got.add((i, int(j[k])) + tuple(int(v) for v in img[k]))
    assert got == golden.nl_set()


def test_energy_force_virial_fp32(golden):
    with _nnap(golden.model_json) as p:
        o = p.calEnergyForceVirials(_S(golden))
        assert p.lastLaunchCount() > 0
    escale = max(1.0, float(np.abs(golden.energies).max()))
    assert np.abs(o["energies"] - golden.energies).max() <= 2e-5 * escale
    assert abs(o["energy"] - golden.energies.sum()) <= 2e-5 * escale * max(1, len(golden.types)) ** 0.5
    _close(o["forces"], golden.forces, 1e-3, 2e-4)
    _close(o["virials"], golden.virials, 1e-3, 2e-4)
    np.testing.assert_allclose(o["virial"], golden.virials.sum(0), rtol=1e-3,
                               atol=1e-4 * max(1.0, np.abs(golden.virials).sum(0).max()))


def test_descriptors_fp32(golden):
    with _nnap(golden.model_json) as p:
        fp = p.calFp(_S(golden))
    D = golden.fp.shape[1]
    scale = np.maximum(np.abs(golden.fp).max(0), 1e-6)
    assert (np.abs(fp[:, :D] - golden.fp) / scale).max() <= 1e-4


def test_descriptors_mixed(golden):
    """Mixed precision: spherical descriptors of fuse matrices with one nonzero per row come
    from the tensor cores (FP16 hi + lo operands, three products, FP32 accumulation); they
    keep the FP32 bound against the reference and agree with the FP32 kernels to 1e-5 of
    each column's scale."""
    with _nnap(golden.model_json, "mixed") as p:
        fp = p.calFp(_S(golden))
    with _nnap(golden.model_json) as p:
        fp32 = p.calFp(_S(golden))
    D = golden.fp.shape[1]
    scale = np.maximum(np.abs(golden.fp).max(0), 1e-6)
    assert (np.abs(fp[:, :D] - golden.fp) / scale).max() <= 1e-4
    assert (np.abs(fp[:, :D] - fp32[:, :D]) / scale).max() <= 1e-5


def test_results_are_deterministic(golden):
    with _nnap(golden.model_json) as p:
        a = p.calEnergyForceVirials(_S(golden))
        b = p.calEnergyForceVirials(_S(golden))
    for k in ("energies", "forces", "virials", "virial"):
        assert np.array_equal(a[k], b[k]), k


def test_energy_force_virial_mixed(golden):
    """Mixed precision: split-BF16 tensor-core network (hi*hi + lo*hi + hi*lo, FP32 accumulation),
    hidden widths padded to multiples of 16: every fixture runs, none is skipped."""
    with _nnap(golden.model_json, "mixed") as p:
        o = p.calEnergyForceVirials(_S(golden))
    escale = max(1.0, float(np.abs(golden.energies).max()))
    n = len(golden.types)
    # the split operands keep 16 significant bits of every network input and weight; a model
    # without descriptor normalisation feeds raw descriptors (tens) into the first layer, so the
    # per-atom bound is 5e-5 of the energy scale here; the energy per atom stays within 1e-5 eV
    assert np.abs(o["energies"] - golden.energies).max() <= 5e-5 * escale
    assert abs(o["energy"] - golden.energies.sum()) / n <= 1e-5
    _close(o["forces"], golden.forces, 1e-3, 2e-4)
    _close(o["virials"], golden.virials, 1e-3, 2e-4)
