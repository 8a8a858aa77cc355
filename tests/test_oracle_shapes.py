"""The CPU oracle against the reference's outputs on the shape sweep (tests/golden/shapes):
the reference's default model, radial nmax 0 / 3 / 20, lmax 0 / 1 / 12, five species with
every weight type, deep and narrow networks and a 252-column descriptor.  Agreement pins
the oracle at every shape the GPU shape tests use, and the NEP oracle at NEP shapes beyond
GPUMD's defaults."""
import os

import numpy as np
import pytest

from oracle import model as OM, native as ON, nep_model as NM, nep_oracle as NO
from tests.shapes_common import NEP_SHAPES, NNAP_SHAPES, ShapeCase


def test_sweep_present():
    assert len(NNAP_SHAPES) >= 20 and len(NEP_SHAPES) >= 2


@pytest.mark.parametrize("path", NNAP_SHAPES, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_matches_reference_shapes(path):
    c = ShapeCase(path)
    pm = OM.load(c.model)
    o = ON.compute(pm, c.x, c.types, c.box_kind, c.box, want_fp=True)
    assert o["nl"].as_set() == c.nl_set()
    np.testing.assert_allclose(o["energies"], c.energies, rtol=1e-11, atol=1e-11 * max(1.0, np.abs(c.energies).max()))
    np.testing.assert_allclose(o["forces"], c.forces, rtol=1e-9, atol=1e-10 * max(1e-3, np.abs(c.forces).max()))
    np.testing.assert_allclose(o["virials"], c.virials, rtol=1e-9, atol=1e-10 * max(1e-3, np.abs(c.virials).max()))
    D = c.fp.shape[1]
    np.testing.assert_allclose(o["fp"][:, :D], c.fp, rtol=1e-9, atol=1e-10 * max(1.0, np.abs(c.fp).max()))


def test_default_model_takes_the_reference_defaults():
    """{"type": "spherical_chebyshev"} alone means nmax 5, lmax 6, rcut 6 (SphericalChebyshev.java:18-19);
    no hidden_dims means [32, 32] (FeedForward.java:28)."""
    c = ShapeCase([p for p in NNAP_SHAPES if p.endswith("default_model_t2.npz")][0])
    assert c.model["models"][0]["basis"] == {"type": "spherical_chebyshev"}
    assert "hidden_dims" not in c.model["models"][0]["nn"]
    pm = OM.load(c.model)
    sb = pm.basis[0].subs[0]
    assert (sb.nmax, sb.lmax, sb.rcut, sb.size_np) == (5, 6, 6.0, 12)
    assert list(pm.nn[0].hidden_dims) == [32, 32]


@pytest.mark.parametrize("path", NEP_SHAPES, ids=lambda p: os.path.basename(p)[:-4])
def test_nep_oracle_matches_reference_shapes(path):
    z = np.load(path)
    m = NM.load(str(z["nep"]))
    xw = ON.wrap(z["x"], int(z["box_kind"]), z["box"])
    nl = ON.neighbors(xw, int(z["box_kind"]), z["box"], max(m.rc_radial, m.rc_angular))
    assert np.max(np.abs(NO.energies(m, z["types"] - 1, nl) - z["energies"])) <= 1e-11
