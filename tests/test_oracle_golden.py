"""The CPU oracle against the golden vectors generated from the reference's own arithmetic.

The golden fixtures (tests/golden/make_golden.py) hold FP64 outputs of the reference's
expanded NNAP headers; agreement here pins the oracle that the GPU tests compare with.
"""
import numpy as np
import pytest

from oracle import model as OM, native as ON


def test_oracle_matches_reference_outputs(golden):
    pm = OM.load(golden.model)
    o = ON.compute(pm, golden.x, golden.types, golden.box_kind, golden.box, want_fp=True)
    np.testing.assert_allclose(o["xw"], golden.xw, rtol=0, atol=0)
    assert o["nl"].as_set() == golden.nl_set()
    scale_e = max(1.0, np.abs(golden.energies).max())
    np.testing.assert_allclose(o["energies"], golden.energies, rtol=1e-11, atol=1e-11 * scale_e)
    scale_f = max(1e-3, np.abs(golden.forces).max())
    np.testing.assert_allclose(o["forces"], golden.forces, rtol=1e-9, atol=1e-10 * scale_f)
    scale_v = max(1e-3, np.abs(golden.virials).max())
    np.testing.assert_allclose(o["virials"], golden.virials, rtol=1e-9, atol=1e-10 * scale_v)
    D = golden.fp.shape[1]
    np.testing.assert_allclose(o["fp"][:, :D], golden.fp, rtol=1e-9, atol=1e-10 * max(1.0, np.abs(golden.fp).max()))


@pytest.mark.parametrize("case", ["sph_small_images", "sph_general_prism", "isolated_and_unwrapped", "sph_binary_tri"])
def test_cell_list_equals_brute_force(case):
    from tests.conftest import Case, GOLDEN_DIR
    import os
    c = Case(os.path.join(GOLDEN_DIR, case + ".npz"))
    rc = OM.load(c.model).rcut_max
    a = ON.neighbors(c.xw, c.box_kind, c.box, rc).as_set()
    b = ON.neighbors(c.xw, c.box_kind, c.box, rc, brute=True).as_set()
    assert a == b
    assert a == c.nl_set()


def test_small_box_contains_self_images():
    from tests.conftest import Case, GOLDEN_DIR
    import os
    c = Case(os.path.join(GOLDEN_DIR, "sph_small_images.npz"))
    s = c.nl_set()
    assert any(i == j for (i, j, *_img) in s), "a box smaller than 2 rcut must list images of the atom itself"
    assert all(not (i == j and img == [0, 0, 0]) for (i, j, *img) in s)
