"""The seeded synthetic-structure generator (random sequential addition in numpy).

Both benchmark arms and the tests build their inputs with it, so it must give the same
structures on every machine (no BLAS arithmetic, PCG64 stream) and keep every pair of
atoms, over all periodic images, at least the minimum separation apart.
"""
import hashlib

import numpy as np
import pytest

from jse_gb300 import workloads as W
from oracle import native as ON


def test_generator_is_pinned():
    s = W.random_liquid(500, 0.060, [0.46, 0.46, 0.08], 2.0, 5, tilt=0.1)
    assert hashlib.sha1(np.ascontiguousarray(s.x).tobytes()).hexdigest()[:12] == "4cd9a21d18cc"
    assert np.bincount(s.types).tolist() == [0, 230, 230, 40]


@pytest.mark.parametrize("n,rho,rmin,tilt", [(32, 0.065, 2.0, 0.1), (700, 0.060, 2.0, None),
                                             (3000, 0.058, 2.1, 0.1)])
def test_minimum_separation_over_all_images(n, rho, rmin, tilt):
    s = W.random_liquid(n, rho, [0.5, 0.5], rmin, 9, tilt=tilt)
    assert s.natoms == n
    xw = ON.wrap(s.x, s.box_kind, s.box)
    assert len(ON.neighbors(xw, s.box_kind, s.box, rmin, brute=n <= 700).j) == 0
    # and the structure is not sparser than asked: about 4 pi/3 rc^3 rho neighbours at 6 A
    nl = ON.neighbors(xw, s.box_kind, s.box, 6.0)
    assert abs(len(nl.j) / n / (4.18879 * 216 * rho) - 1.0) < 0.15
