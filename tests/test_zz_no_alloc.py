"""The allocation-free neighbour count (nnap_neighbor_counts_noalloc) against the neighbour
list of the handle-based entry point (nnap_neighbor_list).

Callers that cannot allocate device memory when they need the answer use this entry
point: an engine that reserves all device memory for its own pool up front, or a loop
where cudaMalloc would synchronise the device.  Its scratch is a fixed array inside the
library, shared by all calls, so the GPU tests call it twice in a row: leftovers of the
first call must not leak into the second.  Counts are integers and must match exactly.
The size and argument checks run before any device work, so they are tested on the CPU.
"""
import ctypes as C

import numpy as np
import pytest

from jse_gb300 import workloads as W

NNAP_ERR_CAPACITY, NNAP_ERR_ARG = 3, 6


def _lib():
    from jse_gb300.nnap import load_library
    L = load_library()
    L.nnap_neighbor_counts_noalloc.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                               C.POINTER(C.c_double), C.c_double, C.c_void_p, C.c_void_p]
    L.nnap_neighbor_counts_noalloc.restype = C.c_int
    return L


def _noalloc_counts(L, s, rcut):
    import torch
    dev = torch.device("cuda", 0)
    x = torch.from_numpy(np.ascontiguousarray(s.x)).to(dev)
    t = torch.from_numpy(np.ascontiguousarray(s.types, dtype=np.int32)).to(dev)
    out = torch.full((s.natoms,), -1, dtype=torch.int32, device=dev)
    box = np.ascontiguousarray(s.box, dtype=np.float64).reshape(9)
    torch.cuda.synchronize(dev)
    rc = L.nnap_neighbor_counts_noalloc(s.natoms, x.data_ptr(), t.data_ptr(), s.box_kind,
                                        box.ctypes.data_as(C.POINTER(C.c_double)), rcut, out.data_ptr(), None)
    assert rc == 0, rc
    return out.cpu().numpy()


def _thin_triclinic(seed):
    """About 90 atoms in a LAMMPS triclinic box whose c planes are 4.8 A apart, below the
    6 A cutoff: the cell list searches two cell layers along c and rows hold images."""
    box = np.array([[18.0, 0.0, 0.0], [3.0, 18.0, 0.0], [2.0, 1.5, 4.8]])
    n = int(0.058 * 18.0 * 18.0 * 4.8)
    x = W._rsa(n, box, 2.0, seed)
    types = (np.arange(n) % 3 + 1).astype(np.int32)
    return W.Structure(x, types, box, W.BOX_LMP)


@pytest.mark.gpu
def test_noalloc_counts_match_neighbor_list_twice():
    from jse_gb300.nnap import NNAP
    L = _lib()
    model = W.model_for("c2")
    s1 = W.random_liquid(3000, 0.060, [0.46, 0.46, 0.08], 2.0, 71, tilt=0.1)
    s2 = W.random_liquid(1200, 0.062, [0.46, 0.46, 0.08], 2.0, 72)
    with NNAP(model) as p:
        ref1 = np.diff(p.neighborList(s1)[0])
        ref2 = np.diff(p.neighborList(s2)[0])
        rcut = p.rcutMax()
    a = _noalloc_counts(L, s1, rcut)
    b = _noalloc_counts(L, s2, rcut)
    assert np.array_equal(a, ref1)
    assert np.array_equal(b, ref2)


@pytest.mark.gpu
def test_noalloc_thin_triclinic_box_twice():
    from jse_gb300.nnap import NNAP
    L = _lib()
    s = _thin_triclinic(73)
    with NNAP(W.model_for("c2")) as p:
        ref = np.diff(p.neighborList(s)[0])
        rcut = p.rcutMax()
    assert ref.max() > 0
    for _ in range(2):
        assert np.array_equal(_noalloc_counts(L, s, rcut), ref)


def test_noalloc_rejects_too_many_atoms():
    L = _lib()
    box = np.diag([200.0, 200.0, 200.0]).reshape(9)
    bp = box.ctypes.data_as(C.POINTER(C.c_double))
    assert L.nnap_neighbor_counts_noalloc(16385, None, None, 0, bp, 6.0, None, None) == NNAP_ERR_CAPACITY


def test_noalloc_rejects_too_many_cells():
    """A 200 A box with a 6 A cutoff needs 33^3 > 16384 cells: refused before any device work."""
    L = _lib()
    box = np.diag([200.0, 200.0, 200.0]).reshape(9)
    bp = box.ctypes.data_as(C.POINTER(C.c_double))
    assert L.nnap_neighbor_counts_noalloc(100, 8, 8, 0, bp, 6.0, 8, None) == NNAP_ERR_CAPACITY


@pytest.mark.parametrize("rcut", [float("inf"), float("nan"), 0.0, -1.0])
def test_noalloc_rejects_bad_cutoff(rcut):
    L = _lib()
    box = np.diag([20.0, 20.0, 20.0]).reshape(9)
    bp = box.ctypes.data_as(C.POINTER(C.c_double))
    assert L.nnap_neighbor_counts_noalloc(10, 8, 8, 0, bp, rcut, 8, None) == NNAP_ERR_ARG


@pytest.mark.parametrize("box", [np.diag([np.inf, 20.0, 20.0]), np.diag([20.0, -20.0, 20.0]),
                                 np.diag([20.0, 20.0, 1e-9]),
                                 np.array([[20.0, 0, 0], [0, 20.0, 0], [20.0, 20.0, 0.0]])])
def test_noalloc_rejects_bad_box(box):
    """Non-finite, left-handed, far too thin and flat boxes fail the shared geometry checks."""
    L = _lib()
    b = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
    assert L.nnap_neighbor_counts_noalloc(10, 8, 8, 2, b.ctypes.data_as(C.POINTER(C.c_double)), 6.0, 8,
                                          None) == NNAP_ERR_ARG
