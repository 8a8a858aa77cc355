"""The allocation-free neighbour count (nnap_neighbor_counts_noalloc) against the neighbour
list of the handle-based entry point (nnap_neighbor_list).

Callers that cannot allocate device memory when they need the answer use this entry
point: a program capturing a CUDA graph in global mode, or an engine that reserves all
device memory up front.  Its scratch is a fixed array inside the library, shared by all
calls, so the test calls it twice in a row: leftovers of the first call must not leak
into the second.  Counts are integers and must match exactly.
"""
import ctypes as C

import numpy as np
import pytest

from jse_gb300 import workloads as W

pytestmark = pytest.mark.gpu


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


def test_noalloc_rejects_sizes_beyond_its_scratch():
    L = _lib()
    box = np.diag([200.0, 200.0, 200.0]).reshape(9)
    bp = box.ctypes.data_as(C.POINTER(C.c_double))
    assert L.nnap_neighbor_counts_noalloc(16385, None, None, 0, bp, 6.0, None, None) == 3  # NNAP_ERR_CAPACITY
