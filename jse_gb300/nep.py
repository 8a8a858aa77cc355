"""GB300 NEP potential: the reference's ``jsex.nep.NEP`` over the NNAP descriptor pipeline.

``NEP(path_or_text)`` loads a nep.txt potential (NEP.java:98-100, loader NEP.java:786-1010;
nep3 / nep4 / nep5 potential models, with or without ZBL and type-wise cutoffs) through
``nnap_create_nep``; every evaluation method of :class:`jse_gb300.nnap.NNAP` applies
(energies, forces and virials of single structures, batches, device buffers, the
LAMMPS-style boundary and the serving loop).  Species are 1-based, as the reference's
``IPairPotential`` callers pass them (``symbol(1)`` is the first symbol of the file).
"""
from __future__ import annotations

import ctypes as C
import os

from .nnap import NNAP, NNAP_ERR_BAD_MODEL, NNAP_ERR_UNSUPPORTED, NNAP_OK, PREC, NNAPError, load_library


class NEP(NNAP):
    """NEP potential on the GPU.  ``potential`` is a nep.txt path or the file's text."""

    def __init__(self, potential: str, precision: str = "fp32", device: int = 0):
        L = load_library()
        if precision not in PREC:
            raise ValueError("precision must be 'fp32' or 'mixed'")
        h = C.c_void_p()
        if "\n" not in potential and os.path.exists(potential):
            rc = L.nnap_create_nep_from_file(potential.encode(), PREC[precision], device, C.byref(h))
        else:
            b = potential.encode()
            rc = L.nnap_create_nep(b, len(b), PREC[precision], device, C.byref(h))
        if rc != NNAP_OK:
            why = {NNAP_ERR_BAD_MODEL: "invalid nep.txt", NNAP_ERR_UNSUPPORTED: "unsupported NEP variant or shape"}
            raise NNAPError(rc, why.get(rc, "handle creation failed"))
        self._h = h
        self._L = L
        self.precision = precision
