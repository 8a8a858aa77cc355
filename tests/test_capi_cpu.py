"""C ABI checks that need no GPU: every declared symbol is exported, and invalid model
files are rejected with NNAP_ERR_BAD_MODEL before any device work (the reference throws
IllegalArgumentException from its loader: NNAP.java:131-176, Basis.java:22-68,
FeedForward.java:131-221)."""
import ctypes as C
import json
import os
import re

import pytest

from tests.conftest import ROOT

HEADER = os.path.join(ROOT, "include", "nnap_gb300.h")


def _lib():
    from jse_gb300 import nnap
    if not os.path.exists(nnap.LIB_PATH):
        from jse_gb300 import build
        build.build()
    return nnap.load_library()


def test_library_exports_every_declared_symbol():
    text = open(HEADER).read()
    declared = set(re.findall(r"^\s*(?:int|const char\s*\*)\s+(nnap_[a-z_]+)\s*\(", text, re.M))
    assert {"nnap_create", "nnap_compute", "nnap_compute_batch", "nnap_compute_device"} <= declared
    L = _lib()
    missing = [s for s in sorted(declared) if not hasattr(L, s)]
    assert not missing, missing


GOOD = {"version": 6, "models": [{"symbol": "Cu", "basis": {"type": "chebyshev", "nmax": 2, "rcut": 4.0},
                                  "nn": {"hidden_dims": [4]}}]}


def _bad(mut):
    m = json.loads(json.dumps(GOOD))
    mut(m)
    return json.dumps(m)


@pytest.mark.parametrize("text", [
    "", "{", "[1,2]", '{"models": []}', '{"version": 7, "models": [{"symbol": "A"}]}',
    _bad(lambda m: m["models"][0].pop("symbol")),
    _bad(lambda m: m["models"][0].update(torch={})),
    _bad(lambda m: m["models"][0]["basis"].update(type="unknown")),
    _bad(lambda m: m["models"][0]["basis"].update(type="spherical_chebyshev", lmax=13)),
    _bad(lambda m: m["models"][0]["basis"].update(nmax=21)),
    _bad(lambda m: m["models"][0]["basis"].update(wtype="weird")),
    _bad(lambda m: m["models"][0]["basis"].update(wtype="rfuse")),
    _bad(lambda m: m["models"][0]["nn"].update(hidden_dims=[])),
    _bad(lambda m: m["models"][0]["nn"].update(input_dim=5)),
    _bad(lambda m: m["models"][0]["nn"].update(hidden_weights=[[[0.0]]])),
    _bad(lambda m: m["models"][0].update(norm_mu=[0.0])),
])
def test_invalid_models_are_rejected(text):
    L = _lib()
    h = C.c_void_p()
    b = text.encode()
    assert L.nnap_create(b, len(b), 0, 0, C.byref(h)) == 1  # NNAP_ERR_BAD_MODEL
    assert not h.value


def test_null_arguments_are_rejected():
    L = _lib()
    assert L.nnap_create(None, 0, 0, 0, None) == 6  # NNAP_ERR_ARG
    assert L.nnap_destroy(None) == 6
