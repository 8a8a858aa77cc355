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


def _mirror_model():
    import numpy as np
    z = np.load(os.path.join(ROOT, "tests", "golden", "mirror_share_sph.npz"))
    return json.loads(str(z["model_json"]))


def _bad_mirror(mut):
    m = _mirror_model()
    mut(m)
    return m


MIRROR_BAD = [
    _bad_mirror(lambda m: m["models"][1]["basis"].update(mirror=2)),            # mirror of a mirror basis
    _bad_mirror(lambda m: m["models"][1]["basis"].update(mirror=3)),            # mirror of a shared basis
    _bad_mirror(lambda m: m["models"][1]["basis"].pop("mirror")),               # no source
    _bad_mirror(lambda m: m["models"][1].update(nn={"hidden_dims": [8, 8]})),   # a mirror has no network
    _bad_mirror(lambda m: m["models"][1].update(ref_eng=0.5)),                  # nor its own normalisation
    _bad_mirror(lambda m: m["models"][1].update(norm_mu=[0.0])),
    _bad_mirror(lambda m: m["models"][2]["basis"].update(share=7)),             # source out of range
    _bad_mirror(lambda m: m["models"][2]["nn"].update(share=2)),                # base network is not plain
    _bad_mirror(lambda m: m["models"][2]["nn"].pop("shared_hidden_dims")),
    _bad_mirror(lambda m: m["models"][2]["nn"].update(shared_hidden_dims=[9, 8])),
    _bad_mirror(lambda m: m["models"][2]["nn"]["hidden_weights"][0].pop()),      # 3 own rows instead of 4
    _bad_mirror(lambda m: m["models"][2]["nn"].update(shared_flags=[True, False])),
]


@pytest.mark.parametrize("model", MIRROR_BAD)
def test_invalid_mirror_and_shared_models_are_rejected(model):
    """Mirror / shared bases and shared networks: the GPU loader and the oracle's restatement
    of the reference loader both refuse the same malformed files."""
    from oracle import model as OM
    L = _lib()
    h = C.c_void_p()
    b = json.dumps(model).encode()
    assert L.nnap_create(b, len(b), 0, 0, C.byref(h)) == 1  # NNAP_ERR_BAD_MODEL
    with pytest.raises((ValueError, KeyError, TypeError)):
        OM.load(model)


def test_valid_mirror_and_shared_model_passes_the_loader():
    """The well-formed model gets past model loading (without a GPU, creation then stops at
    the first CUDA call with NNAP_ERR_CUDA rather than NNAP_ERR_BAD_MODEL)."""
    from oracle import model as OM
    m = _mirror_model()
    pm = OM.load(m)
    assert [b.kind for b in pm.basis] == ["plain", "mirror", "share"]
    L = _lib()
    h = C.c_void_p()
    b = json.dumps(m).encode()
    rc = L.nnap_create(b, len(b), 0, 0, C.byref(h))
    if rc == 0:
        L.nnap_destroy(h)
    assert rc != 1


def _nep_text(**kw):
    from oracle import nep_model as NM
    return NM.write(["Si", "O"], neurons=4, seed=2, **kw)


def _nep_lines(mut):
    lines = _nep_text().splitlines()
    mut(lines)
    return "\n".join(lines) + "\n"


NEP_BAD = [
    ("", 1), ("nep4 2 Si\n", 1), ("lj 1 Ar\n", 1),
    (_nep_lines(lambda ls: ls.__setitem__(0, "nep4_zbl 2 Si O")), 1),            # ZBL without its zbl line
    (_nep_lines(lambda ls: ls.__setitem__(0, "nep4_polarizability 2 Si O")), 5),
    (_nep_lines(lambda ls: ls.__setitem__(0, "nep3_dipole 2 Si O")), 5),
    (_nep_lines(lambda ls: ls.__setitem__(1, "cutoff 5 4 100 100 1.5 1.5")), 1),    # two of three factors
    (_nep_lines(lambda ls: ls.__setitem__(2, "n_max 4")), 1),
    (_nep_lines(lambda ls: ls.__setitem__(4, "l_max 4 2")), 1),
    (_nep_lines(lambda ls: ls.pop()), 1),                                        # one scale short
    (_nep_lines(lambda ls: ls.append("0.5")), 1),                                # one number too many
    (_nep_lines(lambda ls: ls.__setitem__(9, "abc")), 1),
]


@pytest.mark.parametrize("text,status", NEP_BAD)
def test_invalid_nep_files_are_rejected(text, status):
    """nnap_create_nep parses before any device work: malformed files return
    NNAP_ERR_BAD_MODEL (the reference loader throws IllegalArgumentException, NEP.java:795-981)
    and valid files of variants the GPU path does not evaluate NNAP_ERR_UNSUPPORTED."""
    L = _lib()
    h = C.c_void_p()
    b = text.encode()
    assert L.nnap_create_nep(b, len(b), 0, 0, C.byref(h)) == status
    assert not h.value
    assert L.nnap_create_nep(None, 0, 0, 0, None) == 6


@pytest.mark.parametrize("zbl,typewise", [(None, None), ((1.6, 2.3), None), ("flexible", None),
                                          (None, (1.5, 1.5, 0.0)), ((1.6, 2.3), (2.0, 1.6, 0.6))])
def test_valid_nep_file_passes_the_loader(zbl, typewise):
    L = _lib()
    h = C.c_void_p()
    b = _nep_text(zbl=zbl, typewise=typewise).encode()
    rc = L.nnap_create_nep(b, len(b), 0, 0, C.byref(h))
    if rc == 0:
        L.nnap_destroy(h)
    assert rc not in (1, 5, 6)
