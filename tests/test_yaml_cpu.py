"""YAML model files (NNAP.java:407-411: .yaml / .yml files are read with IO.yaml2map).

Every golden model, written as YAML in the block style of Groovy's YamlBuilder (nested
sequences as "- - x") and with flow lists, loads to exactly the model its JSON loads to:
the digest of nnap_model_check covers every value the kernels consume.  Malformed YAML
gives NNAP_ERR_BAD_MODEL.  No GPU is needed.
"""
import glob
import json
import os

import numpy as np
import pytest

from jse_gb300 import workloads as W
from jse_gb300.nnap import NNAP_ERR_BAD_MODEL, NNAPError, model_check
from tests.conftest import GOLDEN_DIR
from tests.yaml_emit import dump

MODELS = sorted(glob.glob(os.path.join(GOLDEN_DIR, "*.npz")) + glob.glob(os.path.join(GOLDEN_DIR, "shapes", "*.npz")))
MODELS = [p for p in MODELS if not os.path.basename(p).startswith("nep_")]


@pytest.mark.parametrize("path", MODELS, ids=lambda p: os.path.basename(p)[:-4])
@pytest.mark.parametrize("flow", [False, True])
def test_yaml_loads_the_same_model_as_json(path, flow):
    text = str(np.load(path)["model_json"])
    ref = model_check(text)
    y = dump(json.loads(text), flow_lists=flow, comments=True)
    assert not y.lstrip().startswith("{")
    got = model_check(y)
    assert got == ref


def test_yaml_file_and_defaults(tmp_path):
    """A .yaml file on disk; keys left out take the reference's defaults as in JSON."""
    m = W.model_for("c2")
    p = tmp_path / "model.yaml"
    p.write_text(dump(m))
    assert model_check(str(p)) == model_check(m)
    y = dump({"models": [{"symbol": "Cu", "basis": {"type": "chebyshev"},
                          "nn": {"hidden_dims": [4], "hidden_weights": [[[0.1] * 6] * 4], "hidden_biases": [[0.0] * 4],
                                 "output_weight": [1.0] * 4, "output_bias": 0.0}}]})
    assert model_check(y)["ntypes"] == 1


@pytest.mark.parametrize("bad", [
    "models:\n- symbol: A\n  basis: [1, 2\n",                 # unclosed flow sequence
    "models:\n\t- symbol: A\n",                                # tab indentation
    "models: &x\n- symbol: A\n",                               # anchors are not read
    "models:\n- symbol: A\n   basis: 1\n",                     # inconsistent indentation
    "version: 6\nversion: 6\nmodels: []\n",                    # duplicate key
    "models:\n- symbol: A\n  nn: |\n    text\n",               # block scalar
])
def test_malformed_yaml_is_a_bad_model(bad):
    with pytest.raises(NNAPError) as e:
        model_check(bad)
    assert e.value.status == NNAP_ERR_BAD_MODEL
