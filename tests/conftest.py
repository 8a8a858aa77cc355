"""Shared pytest configuration: the ``gpu`` marker and fixtures for the golden cases."""
import glob
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libnnap_gb300.so")


class Case:
    """One golden fixture: model text, structure and the reference's FP64 outputs."""

    def __init__(self, path):
        z = np.load(path)
        self.name = os.path.basename(path)[:-4]
        self.model_json = str(z["model_json"])
        self.model = json.loads(self.model_json)
        self.x = z["x"]
        self.types = z["types"].astype(np.int32)
        self.box = z["box"]
        self.box_kind = int(z["box_kind"])
        self.xw = z["xw"]
        self.nl_offsets, self.nl_j, self.nl_img = z["nl_offsets"], z["nl_j"], z["nl_img"]
        self.energies, self.forces, self.virials, self.fp = z["energies"], z["forces"], z["virials"], z["fp"]
        # training gradients of L = bE.E + bF.F + bW.W (reference C-level parameter layouts)
        self.train_be, self.train_bf, self.train_bw = z["train_be"], z["train_bf"], z["train_bw"]
        self.train_grad_fp, self.train_grad_nn = z["train_grad_fp"], z["train_grad_nn"]

    def nl_set(self):
        out = set()
        for i in range(len(self.types)):
            for k in range(self.nl_offsets[i], self.nl_offsets[i + 1]):
                out.add((i, int(self.nl_j[k])) + tuple(int(v) for v in self.nl_img[k]))
        return out


GOLDEN = sorted(p for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz")) if not os.path.basename(p).startswith("nep_"))


@pytest.fixture(params=GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def golden(request):
    return Case(request.param)
