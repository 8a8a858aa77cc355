"""Shared loader of the shape-sweep fixtures (tests/golden/shapes, made by
tests/golden/make_golden_shapes.py from the reference's own arithmetic)."""
import glob
import json
import os

import numpy as np

from tests.conftest import GOLDEN_DIR

SHAPES_DIR = os.path.join(GOLDEN_DIR, "shapes")
NNAP_SHAPES = sorted(p for p in glob.glob(os.path.join(SHAPES_DIR, "*.npz")) if not os.path.basename(p).startswith("nep_"))
NEP_SHAPES = sorted(glob.glob(os.path.join(SHAPES_DIR, "nep_*.npz")))


class ShapeCase:
    def __init__(self, path):
        z = np.load(path)
        self.name = os.path.basename(path)[:-4]
        self.model_json = str(z["model_json"])
        self.model = json.loads(self.model_json)
        self.x, self.types = z["x"], z["types"].astype(np.int32)
        self.box, self.box_kind = z["box"], int(z["box_kind"])
        self.xw = z["xw"]
        self.nl_offsets, self.nl_j, self.nl_img = z["nl_offsets"], z["nl_j"], z["nl_img"]
        self.energies, self.forces, self.virials, self.fp = z["energies"], z["forces"], z["virials"], z["fp"]

    def nl_set(self):
        out = set()
        for i in range(len(self.types)):
            for k in range(self.nl_offsets[i], self.nl_offsets[i + 1]):
                out.add((i, int(self.nl_j[k])) + tuple(int(v) for v in self.nl_img[k]))
        return out
