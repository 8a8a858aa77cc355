"""Expansion of the reference's NEP sources for one model (NEPGEN).

TEST INFRASTRUCTURE ONLY.  Restates NEP.processLines_ / baseReplace_ (NEP.java:689-760):
``// >>> NEPGEN REMOVE`` .. ``// <<< NEPGEN REMOVE`` blocks are dropped; a
``// >>> NEPGEN PICK`` block keeps the lines of its ``// --- NEPGEN PICK: <case>`` whose
case equals the value of the key named after ``// <<< NEPGEN PICK`` (recursively
expanded); every other line has each ``__NEPGEN_KEY__`` replaced by its value.  The keys
are those of NEP.initGenMap_ (NEP.java:645-672) with the CPU / double-precision picks.
"""
from __future__ import annotations

import os
from typing import Dict, List

from .nep_model import NEPModel

REMOVE_START, REMOVE_END = "// >>> NEPGEN REMOVE", "// <<< NEPGEN REMOVE"
PICK_START, PICK_CASE, PICK_END = "// >>> NEPGEN PICK", "// --- NEPGEN PICK:", "// <<< NEPGEN PICK"


def gen_map(m: NEPModel) -> Dict[str, object]:
    return {
        "NEPGEN_USE_TABLE": 0, "NEPGEN_VERSION": m.version, "NEPGEN_NTYPES": m.ntypes,
        # type-wise cutoffs (NEP.java:650-654): the file's factors, else NEP's defaults
        "NEPGEN_USE_TYPEWISE_CUTOFF": 1 if m.typewise_descriptors else 0,
        "NEPGEN_USE_TYPEWISE_CUTOFF_ZBL": 1 if m.typewise_zbl else 0,
        "NEPGEN_TYPEWISE_CUTOFF_FACTOR_R": repr(float(m.typewise[0])) if any(m.typewise) else 2.5,
        "NEPGEN_TYPEWISE_CUTOFF_FACTOR_A": repr(float(m.typewise[1])) if any(m.typewise) else 2.0,
        "NEPGEN_TYPEWISE_CUTOFF_FACTOR_ZBL": repr(float(m.typewise[2])) if any(m.typewise) else 0.65,
        "NEPGEN_RCUT_R": repr(float(m.rc_radial)), "NEPGEN_RCUT_A": repr(float(m.rc_angular)),
        "NEPGEN_RCUT_INNER_ZBL": repr(float(m.zbl_rc_inner)) if m.zbl else "1.0",
        "NEPGEN_RCUT_OUTER_ZBL": repr(float(m.zbl_rc_outer)) if m.zbl else "2.0",
        "NEPGEN_NMAX_R": m.n_max_radial, "NEPGEN_NMAX_A": m.n_max_angular,
        "NEPGEN_BSIZE_R": m.basis_size_radial, "NEPGEN_BSIZE_A": m.basis_size_angular,
        "NEPGEN_NUMC_R": m.num_c_radial, "NEPGEN_LMAX": m.l_max, "NEPGEN_NUML": m.num_L,
        "NEPGEN_ANN_DIM_A": m.dim_angular, "NEPGEN_ANN_DIM": m.dim, "NEPGEN_NUM_NEURONS1": m.num_neurons,
        "NEPGEN_NUM_PARA": m.num_para_ann + m.num_para_descriptor, "NEPGEN_NUM_PARA_ANN": m.num_para_ann,
        "NEPGEN_ZBL": 1 if m.zbl else 0, "NEPGEN_ZBL_FLEXIBLED": 1 if m.zbl_flexible else 0,
        "[PRECISION]": "double", "[ARCH]": "cpu",
    }


def _replace(line: str, gen: Dict[str, object]) -> str:
    for k, v in gen.items():
        if k.startswith("["):
            continue
        line = line.replace("__" + k + "__", str(v))
    return line


def process(lines: List[str], gen: Dict[str, object]) -> List[str]:
    out: List[str] = []
    state, buf = "normal", []
    for line in lines:
        t = line.strip()
        if state == "normal":
            if t == REMOVE_START:
                state = "remove"
            elif t == PICK_START:
                state, buf = "pick", []
            else:
                out.append(_replace(line, gen))
        elif state == "remove":
            if t == REMOVE_END:
                state = "normal"
        else:
            if t.startswith(PICK_END):
                key = t[len(PICK_END):].strip()
                if key not in gen:
                    raise KeyError("missing pick key " + key)
                chosen, inside = [], False
                for b in buf:
                    bt = b.strip()
                    if inside:
                        if bt.startswith(PICK_CASE):
                            break
                        chosen.append(b.replace("NEPGENO", "NEPGEN"))
                    elif bt.startswith(PICK_CASE) and bt[len(PICK_CASE):].strip() == gen[key]:
                        inside = True
                out += process(chosen, gen)
                state = "normal"
            else:
                buf.append(line)
    if state != "normal":
        raise ValueError("unterminated NEPGEN block")
    return out


def expand(src_dir: str, out_dir: str, m: NEPModel) -> None:
    gen = gen_map(m)
    os.makedirs(out_dir, exist_ok=True)
    for name in ("nep_core.hpp", "nep_interface.cpp"):
        with open(os.path.join(src_dir, name)) as f:
            lines = f.read().split("\n")
        with open(os.path.join(out_dir, name), "w") as f:
            f.write("\n".join(process(lines, gen)))
