"""Generate the golden fixtures in this directory from the reference's own arithmetic.

Run from the repository root, where a reference checkout is available
(``$JSE_REFERENCE``, else a ``reference`` folder beside the repository):

    python -m tests.golden.make_golden

For every case the reference's NNAP headers are expanded for the model's shape
(``oracle/nnapgen.py``) and compiled without fast-math (``oracle/build.py``); the
per-atom function ``jse_nnap_calEnergyForce`` then evaluates each atom over the
neighbour list of the oracle's restatement of ``NeighborListGetter``, and the
driver (``oracle/ref_driver.cpp``) scatters energies, forces and per-atom virials
like ``NNAP.calEnergyForceVirial``.  Descriptors come from ``jse_nnap_calFp``.

Each ``<case>.npz`` holds the model JSON text, the structure, the neighbour set
(offsets, j, image) and the reference's FP64 outputs, including the parameter
gradients of a seeded energy / force / virial loss through the reference's training
pair ``jse_nnap_forwardEnergyForce`` / ``jse_nnap_backwardEnergyForce``
(``train_*`` keys; ``ref_train_grad`` in ``oracle/ref_driver.cpp``).
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from jse_gb300 import workloads as W  # noqa: E402
from oracle import model as OM, native as ON  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def _sph(nmax, lmax, rcut, wtype="default", **kw):
    d = {"type": "spherical_chebyshev", "nmax": nmax, "lmax": lmax, "rcut": rcut, "wtype": wtype}
    d.update(kw)
    return d


def _model(symbols, basis, hidden, seed, **kw):
    """A model with random weights; basis may carry explicit fuse/rfuse weights or be merged."""
    D = OM.load({"models": [{"symbol": s, "basis": basis} for s in symbols]}).basis[0].size
    rng = np.random.default_rng(seed)
    models = []
    for s in symbols:
        hw, hb, fan = [], [], D
        for h in hidden:
            hw.append(rng.normal(0, (1 / fan) ** 0.5, (h, fan)).tolist())
            hb.append(rng.normal(0, (1 / fan) ** 0.5, h).tolist())
            fan = h
        models.append({"symbol": s, "basis": basis,
                       "nn": {"type": "feed_forward", "input_dim": D, "hidden_dims": list(hidden),
                              "hidden_weights": hw, "hidden_biases": hb,
                              "output_weight": rng.normal(0, (1 / fan) ** 0.5, fan).tolist(),
                              "output_bias": float(rng.normal())}})
    models[0]["norm_mu_eng"] = -2.0
    models[0]["norm_sigma_eng"] = 0.5
    return {"version": 6, "units": "metal", "models": models}


def _normalised(model: dict, s: W.Structure) -> dict:
    """Set norm_mu / norm_sigma to the descriptor statistics of the structure (per species)."""
    pm = OM.load(model)
    o = ON.compute(pm, s.x, s.types, s.box_kind, s.box, want_fp=True)
    for t, mm in enumerate(model["models"]):
        D = pm.basis[t].size
        sel = o["fp"][s.types == t + 1, :D]
        if len(sel) == 0:
            continue
        mm["norm_mu"] = sel.mean(0).tolist()
        mm["norm_sigma"] = (sel.std(0) + 1e-3).tolist()
        mm["ref_eng"] = 0.1 * (t + 1)
    return model


def cases():
    rng = np.random.default_rng(1234)
    out = {}
    # radial Chebyshev, single element, perturbed FCC (shape of the 4000-atom FCC workload)
    s = W.fcc(3.61, 3, 0.05, 21)
    out["radial_fcc"] = (W.model_for("c1", seed=31), s)
    # spherical Chebyshev, three species, orthogonal liquid (basis shape of the 32000-atom liquid)
    s = W.random_liquid(160, 0.060, [0.46, 0.46, 0.08], 2.0, 22)
    out["sph_ternary_ortho"] = (_normalised(W.write_model(["A", "B", "C"], W.C2_BASIS, [16, 16], 32), s), s)
    # spherical Chebyshev, two species, LAMMPS triclinic (basis shape of the 1M-atom glass)
    s = W.random_liquid(200, 0.058, [0.64, 0.36], 2.1, 23, tilt=0.1)
    out["sph_binary_tri"] = (_normalised(W.write_model(["A", "B"], W.C3_BASIS, [16, 16], 33), s), s)
    # small triclinic box: several images of the same neighbour and of the atom itself
    s = W.random_liquid(12, 0.062, [0.46, 0.46, 0.08], 2.0, 24, tilt=0.1)
    out["sph_small_images"] = (W.write_model(["A", "B", "C"], W.C2_BASIS, [16, 16], 34), s)
    # unperturbed FCC: neighbours exactly on the z axis (the spherical-harmonic pole branch)
    s = W.fcc(3.61, 3, 0.0, 25)
    out["sph_fcc_pole"] = (W.write_model(["Cu"], _sph(4, 4, 5.2), [16, 16], 35), s)
    # weight types and fused radial weights
    s = W.random_liquid(120, 0.06, [0.5, 0.5], 2.0, 26)
    for wt in ("none", "full", "exfull"):
        out["wtype_" + wt] = (W.write_model(["A", "B"], _sph(3, 2, 5.0, wt), [8, 8], 36), s)
    NP, sn = 5, 2 * 4
    rw = rng.uniform(-1, 1, NP * sn).tolist()
    out["wtype_rfuse_ws"] = (_model(["A", "B"], _sph(3, 3, 5.0, "rfuse", rfuse_size=NP, rfuse_weight=rw,
                                                     rfuse_scale=0.4, weight_standardization=True), [8, 8], 37), s)
    fw = rng.uniform(-1, 1, 2 * 3).tolist()
    out["wtype_fuse"] = (_model(["A", "B"], _sph(3, 2, 5.0, "fuse", fuse_size=3, fuse_weight=fw), [8, 8], 38), s)
    out["wtype_exfuse"] = (_model(["A", "B"], _sph(3, 2, 5.0, "exfuse", fuse_size=3, fuse_weight=fw), [8, 8], 39), s)
    # merged basis: radial + spherical with different cutoffs
    merged = {"type": "merge", "basis": [{"type": "chebyshev", "nmax": 5, "rcut": 5.5},
                                          _sph(4, 3, 4.2)]}
    out["merged_basis"] = (_model(["A", "B"], merged, [8, 8], 40), s)
    # general (non-LAMMPS) prism box
    base = W.random_liquid(90, 0.06, [0.5, 0.5], 2.0, 27)
    L = base.box[0, 0]
    box = np.array([[L, 0.05 * L, -0.03 * L], [0.1 * L, 0.95 * L, 0.02 * L], [-0.08 * L, 0.07 * L, 1.02 * L]])
    frac = base.x @ np.linalg.inv(base.box)
    xp = frac @ box + rng.normal(0, 0.01, base.x.shape)
    sp = W.Structure(xp, base.types, box, W.BOX_PRISM)
    out["sph_general_prism"] = (W.write_model(["A", "B"], _sph(4, 3, 5.0), [8, 8], 41), sp)
    # one atom far from every other one (zero neighbours) plus atoms outside the box
    xs = np.array([[1.0, 1.0, 1.0], [3.2, 1.1, 0.9], [2.0, 3.0, 1.5], [15.0, 15.0, 15.0], [-1.0, 31.5, 7.0]])
    s = W.Structure(xs, np.array([1, 2, 1, 2, 1], dtype=np.int32), np.diag([30.0, 30.0, 30.0]), W.BOX_ORTHO)
    out["isolated_and_unwrapped"] = (W.write_model(["A", "B"], _sph(4, 3, 5.0), [8, 8], 42), s)
    # mirror and shared bases with a partly shared network: B mirrors A (its own species and
    # A swapped among the neighbours, A's network and normalisation), C uses A's basis and
    # shares A's network except the first 4 rows of the first hidden layer and the output
    s3 = W.random_liquid(120, 0.06, [0.4, 0.4, 0.2], 2.0, 28)
    for name, basis in (("mirror_share_sph", _sph(3, 2, 5.0, "full")),
                        ("mirror_share_radial", {"type": "chebyshev", "nmax": 3, "rcut": 5.5, "wtype": "full"})):
        m = _model(["A", "B", "C"], basis, [8, 8], 43)
        D = OM.load(m).basis[0].size
        nrm = _normalised(json.loads(json.dumps(m)), s3)["models"][0]
        m["models"][0].update({k: nrm[k] for k in ("norm_mu", "norm_sigma", "ref_eng")})
        m["models"][1] = {"symbol": "B", "basis": {"type": "mirror", "mirror": 1}}
        m["models"][2]["basis"] = {"type": "share", "share": 1}
        m["models"][2]["nn"] = {"type": "shared_feed_forward", "share": 1, "shared_hidden_dims": [4, 8],
                                "hidden_weights": [rng.normal(0, D ** -0.5, (4, D)).tolist(), []],
                                "hidden_biases": [rng.normal(0, 0.3, 4).tolist(), []],
                                "output_weight": rng.normal(0, 0.35, 8).tolist(), "output_bias": 0.2}
        out[name] = (m, s3)
    # fused radial weights behind a mirror and a shared basis: their gradients belong to A
    fw3 = rng.uniform(-1, 1, 3 * 3).tolist()
    m = _model(["A", "B", "C"], _sph(3, 2, 5.0, "fuse", fuse_size=3, fuse_weight=fw3), [8, 8], 44)
    m["models"][1] = {"symbol": "B", "basis": {"type": "mirror", "mirror": 1}}
    m["models"][2]["basis"] = {"type": "share", "share": 1}
    out["mirror_share_fuse"] = (m, s3)
    # three- and four-body invariant columns (l3max / l4max), including an expansion whose
    # largest l comes from l3max rather than lmax
    s2 = W.random_liquid(120, 0.06, [0.5, 0.5], 2.0, 26)
    out["sph_bispectrum"] = (_model(["A", "B"], _sph(3, 3, 5.0, "full", l3max=3, l4max=2), [8, 8], 45), s2)
    s1 = W.random_liquid(100, 0.06, [1.0], 2.0, 29)
    out["sph_bispectrum_high"] = (_model(["A"], _sph(4, 2, 5.0, "default", l3max=4, l4max=3), [8, 8], 46), s1)
    fw2 = rng.uniform(-1, 1, 2 * 2).tolist()
    out["sph_bispectrum_fuse"] = (_model(["A", "B"], _sph(3, 3, 5.0, "fuse", fuse_size=2, fuse_weight=fw2, l3max=3,
                                                          l4max=2), [8, 8], 47), s2)
    return out


def main():
    only = set(sys.argv[1:])  # optional case names: regenerate only those
    for name, (model, s) in cases().items():
        if only and name not in only:
            continue
        pm = OM.load(model)
        o = ON.compute(pm, s.x, s.types, s.box_kind, s.box)
        nl = o["nl"]
        ref = ON.RefLib(pm)
        r = ref.compute(s.types, nl)
        fp = ref.fp(s.types, nl)
        # training gradients of L = bE.E + bF.F + bW.W for seeded upstream gradients
        n = len(s.types)
        rng = np.random.default_rng(len(name) * 7919 + n)
        be, bf, bw = rng.normal(size=n), rng.normal(size=(n, 3)), rng.normal(size=9)
        tg = ref.train_grad(s.types, nl, be, bf, bw)
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            model_json=np.array(json.dumps(model)), x=s.x, types=s.types, box=s.box, box_kind=np.array(s.box_kind),
            xw=o["xw"], nl_offsets=nl.offsets, nl_j=nl.j, nl_img=nl.img,
            energies=r["energies"], forces=r["forces"], virials=r["virials"], fp=fp,
            train_be=be, train_bf=bf, train_bw=bw, train_grad_fp=np.concatenate(tg["grad_fp"]),
            train_grad_nn=np.concatenate(tg["grad_nn"]))
        print("%-24s n=%4d pairs=%6d E=%.10f" % (name, len(s.types), len(nl.j), r["energy"]))


if __name__ == "__main__":
    main()
