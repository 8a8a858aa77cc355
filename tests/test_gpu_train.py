"""Force-training gradients on the GPU (nnap_train_grad_batch).

* Against the golden fixtures: the reference's own gradients of a seeded loss
  L = bE.E + bF.F + bW.W through jse_nnap_forwardEnergyForce / jse_nnap_backwardEnergyForce,
  for every fixture (weight types, merged, mirror and shared bases, pole neighbours,
  isolated atoms, small boxes with self-images).
* At the production network shape (126 -> 64 -> 64 -> 1) and several thousand atoms,
  where the oracle's per-atom loop would be slow to drive through the reference, against
  central differences of the FP64 oracle's loss along random parameter directions.
* Batches: the gradient of a batch is the sum of its structures' gradients, with the
  virial upstream gradient applied per structure; repeated calls are bit-identical.
"""
import json
import os

import numpy as np
import pytest

from jse_gb300 import workloads as W
from oracle import model as OM, native as ON

pytestmark = pytest.mark.gpu

# FP32 descriptors and network against the FP64 reference: largest gradient component
# difference relative to the largest gradient component.
G_TOL = 2e-4


def _nnap(model, precision="fp32"):
    from jse_gb300.nnap import NNAP
    return NNAP(json.dumps(model) if isinstance(model, dict) else model, precision=precision)


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30))


def test_golden_gradients(golden):
    pm = OM.load(golden.model)
    fused = any(sb.internal_wtype in (OM.WTYPE_FUSE, OM.WTYPE_RFUSE, OM.WTYPE_EXFUSE)
                for b in pm.basis for sb in b.subs)
    s = W.Structure(golden.x, golden.types, golden.box, golden.box_kind)
    with _nnap(golden.model_json) as p:
        out = p.backwardEnergyForceBatch([s], golden.train_be, golden.train_bf, golden.train_bw[None, :],
                                         want_fp=False)
        got = np.concatenate(out["grad_nn"])
        assert got.shape == golden.train_grad_nn.shape
        assert _rel(got, golden.train_grad_nn) <= G_TOL, _rel(got, golden.train_grad_nn)
        out = p.backwardEnergyForceBatch([s], golden.train_be, golden.train_bf, golden.train_bw[None, :],
                                         want_fp=True)
        gfp = np.concatenate(out["grad_fp"])
        assert gfp.shape == golden.train_grad_fp.shape
        assert np.array_equal(np.concatenate(out["grad_nn"]), got)
        if fused:
            assert _rel(gfp, golden.train_grad_fp) <= G_TOL, _rel(gfp, golden.train_grad_fp)
        else:
            assert not np.any(golden.train_grad_fp) and not np.any(gfp)


def _set_cparam(nn, vec):
    k = 0
    for i, w in enumerate(nn.hidden_weights):
        nn.hidden_weights[i] = vec[k:k + w.size].reshape(w.shape)
        k += w.size
    nn.output_weight = vec[k:k + nn.output_weight.size].copy()
    k += nn.output_weight.size
    for i, b in enumerate(nn.hidden_biases):
        nn.hidden_biases[i] = vec[k:k + b.size].copy()
        k += b.size
    nn.output_bias = float(vec[k])


def _fd(model, structs, be, bf, bw, vs, h=1e-5):
    """Central difference of the oracle's loss along parameter directions vs (per species)."""
    pm = OM.load(model)
    base = [pm.nn[t].cparam.copy() for t in range(pm.ntypes)]

    def loss():
        tot, a0 = 0.0, 0
        for k, s in enumerate(structs):
            o = ON.compute(pm, s.x, s.types, s.box_kind, s.box)
            n = len(s.types)
            tot += be[a0:a0 + n] @ o["energies"] + np.sum(bf[a0:a0 + n] * o["forces"]) + bw[k] @ o["virial"]
            a0 += n
        return tot

    vals = []
    for sgn in (1.0, -1.0):
        for t in range(pm.ntypes):
            _set_cparam(pm.nn[t], base[t] + sgn * h * vs[t])
        vals.append(loss())
    return (vals[0] - vals[1]) / (2 * h)


@pytest.mark.parametrize("n,seed", [(3000, 71), (700, 72)])
def test_production_shape_against_oracle_differences(n, seed):
    model = W.model_for("c2")
    s = W.random_liquid(n, 0.060, [0.46, 0.46, 0.08], 2.0, seed, tilt=0.1)
    rng = np.random.default_rng(seed)
    be = rng.normal(size=n)
    bf = rng.normal(size=(n, 3))
    bw = rng.normal(size=(1, 9))
    with _nnap(model) as p:
        g = p.backwardEnergyForceBatch([s], be, bf, bw)["grad_nn"]
    pm = OM.load(model)
    for trial in range(2):
        vs = [rng.normal(size=pm.nn[t].cparam.size) for t in range(pm.ntypes)]
        pred = sum(float(g[t] @ vs[t]) for t in range(pm.ntypes))
        fd = _fd(model, [s], be, bf, bw, vs)
        assert abs(pred - fd) <= 2e-4 * abs(fd), (pred, fd)


def test_batch_is_the_sum_of_its_structures_and_deterministic():
    model = W.model_for("c2")
    structs = [W.random_liquid(n, 0.060, [0.46, 0.46, 0.08], 2.0, 80 + k, tilt=0.1 * (k % 2))
               for k, n in enumerate([40, 300, 1500])]
    rng = np.random.default_rng(9)
    N = sum(len(s.types) for s in structs)
    be = rng.normal(size=N)
    bf = rng.normal(size=(N, 3))
    bw = rng.normal(size=(3, 9))
    with _nnap(model) as p:
        a = p.backwardEnergyForceBatch(structs, be, bf, bw)["grad_nn"]
        b = p.backwardEnergyForceBatch(structs, be, bf, bw)["grad_nn"]
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
        parts, a0 = [], 0
        for k, s in enumerate(structs):
            n = len(s.types)
            parts.append(p.backwardEnergyForceBatch([s], be[a0:a0 + n], bf[a0:a0 + n], bw[k:k + 1])["grad_nn"])
            a0 += n
    for t in range(len(a)):
        tot = sum(pp[t] for pp in parts)
        assert _rel(a[t], tot) <= 1e-5
    # and against the oracle along a random direction
    pm = OM.load(model)
    vs = [rng.normal(size=pm.nn[t].cparam.size) for t in range(pm.ntypes)]
    pred = sum(float(a[t] @ vs[t]) for t in range(pm.ntypes))
    fd = _fd(model, structs, be, bf, bw, vs)
    assert abs(pred - fd) <= 2e-4 * abs(fd), (pred, fd)


def test_upstream_terms_separately():
    """Energy-only, force-only and virial-only losses, and a zero loss."""
    model = W.model_for("c3")
    s = W.random_liquid(500, 0.058, [0.64, 0.36], 2.1, 91, tilt=0.1)
    n = len(s.types)
    rng = np.random.default_rng(3)
    pm = OM.load(model)
    vs = [rng.normal(size=pm.nn[t].cparam.size) for t in range(pm.ntypes)]
    zero_e, zero_f, zero_w = np.zeros(n), np.zeros((n, 3)), np.zeros((1, 9))
    with _nnap(model) as p:
        g0 = p.backwardEnergyForceBatch([s])["grad_nn"]
        assert all(not np.any(x) for x in g0)
        for be, bf, bw in ((rng.normal(size=n), None, None), (None, rng.normal(size=(n, 3)), None),
                           (None, None, rng.normal(size=(1, 9)))):
            g = p.backwardEnergyForceBatch([s], be, bf, bw)["grad_nn"]
            pred = sum(float(g[t] @ vs[t]) for t in range(pm.ntypes))
            fd = _fd(model, [s], zero_e if be is None else be, zero_f if bf is None else bf,
                     zero_w if bw is None else bw, vs)
            assert abs(pred - fd) <= 2e-4 * max(abs(fd), 1e-6), (pred, fd)


def test_mixed_precision_handle_gives_the_fp32_gradients():
    model = W.model_for("c2")
    s = W.random_liquid(400, 0.060, [0.46, 0.46, 0.08], 2.0, 93)
    rng = np.random.default_rng(4)
    n = len(s.types)
    be, bf = rng.normal(size=n), rng.normal(size=(n, 3))
    with _nnap(model, "fp32") as a, _nnap(model, "mixed") as b:
        ga = a.backwardEnergyForceBatch([s], be, bf)["grad_nn"]
        gb = b.backwardEnergyForceBatch([s], be, bf)["grad_nn"]
    for x, y in zip(ga, gb):
        assert np.array_equal(x, y)
