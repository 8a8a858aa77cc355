"""Training gradients of the golden fixtures against finite differences of the oracle.

The fixtures hold the reference's parameter gradients of the loss
    L = sum_i bE_i E_i + sum_i bF_i . F_i + sum_ab bW_ab W_ab
(E per-atom energies, F forces, W the total virial) through its training pair
jse_nnap_forwardEnergyForce / jse_nnap_backwardEnergyForce (nnap_interface.cpp:142-232),
driven like TrainerNNAP's force branch (TrainerNNAP.java:1006-1175).  Here the
gradient's projection on a random direction of parameter space is compared with the
central difference of L evaluated by the oracle's own FP64 restatement, for the network
parameters of every species and for the radial-fuse matrices where the basis has them.
"""
import os

import numpy as np
import pytest

from oracle import model as OM, native as ON


def set_cparam(nn, vec):
    """Write ``hidden W | output W | hidden b | output b`` back into a FeedForward."""
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
    assert k + 1 == vec.size


def train_loss(pm, c, nl, be, bf, bw):
    o = ON.compute(pm, c.x, c.types, c.box_kind, c.box, nl=nl)
    return be @ o["energies"] + np.sum(bf * o["forces"]) + bw @ o["virial"]


def split(vec, sizes):
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(int)
    return [vec[off[t]:off[t + 1]] for t in range(len(sizes))]


def fd_directional(c, which, h=1e-5, seed=0):
    """(gradient . v, central difference along v) for network ('nn') or basis ('fp') parameters."""
    pm = OM.load(c.model)
    nl = ON.compute(pm, c.x, c.types, c.box_kind, c.box)["nl"]
    T = pm.ntypes
    rng = np.random.default_rng(seed)
    if which == "nn":
        sizes = [pm.nn[t].cparam.size for t in range(T)]
        grads = split(c.train_grad_nn, sizes)
        base = [pm.nn[t].cparam.copy() for t in range(T)]
        vs = [rng.normal(size=s) for s in sizes]

        def put(sgn):
            for t in range(T):
                set_cparam(pm.nn[t], base[t] + sgn * h * vs[t])
    else:
        # the radial-fuse matrix of every sub-basis object once (mirror / share species
        # point at the same matrix as their source)
        subs = {}
        for t in range(T):
            for sb in pm.basis[t].subs:
                subs.setdefault(id(sb), (t, sb))
        sizes = [pm.basis[t].param.size for t in range(T)]
        grads = split(c.train_grad_fp, sizes)
        vs = [rng.normal(size=s) for s in sizes]
        base = {k: sb.param.copy() for k, (t, sb) in subs.items()}
        offs = {}
        for t in range(T):
            o = 0
            for sb in pm.basis[t].subs:
                offs.setdefault(id(sb), (t, o))
                o += sb.param.size

        def put(sgn):
            for k, (t, sb) in subs.items():
                tt, o = offs[k]
                sb.param = base[k] + sgn * h * vs[tt][o:o + base[k].size]
    pred = sum(float(g @ v) for g, v in zip(grads, vs))
    put(1.0)
    lp = train_loss(pm, c, nl, c.train_be, c.train_bf, c.train_bw)
    put(-1.0)
    lm = train_loss(pm, c, nl, c.train_be, c.train_bf, c.train_bw)
    return pred, (lp - lm) / (2 * h)


def test_network_gradients_match_finite_differences(golden):
    pred, fd = fd_directional(golden, "nn")
    assert abs(pred - fd) <= 1e-6 * max(1.0, abs(fd)), (pred, fd)


def test_basis_gradients_match_finite_differences(golden):
    if not np.any(golden.train_grad_fp):
        pm = OM.load(golden.model)
        fused = any(sb.internal_wtype in (OM.WTYPE_FUSE, OM.WTYPE_RFUSE, OM.WTYPE_EXFUSE)
                    for b in pm.basis for sb in b.subs)
        assert not fused, "a fused radial basis has parameters and a nonzero gradient"
        pytest.skip("the basis has no trainable parameters (the reference computes no gradient)")
    pred, fd = fd_directional(golden, "fp")
    assert abs(pred - fd) <= 1e-6 * max(1.0, abs(fd)), (pred, fd)


def test_reference_driver_reproduces_the_fixture(golden):
    """Where the reference sources are present, the training pair reproduces the fixture."""
    pm = OM.load(golden.model)
    try:
        ref = ON.RefLib(pm)
    except (FileNotFoundError, OSError):
        pytest.skip("reference sources for this shape are not expanded here")
    nl = ON.compute(pm, golden.x, golden.types, golden.box_kind, golden.box)["nl"]
    g = ref.train_grad(golden.types, nl, golden.train_be, golden.train_bf, golden.train_bw, nthreads=2)
    np.testing.assert_allclose(np.concatenate(g["grad_nn"]), golden.train_grad_nn, rtol=1e-10,
                               atol=1e-10 * max(1.0, np.abs(golden.train_grad_nn).max()))
    np.testing.assert_allclose(np.concatenate(g["grad_fp"]), golden.train_grad_fp, rtol=1e-10,
                               atol=1e-10 * max(1.0, np.abs(golden.train_grad_fp).max()))
