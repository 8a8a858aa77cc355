"""Why the mixed-precision network splits its BF16 operands (CPU, numpy emulation).

The tensor-core network multiplies BF16 operands with FP32 accumulation.  This test
evaluates the liquid benchmark model's network (126 -> 64 -> 64 -> 1, SiLU, the committed
normalisation) on FP64 oracle descriptors of 400 liquid atoms with every matrix product
done four ways: FP64; operands rounded to BF16; operands rounded to FP16; and operands
split as x = hi + lo (both BF16) with hi*hi + lo*hi + hi*lo, as k_net_tc does.  The
per-atom energy error of the split form meets the 1e-5 eV target; single BF16 or FP16
operands do not.
"""
import numpy as np

import bench
from jse_gb300 import workloads as W
from oracle import model as OM, native as ON


def _bf16(a):
    """Round FP32 values to BF16 (round to nearest, ties to even), returned as FP32."""
    u = np.asarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def _mm(x, w, mode):
    """x [n][k] times w^T ([m][k]) with the operands as the given precision, FP32 sums."""
    x = np.asarray(x, dtype=np.float32)
    w = np.asarray(w, dtype=np.float32)
    if mode == "fp64":
        return np.asarray(x, np.float64) @ np.asarray(w, np.float64).T
    if mode == "bf16":
        return (_bf16(x).astype(np.float64) @ _bf16(w).astype(np.float64).T).astype(np.float32)
    if mode == "fp16":
        return (x.astype(np.float16).astype(np.float64) @ w.astype(np.float16).astype(np.float64).T).astype(np.float32)
    xh, wh = _bf16(x), _bf16(w)
    xl, wl = _bf16(x - xh), _bf16(w - wh)
    f = lambda a, b: a.astype(np.float64) @ b.astype(np.float64).T  # noqa: E731
    return (f(xh, wh) + f(xl, wh) + f(xh, wl)).astype(np.float32)


def _silu(z):
    return z / (1.0 + np.exp(-z))


def _energies(model_nn, norm, fp, mode):
    mu, sg = norm["mu"], norm["sigma"]
    h = (fp - mu) / sg
    for Wl, bl in zip(model_nn["hidden_weights"], model_nn["hidden_biases"]):
        h = _silu(_mm(h, np.asarray(Wl), mode) + np.asarray(bl))
    return h @ np.asarray(model_nn["output_weight"]) + model_nn["output_bias"]


def test_split_bf16_meets_the_energy_target_and_plain_operands_do_not():
    model = bench.bench_model("c2")
    s = W.random_liquid(400, 0.060, [0.46, 0.46, 0.08], 2.0, 123)
    fp = ON.compute(OM.load(model), s.x, s.types, s.box_kind, s.box, want_fp=True)["fp"]
    sig_e = model["models"][0]["norm_sigma_eng"]
    err = {}
    for mode in ("bf16", "fp16", "split"):
        worst = 0.0
        for t, mm in enumerate(model["models"]):
            sel = s.types == t + 1
            norm = {"mu": np.asarray(mm["norm_mu"]), "sigma": np.asarray(mm["norm_sigma"])}
            ref = _energies(mm["nn"], norm, fp[sel, :126], "fp64")
            got = _energies(mm["nn"], norm, fp[sel, :126], mode)
            worst = max(worst, float(np.abs(got - ref).max()) * sig_e)
        err[mode] = worst
    print("max per-atom energy error (eV): %s" % {k: "%.2e" % v for k, v in err.items()})
    assert err["split"] <= 1e-5
    assert err["bf16"] > 1e-4 and err["fp16"] > 1e-5
