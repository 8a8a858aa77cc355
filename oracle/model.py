"""FP64 model-file loader and parameter packing for the NNAP oracle.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Restates how the reference turns a model file into the flat C parameter blocks its
per-atom C++ arithmetic consumes:

* model keys and defaults: ``NNAP.java:129-176`` (version <= 6, ``models[].symbol``,
  basis default ``spherical_chebyshev``), ``Basis.java:22-68``,
  ``Chebyshev.java:33-69``, ``SphericalChebyshev.java:60-103``,
  ``MergedBasis.java:193-229``, ``FeedForward.java:131-221``;
* basis parameter block per species: the internal radial-fuse matrix
  ``W[(t_nei-1)*NP + np][n]`` built by ``WTypeBasis.updateParameters_``
  (``WTypeBasis.java:202-304``), followed by the hyper-parameter block ``[rcut]``
  (``MergeableBasis.java:24-30``, packing order ``NNAP.java:249-261``);
* network block: ``hidden W | output W | hidden b | output b`` (``FeedForward.java:310-316``);
* normalisation block: ``[norm_mu_eng + ref_eng, norm_sigma_eng, mu[D], sigma[D]]``
  (``NNAP.java:270-307``).
"""
from __future__ import annotations

import json
import math
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

WTYPES = {"default": 0, "none": -1, "full": 2, "exfull": 3, "fuse": 4, "rfuse": 5, "exfuse": 6}
WTYPE_DEFAULT, WTYPE_NONE, WTYPE_FULL, WTYPE_EXFULL, WTYPE_FUSE, WTYPE_RFUSE, WTYPE_EXFUSE = 0, -1, 2, 3, 4, 5, 6
L3NCOLS = [0, 0, 2, 4, 9, 14, 23]
L4NCOLS = [0, 1, 3, 9]
WS_EPS = 1e-5


def _get(m, *keys, default=None):
    for k in keys:
        if k in m and m[k] is not None:
            return m[k]
    return default


def size_n(wtype: int, T: int, nmax: int, fuse_size: int) -> int:
    """``WTypeBasis.getSizeN_`` (WTypeBasis.java:331-354)."""
    if wtype == WTYPE_EXFULL:
        return (T + 1) * (nmax + 1) if T > 1 else nmax + 1
    if wtype in (WTYPE_FULL, WTYPE_RFUSE):
        return T * (nmax + 1)
    if wtype == WTYPE_NONE:
        return nmax + 1
    if wtype == WTYPE_DEFAULT:
        return 2 * nmax + 2 if T > 1 else nmax + 1
    if wtype == WTYPE_FUSE:
        return fuse_size * (nmax + 1)
    if wtype == WTYPE_EXFUSE:
        return (fuse_size + 1) * (nmax + 1)
    raise ValueError("bad wtype %r" % wtype)


@dataclass
class SubBasis:
    kind: str            # "chebyshev" | "spherical_chebyshev"
    T: int
    nmax: int
    rcut: float
    wtype: int
    typed_wtype: int
    internal_wtype: int
    size_np: int
    size_nn: int
    lmax: int = 0
    l3max: int = 0
    l4max: int = 0
    param: np.ndarray = field(default=None)  # internal fuse matrix, (T*NP*(nmax+1),)

    @property
    def size(self) -> int:
        if self.kind == "chebyshev":
            return self.size_np
        return self.size_np * ((self.lmax + 1) + L3NCOLS[self.l3max] + L4NCOLS[self.l4max])

    @property
    def param_size(self) -> int:
        return self.size_np * self.T * (self.nmax + 1)

    def genkey(self):
        return (self.kind, self.size, self.param_size, self.wtype, self.nmax, self.size_np,
                self.internal_wtype, self.lmax, self.l3max, self.l4max)


def _load_sub(kind: str, T: int, m: dict) -> SubBasis:
    """``Chebyshev.load`` / ``SphericalChebyshev.load`` + ``WTypeBasis`` ctor."""
    nmax = int(_get(m, "nmax", default=5))
    rcut = float(_get(m, "rcut", default=6.0))
    lmax = l3max = l4max = 0
    if kind == "spherical_chebyshev":
        lmax = int(_get(m, "lmax", default=6))
        l3max = int(_get(m, "l3max", default=0))
        l4max = int(_get(m, "l4max", default=0))
        if not (0 <= max(lmax, l3max, l4max) <= 12) or l3max > 6 or l4max > 3:
            raise ValueError("lmax/l3max/l4max out of range")
    if not 0 <= nmax <= 20:
        raise ValueError("nmax out of range")
    wt = _get(m, "wtype")
    if wt is None:
        wtype = WTYPE_DEFAULT
    elif isinstance(wt, (int, float)) and not isinstance(wt, bool):
        wtype = int(wt)
    else:
        if wt not in WTYPES:
            raise ValueError("bad wtype %r" % wt)
        wtype = WTYPES[wt]
    ws = bool(_get(m, "weight_standardization", "ws", default=False))
    fuse_w = None
    fuse_size = 0
    if wtype in (WTYPE_FUSE, WTYPE_EXFUSE):
        fw = m.get("fuse_weight")
        fs = _get(m, "fuse_size")
        if fw is None:
            if fs is None:
                raise ValueError("fuse_weight or fuse_size required")
            fuse_w = np.zeros(T * int(fs))
        elif fs is None:   # legacy: column-wise
            fuse_w = np.asarray(fw, dtype=np.float64).T.reshape(-1)
        elif isinstance(fw[0], list):
            fuse_w = np.asarray(fw, dtype=np.float64).reshape(-1)
        else:
            fuse_w = np.asarray(fw, dtype=np.float64)
        fuse_size = fuse_w.size // T
    sn = size_n(wtype, T, nmax, fuse_size)
    rfuse_w = None
    rfuse_scale = 1.0
    if wtype == WTYPE_RFUSE:
        rw = m.get("rfuse_weight")
        if rw is None:
            rs = m.get("rfuse_size")
            if rs is None:
                raise ValueError("rfuse_weight or rfuse_size required")
            rw = np.zeros(int(rs) * sn)
        rfuse_w = np.asarray(rw, dtype=np.float64).reshape(-1)
        rfuse_scale = float(_get(m, "rfuse_scale", default=1.0))
    elif m.get("post_fuse_weight") is not None and m.get("post_fuse") is not False:
        pw = np.asarray(m["post_fuse_weight"], dtype=np.float64).reshape(-1)
        rfuse_scale = float(_get(m, "post_fuse_scale", default=1.0))
        rfuse_w = _post_fuse_to_rfuse(pw, wtype, T, nmax, sn, fuse_w, fuse_size)
        wtype = WTYPE_RFUSE
        fuse_w = None
        sn = size_n(WTYPE_RFUSE, T, nmax, 0)
    typed = wtype
    if T == 1 and wtype in (WTYPE_EXFULL, WTYPE_FULL, WTYPE_NONE, WTYPE_DEFAULT):
        typed = WTYPE_NONE
    size_np = sn if rfuse_w is None else rfuse_w.size // sn
    internal = typed if rfuse_w is None else WTYPE_RFUSE
    sb = SubBasis(kind, T, nmax, rcut, wtype, typed, internal, size_np, sn, lmax, l3max, l4max)
    sb.param = _internal_fuse(sb, fuse_w, fuse_size, rfuse_w, rfuse_scale, ws)
    return sb


def _post_fuse_to_rfuse(pw, wtype, T, nmax, sn, fuse_w, fuse_size):
    """``WTypeBasis.postFuse2RFuse_`` (WTypeBasis.java:412-526)."""
    NP = pw.size // sn
    N1 = nmax + 1
    out = np.zeros(T * NP * N1)
    typed = wtype
    if T == 1 and wtype in (WTYPE_EXFULL, WTYPE_FULL, WTYPE_NONE, WTYPE_DEFAULT):
        typed = WTYPE_NONE
    for t in range(1, T + 1):
        for np_ in range(NP):
            L = ((t - 1) * NP + np_) * N1
            R = np_ * sn
            if typed == WTYPE_FUSE:
                for k in range(fuse_size):
                    out[L:L + N1] += fuse_w[(t - 1) * fuse_size + k] * pw[R + k * N1:R + k * N1 + N1]
            elif typed == WTYPE_EXFUSE:
                out[L:L + N1] = pw[R:R + N1]
                for k in range(fuse_size):
                    s = R + (k + 1) * N1
                    out[L:L + N1] += fuse_w[(t - 1) * fuse_size + k] * pw[s:s + N1]
            elif typed == WTYPE_FULL:
                s = R + (t - 1) * N1
                out[L:L + N1] = pw[s:s + N1]
            elif typed == WTYPE_EXFULL:
                out[L:L + N1] = pw[R:R + N1]
                out[L:L + N1] += pw[R + t * N1:R + t * N1 + N1]
            elif typed == WTYPE_NONE:
                out[L:L + N1] = pw[R:R + N1]
            elif typed == WTYPE_DEFAULT:
                wt = float(t if (t & 1) == 1 else -t)
                out[L:L + N1] = pw[R:R + N1]
                out[L:L + N1] += wt * pw[R + N1:R + 2 * N1]
    return out


def _internal_fuse(sb: SubBasis, fuse_w, fuse_size, rfuse_w, scale, ws) -> np.ndarray:
    """``WTypeBasis.updateParameters_`` (WTypeBasis.java:202-304)."""
    T, NP, N1 = sb.T, sb.size_np, sb.nmax + 1
    W = np.zeros(NP * T * N1)

    def put(t, row, n, v):
        W[((t - 1) * NP + row) * N1 + n] = v

    tw = sb.typed_wtype
    if tw == WTYPE_RFUSE:
        if not ws:
            W[:] = rfuse_w
        else:
            for np_ in range(NP):
                norm = WS_EPS
                for t in range(1, T + 1):
                    s = ((t - 1) * NP + np_) * N1
                    for n in range(N1):
                        norm += abs(rfuse_w[s + n])
                norm /= sb.size_nn
                for t in range(1, T + 1):
                    s = ((t - 1) * NP + np_) * N1
                    for n in range(N1):
                        W[s + n] = rfuse_w[s + n] / norm
        W *= scale
    elif tw == WTYPE_FUSE:
        for t in range(1, T + 1):
            for k in range(fuse_size):
                for n in range(N1):
                    put(t, k * N1 + n, n, fuse_w[(t - 1) * fuse_size + k])
    elif tw == WTYPE_EXFUSE:
        for t in range(1, T + 1):
            for n in range(N1):
                put(t, n, n, 1.0)
            for k in range(fuse_size):
                for n in range(N1):
                    put(t, (k + 1) * N1 + n, n, fuse_w[(t - 1) * fuse_size + k])
    elif tw == WTYPE_FULL:
        for t in range(1, T + 1):
            for n in range(N1):
                put(t, (t - 1) * N1 + n, n, 1.0)
    elif tw == WTYPE_EXFULL:
        for t in range(1, T + 1):
            for n in range(N1):
                put(t, n, n, 1.0)
                put(t, t * N1 + n, n, 1.0)
    elif tw == WTYPE_NONE:
        for t in range(1, T + 1):
            for n in range(N1):
                put(t, n, n, 1.0)
    elif tw == WTYPE_DEFAULT:
        for t in range(1, T + 1):
            wt = float(t if (t & 1) == 1 else -t)
            for n in range(N1):
                put(t, n, n, 1.0)
                put(t, N1 + n, n, wt)
    else:
        raise ValueError("bad typed wtype")
    return W


@dataclass
class Basis:
    subs: List[SubBasis]
    kind: str = "plain"    # "plain" (single or merged), "mirror" or "share"
    src: int = 0           # mirror / share: the 1-based species whose basis is used

    @property
    def size(self) -> int:
        return sum(s.size for s in self.subs)

    @property
    def rcut_max(self) -> float:
        return max(s.rcut for s in self.subs)

    @property
    def param(self) -> np.ndarray:
        return np.concatenate([s.param for s in self.subs])

    @property
    def hparam(self) -> np.ndarray:
        return np.array([s.rcut for s in self.subs], dtype=np.float64)


@dataclass
class FeedForward:
    input_dim: int
    hidden_dims: List[int]
    hidden_weights: List[np.ndarray]   # [out][in] per layer
    hidden_biases: List[np.ndarray]
    output_weight: np.ndarray
    output_bias: float

    @property
    def hidden_weight_size(self) -> int:
        return sum(w.size for w in self.hidden_weights)

    @property
    def hidden_bias_size(self) -> int:
        return sum(self.hidden_dims)

    @property
    def cparam(self) -> np.ndarray:
        """``hidden W | output W | hidden b | output b`` (FeedForward.java:310-316)."""
        return np.concatenate([w.reshape(-1) for w in self.hidden_weights] + [self.output_weight] +
                              list(self.hidden_biases) + [np.array([self.output_bias])])


def _load_shared_nn(D: int, base: FeedForward, m: dict) -> FeedForward:
    """``SharedFeedForward.load`` + ``updateParameters_`` (SharedFeedForward.java:162-339):
    the base network with, per hidden layer, its first H - S rows (and biases) replaced
    by the species' own values (zeros when absent); the output layer is the base's when
    the last shared dimension is 1, else the species' own."""
    if m.get("shared_flags") is not None:
        raise ValueError("shared in layer nn is invalid now")
    ind = _get(m, "input_dim")
    if ind is not None and int(ind) != D:
        raise ValueError("input dimension mismatch: %d vs %d" % (int(ind), D))
    if D != base.input_dim:
        raise ValueError("input dimensions mismatch for shared nn")
    sh = _get(m, "shared_hidden_dims", "shared_nnarch")
    if sh is None:
        raise ValueError("Key `shared_hidden_dims` required for shared_feed_forward")
    sh = [int(v) for v in sh]
    L = len(base.hidden_dims)
    if len(sh) == L:
        sh = sh + [0]
    if len(sh) - 1 != L:
        raise ValueError("the number of hidden layers mismatch")
    hw, hb = m.get("hidden_weights"), m.get("hidden_biases")
    if hw is not None and len(hw) != L:
        raise ValueError("the number of hidden weights mismatch")
    if hb is not None and len(hb) != L:
        raise ValueError("the number of hidden biases mismatch")
    ws, bs, fan = [], [], D
    for i, h in enumerate(base.hidden_dims):
        if sh[i] < 0 or sh[i] > h:
            raise ValueError("invalid shared dimension")
        u = h - sh[i]
        w = base.hidden_weights[i].copy()
        b = base.hidden_biases[i].copy()
        if hw is None or u == 0:
            own_w = np.zeros((u, fan))
        else:
            own_w = np.asarray(hw[i], dtype=np.float64)
        if own_w.shape != (u, fan):
            raise ValueError("hidden weight %d shape mismatch" % i)
        own_b = np.zeros(u) if hb is None else np.asarray(hb[i], dtype=np.float64)
        if own_b.shape != (u,):
            raise ValueError("hidden bias %d size mismatch" % i)
        w[:u] = own_w
        b[:u] = own_b
        ws.append(w)
        bs.append(b)
        fan = h
    if sh[L] not in (0, 1):
        raise ValueError("invalid shared output dimension")
    if sh[L] == 1:
        ow, ob = base.output_weight.copy(), base.output_bias
    else:
        ow = np.asarray(m["output_weight"], dtype=np.float64) if m.get("output_weight") is not None \
            else np.zeros(fan)
        if ow.shape != (fan,):
            raise ValueError("output weight size mismatch")
        ob = float(m.get("output_bias", 0.0) or 0.0)
    return FeedForward(D, list(base.hidden_dims), ws, bs, ow, ob)


def _load_nn(D: int, m: dict) -> FeedForward:
    """``FeedForward.load`` (FeedForward.java:131-221)."""
    if _get(m, "type", default="feed_forward") != "feed_forward":
        raise ValueError("unsupported nn type %r" % m.get("type"))
    ind = _get(m, "input_dim")
    if ind is not None and int(ind) != D:
        raise ValueError("input dimension mismatch: %d vs %d" % (int(ind), D))
    hd = [int(h) for h in _get(m, "hidden_dims", "nnarch", default=[32, 32])]
    if not hd:
        raise ValueError("at least one hidden layer is required")
    hw = m.get("hidden_weights")
    hb = m.get("hidden_biases")
    ws, bs = [], []
    fan = D
    for i, h in enumerate(hd):
        if hw is not None:
            w = np.asarray(hw[i], dtype=np.float64)
            if w.shape != (h, fan):
                raise ValueError("hidden weight %d shape %r != %r" % (i, w.shape, (h, fan)))
        else:
            w = np.zeros((h, fan))
        b = np.asarray(hb[i], dtype=np.float64) if hb is not None else np.zeros(h)
        if b.shape != (h,):
            raise ValueError("hidden bias %d size mismatch" % i)
        ws.append(w)
        bs.append(b)
        fan = h
    ow = np.asarray(m["output_weight"], dtype=np.float64) if m.get("output_weight") is not None else np.zeros(hd[-1])
    if ow.shape != (hd[-1],):
        raise ValueError("output weight size mismatch")
    ob = float(m.get("output_bias", 0.0) or 0.0)
    return FeedForward(D, hd, ws, bs, ow, ob)


@dataclass
class PackedModel:
    symbols: List[str]
    units: Optional[str]
    basis: List[Basis]
    nn: List[FeedForward]
    norm: List[np.ndarray]  # [mu_eng+ref_eng, sigma_eng, mu[D], sigma[D]]

    @property
    def ntypes(self) -> int:
        return len(self.symbols)

    @property
    def rcut_max(self) -> float:
        return max(b.rcut_max for b in self.basis)


def load(source) -> PackedModel:
    """Load a model from a dict, a JSON string or a ``.json`` path."""
    if isinstance(source, dict):
        info = source
    elif isinstance(source, str) and source.lstrip().startswith("{"):
        info = json.loads(source)
    else:
        with open(source) as f:
            info = json.load(f)
    ver = info.get("version")
    if ver is not None and int(ver) > 6:
        raise ValueError("unsupported version %r" % ver)
    models = info.get("models")
    if models is None:
        raise ValueError("no models")
    T = len(models)
    symbols = []
    for mm in models:
        if mm.get("symbol") is None:
            raise ValueError("no symbol in model")
        symbols.append(str(mm["symbol"]))
    basis = []
    for mm in models:
        bm = mm.get("basis") or {"type": "spherical_chebyshev"}
        bt = bm.get("type") or "spherical_chebyshev"
        if bt in ("spherical_chebyshev", "sph_cheby"):
            basis.append(Basis([_load_sub("spherical_chebyshev", T, bm)]))
        elif bt in ("chebyshev", "cheby"):
            basis.append(Basis([_load_sub("chebyshev", T, bm)]))
        elif bt in ("merge", "merged_basis"):
            subs = []
            for sm in bm["basis"]:
                st = sm.get("type") or "spherical_chebyshev"
                kind = {"spherical_chebyshev": "spherical_chebyshev", "sph_cheby": "spherical_chebyshev",
                        "chebyshev": "chebyshev", "cheby": "chebyshev"}.get(st)
                if kind is None:
                    raise ValueError("unsupported merged basis type %r" % st)
                subs.append(_load_sub(kind, T, sm))
            basis.append(Basis(subs))
        elif bt in ("mirror", "mirror_basis", "share", "shared_basis"):
            basis.append(None)  # resolved below, after every concrete basis (Basis.java:50-66)
        else:
            raise ValueError("unsupported basis type %r" % bt)
    for t, mm in enumerate(models):
        if basis[t] is not None:
            continue
        bm = mm["basis"]
        mirror = bm["type"] in ("mirror", "mirror_basis")
        key = "mirror" if mirror else "share"
        if bm.get(key) is None:
            raise ValueError("Key `%s` required" % key)
        src = int(bm[key])
        if not 1 <= src <= T or basis[src - 1] is None or basis[src - 1].kind != "plain":
            # a mirror or shared basis of a mirror or shared basis reads an empty parameter
            # block in the reference's generated code, so only plain sources are accepted
            raise ValueError("the source of a mirror or shared basis must be a plain basis")
        basis[t] = Basis(basis[src - 1].subs, "mirror" if mirror else "share", src)
    nns = [None] * T
    for t, (mm, b) in enumerate(zip(models, basis)):
        if mm.get("torch") is not None:
            raise ValueError("torch model is invalid")
        if b.kind == "mirror":
            if mm.get("nn") is not None:
                raise ValueError("nn data in mirror ModelInfo MUST be empty")
            continue
        nm = mm.get("nn") or {}
        if _get(nm, "type", default="feed_forward") == "shared_feed_forward":
            continue
        nns[t] = _load_nn(b.size, nm)
    plain = [n is not None for n in nns]  # plain feed_forward networks (the only valid bases)
    for t, (mm, b) in enumerate(zip(models, basis)):
        if plain[t]:
            continue
        src = b.src if b.kind == "mirror" else int((mm.get("nn") or {}).get("share", 0))
        if not 1 <= src <= T or not plain[src - 1]:
            raise ValueError("a shared network needs a plain feed_forward source")
        if b.kind == "mirror":  # SharedFeedForward.full: every layer shared
            base = nns[src - 1]
            nns[t] = FeedForward(base.input_dim, list(base.hidden_dims), [w.copy() for w in base.hidden_weights],
                                 [v.copy() for v in base.hidden_biases], base.output_weight.copy(), base.output_bias)
        else:
            nns[t] = _load_shared_nn(b.size, nns[src - 1], mm["nn"])
    sig_e = next((mm["norm_sigma_eng"] for mm in models if mm.get("norm_sigma_eng") is not None), 1.0)
    mu_e = next((mm["norm_mu_eng"] for mm in models if mm.get("norm_mu_eng") is not None), 0.0)
    norms = []
    for mm, b in zip(models, basis):
        if b.kind == "mirror":  # a mirror species takes its source's normalisation (NNAP.java:281-289)
            if mm.get("ref_eng") is not None:
                raise ValueError("ref_eng in mirror_basis MUST be empty")
            if _get(mm, "norm_vec", "norm_sigma", "norm_mu") is not None:
                raise ValueError("norm_vec/norm_sigma/norm_mu in mirror_basis MUST be empty")
            mm = models[b.src - 1]
        D = b.size
        ref = float(mm.get("ref_eng") or 0.0)
        sig = _get(mm, "norm_sigma", "norm_vec")
        mu = mm.get("norm_mu")
        v = np.empty(2 + 2 * D)
        v[0] = float(mu_e) + ref
        v[1] = float(sig_e)
        v[2:2 + D] = 0.0 if mu is None else np.asarray(mu, dtype=np.float64)
        v[2 + D:] = 1.0 if sig is None else np.asarray(sig, dtype=np.float64)
        norms.append(v)
    return PackedModel(symbols, info.get("units"), basis, nns, norms)
