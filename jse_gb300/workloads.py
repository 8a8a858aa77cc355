"""Seeded synthetic structures and NNAP model files for the benchmark workloads.

The reference repository ships no NNAP model files and no benchmark structures, so
the workloads are generated here, deterministically from a seed:

* ``fcc``             -- perturbed FCC lattice (single element).
* ``random_liquid``   -- uniform random positions with a minimum pair separation,
                         enforced by rejection (random sequential addition on a grid),
                         in an orthogonal or LAMMPS-style triclinic periodic box.
* ``write_model``     -- a model dict in the reference's JSON model format
                         (``NNAP.java:129-307``, ``FeedForward.java:131-221``,
                         ``SphericalChebyshev.java:60-103``, ``Chebyshev.java:33-69``)
                         with feed-forward weights ~ N(0, 1/fan_in) and biases ~ N(0, 1/fan_in).

Boxes are 3x3 row matrices ``[a; b; c]``.  ``box_kind`` 0 is orthogonal (diagonal only),
1 is the LAMMPS lower-triangular form ``a=(lx,0,0), b=(xy,ly,0), c=(xz,yz,lz)``.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

BOX_ORTHO, BOX_LMP, BOX_PRISM = 0, 1, 2


@dataclass
class Structure:
    x: np.ndarray        # (n, 3) float64 Cartesian positions
    types: np.ndarray    # (n,) int32, 1-based species
    box: np.ndarray      # (3, 3) float64 rows a, b, c
    box_kind: int

    @property
    def natoms(self) -> int:
        return len(self.types)


def fcc(a: float, reps: int, sigma: float, seed: int) -> Structure:
    """FCC lattice of ``reps^3`` cubic cells, Gaussian-perturbed by ``sigma``."""
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.stack(np.meshgrid(np.arange(reps), np.arange(reps), np.arange(reps), indexing="ij"), -1).reshape(-1, 3)
    x = ((g[:, None, :] + base[None, :, :]).reshape(-1, 3)) * a
    rng = np.random.default_rng(seed)
    x = x + rng.normal(0.0, sigma, size=x.shape)
    L = a * reps
    return Structure(x, np.ones(len(x), dtype=np.int32), np.diag([L, L, L]), BOX_ORTHO)


def _lmp_box(L: float, tilt: float) -> np.ndarray:
    return np.array([[L, 0.0, 0.0], [tilt * L, L, 0.0], [tilt * L, tilt * L, L]])


def _cross(u, v):
    return (u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0])


def _norm(u):
    return math.sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2])


def _rsa_grid(box, rmin: float):
    """Cell grid for random sequential addition: cells whose longest diagonal is below
    rmin (so a cell holds at most one accepted point) and the cell offsets along a, b, c
    that reach every point within rmin.  Scalar Python arithmetic (no BLAS), so the grid
    is the same on every machine."""
    A, B, C = [[float(v) for v in row] for row in box]
    bc, ca, ab = _cross(B, C), _cross(C, A), _cross(A, B)
    vol = abs(A[0] * bc[0] + A[1] * bc[1] + A[2] * bc[2])
    h = [vol / _norm(bc), vol / _norm(ca), vol / _norm(ab)]
    nc = [max(1, int(math.floor(_norm(r) * math.sqrt(3.0) * 1.15 / rmin))) for r in (A, B, C)]
    while True:
        worst = 0.0
        for sa, sb, sc in ((1, 1, 1), (1, 1, -1), (1, -1, 1), (-1, 1, 1)):
            v = [sa * A[d] / nc[0] + sb * B[d] / nc[1] + sc * C[d] / nc[2] for d in range(3)]
            worst = max(worst, _norm(v))
        if worst < rmin * 0.999:
            break
        nc = [k + 1 for k in nc]
    R = [int(math.ceil(rmin * nc[d] / h[d])) for d in range(3)]
    return np.array(nc, dtype=np.int64), np.array(R, dtype=np.int64), vol


def _to_cart(f, box):
    """Direct coordinates [m, 3] to Cartesian, elementwise (no BLAS, so no machine-dependent
    fused multiply-adds)."""
    return np.stack([f[:, 0] * box[0, d] + f[:, 1] * box[1, d] + f[:, 2] * box[2, d] for d in range(3)], axis=1)


def _rsa(n: int, box: np.ndarray, rmin: float, seed: int) -> np.ndarray:
    """Uniform random points with every pair distance >= rmin under periodic boundaries
    (all images), by random sequential addition in batches.

    Candidates are drawn uniformly in direct coordinates from numpy's PCG64 stream of
    ``seed`` and are accepted in draw order.  A candidate is rejected when an accepted
    point lies within rmin, or when an earlier candidate of its batch that passed that
    test lies within rmin (earlier candidates that are themselves rejected still count, so
    a batch can reject a little more than one-at-a-time addition would).  Batches are
    sized from the last batch's acceptance rate so that they accept about one point per
    16 exclusion volumes of the box, which keeps such in-batch conflicts rare.  Pure
    numpy, so structures are identical on every machine."""
    box = np.asarray(box, dtype=np.float64).reshape(3, 3)
    if n <= 0:
        return np.zeros((0, 3))
    rng = np.random.default_rng(int(seed) & ((1 << 63) - 1))
    nc, R, vol = _rsa_grid(box, rmin)
    ncell = int(nc.prod())
    occ = np.full(ncell, -1, dtype=np.int32)   # accepted point of each cell
    tmp = np.full(ncell, -1, dtype=np.int32)   # first passing candidate of each cell, per batch
    frac = np.zeros((n, 3))
    # stencil: cell offsets whose cells can hold a point within rmin, the 27 nearest first.
    # Points of cells o apart differ by at least max(|o_d| - 1, 0) / nc_d in direct
    # coordinate d, and |x| >= s_min |f| for the box's smallest singular value s_min; an
    # offset is left out only with a 1 % margin on that bound
    s_min = math.sqrt(max(0.0, float(np.linalg.eigvalsh(box @ box.T)[0])))
    g = np.stack(np.meshgrid(*[np.arange(-R[d], R[d] + 1) for d in range(3)], indexing="ij"), -1).reshape(-1, 3)
    gap = np.maximum(np.abs(g) - 1, 0) / nc
    keep = s_min * np.sqrt((gap * gap).sum(1)) < 1.01 * rmin
    inner = np.abs(g).max(1) <= 1
    offs = np.concatenate([g[inner], g[keep & ~inner]])
    n_in = int(inner.sum())
    centre = int(np.nonzero((offs == 0).all(1))[0][0])
    r2 = rmin * rmin
    target = max(4.0, vol / (4.0 / 3.0 * math.pi * rmin ** 3) / 16.0)
    placed, stalled, rate = 0, 0, 1.0

    # per axis: the flat-index contribution of cell (c_d + o_d) mod nc_d, [nc_d][2 R_d + 1]
    tab, stride = [], 1
    for d in range(3):
        q = np.arange(nc[d])[:, None] + np.arange(-R[d], R[d] + 1)[None, :]
        tab.append(((q - np.floor_divide(q, nc[d]) * nc[d]) * stride).astype(np.int32))
        stride *= int(nc[d])
    oidx = offs + R  # column of each offset in the tables

    def stencil(c, o_rows):
        """Flat cell index [m, len(o_rows)] of the stencil cells (rows of offs) of each
        candidate cell."""
        return (tab[0][c[:, 0, None], oidx[None, o_rows, 0]] + tab[1][c[:, 1, None], oidx[None, o_rows, 1]] +
                tab[2][c[:, 2, None], oidx[None, o_rows, 2]])

    def too_close(cc, oo, other_frac, mine):
        """Distances of the point pairs (candidate cell cc, stencil offset oo) below rmin."""
        q = cc + oo
        df = other_frac - mine + np.floor_divide(q, nc)
        v = _to_cart(df, box)
        return v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1] + v[:, 2] * v[:, 2] < r2

    while placed < n:
        nb = int(min(max(16.0, target / rate), 65536))
        s = rng.random((nb, 3))
        c = np.minimum((s * nc).astype(np.int64), nc - 1)
        ok = np.ones(nb, dtype=bool)
        # the 27 nearest cells first: they reject most candidates; then the rest of the
        # stencil for the candidates still standing
        for lo, hi in ((0, n_in), (n_in, len(offs))):
            live = np.nonzero(ok)[0]
            if hi == lo or len(live) == 0:
                continue
            o = occ[stencil(c[live], np.arange(lo, hi))]
            ci, oi = np.nonzero(o >= 0)
            if len(ci):
                bad = too_close(c[live[ci]], offs[lo + oi], frac[o[ci, oi]], s[live[ci]])
                ok[live[ci[bad]]] = False
        # conflicts with earlier passing candidates of the same batch
        cand = np.nonzero(ok)[0]
        if len(cand) > 1:
            fl = stencil(c[cand], np.arange(len(offs)))
            fc = fl[:, centre]
            # the first candidate of each cell claims it (assignments in reverse order leave
            # the earliest); later ones in that cell are too close
            tmp[fc[::-1]] = cand[::-1].astype(np.int32)
            reject = tmp[fc] != cand
            o2 = tmp[fl]
            m = (o2 >= 0) & (o2 < cand[:, None])
            ci, oi = np.nonzero(m)
            if len(ci):
                bad = too_close(c[cand[ci]], offs[oi], s[o2[ci, oi]], s[cand[ci]])
                reject[ci[bad]] = True
            tmp[fc] = -1
            ok[cand[reject]] = False
        acc = np.nonzero(ok)[0][: n - placed]
        rate = max(len(acc), 0.5) / nb
        if len(acc) == 0:
            stalled += nb
            if stalled > 100000:
                raise RuntimeError("random sequential addition stalled at %d of %d points" % (placed, n))
            continue
        stalled = 0
        frac[placed:placed + len(acc)] = s[acc]
        occ[stencil(c[acc], np.array([centre]))[:, 0]] = np.arange(placed, placed + len(acc))
        placed += len(acc)
    return _to_cart(frac, box)


def random_liquid(n: int, density: float, fractions: Sequence[float], rmin: float, seed: int,
                  tilt: Optional[float] = None) -> Structure:
    """Uniform random structure at number density ``density`` (1/A^3) with min separation."""
    rng = np.random.default_rng(seed)
    L = (n / density) ** (1.0 / 3.0)
    if tilt is None:
        box, kind = np.diag([L, L, L]), BOX_ORTHO
    else:
        box, kind = _lmp_box(L, tilt), BOX_LMP
    x = _rsa(n, box, rmin, int(rng.integers(0, 2 ** 63)))
    counts = [int(round(f * n)) for f in fractions]
    counts[0] += n - sum(counts)
    types = np.concatenate([np.full(c, t + 1, dtype=np.int32) for t, c in enumerate(counts)])
    rng.shuffle(types)
    return Structure(x, types, box, kind)


def write_model(symbols: List[str], basis: dict, hidden: Sequence[int], seed: int,
                norm_mu=None, norm_sigma=None, norm_mu_eng: float = 0.0, norm_sigma_eng: float = 1.0,
                ref_eng=None) -> dict:
    """Model dict in the reference's JSON format with random feed-forward weights."""
    T = len(symbols)
    D = descriptor_size(basis, T)
    rng = np.random.default_rng(seed)
    models = []
    for t, sym in enumerate(symbols):
        hw, hb = [], []
        fan = D
        for h in hidden:
            hw.append(rng.normal(0.0, math.sqrt(1.0 / fan), size=(h, fan)).tolist())
            hb.append(rng.normal(0.0, math.sqrt(1.0 / fan), size=h).tolist())
            fan = h
        ow = rng.normal(0.0, math.sqrt(1.0 / fan), size=fan).tolist()
        ob = float(rng.normal(0.0, math.sqrt(1.0 / fan)))
        m = {"symbol": sym, "basis": dict(basis),
             "nn": {"type": "feed_forward", "input_dim": D, "hidden_dims": list(hidden),
                    "hidden_weights": hw, "hidden_biases": hb, "output_weight": ow, "output_bias": ob}}
        if norm_mu is not None:
            m["norm_mu"] = list(map(float, norm_mu[t]))
        if norm_sigma is not None:
            m["norm_sigma"] = list(map(float, norm_sigma[t]))
        if ref_eng is not None:
            m["ref_eng"] = float(ref_eng[t])
        models.append(m)
    models[0]["norm_mu_eng"] = float(norm_mu_eng)
    models[0]["norm_sigma_eng"] = float(norm_sigma_eng)
    return {"version": 6, "units": "metal", "models": models}


def descriptor_size(basis: dict, T: int) -> int:
    """Descriptor length of a single (non-merged) basis dict without fuse/rfuse weights."""
    nmax = int(basis.get("nmax", 5))
    wt = basis.get("wtype", "default")
    if wt == "default":
        P = 2 * (nmax + 1) if T > 1 else nmax + 1
    elif wt == "none":
        P = nmax + 1
    elif wt == "full":
        P = T * (nmax + 1) if T > 1 else nmax + 1
    elif wt == "exfull":
        P = (T + 1) * (nmax + 1) if T > 1 else nmax + 1
    else:
        raise ValueError("descriptor_size only handles default/none/full/exfull")
    if basis.get("type", "spherical_chebyshev") in ("chebyshev", "cheby"):
        return P
    return P * (int(basis.get("lmax", 6)) + 1)


# ------------------------------------------------------------------ named workloads
C1_BASIS = {"type": "chebyshev", "nmax": 10, "rcut": 6.0}
C2_BASIS = {"type": "spherical_chebyshev", "nmax": 8, "lmax": 6, "rcut": 6.0, "wtype": "default"}
C3_BASIS = {"type": "spherical_chebyshev", "nmax": 8, "lmax": 4, "rcut": 5.5, "wtype": "default"}


_CACHE_DIR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), ".cache", "workloads")
_GEN_VERSION = 3  # bump when the generator's output changes


def _cached(key: str, make):
    """Structures made by ``make()``, kept as an .npz under the repository's .cache folder
    (not committed) so that the benchmark's arms and the tests generate each large
    workload once per machine."""
    path = os.path.join(_CACHE_DIR, "%s_v%d.npz" % (key, _GEN_VERSION))
    try:
        z = np.load(path)
        k = int(z["count"])
        return [Structure(z["x%d" % i], z["t%d" % i], z["b%d" % i], int(z["k%d" % i])) for i in range(k)]
    except (OSError, KeyError, ValueError):
        pass
    out = make()
    try:
        os.makedirs(_CACHE_DIR, exist_ok=True)
        arrs = {"count": np.array(len(out))}
        for i, st in enumerate(out):
            arrs["x%d" % i], arrs["t%d" % i], arrs["b%d" % i], arrs["k%d" % i] = st.x, st.types, st.box, np.array(st.box_kind)
        tmp = path + ".%d.tmp.npz" % os.getpid()
        np.savez(tmp, **arrs)
        os.replace(tmp, path)
    except OSError:
        pass
    return out


def c1_structure(seed: int = 1) -> Structure:
    """FCC a=3.61 A, 10x10x10 cells (4000 atoms), sigma=0.05 A."""
    return fcc(3.61, 10, 0.05, seed)


def c2_structure(n: int = 32000, seed: int = 2) -> Structure:
    """Ternary liquid, density 0.060 /A^3, fractions 0.46/0.46/0.08, min separation 2.0 A."""
    return _cached("c2_%d_%d" % (n, seed), lambda: [random_liquid(n, 0.060, [0.46, 0.46, 0.08], 2.0, seed)])[0]


def c3_structure(n: int = 1048576, seed: int = 3) -> Structure:
    """Binary glass, density 0.058 /A^3, fractions 0.64/0.36, min separation 2.1 A, tilt 0.1."""
    return _cached("c3_%d_%d" % (n, seed), lambda: [random_liquid(n, 0.058, [0.64, 0.36], 2.1, seed, tilt=0.1)])[0]


def c4_structures(count: int = 1024, seed: int = 4) -> List[Structure]:
    """Mixed batch: n ~ log-uniform[32, 2048], half orthogonal / half triclinic (tilt 0.1),
    density ~ U[0.055, 0.065], ternary species as the liquid workload, min separation 2.0 A."""
    return _cached("c4_%d_%d" % (count, seed), lambda: _c4_make(count, seed))


def _c4_make(count: int, seed: int) -> List[Structure]:
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n = int(round(math.exp(rng.uniform(math.log(32), math.log(2048)))))
        rho = float(rng.uniform(0.055, 0.065))
        tilt = 0.1 if (k % 2 == 1) else None
        out.append(random_liquid(n, rho, [0.46, 0.46, 0.08], 2.0, seed * 100003 + k, tilt=tilt))
    return out


def model_for(config: str, seed: int = 11, norm_mu=None, norm_sigma=None) -> dict:
    """Model dict for the named workload; normalisation statistics may be supplied."""
    if config == "c1":
        return write_model(["Cu"], C1_BASIS, [32, 32], seed, norm_mu, norm_sigma, -3.5, 0.1)
    if config in ("c2", "c4", "c5"):
        return write_model(["A", "B", "C"], C2_BASIS, [64, 64], seed, norm_mu, norm_sigma, -3.0, 0.1)
    if config == "c3":
        return write_model(["A", "B"], C3_BASIS, [64, 64], seed, norm_mu, norm_sigma, -3.0, 0.1)
    raise ValueError(config)


def c5_pool(count: int = 512, seed: int = 5, sigma: float = 1.0) -> List[Structure]:
    """Structures for the serving workload: n ~ log-normal (median 500, log-sd ``sigma``)
    clipped to [50, 20000]; ternary liquids as the 32000-atom workload (cubic box,
    density 0.060 /A^3, fractions 0.46/0.46/0.08, min separation 2.0 A).  Requests draw
    their starting structure from this pool."""
    return _cached("c5_%d_%d_%g" % (count, seed, sigma), lambda: _c5_make(count, seed, sigma))


def _c5_make(count: int, seed: int, sigma: float) -> List[Structure]:
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n = int(min(20000, max(50, round(math.exp(math.log(500.0) + sigma * rng.standard_normal())))))
        out.append(random_liquid(n, 0.060, [0.46, 0.46, 0.08], 2.0, seed * 100003 + k))
    return out


def random_nep_text(symbols: Sequence[str], version: int = 4, rc=(8.0, 4.0), n_max=(4, 4), basis=(8, 8),
                    l_max=(4, 2, 1), neurons: int = 30, seed: int = 0) -> str:
    """A seeded random NEP potential file (nep.txt) of the given hyperparameters (defaults:
    GPUMD's nep.in defaults, cutoff 8 / 4 A, n_max 4 4, basis_size 8 8, l_max 4 2 1, 30
    neurons).  Network weights ~ N(0, 1/dim), descriptor coefficients ~ U(-1, 1), descriptor
    scales ~ U(0.5, 2)."""
    rng = np.random.default_rng(seed)
    T = len(symbols)
    numL = l_max[0] + (1 if l_max[1] == 2 else 0) + (1 if l_max[2] == 1 else 0)
    dim = (n_max[0] + 1) + (n_max[1] + 1) * numL
    if version == 3:
        nann = (dim + 2) * neurons + 1
    elif version == 4:
        nann = (dim + 2) * neurons * T + 1
    else:
        nann = ((dim + 2) * neurons + 1) * T + 1
    ndesc = T * T * ((n_max[0] + 1) * (basis[0] + 1) + (n_max[1] + 1) * (basis[1] + 1))
    vals = np.concatenate([rng.normal(0.0, 1.0 / math.sqrt(dim), nann), rng.uniform(-1.0, 1.0, ndesc),
                           rng.uniform(0.5, 2.0, dim)])
    head = ["nep%d %d %s" % (version, T, " ".join(symbols)), "cutoff %g %g 100 100" % tuple(rc),
            "n_max %d %d" % tuple(n_max), "basis_size %d %d" % tuple(basis), "l_max %d %d %d" % tuple(l_max),
            "ANN %d 0" % neurons]
    return "\n".join(head + ["%.17g" % v for v in vals]) + "\n"


# NEP benchmark: a binary liquid at 0.060 /A^3 under a nep4 potential of GPUMD's default
# hyperparameters.
NEP_BENCH_ATOMS = 32000


def nep_bench(n: int = NEP_BENCH_ATOMS, seed: int = 21):
    return random_nep_text(["Si", "O"], seed=seed), random_liquid(n, 0.060, [0.5, 0.5], 2.0, seed)


def lammps_form(s: Structure, offsets, j, img):
    """A structure in the form LAMMPS hands a pair style: the local atoms, then one ghost
    atom per (atom, periodic image) that appears in a full neighbour list, and per local
    atom the list of its neighbours as indices into local + ghost atoms.  ``offsets, j,
    img`` is a full neighbour list of ``s`` with image offsets (``NNAP.neighborList``);
    the positions must lie inside the box (direct coordinates in [0, 1)), as the list's
    images refer to wrapped positions.  Returns (x_all, types_all, lists, owner) with
    owner[g] the local atom of ghost n + g."""
    x = np.asarray(s.x, dtype=np.float64).reshape(-1, 3)
    box = np.asarray(s.box, dtype=np.float64).reshape(3, 3)
    frac = x @ np.linalg.inv(box)
    if (frac < 0.0).any() or (frac >= 1.0).any():
        raise ValueError("positions must lie inside the box")
    n = len(x)
    j = np.asarray(j, dtype=np.int64)
    img = np.asarray(img, dtype=np.int64).reshape(-1, 3)
    shifted = img.any(axis=1)
    keys, inv = np.unique(np.column_stack([j[shifted], img[shifted]]), axis=0, return_inverse=True)
    idx = j.copy()
    idx[shifted] = n + inv.reshape(-1)
    x_all = np.concatenate([x, x[keys[:, 0]] + keys[:, 1:] @ box]) if len(keys) else x.copy()
    types = np.asarray(s.types, dtype=np.int32)
    t_all = np.concatenate([types, types[keys[:, 0]]]) if len(keys) else types.copy()
    lists = np.split(idx.astype(np.int32), np.asarray(offsets[1:-1], dtype=np.int64))
    return x_all, t_all.astype(np.int32), lists, keys[:, 0].astype(np.int64) if len(keys) else np.zeros(0, np.int64)
