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


_RSA = None


def _rsa_lib():
    """The C generator (jse_gb300/csrc/rsa.c), compiled on first use."""
    global _RSA
    if _RSA is None:
        import ctypes as C
        import os
        import subprocess
        here = os.path.dirname(os.path.abspath(__file__))
        src = os.path.join(here, "csrc", "rsa.c")
        lib = os.path.join(here, "librsa.so")
        if not os.path.exists(lib) or os.path.getmtime(lib) < os.path.getmtime(src):
            subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", src, "-o", lib, "-lm"], check=True)
        L = C.CDLL(lib)
        L.rsa_generate.argtypes = [C.c_int, C.POINTER(C.c_double), C.c_double, C.c_uint64, C.c_int,
                                   C.POINTER(C.c_double)]
        L.rsa_generate.restype = C.c_int
        _RSA = L
    return _RSA


def _rsa(n: int, box: np.ndarray, rmin: float, seed: int) -> np.ndarray:
    """Random sequential addition of ``n`` points with pair distance >= rmin under PBC."""
    import ctypes as C
    L = _rsa_lib()
    b = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
    out = np.zeros((max(n, 1), 3))
    got = L.rsa_generate(n, b.ctypes.data_as(C.POINTER(C.c_double)), float(rmin), int(seed) & ((1 << 64) - 1),
                         100000, out.ctypes.data_as(C.POINTER(C.c_double)))
    if got != n:
        raise RuntimeError("random sequential addition stalled at %d of %d points" % (got, n))
    return out[:n]


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


def c1_structure(seed: int = 1) -> Structure:
    """FCC a=3.61 A, 10x10x10 cells (4000 atoms), sigma=0.05 A."""
    return fcc(3.61, 10, 0.05, seed)


def c2_structure(n: int = 32000, seed: int = 2) -> Structure:
    """Ternary liquid, density 0.060 /A^3, fractions 0.46/0.46/0.08, min separation 2.0 A."""
    return random_liquid(n, 0.060, [0.46, 0.46, 0.08], 2.0, seed)


def c3_structure(n: int = 1048576, seed: int = 3) -> Structure:
    """Binary glass, density 0.058 /A^3, fractions 0.64/0.36, min separation 2.1 A, tilt 0.1."""
    return random_liquid(n, 0.058, [0.64, 0.36], 2.1, seed, tilt=0.1)


def c4_structures(count: int = 1024, seed: int = 4) -> List[Structure]:
    """Mixed batch: n ~ log-uniform[32, 2048], half orthogonal / half triclinic (tilt 0.1),
    density ~ U[0.055, 0.065], ternary species as the liquid workload, min separation 2.0 A."""
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
