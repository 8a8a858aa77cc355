"""NEP model files (nep.txt) for the oracle.

TEST INFRASTRUCTURE ONLY.  Restates the subset of NEP.java's loader (NEP.java:786-1010)
and of its parameter split (update_potential, NEP.java:1097-1140) that the GPU path
supports: potential models of versions 3, 4 and 5 (``nep3``, ``nep4``, ``nep5``), with or
without ZBL (``nepV_zbl``: a ``zbl rc_inner rc_outer`` line after the first; both zero
select the flexible form, whose 10 parameters per species pair follow the descriptor
scales), with or without type-wise cutoffs (three factors after the cutoff line's
neighbour counts: radial, angular, ZBL).  Other variants raise ValueError.

The file is whitespace-separated text:
    nepV T sym_1 .. sym_T
    cutoff rc_radial rc_angular MN_radial MN_angular [radial_factor angular_factor zbl_factor]
    n_max n_max_radial n_max_angular
    basis_size basis_size_radial basis_size_angular
    l_max l_max_3body l_max_4body l_max_5body
    ANN num_neurons 0
followed by one number per line: the network parameters, the descriptor coefficients
c and the dim descriptor scales q_scaler.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List

import numpy as np


# Element symbols in periodic-table order (H .. Pu): a species' atomic number is its index + 1
ELEMENTS = ("H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge "
            "As Se Br Kr Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm "
            "Eu Gd Tb Dy Ho Er Tm Yb Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn Fr Ra Ac Th Pa U "
            "Np Pu").split()


# Covalent radii (A) by periodic-table index, scaled by the type-wise cutoffs
# (COVALENT_RADIUS, nep_core.hpp:247-258)
COVALENT_RADIUS = (
    0.426667, 0.613333, 1.6, 1.25333, 1.02667, 1.0, 0.946667, 0.84, 0.853333, 0.893333,
    1.86667, 1.66667, 1.50667, 1.38667, 1.46667, 1.36, 1.32, 1.28, 2.34667, 2.05333,
    1.77333, 1.62667, 1.61333, 1.46667, 1.42667, 1.38667, 1.33333, 1.32, 1.34667, 1.45333,
    1.49333, 1.45333, 1.53333, 1.46667, 1.52, 1.56, 2.52, 2.22667, 1.96, 1.85333,
    1.76, 1.65333, 1.53333, 1.50667, 1.50667, 1.44, 1.53333, 1.64, 1.70667, 1.68,
    1.68, 1.64, 1.76, 1.74667, 2.78667, 2.34667, 2.16, 1.96, 2.10667, 2.09333,
    2.08, 2.06667, 2.01333, 2.02667, 2.01333, 2.0, 1.98667, 1.98667, 1.97333, 2.04,
    1.94667, 1.82667, 1.74667, 1.64, 1.57333, 1.54667, 1.48, 1.49333, 1.50667, 1.76,
    1.73333, 1.73333, 1.81333, 1.74667, 1.84, 1.89333, 2.68, 2.41333, 2.22667, 2.10667,
    2.02667, 2.04, 2.05333, 2.06667,
)

@dataclass
class NEPModel:
    version: int
    symbols: List[str]
    rc_radial: float
    rc_angular: float
    n_max_radial: int
    n_max_angular: int
    basis_size_radial: int
    basis_size_angular: int
    l_max: int
    l_max_4body: int
    l_max_5body: int
    num_neurons: int
    params: np.ndarray = field(repr=False)     # network then descriptor parameters
    q_scaler: np.ndarray = field(repr=False)
    zbl: bool = False                          # ZBL short-range term (nepV_zbl)
    zbl_rc_inner: float = 0.0
    zbl_rc_outer: float = 0.0
    zbl_para: np.ndarray = field(default_factory=lambda: np.zeros(0), repr=False)  # flexible: 10 per pair
    typewise: tuple = (0.0, 0.0, 0.0)          # type-wise cutoff factors: radial, angular, ZBL

    def pair_cutoff(self, rc: float, factor: float, ti, tj):
        """A species pair's type-wise cutoff min(rc, (R_cov,i + R_cov,j) factor)
        (find_descriptor / find_force_ZBL, nep_core.hpp:1078, 1121, 1371); ti, tj may be arrays."""
        R = np.asarray(COVALENT_RADIUS)[self.atomic_numbers0]
        return np.minimum(rc, (R[ti] + R[tj]) * factor)

    @property
    def typewise_descriptors(self) -> bool:
        return self.typewise[0] > 0.0

    @property
    def typewise_zbl(self) -> bool:
        return self.typewise[2] > 0.0

    @property
    def zbl_flexible(self) -> bool:
        return self.zbl and self.zbl_rc_inner == 0.0 and self.zbl_rc_outer == 0.0

    @property
    def atomic_numbers0(self) -> np.ndarray:
        """0-based element index of each species (0 for a symbol outside the table)."""
        return np.array([ELEMENTS.index(x) if x in ELEMENTS else 0 for x in self.symbols], dtype=np.int32)

    @property
    def ntypes(self) -> int:
        return len(self.symbols)

    @property
    def num_L(self) -> int:
        return self.l_max + (1 if self.l_max_4body == 2 else 0) + (1 if self.l_max_5body == 1 else 0)

    @property
    def dim_angular(self) -> int:
        return (self.n_max_angular + 1) * self.num_L

    @property
    def dim(self) -> int:
        return (self.n_max_radial + 1) + self.dim_angular

    @property
    def num_para_ann(self) -> int:
        T, d, h = self.ntypes, self.dim, self.num_neurons
        if self.version == 3:
            return (d + 2) * h + 1
        if self.version == 4:
            return (d + 2) * h * T + 1
        return ((d + 2) * h + 1) * T + 1

    @property
    def num_c_radial(self) -> int:
        return self.ntypes ** 2 * (self.n_max_radial + 1) * (self.basis_size_radial + 1)

    @property
    def num_para_descriptor(self) -> int:
        return self.ntypes ** 2 * ((self.n_max_radial + 1) * (self.basis_size_radial + 1) +
                                   (self.n_max_angular + 1) * (self.basis_size_angular + 1))

    def ann(self, t: int):
        """(w0 [h][dim], b0 [h], w1 [h], extra output bias) of species t (0-based)."""
        d, h = self.dim, self.num_neurons
        per = (d + 2) * h + (1 if self.version == 5 else 0)
        off = 0 if self.version == 3 else t * per
        p = self.params
        w0 = p[off:off + h * d].reshape(h, d)
        b0 = p[off + h * d:off + h * d + h]
        w1 = p[off + h * d + h:off + h * d + 2 * h]
        extra = float(p[off + h * d + 2 * h]) if self.version == 5 else 0.0
        return w0, b0, w1, extra

    @property
    def b1(self) -> float:
        return float(self.params[self.num_para_ann - 1])

    @property
    def c(self) -> np.ndarray:
        return self.params[self.num_para_ann:self.num_para_ann + self.num_para_descriptor]


def load(text: str) -> NEPModel:
    lines = [ln.split() for ln in text.splitlines() if ln.split()]
    head = lines[0]
    versions = {"nep3": 3, "nep4": 4, "nep5": 5}
    name = head[0][:-4] if head[0].endswith("_zbl") else head[0]
    if name not in versions:
        raise ValueError("unsupported NEP variant %r (potential models nep3/nep4/nep5, with or without ZBL)" % head[0])
    zbl = head[0].endswith("_zbl")
    T = int(head[1])
    if len(head) != 2 + T:
        raise ValueError("the first line must list %d symbols" % T)
    if zbl:
        z = lines.pop(1)
        if z[0] != "zbl" or len(z) != 3:
            raise ValueError("expected: zbl rc_inner rc_outer")
        zin, zout = float(z[1]), float(z[2])
    cut = lines[1]
    if cut[0] != "cutoff" or len(cut) not in (5, 8):
        raise ValueError("expected: cutoff rc_radial rc_angular MN_radial MN_angular [factors]")
    nmax, bsize, lmax, ann = lines[2], lines[3], lines[4], lines[5]
    if nmax[0] != "n_max" or bsize[0] != "basis_size" or lmax[0] != "l_max" or ann[0] != "ANN":
        raise ValueError("unexpected header line order")
    m = NEPModel(version=versions[name], symbols=head[2:], rc_radial=float(cut[1]), rc_angular=float(cut[2]),
                 n_max_radial=int(nmax[1]), n_max_angular=int(nmax[2]), basis_size_radial=int(bsize[1]),
                 basis_size_angular=int(bsize[2]), l_max=int(lmax[1]), l_max_4body=int(lmax[2]),
                 l_max_5body=int(lmax[3]), num_neurons=int(ann[1]), params=np.zeros(0), q_scaler=np.zeros(0))
    if len(cut) == 8:
        m.typewise = (float(cut[5]), float(cut[6]), float(cut[7]))
    vals = np.array([float(x[0]) for x in lines[6:]], dtype=np.float64)
    npar = m.num_para_ann + m.num_para_descriptor
    if zbl:
        m.zbl, m.zbl_rc_inner, m.zbl_rc_outer = True, zin, zout
    nz = 10 * T * (T + 1) // 2 if m.zbl_flexible else 0
    if len(vals) != npar + m.dim + nz:
        raise ValueError("expected %d numbers after the header, found %d" % (npar + m.dim + nz, len(vals)))
    m.params = vals[:npar]
    m.q_scaler = vals[npar:npar + m.dim]
    m.zbl_para = vals[npar + m.dim:]
    return m


def write(symbols, version=4, rc=(5.0, 4.0), n_max=(4, 4), basis=(8, 8), l_max=(4, 2, 1), neurons=16, seed=0,
          zbl=None, typewise=None) -> str:
    """A random model file (seeded), for tests and benchmarks.  ``zbl``: None, (rc_inner,
    rc_outer) for the fixed ZBL form, or "flexible" for per-pair parameters; ``typewise``:
    None or the three type-wise cutoff factors (radial, angular, ZBL)."""
    rng = np.random.default_rng(seed)
    T = len(symbols)
    m = NEPModel(version=version, symbols=list(symbols), rc_radial=rc[0], rc_angular=rc[1], n_max_radial=n_max[0],
                 n_max_angular=n_max[1], basis_size_radial=basis[0], basis_size_angular=basis[1], l_max=l_max[0],
                 l_max_4body=l_max[1], l_max_5body=l_max[2], num_neurons=neurons, params=np.zeros(0),
                 q_scaler=np.zeros(0))
    ann = rng.normal(0.0, 1.0 / np.sqrt(m.dim), m.num_para_ann)
    c = rng.uniform(-1.0, 1.0, m.num_para_descriptor)
    qs = rng.uniform(0.5, 2.0, m.dim)
    out = ["nep%d%s %d %s" % (version, "_zbl" if zbl else "", T, " ".join(symbols))]
    extra = np.zeros(0)
    if zbl == "flexible":
        out.append("zbl 0 0")
        pairs = T * (T + 1) // 2
        extra = np.concatenate([[rng.uniform(1.0, 1.4), rng.uniform(2.0, 2.4), rng.uniform(0.1, 0.3),
                                 rng.uniform(2.5, 3.5), rng.uniform(0.4, 0.6), rng.uniform(0.8, 1.0),
                                 rng.uniform(0.2, 0.3), rng.uniform(0.3, 0.5), rng.uniform(0.02, 0.04),
                                 rng.uniform(0.15, 0.25)] for _ in range(pairs)])
    elif zbl:
        out.append("zbl %g %g" % tuple(zbl))
    cutline = "cutoff %g %g 100 100" % rc + ("" if typewise is None else " %g %g %g" % tuple(typewise))
    out += [cutline, "n_max %d %d" % n_max, "basis_size %d %d" % basis,
            "l_max %d %d %d" % l_max, "ANN %d 0" % neurons]
    out += ["%.17g" % v for v in np.concatenate([ann, c, qs, extra])]
    return "\n".join(out) + "\n"
