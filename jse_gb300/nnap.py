"""Python mirror of jse's ``jsex.nnap.NNAP`` potential over the C ABI of ``libnnap_gb300.so``.

Method names, argument meaning and error behaviour follow the reference:

* ``NNAP(model, ...)``                      -- ``NNAP(Map|String)`` (NNAP.java:402-426);
* ``ntypes() / rcutMax() / symbol(t) / units()`` (NNAP.java:86-90, 489-491);
* ``calEnergyForceVirials(data, ...)``      -- ``IPairPotential.calEnergyForceVirials``
                                               (IPairPotential.java:811-1022, 1137);
* ``calEnergy / calEnergies / calForces / calStress / calStresses``
                                            -- the ``IPotential`` conveniences
                                               (IPotential.java:145-311, IPairPotential.java:129-303);
* ``calFp(data)``                           -- ``NNAP.calFp(IAtomData)`` (NNAP.java:596-632);
* ``close()`` / ``isClosed()``              -- ``NNAP.close`` (NNAP.java:472-486); a closed object
                                               raises ``IllegalStateError("This NNAP is dead")``.

Atom data is anything with ``x`` (n x 3 Cartesian), ``types`` (1-based), ``box`` (3 x 3 rows
a, b, c) and ``box_kind`` (0 orthogonal, 1 LAMMPS triclinic, 2 general prism), such as
:class:`jse_gb300.workloads.Structure`.  All work runs on the GPU through the CUDA
library; there is no CPU path and the import fails loudly when the library is missing.
"""
from __future__ import annotations

import ctypes as C
import json
import os
from typing import Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libnnap_gb300.so")

NNAP_OK, NNAP_ERR_BAD_MODEL, NNAP_ERR_BAD_TYPE, NNAP_ERR_CAPACITY, NNAP_ERR_CUDA, NNAP_ERR_UNSUPPORTED, \
    NNAP_ERR_ARG, NNAP_ERR_TIMEOUT, NNAP_ERR_DEAD, NNAP_ERR_BUSY = range(10)
PREC = {"fp32": 0, "single": 0, "mixed": 1}
WANT_ENERGY, WANT_ENERGIES, WANT_FORCES, WANT_VIRIAL, WANT_VIRIALS = 1, 2, 4, 8, 16

EXPORTS = ["nnap_create", "nnap_create_from_file", "nnap_destroy", "nnap_ntypes", "nnap_rcut_max", "nnap_symbol",
           "nnap_descriptor_size", "nnap_last_error", "nnap_compute", "nnap_compute_device", "nnap_compute_batch",
           "nnap_compute_fp", "nnap_neighbor_list", "nnap_last_launch_count", "nnap_set_profiling",
           "nnap_stage_times", "nnap_compute_batch_device", "nnap_set_graphs", "nnap_neighbor_counts_noalloc",
           "nnap_server_create", "nnap_server_destroy", "nnap_server_admit", "nnap_server_release",
           "nnap_server_step", "nnap_server_neighbor_list", "nnap_server_stats", "nnap_set_autotune",
           "nnap_get_tuning", "nnap_set_tuning", "nnap_compute_lammps", "nnap_param_sizes", "nnap_train_grad_batch",
           "nnap_create_nep", "nnap_create_nep_from_file", "nnap_compute_lammps_nl", "nnap_model_check",
           "nnap_server_submit", "nnap_server_collect"]


class IllegalStateError(RuntimeError):
    """Raised where the reference throws IllegalStateException."""


class NNAPError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("NNAP status %d: %s" % (status, msg))
        self.status = status


_lib = None


def load_library(path: str = LIB_PATH):
    """Load the CUDA library (raises OSError when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError("libnnap_gb300.so is missing; build it with `python -m jse_gb300.build`")
    L = C.CDLL(path)
    P, I, D, S = C.c_void_p, C.c_int, C.c_double, C.c_size_t
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
    L.nnap_create.argtypes = [C.c_char_p, S, I, I, C.POINTER(P)]
    L.nnap_create_from_file.argtypes = [C.c_char_p, I, I, C.POINTER(P)]
    L.nnap_model_check.argtypes = [C.c_char_p, S, ip, C.POINTER(C.c_uint64), C.c_char_p, S]
    L.nnap_destroy.argtypes = [P]
    L.nnap_ntypes.argtypes = [P, ip]
    L.nnap_rcut_max.argtypes = [P, dp]
    L.nnap_symbol.argtypes = [P, I, C.c_char_p, S]
    L.nnap_descriptor_size.argtypes = [P, I, ip]
    L.nnap_last_error.argtypes = [P]
    L.nnap_last_error.restype = C.c_char_p
    L.nnap_compute.argtypes = [P, I, dp, ip, I, dp, I, dp, dp, dp, dp, dp]
    L.nnap_compute_device.argtypes = [P, I, P, P, I, dp, I, P, P, P, P, P, P]
    L.nnap_compute_batch.argtypes = [P, I, ip, dp, ip, ip, dp, I, dp, dp, dp, dp, dp]
    L.nnap_compute_fp.argtypes = [P, I, dp, ip, I, dp, dp, I]
    L.nnap_neighbor_list.argtypes = [P, I, dp, ip, I, dp, ip, C.c_longlong, ip, ip, C.POINTER(C.c_longlong)]
    L.nnap_last_launch_count.argtypes = [P, ip]
    L.nnap_set_profiling.argtypes = [P, I]
    L.nnap_stage_times.argtypes = [P, dp]
    L.nnap_compute_batch_device.argtypes = [P, I, ip, P, P, ip, dp, I, P, P, P, P, P, P]
    L.nnap_set_graphs.argtypes = [P, I]
    L.nnap_compute_lammps.argtypes = [P, I, I, ip, ip, C.POINTER(ip), dp, ip, ip, I, I, I, I, I, dp, dp, dp, dp,
                                      dp, dp]
    L.nnap_set_autotune.argtypes = [P, I]
    L.nnap_get_tuning.argtypes = [P, I, ip, ip]
    L.nnap_set_tuning.argtypes = [P, I, ip]
    L.nnap_server_create.argtypes = [P, D, S, I, C.POINTER(P)]
    L.nnap_server_destroy.argtypes = [P]
    L.nnap_server_admit.argtypes = [P, I, ip, I, dp, ip]
    L.nnap_server_release.argtypes = [P, I]
    L.nnap_server_step.argtypes = [P, I, ip, dp, I, dp, dp, dp, dp, dp]
    L.nnap_server_submit.argtypes = [P, I, ip, C.POINTER(dp), I]
    L.nnap_server_collect.argtypes = [P, dp, dp, dp, dp, dp]
    L.nnap_server_neighbor_list.argtypes = [P, I, ip, C.c_longlong, ip, ip, C.POINTER(C.c_longlong)]
    L.nnap_server_stats.argtypes = [P, C.POINTER(C.c_longlong)]
    L.nnap_param_sizes.argtypes = [P, I, ip, ip]
    L.nnap_train_grad_batch.argtypes = [P, I, ip, dp, ip, ip, dp, dp, dp, dp, dp, dp]
    L.nnap_compute_lammps_nl.argtypes = [P, I, I, I, ip, ip, C.POINTER(ip), dp, ip, ip, I, I, I, I, I, dp, dp, dp,
                                         dp, dp, dp]
    L.nnap_create_nep.argtypes = [C.c_char_p, S, I, I, C.POINTER(P)]
    L.nnap_create_nep_from_file.argtypes = [C.c_char_p, I, I, C.POINTER(P)]
    _lib = L
    return L


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int)) if a is not None else None


def _unpack(data):
    x = np.ascontiguousarray(data.x, dtype=np.float64).reshape(-1, 3)
    t = np.ascontiguousarray(data.types, dtype=np.int32).reshape(-1)
    box = np.ascontiguousarray(data.box, dtype=np.float64).reshape(9)
    return x, t, box, int(getattr(data, "box_kind", 0))


def model_check(model) -> dict:
    """Parse and validate model text (JSON or YAML), a dict or a model file without a GPU
    (nnap_model_check): {"ntypes", "digest"}; raises NNAPError for an invalid model."""
    L = load_library()
    if isinstance(model, dict):
        model = json.dumps(model)
    if isinstance(model, str) and os.path.isfile(model):
        with open(model, "rb") as f:
            b = f.read()
    else:
        b = model.encode() if isinstance(model, str) else bytes(model)
    nt = C.c_int()
    dig = C.c_uint64()
    err = C.create_string_buffer(512)
    rc = L.nnap_model_check(b, len(b), C.byref(nt), C.byref(dig), err, 512)
    if rc != NNAP_OK:
        raise NNAPError(rc, err.value.decode(errors="replace"))
    return {"ntypes": nt.value, "digest": dig.value}


class NNAP:
    """GB300 NNAP potential.  ``model`` is a path to a JSON model file, JSON text or a dict."""

    def __init__(self, model, precision: str = "fp32", device: int = 0):
        L = load_library()
        if precision not in PREC:
            raise ValueError("precision must be 'fp32' or 'mixed'")
        h = C.c_void_p()
        if isinstance(model, dict):
            model = json.dumps(model)
        if isinstance(model, str) and not model.lstrip().startswith("{") and os.path.isfile(model):
            rc = L.nnap_create_from_file(model.encode(), PREC[precision], device, C.byref(h))
        else:
            b = model.encode() if isinstance(model, str) else bytes(model)
            rc = L.nnap_create(b, len(b), PREC[precision], device, C.byref(h))
        if rc != NNAP_OK:
            raise NNAPError(rc, "model could not be loaded" if rc == NNAP_ERR_BAD_MODEL else "handle creation failed")
        self._h = h
        self._L = L
        self.precision = precision

    # ----------------------------------------------------------- lifetime
    def close(self):
        if self._h is not None:
            self._L.nnap_destroy(self._h)
            self._h = None

    def isClosed(self) -> bool:
        return self._h is None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _handle(self):
        if self._h is None:
            raise IllegalStateError("This NNAP is dead")
        return self._h

    def _check(self, rc: int):
        if rc != NNAP_OK:
            msg = self._L.nnap_last_error(self._h).decode() if self._h is not None else ""
            if rc == NNAP_ERR_BAD_TYPE:
                raise ValueError("Exist type greater than the input ntypes: " + msg)
            raise NNAPError(rc, msg)

    # ----------------------------------------------------------- model queries
    def ntypes(self) -> int:
        v = C.c_int()
        self._check(self._L.nnap_ntypes(self._handle(), C.byref(v)))
        return v.value

    def rcutMax(self) -> float:
        v = C.c_double()
        self._check(self._L.nnap_rcut_max(self._handle(), C.byref(v)))
        return v.value

    def symbol(self, t: int) -> str:
        buf = C.create_string_buffer(64)
        self._check(self._L.nnap_symbol(self._handle(), t, buf, 64))
        return buf.value.decode()

    def symbols(self):
        return [self.symbol(t) for t in range(1, self.ntypes() + 1)]

    def descriptorSize(self, t: int) -> int:
        v = C.c_int()
        self._check(self._L.nnap_descriptor_size(self._handle(), t, C.byref(v)))
        return v.value

    def lastLaunchCount(self) -> int:
        v = C.c_int()
        self._check(self._L.nnap_last_launch_count(self._handle(), C.byref(v)))
        return v.value

    def setGraphs(self, on: bool):
        """CUDA-graph replay of repeated evaluations of the same layout (on by default)."""
        self._check(self._L.nnap_set_graphs(self._handle(), 1 if on else 0))

    def setAutotune(self, on: bool):
        """Tune launch shapes on the first evaluation of each atom-count bucket."""
        self._check(self._L.nnap_set_autotune(self._handle(), 1 if on else 0))

    TUNING_KEYS = ("desc_fwd_warps", "desc_bwd_warps", "nb_warps", "gather_block", "net_split")

    def tuning(self, natoms: int) -> dict:
        """Launch shapes used for ``natoms`` atoms (and whether they were tuned)."""
        v = np.zeros(5, dtype=np.int32)
        t = C.c_int()
        self._check(self._L.nnap_get_tuning(self._handle(), int(natoms), _iptr(v), C.byref(t)))
        d = dict(zip(self.TUNING_KEYS, (int(x) for x in v)))
        d["tuned"] = bool(t.value)
        return d

    def setTuning(self, natoms: int, shapes: dict):
        v = np.array([shapes[k] for k in self.TUNING_KEYS], dtype=np.int32)
        self._check(self._L.nnap_set_tuning(self._handle(), int(natoms), _iptr(v)))

    def setProfiling(self, on: bool):
        self._check(self._L.nnap_set_profiling(self._handle(), 1 if on else 0))

    def stageTimes(self) -> np.ndarray:
        """Device ms of [neighbours, descriptors fwd, network, descriptors bwd, scatter] of the last call."""
        out = np.zeros(5)
        self._check(self._L.nnap_stage_times(self._handle(), _dptr(out)))
        return out

    # ----------------------------------------------------------- evaluation
    def calEnergyForceVirials(self, data, energies: bool = True, forces: bool = True, virials: bool = True,
                              per_atom_virial: bool = True) -> dict:
        """Energies (per atom), forces and virials of one structure.

        Returns a dict with ``energy`` (total), ``energies`` (n), ``forces`` (n x 3),
        ``virial`` (9: xx, yy, zz, xy, xz, yz, yx, zx, zy) and, when requested,
        ``virials`` (n x 9, the pair term assigned to the neighbour).
        """
        x, t, box, kind = _unpack(data)
        n = len(t)
        flags = WANT_ENERGY | WANT_VIRIAL
        e = np.zeros(1)
        ea = np.zeros(n) if energies else None
        f = np.zeros((n, 3)) if forces else None
        v = np.zeros(9)
        va = np.zeros((n, 9)) if per_atom_virial and virials else None
        if energies:
            flags |= WANT_ENERGIES
        if forces:
            flags |= WANT_FORCES
        if va is not None:
            flags |= WANT_VIRIALS
        self._check(self._L.nnap_compute(self._handle(), n, _dptr(x), _iptr(t), kind, _dptr(box), flags, _dptr(e),
                                         _dptr(ea), _dptr(f), _dptr(v), _dptr(va)))
        out = {"energy": float(e[0]), "virial": v}
        if energies:
            out["energies"] = ea
        if forces:
            out["forces"] = f
        if va is not None:
            out["virials"] = va
        return out

    def calEnergy(self, data) -> float:
        return self.calEnergyForceVirials(data, energies=False, forces=False, virials=False)["energy"]

    def calEnergies(self, data) -> np.ndarray:
        return self.calEnergyForceVirials(data, forces=False, virials=False)["energies"]

    def calForces(self, data) -> np.ndarray:
        return self.calEnergyForceVirials(data, energies=False, virials=False)["forces"]

    def calStress(self, data) -> list:
        """[xx, yy, zz, xy, xz, yz] = -virial / volume (IPotential.java:264-311, without the ideal-gas term)."""
        v = self.calEnergyForceVirials(data, energies=False, forces=False, per_atom_virial=False)["virial"]
        vol = abs(np.linalg.det(np.asarray(data.box, dtype=np.float64).reshape(3, 3)))
        return [-v[k] / vol for k in range(6)]

    def calStresses(self, data) -> np.ndarray:
        """Per-atom stresses [n x 6] = -per-atom virial (IPairPotential.java:224-257 without volume)."""
        va = self.calEnergyForceVirials(data, energies=False, forces=False)["virials"]
        return -va[:, :6]

    def calFp(self, data) -> np.ndarray:
        """Descriptor vector of every atom (rows padded with zeros to the largest size)."""
        x, t, box, kind = _unpack(data)
        n = len(t)
        D = max(self.descriptorSize(s) for s in range(1, self.ntypes() + 1))
        out = np.zeros((n, D))
        self._check(self._L.nnap_compute_fp(self._handle(), n, _dptr(x), _iptr(t), kind, _dptr(box), _dptr(out), D))
        return out

    def neighborList(self, data):
        """Full neighbour list with the largest cutoff: (offsets[n+1], j, image[n_pairs x 3])."""
        x, t, box, kind = _unpack(data)
        n = len(t)
        counts = np.zeros(n, dtype=np.int32)
        total = C.c_longlong()
        self._check(self._L.nnap_neighbor_list(self._handle(), n, _dptr(x), _iptr(t), kind, _dptr(box),
                                               _iptr(counts), 0, None, None, C.byref(total)))
        j = np.zeros(max(total.value, 1), dtype=np.int32)
        img = np.zeros((max(total.value, 1), 3), dtype=np.int32)
        self._check(self._L.nnap_neighbor_list(self._handle(), n, _dptr(x), _iptr(t), kind, _dptr(box),
                                               _iptr(counts), total.value, _iptr(j), _iptr(img), C.byref(total)))
        off = np.zeros(n + 1, dtype=np.int64)
        np.cumsum(counts, out=off[1:])
        return off, j[:total.value], img[:total.value]

    def calEnergyForceVirialsBatch(self, structures: Sequence, per_atom_virial: bool = False) -> list:
        """Evaluate many independent structures in one batched launch sequence."""
        xs, ts, kinds, boxes, ns = [], [], [], [], []
        for s in structures:
            x, t, box, kind = _unpack(s)
            xs.append(x); ts.append(t); kinds.append(kind); boxes.append(box); ns.append(len(t))
        S = len(ns)
        x = np.ascontiguousarray(np.concatenate(xs)) if S else np.zeros((0, 3))
        t = np.ascontiguousarray(np.concatenate(ts)).astype(np.int32)
        nat = np.asarray(ns, dtype=np.int32)
        kd = np.asarray(kinds, dtype=np.int32)
        bx = np.ascontiguousarray(np.concatenate(boxes))
        N = int(nat.sum())
        e = np.zeros(S)
        ea = np.zeros(N)
        f = np.zeros((N, 3))
        v = np.zeros((S, 9))
        va = np.zeros((N, 9)) if per_atom_virial else None
        flags = WANT_ENERGY | WANT_ENERGIES | WANT_FORCES | WANT_VIRIAL | (WANT_VIRIALS if per_atom_virial else 0)
        self._check(self._L.nnap_compute_batch(self._handle(), S, _iptr(nat), _dptr(x), _iptr(t), _iptr(kd),
                                               _dptr(bx), flags, _dptr(e), _dptr(ea), _dptr(f), _dptr(v), _dptr(va)))
        out, a0 = [], 0
        for s in range(S):
            n = ns[s]
            r = {"energy": float(e[s]), "energies": ea[a0:a0 + n], "forces": f[a0:a0 + n], "virial": v[s]}
            if va is not None:
                r["virials"] = va[a0:a0 + n]
            out.append(r)
            a0 += n
        return out

    def paramSizes(self, t: int):
        """(basis parameters, network parameters) of species t (1-based), C-level layouts."""
        a, b = C.c_int(0), C.c_int(0)
        self._check(self._L.nnap_param_sizes(self._handle(), int(t), C.byref(a), C.byref(b)))
        return a.value, b.value

    def backwardEnergyForceBatch(self, structures: Sequence, bgrad_energies=None, bgrad_forces=None,
                                 bgrad_virial=None, want_fp: bool = False) -> dict:
        """Parameter gradients of L = sum bE.E + sum bF.F + sum bW.W over a batch of structures.

        The structure-level form of the reference's training pair forwardEnergyForce /
        backwardEnergyForce (NNAP.java:823-869) as TrainerNNAP drives it: ``bgrad_energies``
        holds dL/dE_i per atom, ``bgrad_forces`` dL/dF_i (n x 3), ``bgrad_virial`` dL/dW per
        structure (9 components xx, yy, zz, xy, xz, yz, yx, zx, zy); each may be None.
        Returns per-species lists ``grad_nn`` (hidden W | output W | hidden b | output b)
        and, with ``want_fp``, ``grad_fp`` (radial-fuse matrices)."""
        xs, ts, kinds, boxes, ns = [], [], [], [], []
        for s in structures:
            x, t, box, kind = _unpack(s)
            xs.append(x); ts.append(t); kinds.append(kind); boxes.append(box); ns.append(len(t))
        S = len(ns)
        x = np.ascontiguousarray(np.concatenate(xs)) if S else np.zeros((0, 3))
        t = np.ascontiguousarray(np.concatenate(ts)).astype(np.int32)
        nat = np.asarray(ns, dtype=np.int32)
        kd = np.asarray(kinds, dtype=np.int32)
        bx = np.ascontiguousarray(np.concatenate(boxes))
        N = int(nat.sum())
        be = None if bgrad_energies is None else np.ascontiguousarray(bgrad_energies, dtype=np.float64).reshape(N)
        bf = None if bgrad_forces is None else np.ascontiguousarray(bgrad_forces, dtype=np.float64).reshape(N, 3)
        bw = None if bgrad_virial is None else np.ascontiguousarray(bgrad_virial, dtype=np.float64).reshape(S, 9)
        T = self.ntypes()
        sizes = [self.paramSizes(k + 1) for k in range(T)]
        gfp = np.zeros(max(sum(a for a, _ in sizes), 1)) if want_fp else None
        gnn = np.zeros(max(sum(b for _, b in sizes), 1))
        self._check(self._L.nnap_train_grad_batch(self._handle(), S, _iptr(nat), _dptr(x), _iptr(t), _iptr(kd),
                                                  _dptr(bx), _dptr(be), _dptr(bf), _dptr(bw), _dptr(gfp),
                                                  _dptr(gnn)))
        out = {"grad_nn": [], "grad_fp": [] if want_fp else None}
        on = of = 0
        for a, b in sizes:
            out["grad_nn"].append(gnn[on:on + b].copy())
            on += b
            if want_fp:
                out["grad_fp"].append(gfp[of:of + a].copy())
                of += a
        return out

    def computeLammps(self, ilist, neighbors, x, types, type_map=None, eflag=True, vflag=True, eflag_atom=True,
                      vflag_atom=False, cvflag_atom=True, nlflag=True) -> dict:
        """LAMMPS-style evaluation (``PairNNAP_gpu``): ``ilist`` local atoms, ``neighbors[i]``
        the full list of local atom i (indices into the nall = len(x) local + ghost atoms),
        ``types`` LAMMPS types (mapped through ``type_map`` when given).  ``nlflag=False``
        reuses the list sent by the last call with ``nlflag=True`` (``neighbors`` is then not
        read).  Returns fresh accumulators: forces on every atom (ghosts included), eng,
        eatom, virial[6], vatom (nall x 6), cvatom (nall x 9)."""
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        t = np.ascontiguousarray(types, dtype=np.int32)
        il = np.ascontiguousarray(ilist, dtype=np.int32)
        nall = len(x)
        lists = [np.ascontiguousarray(neighbors[i], dtype=np.int32) if i < len(neighbors) and neighbors[i] is not None
                 else np.zeros(0, dtype=np.int32) for i in range(nall)]
        num = np.array([len(a) for a in lists], dtype=np.int32)
        ptrs = (C.POINTER(C.c_int) * max(nall, 1))(*[_iptr(a) for a in lists])
        tm = None if type_map is None else np.ascontiguousarray(type_map, dtype=np.int32)
        f = np.zeros((nall, 3))
        eng = np.zeros(1)
        eatom = np.zeros(nall)
        vir = np.zeros(6)
        vatom = np.zeros((nall, 6))
        cvatom = np.zeros((nall, 9))
        self._check(self._L.nnap_compute_lammps_nl(self._handle(), int(bool(nlflag)), len(il), nall, _iptr(il),
                                                   _iptr(num), ptrs, _dptr(x), _iptr(t), _iptr(tm), int(eflag),
                                                   int(vflag), int(eflag_atom), int(vflag_atom), int(cvflag_atom),
                                                   _dptr(f), _dptr(eng), _dptr(eatom), _dptr(vir), _dptr(vatom),
                                                   _dptr(cvatom)))
        return {"forces": f, "eng": float(eng[0]), "eatom": eatom, "virial": vir, "vatom": vatom, "cvatom": cvatom}

    def computeBatchDevice(self, natoms, x_ptr: int, type_ptr: int, box_kinds, boxes, flags: int,
                           energy_ptr: int = 0, energies_ptr: int = 0, forces_ptr: int = 0, virial_ptr: int = 0,
                           virials_ptr: int = 0, stream: int = 0):
        """Batched device-resident evaluation; natoms/box_kinds/boxes are host sequences."""
        nat = np.ascontiguousarray(natoms, dtype=np.int32)
        kd = np.ascontiguousarray(box_kinds, dtype=np.int32)
        bx = np.ascontiguousarray(boxes, dtype=np.float64).reshape(-1)
        self._check(self._L.nnap_compute_batch_device(self._handle(), len(nat), _iptr(nat), x_ptr, type_ptr,
                                                      _iptr(kd), _dptr(bx), flags, energy_ptr or None,
                                                      energies_ptr or None, forces_ptr or None, virial_ptr or None,
                                                      virials_ptr or None, stream or None))

    def computeDevice(self, n: int, x_ptr: int, type_ptr: int, box, box_kind: int, flags: int, energy_ptr: int = 0,
                      energies_ptr: int = 0, forces_ptr: int = 0, virial_ptr: int = 0, virials_ptr: int = 0,
                      stream: int = 0):
        """Device-resident evaluation (pointers are raw device addresses, e.g. ``tensor.data_ptr()``)."""
        box = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
        self._check(self._L.nnap_compute_device(self._handle(), n, x_ptr, type_ptr, box_kind, _dptr(box), flags,
                                                energy_ptr or None, energies_ptr or None, forces_ptr or None,
                                                virial_ptr or None, virials_ptr or None, stream or None))
