"""Serving over the C ABI: resident structures evaluated by continuous batching.

The reference evaluates one structure per call.  High-throughput and rare-event
workflows instead keep many structures alive and evaluate each of them again and
again after small moves.  Two pieces serve them:

* :class:`NNAPServer` wraps ``nnap_server_*``.  A structure is admitted once.  Its
  species, box and neighbour rows at rcut + skin stay on the GPU.  ``step`` evaluates
  any set of admitted structures in one batched launch sequence.  Neighbour rows are
  rebuilt only for structures with an atom displaced by more than skin/2 since their
  last rebuild.
* :class:`RequestLoop` is the scheduler.  Requests arrive over time and wait in a FIFO
  queue.  They are admitted as soon as the server's memory budget and slot table allow.
  Each admitted request runs one evaluation per step, alongside every other admitted
  request; requests that arrive meanwhile join at the next step.  A request releases its
  slot after its last evaluation.  The loop reports p50/p99 latencies and throughput.
"""
from __future__ import annotations

import ctypes as C
import time
from collections import deque
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from .nnap import (NNAP, NNAP_ERR_BUSY, NNAP_OK, NNAPError, WANT_ENERGY, WANT_ENERGIES, WANT_FORCES,
                   WANT_VIRIAL, WANT_VIRIALS, _dptr, _iptr, _unpack)


class NNAPServer:
    """Resident structures on one handle (the handle is reserved for the server)."""

    def __init__(self, nnap: NNAP, skin: float = 0.5, memory_budget: float = 120e9, max_structs: int = 0):
        self._nnap = nnap
        self._L = nnap._L
        s = C.c_void_p()
        nnap._check(self._L.nnap_server_create(nnap._handle(), float(skin), int(memory_budget), int(max_structs),
                                               C.byref(s)))
        self._s = s
        self.skin = skin
        self._n = {}
        self._pending = None

    def close(self):
        if self._s is not None:
            self._L.nnap_server_destroy(self._s)
            self._s = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _srv(self):
        if self._s is None:
            raise RuntimeError("server is closed")
        return self._s

    def admit(self, data) -> Optional[int]:
        """Make a structure resident; returns its slot, or None while the server is full."""
        x, t, box, kind = _unpack(data)
        slot = C.c_int(-1)
        rc = self._L.nnap_server_admit(self._srv(), len(t), _iptr(t), kind, _dptr(box), C.byref(slot))
        if rc == NNAP_ERR_BUSY:
            return None
        self._nnap._check(rc)
        self._n[slot.value] = len(t)
        return slot.value

    def release(self, slot: int):
        self._nnap._check(self._L.nnap_server_release(self._srv(), int(slot)))
        self._n.pop(slot, None)

    def step(self, slots: Sequence[int], xs, energies: bool = False, forces: bool = True,
             per_atom_virial: bool = False) -> dict:
        """Evaluate ``slots`` at positions ``xs`` (one (n, 3) array per slot, or all of them
        concatenated).  Returns concatenated outputs: ``energy`` and ``virial`` per slot,
        ``forces`` / ``energies`` / ``virials`` per atom in slot order."""
        sl = np.ascontiguousarray(slots, dtype=np.int32)
        if isinstance(xs, np.ndarray):
            x = np.ascontiguousarray(xs, dtype=np.float64)
        else:
            x = np.ascontiguousarray(np.concatenate(xs), dtype=np.float64)
        N = sum(self._n[int(s)] for s in sl)
        if x.size != 3 * N:
            raise ValueError("positions do not match the slots' atom counts")
        S = len(sl)
        e = np.zeros(S)
        v = np.zeros((S, 9))
        flags = WANT_ENERGY | WANT_VIRIAL
        f = ea = va = None
        if forces:
            f = np.zeros((N, 3))
            flags |= WANT_FORCES
        if energies:
            ea = np.zeros(N)
            flags |= WANT_ENERGIES
        if per_atom_virial:
            va = np.zeros((N, 9))
            flags |= WANT_VIRIALS
        self._nnap._check(self._L.nnap_server_step(self._srv(), S, _iptr(sl), _dptr(x), flags, _dptr(e), _dptr(ea),
                                                   _dptr(f), _dptr(v), _dptr(va)))
        out = {"energy": e, "virial": v}
        if forces:
            out["forces"] = f
        if energies:
            out["energies"] = ea
        if per_atom_virial:
            out["virials"] = va
        return out

    def submit(self, slots: Sequence[int], xs: Sequence[np.ndarray], energies: bool = False, forces: bool = True,
               per_atom_virial: bool = False):
        """Queue a step over ``slots`` at positions ``xs`` (one C-contiguous float64 (n, 3)
        array per slot) and return at once: the positions are staged, so the arrays may be
        changed while the step runs.  :meth:`collect` returns its outputs."""
        sl = np.ascontiguousarray(slots, dtype=np.int32)
        ptrs = (C.POINTER(C.c_double) * len(sl))()
        N = 0
        for q, (s, x) in enumerate(zip(sl, xs)):
            n = self._n[int(s)]
            if x.dtype != np.float64 or not x.flags.c_contiguous or x.size != 3 * n:
                raise ValueError("positions of slot %d must be a contiguous float64 (%d, 3) array" % (s, n))
            ptrs[q] = _dptr(x)
            N += n
        flags = WANT_ENERGY | WANT_VIRIAL
        flags |= WANT_FORCES if forces else 0
        flags |= WANT_ENERGIES if energies else 0
        flags |= WANT_VIRIALS if per_atom_virial else 0
        self._nnap._check(self._L.nnap_server_submit(self._srv(), len(sl), _iptr(sl), ptrs, flags))
        self._pending = (len(sl), N, flags)

    def submit_prepared(self, slots: np.ndarray, ptrs: np.ndarray, natoms: int, energies: bool = False,
                        forces: bool = True, per_atom_virial: bool = False):
        """:meth:`submit` for a caller that checked its position arrays once (at admission):
        ``slots`` int32, ``ptrs`` the arrays' addresses (uintp), ``natoms`` their total
        atom count.  Skips the per-array checks, which cost more than the launch for
        hundreds of small structures."""
        sl = np.ascontiguousarray(slots, dtype=np.int32)
        pa = np.ascontiguousarray(ptrs, dtype=np.uintp)
        flags = WANT_ENERGY | WANT_VIRIAL
        flags |= WANT_FORCES if forces else 0
        flags |= WANT_ENERGIES if energies else 0
        flags |= WANT_VIRIALS if per_atom_virial else 0
        self._nnap._check(self._L.nnap_server_submit(self._srv(), len(sl), _iptr(sl),
                                                     pa.ctypes.data_as(C.POINTER(C.POINTER(C.c_double))), flags))
        self._pending = (len(sl), int(natoms), flags)

    def collect(self) -> dict:
        """Wait for the submitted step; outputs as :meth:`step`."""
        S, N, flags = self._pending
        self._pending = None
        e, v = np.zeros(S), np.zeros((S, 9))
        f = np.zeros((N, 3)) if flags & WANT_FORCES else None
        ea = np.zeros(N) if flags & WANT_ENERGIES else None
        va = np.zeros((N, 9)) if flags & WANT_VIRIALS else None
        self._nnap._check(self._L.nnap_server_collect(self._srv(), _dptr(e), _dptr(ea), _dptr(f), _dptr(v),
                                                      _dptr(va)))
        out = {"energy": e, "virial": v}
        if f is not None:
            out["forces"] = f
        if ea is not None:
            out["energies"] = ea
        if va is not None:
            out["virials"] = va
        return out

    def neighborList(self, slot: int):
        """Neighbour list the last step used for ``slot``: (offsets[n+1], j, image[n_pairs x 3])."""
        n = self._n[slot]
        counts = np.zeros(n, dtype=np.int32)
        total = C.c_longlong()
        self._nnap._check(self._L.nnap_server_neighbor_list(self._srv(), slot, _iptr(counts), 0, None, None,
                                                            C.byref(total)))
        j = np.zeros(max(total.value, 1), dtype=np.int32)
        img = np.zeros((max(total.value, 1), 3), dtype=np.int32)
        self._nnap._check(self._L.nnap_server_neighbor_list(self._srv(), slot, _iptr(counts), total.value, _iptr(j),
                                                            _iptr(img), C.byref(total)))
        off = np.zeros(n + 1, dtype=np.int64)
        np.cumsum(counts, out=off[1:])
        return off, j[:total.value], img[:total.value]

    def stats(self) -> dict:
        a = (C.c_longlong * 8)()
        self._nnap._check(self._L.nnap_server_stats(self._srv(), a))
        keys = ["resident_structs", "resident_atoms", "resident_bytes", "work_bytes", "steps", "rebuilds",
                "row_capacity", "memory_budget"]
        return {k: int(a[i]) for i, k in enumerate(keys)}


class GaussianMoves:
    """Positions of successive evaluations: x_k = x_{k-1} + N(0, sigma^2) per coordinate.

    The noise of request ``rid`` at evaluation ``k`` is a window of a fixed seeded pool
    chosen from (rid, k) alone, so a request follows the same trajectory whatever else
    is being served."""

    def __init__(self, sigma: float = 0.01, seed: int = 7, pool: int = 1 << 22):
        self.sigma = sigma
        self.pool = np.random.default_rng(seed).standard_normal(pool) * sigma

    def window(self, rid: int, k: int, m: int) -> np.ndarray:
        span = self.pool.size - m
        off = ((rid * 1000003 + k * 7919) * 2654435761) % max(span, 1)
        return self.pool[off:off + m]

    def __call__(self, rid: int, k: int, x: np.ndarray) -> np.ndarray:
        return x + self.window(rid, k, x.size).reshape(x.shape)

    def apply(self, rid: int, k: int, x: np.ndarray) -> None:
        """The same move, in place (no new array)."""
        x.reshape(-1).__iadd__(self.window(rid, k, x.size))


@dataclass
class Request:
    """One client request: ``nsteps`` successive evaluations of one structure."""
    rid: int
    structure: object
    nsteps: int
    t_arrival: float                      # seconds after the loop starts
    slot: int = -1
    done: int = 0
    x: Optional[np.ndarray] = None
    t_admit: float = float("nan")
    t_done: float = float("nan")
    t_ready: float = float("nan")
    xptr: int = 0                         # address of x (set at admission; x is updated in place)
    natoms: int = 0
    step_latency: List[float] = field(default_factory=list)
    energies: List[float] = field(default_factory=list)
    forces: List[np.ndarray] = field(default_factory=list)


class RequestLoop:
    """Continuous batching over an :class:`NNAPServer`.

    Every loop turn has one step on the GPU.  While it runs, the loop moves the positions
    of the requests that continue and admits new arrivals (FIFO, they join the next step).
    When it completes, the finished requests release their slots, the next step (the
    continuing and the newly admitted requests) is submitted at once, and only then does
    the loop do the accounting of the step it collected, so the GPU does not wait for the
    host's per-request work.  With nothing admitted, the loop sleeps until the next
    arrival."""

    def __init__(self, server: NNAPServer, requests: Sequence[Request], moves=None, keep_results: bool = False):
        self.server = server
        self.requests = sorted(requests, key=lambda r: r.t_arrival)
        self.moves = moves
        self.keep = keep_results

    def run(self) -> dict:
        srv = self.server
        clock = time.perf_counter
        t0 = clock()
        pending = deque(self.requests)
        queue: deque = deque()
        active: List[Request] = []
        atom_evals = 0
        steps = 0
        max_active = 0
        step_atoms = []

        def admit(now):
            while pending and pending[0].t_arrival <= now:
                queue.append(pending.popleft())
            joined = []
            while queue:
                r = queue[0]
                slot = srv.admit(r.structure)
                if slot is None:
                    break
                queue.popleft()
                r.slot, r.t_admit, r.t_ready = slot, now, now
                r.x = np.array(r.structure.x, dtype=np.float64, order="C", copy=True)
                r.xptr = r.x.ctypes.data
                r.natoms = len(r.structure.types)
                joined.append(r)
            return joined

        prepared = hasattr(srv, "submit_prepared")

        def submit(batch):
            if prepared:
                srv.submit_prepared(np.fromiter((r.slot for r in batch), dtype=np.int32, count=len(batch)),
                                    np.fromiter((r.xptr for r in batch), dtype=np.uintp, count=len(batch)),
                                    sum(r.natoms for r in batch), forces=self.keep)
            else:
                srv.submit([r.slot for r in batch], [r.x for r in batch], forces=self.keep)

        active: List[Request] = []   # the step in flight
        joining: List[Request] = []  # admitted while it runs: they join the next step
        while True:
            if not active:
                active = joining + admit(clock() - t0)
                joining = []
                if not active:
                    if queue:
                        raise RuntimeError("a queued request cannot be admitted into an empty server")
                    if not pending:
                        break
                    time.sleep(max(0.0, pending[0].t_arrival - (clock() - t0)))
                    continue
                submit(active)
            # while the step runs: the next positions of the requests that continue, and
            # admissions of the requests that arrived meanwhile
            if self.moves is not None:
                for r in active:
                    if r.done + 1 < r.nsteps:
                        self.moves.apply(r.rid, r.done + 1, r.x)
            joining += admit(clock() - t0)
            out = srv.collect()
            t = clock() - t0
            steps += 1
            max_active = max(max_active, len(active))
            # the next step goes to the GPU before this one's accounting: the finished
            # requests release their slots, arrivals are admitted, and the rest continue
            nxt = []
            for r in active:
                if r.done + 1 < r.nsteps:
                    nxt.append(r)
                else:
                    srv.release(r.slot)
            nxt += joining
            nxt += admit(clock() - t0)
            joining = []
            if nxt:
                submit(nxt)
            n_now = 0
            a0 = 0
            for q, r in enumerate(active):
                n = r.natoms
                n_now += n
                r.step_latency.append(t - r.t_ready)
                r.t_ready = t
                if self.keep:
                    r.energies.append(float(out["energy"][q]))
                    r.forces.append(out["forces"][a0:a0 + n].copy())
                a0 += n
                r.done += 1
                if r.done >= r.nsteps:
                    r.t_done = t
            atom_evals += n_now
            step_atoms.append(n_now)
            active = nxt
        wall = clock() - t0
        lat = np.array([r.t_done - r.t_arrival for r in self.requests]) * 1e3
        ev = np.concatenate([np.asarray(r.step_latency) for r in self.requests]) * 1e3
        wait = np.array([r.t_admit - r.t_arrival for r in self.requests]) * 1e3
        first = min(r.t_arrival for r in self.requests)
        span = max(r.t_done for r in self.requests) - first
        return {
            "requests": len(self.requests),
            "wall_s": wall,
            "req_per_s": len(self.requests) / span,
            "atom_evals_per_s": atom_evals / span,
            "request_p50_ms": float(np.percentile(lat, 50)),
            "request_p99_ms": float(np.percentile(lat, 99)),
            "eval_p50_ms": float(np.percentile(ev, 50)),
            "eval_p99_ms": float(np.percentile(ev, 99)),
            "queue_wait_p99_ms": float(np.percentile(wait, 99)),
            "steps": steps,
            "max_active": max_active,
            "mean_step_atoms": float(np.mean(step_atoms)) if step_atoms else 0.0,
        }


def poisson_requests(pool: Sequence, count: int, rate: float, nsteps: int = 20, seed: int = 9) -> List[Request]:
    """``count`` requests arriving as a Poisson stream of ``rate`` per second (rate
    ``inf``: all at once); each starts from a structure drawn from ``pool``."""
    rng = np.random.default_rng(seed)
    if np.isinf(rate):
        t = np.zeros(count)
    else:
        t = np.cumsum(rng.exponential(1.0 / rate, size=count))
    pick = rng.integers(0, len(pool), size=count)
    return [Request(k, pool[int(pick[k])], nsteps, float(t[k])) for k in range(count)]
