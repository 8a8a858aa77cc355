"""Benchmark: NNAP energy+force+virial evaluation, atom-evals/s, on one GB300 per rank.

A step evaluates energies, forces and virials of one batch of structures (or one
structure) of the chosen workload.  ``value`` is the device-resident throughput (inputs
already in HBM, outputs left in HBM), timed per step with CUDA events on the caller's
stream with an L2 flush (a 256 MiB write) between steps outside the events.  ``e2e`` is
the same metric through the host-buffer C-ABI call ``nnap_compute_batch`` with pinned host
inputs and outputs: host->device copies of positions and species and the device->host
read of energies, forces and virials are inside the timed region.  ``plain_gpu`` is the
plain FP32 drop-in: one synchronous single-structure ``nnap_compute`` per structure.

Workloads (seeded synthetic inputs; the reference publishes none):
  batch1024   1024 structures, 32..2048 atoms log-uniform, half triclinic, the liquid's model (default)
  liquid32k   ternary liquid, 32000 atoms, spherical Chebyshev nmax 8 lmax 6 rc 6.0, 126->64->64->1
  fcc4000     perturbed FCC Cu, 4000 atoms, radial Chebyshev nmax 10 rc 6.0, 11->32->32->1
  glass1m     binary glass, 1048576 atoms, LAMMPS triclinic, nmax 8 lmax 4 rc 5.5, 90->64->64->1
Every model carries the descriptor normalisation committed in tests/golden/bench_norm.json,
so both arms evaluate the same model file.  The default run also measures the liquid
(``liquid32k`` object), serving, training gradients, NEP and the reference's own CUDA
kernels.

``--impl reference`` times the reference's own per-atom C++ arithmetic (expanded from its
headers, compiled -O3 -ffast-math into oracle/_ref) on all host cores over a bounded
sample of the same workload, driven over neighbour lists built outside the timed region
(the reference's neighbour search is not timed; this build's ``value`` includes its own);
only rank 0 runs it.  With torchrun and N > 1 every rank evaluates its own replica of the
workload (the path has no collective); value = atoms of all ranks / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from jse_gb300 import workloads as W  # noqa: E402

METRIC = "NNAP E+F atom-evals/s"


# ----------------------------------------------------------------------------- workloads
def make_workload(name: str, atoms: int = 0):
    """Structures and a model-factory taking per-species normalisation statistics.  ``atoms``
    resizes the liquid and glass workloads (same density and composition), for profiling."""
    if name == "liquid32k":
        return [W.c2_structure(atoms) if atoms else W.c2_structure()], "c2"
    if name == "fcc4000":
        return [W.c1_structure()], "c1"
    if name == "glass1m":
        return [W.c3_structure(atoms) if atoms else W.c3_structure()], "c3"
    if name == "batch1024":
        return W.c4_structures(), "c4"
    raise SystemExit("unknown workload " + name)


def bench_model(cfg: str) -> dict:
    """The workload's model with the committed descriptor normalisation (per species mean
    and standard deviation of the descriptors of one seeded structure of the workload,
    tests/golden/make_bench_norm.py): the same model file for both arms."""
    with open(os.path.join(ROOT, "tests", "golden", "bench_norm.json")) as f:
        st = json.load(f)["c2" if cfg in ("c4", "c5") else cfg]
    return W.model_for(cfg, norm_mu=[np.asarray(v) for v in st["mu"]], norm_sigma=[np.asarray(v) for v in st["sigma"]])


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.out = tempfile.NamedTemporaryFile("w+", delete=False, suffix=".csv")

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.flush()
        self.out.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out.read().splitlines():
            f = [c.strip() for c in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.out.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------------------- roofline
def stage_costs(model: dict, mean_nei: float):
    """Algorithmic HBM bytes and FP32 FLOPs per atom of each pipeline stage.

    Bytes count every item once (positions, pair rows, descriptors, expansion
    coefficients, gradients, outputs); FLOPs are the per-pair counts of the
    descriptor mathematics: forward 6K + 3Nn + 8 + 2 P Nn + 2 P K, backward
    4 P K + 2 P Nn + 14 K + 3 Nn, with K = (lmax+1)^2 (0 for a radial basis).
    """
    b = model["models"][0]["basis"]
    T = len(model["models"])
    nmax = int(b.get("nmax", 5))
    N1 = nmax + 1
    P = (2 * N1 if T > 1 else N1) if b.get("wtype", "default") == "default" else N1
    sph = b.get("type", "spherical_chebyshev") not in ("chebyshev", "cheby")
    L = int(b.get("lmax", 6)) if sph else -1
    K = (L + 1) ** 2 if sph else 0
    D = P * (L + 1) if sph else P
    nn = mean_nei
    H = model["models"][0]["nn"]["hidden_dims"]
    pk = P * K * 4
    stages = {
        "neighbours": {"bytes": 24 + 4 + 24 + 16 + 4 + nn * (8 + 16 + 4) + 4, "flops": 0.0},
        "descriptors_fwd": {"bytes": nn * 16 + 8 + D * 4 + pk, "flops": nn * (6 * K + 3 * N1 + 8 + 2 * P * N1 + 2 * P * K)},
        "network": {"bytes": 2 * D * 4 + 8, "flops": 4.0 * (D * H[0] + sum(H[i] * H[i + 1] for i in range(len(H) - 1)) + H[-1])},
        "descriptors_bwd": {"bytes": nn * 32 + 8 + D * 4 + pk, "flops": nn * (4 * P * K + 2 * P * N1 + 14 * K + 3 * N1)},
        "scatter": {"bytes": nn * (16 + 4 + 16 + 16) + 4 + 24 + 72 + 8 + 72, "flops": 0.0},
    }
    return stages


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured", float(d.get("sm_max_mhz", 2070.0))
    return 6800.0, "fallback", 2070.0


def load_traffic():
    """DRAM bytes per atom of a stage's dominant kernel, from one ncu capture
    (dram__bytes_read.sum + dram__bytes_write.sum of one launch divided by its atoms):
    liquid32k / descriptors_bwd is k_sph_bwd_n<6,18,9> on the 32000-atom liquid, 159.2 MB
    read + 16.9 MB written (profiles/k_sph_liquid32k.md); batch1024 / descriptors_bwd is the
    same kernel over the 1024-structure batch, 2626.6 MB read + 443.2 MB written for 526124
    atoms (profiles/batch1024_launches_and_top_kernels.md)."""
    return {"liquid32k/descriptors_bwd": (159.2e6 + 16.9e6) / 32000,
            "batch1024/descriptors_bwd": (2626.569e6 + 443.240e6) / 526124}


# ----------------------------------------------------------------------------- reference arm
class _RefSample:
    """A prefix of the workload's structures as one list of independent atoms for the
    reference's per-atom arithmetic: wrapped positions, neighbour lists (built here, outside
    any timed region) and species, concatenated with shifted atom indices.  Structures are
    independent, so one call over the concatenation does the work of one call per
    structure without the per-call thread start-up of the driver."""

    def __init__(self, structures, rcut: float, max_atoms: int):
        from oracle import native as ON
        offs, js, dxs, types, imgs = [np.zeros(1, dtype=np.int64)], [], [], [], []
        n = 0
        self.nstruct = 0
        for s in structures:
            if n and n + s.natoms > max_atoms:
                break
            xw = ON.wrap(s.x, s.box_kind, s.box)
            nl = ON.neighbors(xw, s.box_kind, s.box, rcut)
            offs.append(nl.offsets[1:] + offs[-1][-1])
            js.append(nl.j + n)
            dxs.append(nl.dx)
            imgs.append(nl.img)
            types.append(np.asarray(s.types, dtype=np.int32))
            n += s.natoms
            self.nstruct += 1
        self.natoms = n
        self.types = np.concatenate(types)
        self.nl = ON.NeighborList(np.concatenate(offs), np.concatenate(js).astype(np.int32),
                                  np.concatenate(imgs), np.ascontiguousarray(np.concatenate(dxs)))


def cpu_reference(structures, model: dict, budget_s: float = 12.0, threads: int = 0, single_thread_s: float = 0.0):
    """Time the reference's per-atom arithmetic (oracle/_ref, -O3 -ffast-math) or, when that
    build is absent, the oracle port, on a bounded sample of the workload: the first
    structures up to about ``budget_s`` seconds of work (for a single large structure, its
    first atoms).  Neighbour lists are built before the timed region.  Returns (atoms/s,
    info); with ``single_thread_s`` > 0 info also holds a one-thread rate on a smaller
    sample of the same kind."""
    from oracle import model as OM, native as ON
    threads = threads or os.cpu_count() or 1
    pm = OM.load(model)
    kind = "reference"
    try:
        ref = ON.RefLib(pm, fast=True)
    except (FileNotFoundError, OSError, RuntimeError):
        ref = None
        kind = "port"
    many = len(structures) > 1

    def sample(atoms):
        if many:
            return _RefSample(structures, pm.rcut_max, atoms)
        return _RefSample(structures[:1], pm.rcut_max, structures[0].natoms)

    def run(smp, m, nth):
        t0 = time.perf_counter()
        if ref is not None:
            ref.compute(smp.types, smp.nl, nthreads=nth, n_eval=m)
        else:
            ON.compute(pm, np.zeros((smp.natoms, 3)), smp.types, 0, np.eye(3), nl=smp.nl, n_eval=m)
        return time.perf_counter() - t0

    def measure(budget, nth):
        atoms = 2048
        while True:
            smp = sample(atoms)
            m = smp.natoms if many else min(smp.natoms, atoms)
            dt = run(smp, m, nth)
            if dt >= 0.25 * budget or (many and smp.nstruct == len(structures)) or (not many and m == smp.natoms):
                break
            atoms = int(atoms * min(16.0, max(2.0, 0.5 * budget / max(dt, 1e-3))))
        rate = m / dt
        want = int(rate * budget)
        if want > m:
            smp = sample(want)
            m = smp.natoms if many else min(smp.natoms, want)
            dt = run(smp, m, nth)
        what = ("%d structures (%d atoms) of %d" % (smp.nstruct, m, len(structures)) if many
                else "%d of %d atoms of the structure" % (m, smp.natoms))
        return m / dt, what

    nth = threads if ref is not None else 1
    rate, what = measure(budget_s, nth)
    info = {"kind": kind, "cores": nth,
            "sample": "%s, full neighbour rows built outside the timed region (neighbour search not timed), %s" % (
                what, "reference per-atom C++ (-O3 -ffast-math), %d threads" % nth if ref is not None
                else "FP64 oracle port, 1 thread")}
    if single_thread_s > 0 and ref is not None:
        r1, what1 = measure(single_thread_s, 1)
        info["single_thread"] = {"value": r1, "unit": "atom-evals/s", "cores": 1, "sample": what1}
    return rate, info


# ----------------------------------------------------------------------------- serving
def serve_measurement(device: int, nreq: int = 5000, loads=(0.5, 0.8, 1.0, 1.2), steady: int = 64,
                      curve=(64, 256)) -> dict:
    """Continuous-batching serving of ``nreq`` requests of 20 evaluations each.

    Requests start from structures of a 256-structure pool (n ~ log-normal, median 500,
    log-sd 1.0, clipped to [50, 20000]; ternary liquids at 0.060 /A^3) and move every
    coordinate by N(0, 0.01^2) A between evaluations.  The server keeps neighbour rows at
    rcut + 0.5 A and admits by a 120 GB budget.  ``steady`` lists the request rate
    sustained at a steady resident count R (every request queued at once, at most R slots:
    one is admitted as soon as one finishes); ``saturated`` is that run with 1024 slots.
    The capacity is the rate at ``steady`` resident requests, an operating point of
    millisecond steps; the Poisson runs offer fractions of it with up to 1024 resident
    requests, so a burst is absorbed by larger, more efficient steps.  Latencies are
    wall-clock, host buffers, and include queueing."""
    from jse_gb300.nnap import NNAP
    from jse_gb300.serve import GaussianMoves, NNAPServer, RequestLoop, poisson_requests
    pool = W.c5_pool(256)
    model = bench_model("c5")
    moves = GaussianMoves(sigma=0.01, seed=7)
    out = {"requests": nreq, "evaluations_per_request": 20, "skin_A": 0.5, "memory_budget_GB": 120,
           "max_resident": 1024, "capacity_at_resident": steady,
           "pool": "256 structures, n ~ lognormal(median 500, sd 1.0) in [50, 20000]",
           "mean_atoms": float(np.mean([p.natoms for p in pool])),
           "loop": "submit a step, move the continuing requests and admit arrivals while it runs, collect"}
    with NNAP(model, precision="mixed", device=device) as p:
        def run(rate, slots=1024):
            with NNAPServer(p, skin=0.5, memory_budget=120e9, max_structs=slots) as srv:
                reqs = poisson_requests(pool, nreq, rate, nsteps=20, seed=11)
                st = RequestLoop(srv, reqs, moves=moves).run()
                ss = srv.stats()
                st["rebuilds_per_request"] = ss["rebuilds"] / max(1, nreq)
                return st
        # warm the pool allocator and kernels
        with NNAPServer(p, skin=0.5, memory_budget=120e9, max_structs=1024) as srv:
            RequestLoop(srv, poisson_requests(pool, 64, float("inf"), nsteps=3, seed=1), moves=moves).run()
        sat = run(float("inf"))
        out["saturated"] = {"req_s": sat["req_per_s"], "atom_evals_s": sat["atom_evals_per_s"],
                            "eval_p50_ms": sat["eval_p50_ms"], "max_active": sat["max_active"]}
        out["steady"] = []
        for R in sorted(set(curve) | {steady}):
            st = run(float("inf"), slots=R)
            out["steady"].append({"resident": R, "req_s": st["req_per_s"], "atom_evals_s": st["atom_evals_per_s"],
                                  "eval_p50_ms": st["eval_p50_ms"]})
            if R == steady:
                cap = st["req_per_s"]
                out["capacity_req_s"] = cap
                out["capacity_atom_evals_s"] = st["atom_evals_per_s"]
        runs = []
        for f in loads:
            st = run(f * cap)
            runs.append({"load": f, "offered_req_s": f * cap, "achieved_req_s": st["req_per_s"],
                         "atom_evals_s": st["atom_evals_per_s"], "request_p50_ms": st["request_p50_ms"],
                         "request_p99_ms": st["request_p99_ms"], "eval_p50_ms": st["eval_p50_ms"],
                         "eval_p99_ms": st["eval_p99_ms"], "max_active": st["max_active"],
                         "rebuilds_per_request": st["rebuilds_per_request"]})
        out["runs"] = runs
    return out


# ----------------------------------------------------------------------------- training
def train_measurement(device: int, s, model: dict, steps: int = 5, cpu: bool = True) -> dict:
    """Force-training gradients (nnap_train_grad_batch) of one structure: dL/dparameters of
    L = bE.E + bF.F + bW.W for seeded upstream gradients, host buffers in and out, FP32.
    The CPU baseline runs the reference's training pair (jse_nnap_forwardEnergyForce +
    jse_nnap_backwardEnergyForce per atom, oracle/_ref -O3 -ffast-math, all host threads)
    on a 2000-atom structure of the same liquid."""
    import torch
    from jse_gb300.nnap import NNAP
    n = s.natoms
    rng = np.random.default_rng(17)
    be, bf, bw = rng.normal(size=n), rng.normal(size=(n, 3)), rng.normal(size=(1, 9))
    out = {"unit": "atom-evals/s", "atoms": n, "path": "nnap_train_grad_batch, host buffers, FP32 (network "
           "parameter gradients of an energy + force + virial loss)"}
    with NNAP(model, precision="fp32", device=device) as p:
        for _ in range(3):
            p.backwardEnergyForceBatch([s], be, bf, bw)
        dts = []
        for _ in range(steps):
            torch.cuda.synchronize(device)
            t0 = time.perf_counter()
            p.backwardEnergyForceBatch([s], be, bf, bw)
            dts.append(time.perf_counter() - t0)
        out["gpu_launches"] = p.lastLaunchCount()
    out["value"] = n * len(dts) / sum(dts)
    out["ms_per_step"] = 1e3 * sum(dts) / len(dts)
    if cpu:
        try:
            from oracle import model as OM, native as ON
            pm = OM.load(model)
            ref = ON.RefLib(pm, fast=True)
            smp = W.random_liquid(2000, 0.060, [0.46, 0.46, 0.08], 2.0, 5)
            nl = ON.neighbors(ON.wrap(smp.x, smp.box_kind, smp.box), smp.box_kind, smp.box, pm.rcut_max)
            r2 = np.random.default_rng(18)
            args = (smp.types, nl, r2.normal(size=2000), r2.normal(size=(2000, 3)), r2.normal(size=9))
            threads = os.cpu_count() or 1
            ref.train_grad(*args, nthreads=threads)
            t0 = time.perf_counter()
            reps = 0
            while time.perf_counter() - t0 < 5.0:
                ref.train_grad(*args, nthreads=threads)
                reps += 1
            v = 2000 * reps / (time.perf_counter() - t0)
            out["cpu_baseline"] = {"value": v, "unit": "atom-evals/s", "kind": "reference", "cores": threads,
                                   "sample": "2000-atom liquid of the same density and species, %d repeats" % reps}
        except Exception as ex:
            out["cpu_baseline"] = {"value": None, "error": str(ex)[:200]}
    return out


# ----------------------------------------------------------------------------- reference GPU kernels
def ref_gpu_measurement(device: int, s, model: dict, precision: str, steps: int = 10) -> dict:
    """A baseline leg: the reference's own CUDA kernels (nnap_interface_cuda.cu, FP32, one
    thread per atom, compiled by oracle/ref_cuda.py; the reference is what is measured,
    never this build) beside this build's, on the LAMMPS form of the same structure (local
    atoms, ghost atoms, full neighbour lists from nnap_neighbor_list).
    ``lammps_e2e``: one call of each LAMMPS boundary per step with host arrays in and out
    (reference: jse_nnap_lammps2cuda + jse_nnap_computeLammpsCuda + jse_nnap_cuda2lammps,
    lists sent every step; this build: nnap_compute_lammps); ``_list_reused``: the same with
    the list of the previous step kept on the device (nlflag = 0, as between LAMMPS
    neighbour-list rebuilds).  ``kernels``: the reference's
    jse_nnap_computeLammpsCuda with its inputs on the device (its memsets, three kernels and
    closing synchronisation) against this build's device-resident nnap_compute_device on the
    periodic structure, which also builds its own neighbour list.  L2 flushed between steps."""
    import torch
    from jse_gb300.nnap import NNAP, WANT_ENERGY, WANT_FORCES, WANT_VIRIAL, _dptr, _iptr
    from oracle import ref_cuda as RC
    dev = torch.device("cuda", device)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    n = s.natoms
    out = {"unit": "atom-evals/s", "atoms": n, "reference": "nnap_interface_cuda.cu kernels compiled for sm_103a "
           "(-O3), FP32, driven through their own host functions", "precision_ours": precision}

    def timed(fn, k):
        for _ in range(2):
            fn()
        dts = []
        for _ in range(k):
            flush.zero_()
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize(dev)
            dts.append(time.perf_counter() - t0)
        return n * k / sum(dts), 1e3 * sum(dts) / k
    with NNAP(model, precision=precision, device=device) as p:
        off, j, img = p.neighborList(s)
        x, t, lists, owner = W.lammps_form(s, off, j, img)
        nall = len(x)
        out["ghosts"] = nall - n
        out["mean_neighbours"] = float(len(j)) / n
        il = np.arange(n, dtype=np.int32)
        rows = [np.ascontiguousarray(l, dtype=np.int32) for l in lists] + [np.zeros(0, np.int32)] * (nall - n)
        num = np.array([len(r) for r in rows], dtype=np.int32)
        ptrs = (C.POINTER(C.c_int) * nall)(*[_iptr(r) for r in rows])
        xh = np.ascontiguousarray(x)
        f, eng, eatom, vir = np.zeros((nall, 3)), np.zeros(1), np.zeros(nall), np.zeros(6)

        def ours_lmp():
            p._check(p._L.nnap_compute_lammps(p._handle(), n, nall, _iptr(il), _iptr(num), ptrs, _dptr(xh), _iptr(t),
                                              None, 1, 1, 1, 0, 0, _dptr(f), _dptr(eng), _dptr(eatom), _dptr(vir),
                                              None, None))
        v, ms = timed(ours_lmp, steps)
        out["ours_lammps_e2e"] = {"value": v, "ms_per_step": ms}

        def ours_lmp_reuse():
            p._check(p._L.nnap_compute_lammps_nl(p._handle(), 0, n, nall, _iptr(il), _iptr(num), ptrs, _dptr(xh),
                                                 _iptr(t), None, 1, 1, 1, 0, 0, _dptr(f), _dptr(eng), _dptr(eatom),
                                                 _dptr(vir), None, None))
        v, ms = timed(ours_lmp_reuse, steps)
        out["ours_lammps_e2e_list_reused"] = {"value": v, "ms_per_step": ms}
        x_d = torch.from_numpy(np.ascontiguousarray(s.x)).to(dev)
        t_d = torch.from_numpy(np.ascontiguousarray(s.types, dtype=np.int32)).to(dev)
        e_d = torch.zeros(1, dtype=torch.float64, device=dev)
        f_d = torch.zeros((n, 3), dtype=torch.float64, device=dev)
        v_d = torch.zeros(9, dtype=torch.float64, device=dev)

        def ours_dev():
            p.computeDevice(n, x_d.data_ptr(), t_d.data_ptr(), s.box, s.box_kind, WANT_ENERGY | WANT_FORCES | WANT_VIRIAL,
                            e_d.data_ptr(), 0, f_d.data_ptr(), v_d.data_ptr(), 0,
                            stream=torch.cuda.current_stream(dev).cuda_stream)
        v, ms = timed(ours_dev, steps)
        out["ours_kernels"] = {"value": v, "ms_per_step": ms}
        for a in (f, eng, eatom, vir):  # the LAMMPS boundary accumulates, like a pair style
            a[...] = 0.0
        ours_lmp()
        f_ours = f[:n].copy()
        np.add.at(f_ours, owner, f[n:])
    if precision != "fp32":  # this build in FP32 too, for an FP32-against-FP32 comparison
        with NNAP(model, precision="fp32", device=device) as p32:
            def ours_lmp32():
                p32._check(p32._L.nnap_compute_lammps(p32._handle(), n, nall, _iptr(il), _iptr(num), ptrs, _dptr(xh),
                                                      _iptr(t), None, 1, 1, 1, 0, 0, _dptr(f), _dptr(eng),
                                                      _dptr(eatom), _dptr(vir), None, None))
            v, ms = timed(ours_lmp32, steps)
            out["ours_lammps_e2e_fp32"] = {"value": v, "ms_per_step": ms}

            def ours_dev32():
                p32.computeDevice(n, x_d.data_ptr(), t_d.data_ptr(), s.box, s.box_kind,
                                  WANT_ENERGY | WANT_FORCES | WANT_VIRIAL, e_d.data_ptr(), 0, f_d.data_ptr(),
                                  v_d.data_ptr(), 0, stream=torch.cuda.current_stream(dev).cuda_stream)
            v, ms = timed(ours_dev32, steps)
            out["ours_kernels_fp32"] = {"value": v, "ms_per_step": ms}
    try:
        ref = RC.RefCudaNNAP(model, device)
    except (FileNotFoundError, RuntimeError, OSError, ValueError) as ex:
        out["reference_error"] = str(ex)[:200]
        return out
    ref.setup(x, t, n, lists)
    v, ms = timed(ref.step, steps)
    out["ref_lammps_e2e"] = {"value": v, "ms_per_step": ms}

    def ref_step_reuse():
        ref.to_device(False)
        ref.compute()
        ref.to_host()
    v, ms = timed(ref_step_reuse, steps)
    out["ref_lammps_e2e_list_reused"] = {"value": v, "ms_per_step": ms}
    ref.to_device(True)
    v, ms = timed(ref.compute, steps)
    out["ref_kernels"] = {"value": v, "ms_per_step": ms}
    r = ref.step()
    f_ref = r["forces"][:n].copy()
    np.add.at(f_ref, owner, r["forces"][n:])
    out["max_abs_force_difference"] = float(np.abs(f_ref - f_ours).max())
    out["speedup_lammps_e2e"] = out["ours_lammps_e2e"]["value"] / out["ref_lammps_e2e"]["value"]
    out["speedup_kernels"] = out["ours_kernels"]["value"] / out["ref_kernels"]["value"]
    if "ours_kernels_fp32" in out:  # FP32 against the reference's FP32 kernels
        out["speedup_lammps_e2e_fp32"] = out["ours_lammps_e2e_fp32"]["value"] / out["ref_lammps_e2e"]["value"]
        out["speedup_kernels_fp32"] = out["ours_kernels_fp32"]["value"] / out["ref_kernels"]["value"]
    return out


# ----------------------------------------------------------------------------- NEP
def nep_ref_gpu(device: int, p, s, text: str, flush, steps: int) -> dict:
    """The reference's CUDA NEP kernels (nep_interface_cuda.cu, FP32, one thread per atom,
    compiled by oracle/nep_ref_cuda.py; the reference is what is measured) beside this
    build's LAMMPS boundary on the LAMMPS form of the NEP benchmark structure: host arrays
    in and out, lists sent every step; and the reference's kernels alone with their inputs
    on the device."""
    import torch
    from jse_gb300.nnap import _dptr, _iptr
    dev = torch.device("cuda", device)
    n = s.natoms
    off, j, img = p.neighborList(s)
    x, t, lists, owner = W.lammps_form(s, off, j, img)
    nall = len(x)
    out = {"unit": "atom-evals/s", "ghosts": nall - n}

    def timed(fn):
        for _ in range(2):
            fn()
        dts = []
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize(dev)
            dts.append(time.perf_counter() - t0)
        return {"value": n * steps / sum(dts), "ms_per_step": 1e3 * sum(dts) / steps}
    il = np.arange(n, dtype=np.int32)
    rows = [np.ascontiguousarray(l, dtype=np.int32) for l in lists] + [np.zeros(0, np.int32)] * (nall - n)
    num = np.array([len(r) for r in rows], dtype=np.int32)
    ptrs = (C.POINTER(C.c_int) * nall)(*[_iptr(r) for r in rows])
    xh = np.ascontiguousarray(x)
    f, eng, eatom, vir = np.zeros((nall, 3)), np.zeros(1), np.zeros(nall), np.zeros(6)

    def ours():
        p._check(p._L.nnap_compute_lammps(p._handle(), n, nall, _iptr(il), _iptr(num), ptrs, _dptr(xh), _iptr(t),
                                          None, 1, 1, 1, 0, 0, _dptr(f), _dptr(eng), _dptr(eatom), _dptr(vir),
                                          None, None))
    out["ours_lammps_e2e"] = timed(ours)
    for a in (f, eng, eatom, vir):
        a[...] = 0.0
    ours()
    f_ours = f[:n].copy()
    np.add.at(f_ours, owner, f[n:])
    try:
        from oracle import nep_model as NM, nep_ref_cuda as NRC
        ref = NRC.RefCudaNEP(NM.load(text), device)
    except (FileNotFoundError, RuntimeError, OSError, ValueError) as ex:
        out["reference_error"] = str(ex)[:200]
        return out
    ref.setup(x, t, n, lists)
    out["ref_lammps_e2e"] = timed(ref.step)
    ref.to_device(True)
    out["ref_kernels"] = timed(ref.compute)
    r = ref.step()
    f_ref = r["forces"][:n].copy()
    np.add.at(f_ref, owner, r["forces"][n:])
    out["max_abs_force_difference"] = float(np.abs(f_ref - f_ours).max())
    out["speedup_lammps_e2e"] = out["ours_lammps_e2e"]["value"] / out["ref_lammps_e2e"]["value"]
    return out


def nep_measurement(device: int, steps: int = 10, cpu: bool = True, autotune: bool = True) -> dict:
    """NEP potential through nnap_create_nep on the NEP benchmark: a 32000-atom binary liquid
    (0.060 /A^3) under a seeded nep4 potential of GPUMD's default hyperparameters (cutoff
    8 / 4 A, n_max 4 4, basis_size 8 8, l_max 4 2 1, 30 neurons), FP32.  ``value`` is
    device-resident (CUDA events on the launching stream, L2 flushed between steps); ``e2e``
    goes through nnap_compute with pinned host buffers.  The CPU baseline is the reference's
    NEP arithmetic (oracle/_ref, -O3 -ffast-math) with all host threads on a sample of the
    same structure's atoms (full neighbour rows)."""
    import torch
    from jse_gb300.nep import NEP
    from jse_gb300.nnap import WANT_ENERGY, WANT_FORCES, WANT_VIRIAL, _dptr, _iptr
    text, s = W.nep_bench()
    n = s.natoms
    dev = torch.device("cuda", device)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    x_d = torch.from_numpy(np.ascontiguousarray(s.x)).to(dev)
    t_d = torch.from_numpy(np.ascontiguousarray(s.types, dtype=np.int32)).to(dev)
    e_d = torch.zeros(1, dtype=torch.float64, device=dev)
    f_d = torch.zeros((n, 3), dtype=torch.float64, device=dev)
    v_d = torch.zeros(9, dtype=torch.float64, device=dev)
    flags = WANT_ENERGY | WANT_FORCES | WANT_VIRIAL
    out = {"unit": "atom-evals/s", "atoms": n, "model": "nep4, 2 species, cutoff 8/4 A, n_max 4 4, basis_size 8 8, "
           "l_max 4 2 1, 30 neurons (seeded random weights)", "precision": "FP32"}
    with NEP(text, device=device) as p:
        def dstep():
            p.computeDevice(n, x_d.data_ptr(), t_d.data_ptr(), s.box, s.box_kind, flags, e_d.data_ptr(), 0,
                            f_d.data_ptr(), v_d.data_ptr(), 0, stream=torch.cuda.current_stream(dev).cuda_stream)
        p.setProfiling(True)
        p.setAutotune(autotune)  # shapes picked on the first warm-up step, as for the NNAP liquid
        for _ in range(3):
            flush.zero_()
            dstep()
        torch.cuda.synchronize(dev)
        ms, stages, launches = [], np.zeros(5), 0
        for _ in range(steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            dstep()
            e1.record()
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
            stages += p.stageTimes()
            launches += p.lastLaunchCount()
        out["value"] = n * steps / (sum(ms) / 1e3)
        out["ms_per_step"] = sum(ms) / steps
        out["gpu_launches"] = launches
        out["stage_ms"] = dict(zip(["neighbours", "descriptors_fwd", "network", "descriptors_bwd", "scatter"],
                                   [round(float(v), 5) for v in stages / steps]))
        xh = torch.from_numpy(np.ascontiguousarray(s.x)).pin_memory().numpy()
        th = torch.from_numpy(np.ascontiguousarray(s.types, dtype=np.int32)).pin_memory().numpy()
        fh = torch.zeros((n, 3), dtype=torch.float64).pin_memory().numpy()
        eh = torch.zeros(1, dtype=torch.float64).pin_memory().numpy()
        vh = torch.zeros(9, dtype=torch.float64).pin_memory().numpy()
        box = np.ascontiguousarray(s.box, dtype=np.float64).reshape(9)

        def hstep():
            p._check(p._L.nnap_compute(p._handle(), n, _dptr(xh), _iptr(th), int(s.box_kind), _dptr(box), flags,
                                       _dptr(eh), None, _dptr(fh), _dptr(vh), None))
        for _ in range(3):
            hstep()
        dts = []
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            hstep()
            dts.append(time.perf_counter() - t0)
        out["e2e"] = {"value": n * steps / sum(dts), "unit": "atom-evals/s", "h2d_bytes_per_step": n * 28,
                      "d2h_bytes_per_step": 8 + n * 24 + 72}
        if cpu:  # a baseline leg: the reference's own CUDA NEP on the LAMMPS form of the structure
            out["reference_gpu"] = nep_ref_gpu(device, p, s, text, flush, steps)
    if cpu:
        try:
            from oracle import native as ON, nep_model as NM, nep_ref as NR
            m = NM.load(text)
            ref = NR.RefNEP(m, fast=True)
            nl = ON.neighbors(ON.wrap(s.x, s.box_kind, s.box), s.box_kind, s.box, max(m.rc_radial, m.rc_angular))
            threads = os.cpu_count() or 1
            t0s = s.types - 1
            k = 256
            while True:
                t0 = time.perf_counter()
                ref.compute(t0s, nl, nthreads=threads, n_eval=k)
                dt = time.perf_counter() - t0
                if dt > 1.0 or k >= n:
                    break
                k = min(n, k * 4)
            k = int(min(n, max(k, k / dt * 10.0)))
            t0 = time.perf_counter()
            ref.compute(t0s, nl, nthreads=threads, n_eval=k)
            v = k / (time.perf_counter() - t0)
            out["cpu_baseline"] = {"value": v, "unit": "atom-evals/s", "kind": "reference", "cores": threads,
                                   "sample": "%d of %d atoms, full neighbour rows, reference NEP per-atom C++ "
                                             "(-O3 -ffast-math)" % (k, n)}
        except Exception as ex:  # the baseline is reported, never required
            out["cpu_baseline"] = {"value": None, "error": str(ex)[:200]}
    return out


# ----------------------------------------------------------------------------- device runs
def _sm_count(dev) -> int:
    import torch
    return int(torch.cuda.get_device_properties(dev).multi_processor_count)


def device_run(pot, structures, dev, flush, steps: int, warmup: int, clocks=None, dist=None):
    """Warm-up then ``steps`` timed evaluations of the whole workload with inputs and outputs
    resident on the device (CUDA events on the launching stream, L2 flushed between steps
    outside the events).  Returns timing, per-stage times, kernel launches and the
    device arrays."""
    import torch
    from jse_gb300.nnap import WANT_ENERGY, WANT_FORCES, WANT_VIRIAL
    from jse_gb300.replicas import barrier
    single = len(structures) == 1
    s = structures[0]
    nat = np.array([st.natoms for st in structures], dtype=np.int32)
    kinds = np.array([st.box_kind for st in structures], dtype=np.int32)
    boxes = np.ascontiguousarray(np.concatenate([np.asarray(st.box, dtype=np.float64).reshape(9) for st in structures]))
    x_all = np.ascontiguousarray(np.concatenate([st.x for st in structures]))
    t_all = np.ascontiguousarray(np.concatenate([st.types for st in structures]).astype(np.int32))
    N, S = int(nat.sum()), len(structures)
    x_d = torch.from_numpy(x_all).to(dev)
    t_d = torch.from_numpy(t_all).to(dev)
    e_d = torch.zeros(S, dtype=torch.float64, device=dev)
    f_d = torch.zeros((N, 3), dtype=torch.float64, device=dev)
    v_d = torch.zeros((S, 9), dtype=torch.float64, device=dev)
    flags = WANT_ENERGY | WANT_FORCES | WANT_VIRIAL

    def step():
        st_ = torch.cuda.current_stream(dev).cuda_stream
        if single:
            pot.computeDevice(N, x_d.data_ptr(), t_d.data_ptr(), s.box, s.box_kind, flags, e_d.data_ptr(), 0,
                              f_d.data_ptr(), v_d.data_ptr(), 0, stream=st_)
        else:
            pot.computeBatchDevice(nat, x_d.data_ptr(), t_d.data_ptr(), kinds, boxes, flags, e_d.data_ptr(), 0,
                                   f_d.data_ptr(), v_d.data_ptr(), 0, stream=st_)

    pot.setProfiling(True)
    for _ in range(warmup):
        flush.zero_()
        step()
    torch.cuda.synchronize(dev)
    if clocks is not None:
        clocks.start()
        time.sleep(0.2)
    barrier(dist)
    torch.cuda.synchronize(dev)
    ms, stages, launches, stage_ok = [], np.zeros(5), 0, True
    t_wall = time.perf_counter()
    for _ in range(steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        step()
        e1.record()
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
        if stage_ok:
            try:
                stages += pot.stageTimes()
            except Exception:
                stage_ok = False
        launches += pot.lastLaunchCount()
    torch.cuda.synchronize(dev)
    wall = time.perf_counter() - t_wall
    barrier(dist)
    clk = clocks.stop() if clocks is not None else None
    return {"ms": ms, "stages": stages / steps, "launches": launches, "wall": wall, "clocks": clk, "N": N, "S": S,
            "nat": nat, "kinds": kinds, "boxes": boxes, "x_all": x_all, "t_all": t_all}


def e2e_run(pot, run, dev, flush, steps: int) -> dict:
    """The same evaluations through nnap_compute_batch with pinned host buffers: the copies of
    inputs and outputs are inside the timed region."""
    import torch
    from jse_gb300.nnap import WANT_ENERGY, WANT_FORCES, WANT_VIRIAL, _dptr, _iptr
    N, S = run["N"], run["S"]
    nat, kinds, boxes = run["nat"], run["kinds"], run["boxes"]
    xh = torch.from_numpy(run["x_all"]).pin_memory().numpy()
    th = torch.from_numpy(run["t_all"]).pin_memory().numpy()
    fh = torch.zeros((N, 3), dtype=torch.float64).pin_memory().numpy()
    eh = torch.zeros(S, dtype=torch.float64).pin_memory().numpy()
    vh = torch.zeros((S, 9), dtype=torch.float64).pin_memory().numpy()
    flags = WANT_ENERGY | WANT_FORCES | WANT_VIRIAL

    def host_step():
        pot._check(pot._L.nnap_compute_batch(pot._handle(), S, _iptr(nat), _dptr(xh), _iptr(th), _iptr(kinds),
                                             _dptr(boxes), flags, _dptr(eh), None, _dptr(fh), _dptr(vh), None))
    for _ in range(3):
        host_step()
    dts = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        host_step()
        dts.append(time.perf_counter() - t0)
    return {"value": N * len(dts) / sum(dts), "unit": "atom-evals/s", "h2d_bytes_per_step": N * 28,
            "d2h_bytes_per_step": S * 8 + N * 24 + S * 72, "path": "nnap_compute_batch, pinned host buffers"}


def plain_run(model, run, local, dev, flush, steps: int) -> dict:
    """The plain FP32 drop-in: one synchronous single-structure nnap_compute per structure
    on an FP32 handle, host buffers (graphs off for a batch: every structure has its own
    layout)."""
    import torch
    from jse_gb300.nnap import NNAP, WANT_ENERGY, WANT_FORCES, WANT_VIRIAL, _dptr, _iptr
    N, S = run["N"], run["S"]
    nat, kinds, boxes = run["nat"], run["kinds"], run["boxes"]
    xh, th = run["x_all"], run["t_all"]
    fh, eh, vh = np.zeros((N, 3)), np.zeros(S), np.zeros((S, 9))
    flags = WANT_ENERGY | WANT_FORCES | WANT_VIRIAL
    with NNAP(model, precision="fp32", device=local) as pp:
        if S > 1:
            pp.setGraphs(False)
        offs = np.concatenate([[0], np.cumsum(nat)])

        def plain_step():
            for k in range(S):
                a, b = offs[k], offs[k + 1]
                pp._check(pp._L.nnap_compute(pp._handle(), int(nat[k]), _dptr(xh[a:b]), _iptr(th[a:b]),
                                             int(kinds[k]), _dptr(boxes[9 * k:9 * k + 9]), flags, _dptr(eh[k:k + 1]),
                                             None, _dptr(fh[a:b]), _dptr(vh[k]), None))
        for _ in range(3):
            plain_step()
        pts = []
        for _ in range(max(1, min(steps, 5) if S > 1 else steps)):
            flush.zero_()
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            plain_step()
            pts.append(time.perf_counter() - t0)
    pv = N * len(pts) / sum(pts)
    return {"value": pv, "unit": "atom-evals/s", "ms_per_step": 1e3 * sum(pts) / len(pts),
            "path": "plain FP32, one synchronous nnap_compute per structure, host buffers"}


def mean_neighbours(pot, structures) -> float:
    pairs, atoms = 0, 0
    for s in structures:
        off, j, img = pot.neighborList(s)
        pairs += len(j)
        atoms += s.natoms
    return pairs / max(1, atoms)


def roofline(model, mean_nei: float, stages, natoms_step: int, workload: str, sm_count: int) -> dict:
    """HBM roofline of the dominant stage (algorithmic bytes / stage time against the measured
    copy bandwidth) and its FP32 fraction against this GPU's FP32 peak (SMs x 128 lanes x 2
    x maximum clock)."""
    peak, peak_kind, sm_max = load_peaks()
    costs = stage_costs(model, mean_nei)
    names = list(costs.keys())
    dom = int(np.argmax(stages))
    dname = names[dom]
    t_dom = stages[dom] / 1e3
    achieved = costs[dname]["bytes"] * natoms_step / t_dom / 1e9
    fp32_peak = sm_count * 128 * 2 * sm_max * 1e6 / 1e12
    traffic = load_traffic().get("%s/%s" % (workload, dname))
    return {"bound": "hbm", "kernel_stage": dname, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind,
            "traffic": traffic * natoms_step if traffic else None,
            "algorithmic_bytes_per_atom": costs[dname]["bytes"],
            "fp32": {"achieved_tflops": costs[dname]["flops"] * natoms_step / t_dom / 1e12,
                     "peak_tflops": fp32_peak,
                     "peak_source": "%d SMs (cudaDeviceProp) x 128 lanes x 2 x max clock %.0f MHz" % (sm_count, sm_max),
                     "frac": costs[dname]["flops"] * natoms_step / t_dom / 1e12 / fp32_peak},
            "stage_ms": dict(zip(names, [round(float(x), 5) for x in stages])),
            "mean_neighbours": mean_nei}


# ----------------------------------------------------------------------------- main
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="batch1024", choices=["batch1024", "liquid32k", "fcc4000", "glass1m"])
    ap.add_argument("--precision", default="mixed", choices=["fp32", "mixed"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="only the headline workload (no liquid, serving, "
                    "training, NEP or reference-GPU legs)")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving measurement")
    ap.add_argument("--no-train", action="store_true", help="skip the training-gradient measurement")
    ap.add_argument("--no-nep", action="store_true", help="skip the NEP measurement")
    ap.add_argument("--no-ref-gpu", action="store_true", help="skip the reference-CUDA-kernel comparison")
    ap.add_argument("--only-ref-gpu", action="store_true", help="run only the reference-CUDA-kernel comparison")
    ap.add_argument("--only-nep", action="store_true", help="run only the NEP measurement (profiling runs)")
    ap.add_argument("--only-train", action="store_true", help="run only the training-gradient measurement "
                    "(profiling runs)")
    ap.add_argument("--serve-requests", type=int, default=5000)
    ap.add_argument("--ref-seconds", type=float, default=20.0, help="host seconds of the reference arm's timed "
                    "samples over all steps (plus a 5 s single-thread sample)")
    ap.add_argument("--no-autotune", action="store_true", help="default launch shapes (profiling runs)")
    ap.add_argument("--atoms", type=int, default=0, help="resize the liquid / glass workload (profiling runs)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    from jse_gb300.replicas import barrier, init_from_env, max_over_ranks, whole_job_rate
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist, rank, world = init_from_env("gloo")

    if args.only_nep:
        if rank == 0:
            print(json.dumps({"nep": nep_measurement(local, steps=args.steps, cpu=not args.no_cpu_baseline,
                                                        autotune=not args.no_autotune)}))
        return
    structures, cfg = make_workload(args.workload, args.atoms)
    natoms_step = sum(s.natoms for s in structures)
    config = {"workload": args.workload, "structures": len(structures), "atoms_per_step": natoms_step,
              "precision": args.precision, "l2": "flushed between steps (256 MiB write)",
              "parallelism": "replicas x%d" % world,
              "model": "normalisation from tests/golden/bench_norm.json (same model file in both arms)"}
    model = bench_model(cfg)

    if args.impl == "reference":
        if rank != 0:
            return
        rates = []
        info = None
        for k in range(args.steps):
            r, info = cpu_reference(structures, model, budget_s=max(0.5, args.ref_seconds / max(args.steps, 1)),
                                    single_thread_s=min(5.0, args.ref_seconds / 4) if k == args.steps - 1 else 0.0)
            rates.append(r)
        v = statistics.median(rates)
        line = {"metric": METRIC, "value": v, "unit": "atom-evals/s", "n_gpus": 0, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": natoms_step / v * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
                "config": config, "impl": "reference",
                "timed": "the reference's per-atom energy/force arithmetic and its force/virial scatter; its "
                         "neighbour search is built before the timed region (this build's value includes its own)",
                "cpu_baseline": dict(info, value=v, unit="atom-evals/s"),
                "e2e": {"value": v, "unit": "atom-evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    from jse_gb300.nnap import NNAP
    torch.cuda.set_device(local)
    if args.only_ref_gpu:
        if rank == 0:
            print(json.dumps({"reference_gpu": ref_gpu_measurement(local, structures[0], model, args.precision,
                                                                   steps=args.steps)}))
        return
    if args.only_train:
        if rank == 0:
            print(json.dumps({"training": train_measurement(local, structures[0], model, steps=args.steps,
                                                             cpu=not args.no_cpu_baseline)}))
        return
    dev = torch.device("cuda", local)
    sm_count = _sm_count(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    bench_stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(bench_stream)
    pot = NNAP(model, precision=args.precision, device=local)
    pot.setAutotune(not args.no_autotune)  # shapes picked on the first warm-up step of each size bucket
    run = device_run(pot, structures, dev, flush, args.steps, args.warmup, clocks=ClockSampler(local), dist=dist)
    t_dev = max_over_ranks(sum(run["ms"]) / 1e3, dist)
    value = whole_job_rate(natoms_step, args.steps, world, t_dev)
    e2e = e2e_run(pot, run, dev, flush, args.steps)
    plain = plain_run(model, run, local, dev, flush, args.steps)
    plain["tuned_e2e_over_plain"] = e2e["value"] / plain["value"]
    plain["tuned_value_over_plain"] = value / plain["value"]
    mean_nei = mean_neighbours(pot, structures)
    roof = roofline(model, mean_nei, run["stages"], natoms_step, args.workload, sm_count)
    config["launch_shapes"] = pot.tuning(natoms_step)

    extras = rank == 0 and not args.no_extras
    liquid = None
    if extras and args.workload == "batch1024":  # the 32000-atom liquid of the same model, as an extra object
        ls, _ = make_workload("liquid32k")
        lm = bench_model("c2")
        with NNAP(lm, precision=args.precision, device=local) as lp:
            lp.setAutotune(not args.no_autotune)
            lr = device_run(lp, ls, dev, flush, args.steps, args.warmup)
            lv = ls[0].natoms * args.steps / (sum(lr["ms"]) / 1e3)
            le2e = e2e_run(lp, lr, dev, flush, args.steps)
            lroof = roofline(lm, mean_neighbours(lp, ls), lr["stages"], ls[0].natoms, "liquid32k", sm_count)
            liquid = {"value": lv, "unit": "atom-evals/s", "ms_per_step": sum(lr["ms"]) / args.steps,
                      "atoms": ls[0].natoms, "gpu_launches": lr["launches"], "e2e": le2e, "roofline": lroof,
                      "plain_gpu": plain_run(lm, lr, local, dev, flush, args.steps),
                      "launch_shapes": lp.tuning(ls[0].natoms)}
    else:
        ls = structures
    serving = training = ref_gpu = nep = None
    if extras and not args.no_serve and args.workload in ("batch1024", "liquid32k"):
        serving = serve_measurement(local, args.serve_requests)
    if extras and not args.no_train and args.workload in ("batch1024", "liquid32k"):
        training = train_measurement(local, ls[0], bench_model("c2"), cpu=not args.no_cpu_baseline)
    if extras and not args.no_ref_gpu and not args.no_cpu_baseline and args.workload in ("batch1024", "liquid32k"):
        ref_gpu = ref_gpu_measurement(local, ls[0], bench_model("c2"), args.precision)
    if extras and not args.no_nep and args.workload in ("batch1024", "liquid32k"):
        nep = nep_measurement(local, cpu=not args.no_cpu_baseline, autotune=not args.no_autotune)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            v_cpu, info = cpu_reference(structures, model, budget_s=10.0)
            cpu = dict(info, value=v_cpu, unit="atom-evals/s")
        except Exception as ex:  # the baseline is reported, never required
            cpu = {"value": None, "unit": "atom-evals/s", "error": str(ex)[:200]}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "atom-evals/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.precision == "fp32" else "bf16+f32",
                "data": "synthetic (seeded)", "config": config, "e2e": e2e, "roofline": roof, "cpu_baseline": cpu,
                "clocks": run["clocks"], "gpu_launches": run["launches"], "wall_s_timed": run["wall"],
                "plain_gpu": plain}
        for k, v in (("liquid32k", liquid), ("serving", serving), ("training", training), ("nep", nep),
                     ("reference_gpu", ref_gpu)):
            if v is not None:
                line[k] = v
        print(json.dumps(line))
    pot.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
