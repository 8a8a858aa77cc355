"""Host logic of the request loop (no GPU): FIFO admission under a budget, continuous
batching of requests that arrive while others run, and per-request accounting.  The
server is replaced by a fake with the same interface whose "energy" is a function of
the request's own positions only."""
import numpy as np

from jse_gb300.serve import GaussianMoves, Request, RequestLoop, poisson_requests
from jse_gb300.workloads import Structure


class FakeServer:
    def __init__(self, cap_atoms):
        self.cap = cap_atoms
        self.used = {}
        self.next = 0
        self.steps = []
        self.peak = 0

    def admit(self, s):
        n = len(s.types)
        if sum(self.used.values()) + n > self.cap:
            return None
        k = self.next
        self.next += 1
        self.used[k] = n
        self.peak = max(self.peak, sum(self.used.values()))
        return k

    def release(self, k):
        del self.used[k]

    def step(self, slots, xs, forces=False):
        assert len(set(slots)) == len(slots) and all(k in self.used for k in slots)
        self.steps.append(list(slots))
        x = np.concatenate(xs)
        return {"energy": np.array([float(np.sum(v)) for v in xs]), "forces": x.copy()}

    def submit(self, slots, xs, forces=False):
        # positions are staged: the loop moves them in place while the step runs
        assert getattr(self, "_out", None) is None, "one step in flight at a time"
        self._out = self.step(slots, [np.array(v, copy=True) for v in xs], forces)

    def collect(self):
        out, self._out = self._out, None
        return out


def _pool():
    rng = np.random.default_rng(0)
    out = []
    for n in (5, 17, 40):
        out.append(Structure(rng.uniform(0, 10, size=(n, 3)), np.ones(n, dtype=np.int32), np.eye(3) * 10.0, 0))
    return out


def test_every_request_completes_in_fifo_order_within_budget():
    reqs = poisson_requests(_pool(), 60, rate=2000.0, nsteps=5, seed=1)
    srv = FakeServer(cap_atoms=100)
    st = RequestLoop(srv, reqs, moves=GaussianMoves(0.01, seed=2, pool=1 << 12)).run()
    assert st["requests"] == 60 and all(r.done == 5 for r in reqs)
    assert srv.peak <= 100 and not srv.used
    admits = [r.t_admit for r in sorted(reqs, key=lambda r: r.t_arrival)]
    assert all(a <= b for a, b in zip(admits, admits[1:]))
    # continuous batching: some step mixes requests admitted at different times
    first_step = {}
    for k, slots in enumerate(srv.steps):
        for s in slots:
            first_step.setdefault(s, k)
    assert any(len({first_step[s] for s in slots}) > 1 for slots in srv.steps)
    assert st["request_p99_ms"] >= st["request_p50_ms"] > 0


def test_results_depend_only_on_the_request():
    pool = _pool()
    moves = GaussianMoves(0.01, seed=2, pool=1 << 12)
    alone = Request(7, pool[1], 6, 0.0)
    RequestLoop(FakeServer(1000), [alone], moves=moves, keep_results=True).run()
    mine = Request(7, pool[1], 6, 0.0005)
    others = poisson_requests(pool, 20, rate=5000.0, nsteps=4, seed=3)
    RequestLoop(FakeServer(60), others + [mine], moves=moves, keep_results=True).run()
    assert mine.energies == alone.energies
    assert all(np.array_equal(a, b) for a, b in zip(mine.forces, alone.forces))
