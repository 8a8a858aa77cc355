"""bench.py pieces that need no GPU: the algorithmic counts behind the roofline, the
measured-traffic table, and the reference arm's JSON line (the reference's per-atom
arithmetic on the host cores)."""
import json
import os
import subprocess
import sys

from tests.conftest import ROOT

sys.path.insert(0, ROOT)


def test_stage_costs_are_positive_and_ordered():
    import bench
    from jse_gb300 import workloads as W
    costs = bench.stage_costs(W.model_for("c2"), 53.4)
    assert list(costs) == ["neighbours", "descriptors_fwd", "network", "descriptors_bwd", "scatter"]
    assert all(c["bytes"] > 0 for c in costs.values())
    # the descriptor stages carry the FLOPs; the backward more than the forward
    assert costs["descriptors_bwd"]["flops"] > costs["descriptors_fwd"]["flops"] > costs["network"]["flops"] > 0
    # the liquid's backward: algorithmic bytes per atom agree with its measured DRAM traffic
    traffic = bench.load_traffic()["liquid32k/descriptors_bwd"]
    assert 0.8 < traffic / costs["descriptors_bwd"]["bytes"] < 1.2


def test_reference_arm_line_and_mapped_libraries():
    """One JSON line with the reference arm's fields; and the arm's process maps only
    reference and oracle code, no shared library of the jse_gb300 package (its inputs come
    from the pure-numpy structure generator).  (Without an expanded reference the arm times
    the oracle port on a bounded sample.)"""
    code = ("import runpy, sys\n"
            "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '3', '--ref-seconds', '4']\n"
            "runpy.run_path('bench.py', run_name='__main__')\n"
            "maps = open('/proc/self/maps').read().split()\n"
            "print('MAPPED', sorted({m for m in maps if m.endswith('.so') or '.so.' in m}))\n")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 2 and lines[1].startswith("MAPPED")
    assert "jse_gb300" not in lines[1], lines[1]
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "NNAP E+F atom-evals/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 1 and d["warmup"] == 3
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["kind"] in ("reference", "port")
    assert d["config"]["workload"] == "batch1024" and "neighbour search" in d["timed"]
    if d["cpu_baseline"]["kind"] == "reference":
        assert d["cpu_baseline"]["single_thread"]["value"] > 0
