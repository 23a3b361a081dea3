"""The benchmark's JSON line: the reference arm (`bench.py --impl reference`, the FP64 oracle on
the host cores) runs here without a GPU and prints the keys the GPU arm prints, with the
reference arm's own; the roofline byte counts are the documented formulas."""
import json
import os
import subprocess
import sys

import bench
from fesom2_gb300 import mesh as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--config", "1", "--steps", "1",
                          "--warmup", "1"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["higher_is_better"] is True and d["value"] > 0 and d["steps"] == 1
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_roofline_byte_formulas():
    c = M.config_mesh(1).counts()
    N3, E3, T3 = c["N3"], c["E3"], c["T3"]
    assert bench.algorithmic_bytes(c, 24, 4) == 4 * (24 * (18 * N3 + 3 * E3) + 3 * T3 + 14 * N3)
    sb = bench.stage_bytes(c, 6, 4)
    # the bounds and update passes: 7 N3 + E3 per tracer, hnode_new and areasvol shared
    assert sb["bounds"] == sb["update"] == 4 * (6 * (5 * N3 + E3) + 2 * N3)
    assert set(bench.MEASURED_DRAM_B_PER_TRACER_DOF) <= set(sb)
    # the update with the vertical diffusion as its epilogue: no T* round trip, the factors read
    assert bench.algorithmic_bytes(c, 24, 4, vdiff_fused=True) == 4 * (24 * (16 * N3 + 3 * E3) + 3 * T3 + 14 * N3)
    sf = bench.stage_bytes(c, 6, 4, vdiff_fused=True)
    assert "vdiff" not in sf and sf["update"] == 4 * (6 * (5 * N3 + E3) + 6 * N3)
    assert sum(sf.values()) == sum(sb.values()) - 4 * 6 * 2 * N3


def test_node_order_choice_times_every_candidate(sphere_small, monkeypatch):
    """--order auto times the generators' order, reverse Cuthill-McKee and the Hilbert curve and
    keeps the fastest with its permutation; an explicit order is taken untimed (the trial stubbed:
    no GPU here)."""
    import numpy as np

    mesh = sphere_small
    f = M.make_forcing(mesh, "sphere", seed=3, dt=600.0)
    T = M.make_tracers(mesh, "sphere", ntr=2, seed=4, dtype=np.float32)
    seen = []

    def trial(m, forcing, tracers, dt, args, steps=2):
        seen.append((m.nod2D, tracers.shape))
        return {0: 10.0, 1: 12.0, 2: 9.0}[len(seen) - 1]

    monkeypatch.setattr(bench, "order_trial", trial)
    args = bench.argparse.Namespace(order="auto", no_tune=False, scale=1.0, profile_only=False, width=0)
    r = bench.choose_order(args, mesh, f, T, 600.0, 0)
    assert r["timed"] and set(r["ms_per_step"]) == {"morton", "rcm", "hilbert"} and r["chosen"] == "hilbert"
    assert len(seen) == 3 and all(s == (mesh.nod2D, T.shape) for s in seen)
    assert np.array_equal(np.sort(r["_order"]), np.arange(mesh.nod2D))
    args.order = "rcm"
    r = bench.choose_order(args, mesh, f, T, 600.0, 0)
    assert r["chosen"] == "rcm" and not r["timed"] and len(r["_order"]) == mesh.nod2D
    args.order, args.no_tune = "auto", True
    assert bench.choose_order(args, mesh, f, T, 600.0, 0) == {"chosen": "morton", "timed": False}
