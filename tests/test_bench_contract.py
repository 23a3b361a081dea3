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
