"""bench.py's GPU arm at a small size, every leg on: one JSON line with the
contract's keys (metric, value, timing, the HBM roofline of the dominant
kernel, the CPU baseline, the end-to-end measure, the launch count, the
clock record) and the legs of the other configurations."""
import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_gpu_arm_prints_the_contract_line():
    cmd = [sys.executable, "bench.py", "--nx", "24", "--steps", "3", "--warmup", "3", "--config-cycles", "6",
           "--cpu-seconds", "1", "--ens-instances", "4", "--ens-cycles", "5", "--adj-nx", "8",
           "--adj-cycles", "4", "--adj-every", "2", "--adj-dirs", "1", "--c3-nx", "16", "--c3-cycles", "3"]
    out = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stderr[-3000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    d = json.loads(lines[0])
    for k in ("metric", "unit", "dtype", "data", "scaling"):
        assert isinstance(d[k], str), k
    assert d["n_gpus"] == 1 and d["steps"] == 3 and d["warmup"] == 3
    assert d["value"] > 0 and d["ms_per_step"] > 0 and d["higher_is_better"] is True
    assert d["vs_baseline"] is None and d["dtype"] == "f64"
    assert d["config"]["nx"] == 24 and d["config"]["elements"] == 24 ** 3
    r = d["roofline"]
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and r["peak"] > 0
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    assert d["fp64_roofline"]["step"]["frac"] > 0
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] > 0 and isinstance(cb["sample"], str)
    e2e = d["e2e"]
    assert e2e["unit"] == d["unit"] and 0 < e2e["value"]
    assert e2e["h2d_bytes_per_step"] > 0 and e2e["d2h_bytes_per_step"] > 0
    assert d["gpu_launches"] == 5 * d["steps"]
    assert "sm_mhz" in d["clocks"] and isinstance(d["clocks"]["reasons"], list)
    # the other configurations' legs
    assert d["ensemble"]["instances_completed_rank0"] == 4 and d["ensemble"]["problems_per_s"] > 0
    assert d["adjoint"]["adjoint_over_forward"] > 0
    assert d["c3_unbalanced_regions"]["with_region_reps"]["cycles"] == 3
    c1 = d["c1_to_stoptime"]["corrected_to_stoptime"]
    assert c1["cycles"] == 932 and c1["time"] == 1e-2
    assert c1["origin_energy"] == pytest.approx(2.025075e5, rel=1e-6)
    assert d["blocks"]["blocks"] == 8
