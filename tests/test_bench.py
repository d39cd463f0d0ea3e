"""bench.py's contract pieces that need no GPU: the reference arm's JSON line
(the CPU engine timed on a bounded sample of the workload), and the issue
roofline's arithmetic with the instruction count of the launch shape that ran.
"""
import json
import os
import subprocess
import sys

import pytest

from tests.conftest import ROOT

sys.path.insert(0, ROOT)
import bench  # noqa: E402

KEYS = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
        "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config")


def test_reference_arm_prints_one_contract_line(port):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "1", "--cpu-chains", "16"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in KEYS:
        assert k in d, k
    assert d["impl"] == "reference" and d["metric"] == "ministeps/s" and d["value"] > 0
    assert d["higher_is_better"] is True and d["config"]["chains_per_step"] == 16
    assert d["config"]["chains_full_workload"] == 4096
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("reference", "port") and cb["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": "ministeps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_issue_roofline_uses_the_count_of_the_shape_that_ran():
    clk = {"sm_mhz": 2000.0}
    steps, ms = 6_557_430, 72.0
    r1 = bench.period_roofline("c2", 200, 7, 8, steps, ms, 152, clk, specialised=True,
                               chains=4096, warps_per_chain=1)
    rate = steps / (ms / 1e3)
    assert r1["inst_per_ministep"] == bench.INST_PER_MINISTEP[("c2", True, 1)]
    assert r1["achieved"] == pytest.approx(rate * r1["inst_per_ministep"] / 1e9)
    assert r1["peak"] == pytest.approx(4 * 152 * 2000e6 / 1e9)
    assert r1["frac"] == pytest.approx(r1["achieved"] / r1["peak"])
    assert r1["traffic"] == bench.DRAM_BYTES_PER_LAUNCH[("c2", 4096)]
    assert r1["algorithmic"]["dram"]["GBps"] == pytest.approx(r1["traffic"] / (ms / 1e3) / 1e9)
    # a shape without a measured count reports no issue rate rather than a wrong one
    r8 = bench.period_roofline("c2", 200, 7, 8, steps, ms, 152, clk, specialised=True,
                               chains=4096, warps_per_chain=8)
    assert r8["achieved"] is None and r8["frac"] is None
    # the library kernel has no measured count or traffic
    rl = bench.period_roofline("c2", 200, 7, 8, steps, ms, 152, clk, specialised=False,
                               chains=4096, warps_per_chain=1)
    assert rl["achieved"] is None and rl["traffic"] is None
