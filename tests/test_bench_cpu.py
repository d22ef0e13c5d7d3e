"""The bench's reference arm (the oracle port on the host cores, the CPU
baseline of the default order-9 N=800 workload) prints one JSON line that
keeps the bench contract: metric, value, unit, the same workload string as
the GPU arm, the CPU-baseline description and an e2e object with zero
copies; ms_per_step is the measured time of the sample it ran.  No GPU is
used (under a minute of host time)."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_prints_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "1"], capture_output=True, text=True,
                         timeout=900, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "R^k elements/s"
    sys.path.insert(0, ROOT)
    import bench
    assert d["config"]["workload"] == bench.workload_string(bench.LARGE)
    assert d["full_job_s_extrapolated"] > d["ms_per_step"] / 1e3
    assert d["value"] > 0 and d["ms_per_step"] > 0 and d["higher_is_better"] is True
    assert d["n_gpus"] == 1 and d["gpus_used"] == 0 and d["steps"] == 1
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
