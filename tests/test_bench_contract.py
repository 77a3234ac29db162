"""bench.py's reference arm runs on the host alone (the oracle port, or the
reference's own build where it exists). Its last stdout line must be one
compact JSON object with the keys of the benchmark line: metric, value (> 0),
unit, n_gpus, steps, warmup, ms_per_step, higher_is_better, scaling,
vs_baseline, dtype, data, config, cpu_baseline (value, unit, cores, kind,
sample), e2e (value, unit, host-device bytes) and impl = "reference"."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_prints_one_parseable_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--size", "64",
                        "--steps", "2", "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    last = r.stdout.strip().splitlines()[-1]
    assert len(last) < 1500
    line = json.loads(last)
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0 and line["steps"] == 2 and line["warmup"] == 3
    assert line["higher_is_better"] is True and line["unit"] == "GB/s"
    cb = line["cpu_baseline"]
    assert {"value", "unit", "cores", "kind", "sample"} <= set(cb) and cb["kind"] in ("reference", "port")
    e = line["e2e"]
    assert e["value"] == line["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
    assert "workload" in line["config"]
