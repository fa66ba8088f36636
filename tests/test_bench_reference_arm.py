"""The benchmark's reference arm on the host cores (no GPU): `bench.py --impl reference` prints one
JSON line in the benchmark's contract, for the same metric, unit and workload as the GPU arm, timed
on the reference's own compiled tracer (or the oracle's restatement where the reference is not
built), and the process maps no GPU library of this repository."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


@pytest.fixture(scope="module")
def line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert lines, r.stdout[-2000:]
    return json.loads(lines[-1])


def test_reference_line_follows_the_contract(line):
    import bench
    if "unavailable" in line:
        pytest.skip(line["unavailable"])
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == "paths/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["steps"] == 1 and line["n_gpus"] == 1
    assert line["config"] == dict(bench.WORKLOAD)
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_maps_no_gpu_library(line):
    if "unavailable" in line:
        pytest.skip(line["unavailable"])
    libs = line.get("mapped_repo_libraries") or []
    assert not any(x.startswith("x3dcore2_gb300" + os.sep) for x in libs), libs
