"""The bounds-checked debug build (x3dcore2_gb300/libe8g_checks.so, compiled with -DE8G_CHECKS):
every index a kernel reads through — BVH nodes, triangle records, traversal stacks, vertices,
meshes, materials, lights, wavefront queue entries and slots — is checked on the device, and a
failed check records itself in a check word (nothing traps) that the host turns into
E8G_ERR_INTERNAL. Every integrator on every layout, the ray queries and both batch forms run
through the checked build without a failed check and give the normal build's images."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def run_with(library, out):
    env = dict(os.environ, E8G_LIBRARY=library)
    r = subprocess.run([sys.executable, os.path.join(HERE, "checks_run.py"), str(out)], env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    with open(out) as f:
        return json.load(f)


def test_checked_build_runs_clean_and_equals_the_normal_build(lib, tmp_path):
    from x3dcore2_gb300 import abi
    from x3dcore2_gb300 import build as B
    checked = B.build(checks=True)
    a = run_with(checked, tmp_path / "checked.json")
    b = run_with(abi.LIB_PATH, tmp_path / "normal.json")
    assert a["library"].endswith("libe8g_checks.so")
    bad = [c for c in a["calls"] if c[1] != "OK"]
    assert not bad, bad[:10]
    assert len(a["calls"]) > 100 and [c[0] for c in a["calls"]] == [c[0] for c in b["calls"]]
    for key, img in a["images"].items():
        x, y = np.asarray(img, np.float32), np.asarray(b["images"][key], np.float32)
        close = np.all(np.abs(x - y) <= np.maximum(1e-4 * np.abs(y), 1e-6), axis=-1)
        assert close.mean() >= 0.995, key
