"""The eight-wide quantized BVH on the CPU: tests/cpp/wide_check.cpp builds the binary SAH tree
and its eight-wide collapse with the library's own builder sources, then traces random rays
(from inside and around the scene, from vertices, along triangle planes, exactly axis-parallel) through the same
traversal code the kernels run (csrc/wide_trav.h, compiled for the host) and through brute force
over every triangle. Closest hits must have the brute-force distance bit for bit (and the same
triangle, or one at exactly that distance); any-hit answers must agree."""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from x3dcore2_gb300 import scene as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "x3dcore2_gb300", "csrc")


def cuda_include():
    for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "vector_types.h")):
            return os.path.join(d, "include")
    nvcc = shutil.which("nvcc")
    if nvcc:
        d = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
        if os.path.exists(os.path.join(d, "vector_types.h")):
            return d
    pytest.skip("CUDA headers (vector_types.h) not found")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    exe = tmp_path_factory.mktemp("wide") / "wide_check"
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-pthread", f"-I{CSRC}",
           f"-I{os.path.join(ROOT, 'include')}", f"-I{cuda_include()}",
           os.path.join(ROOT, "tests", "cpp", "wide_check.cpp"), os.path.join(CSRC, "bvh.cpp"),
           os.path.join(CSRC, "bvh_wide.cpp"), "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


def dump(sc, path):
    base = np.repeat(sc.voff[:-1], np.diff(sc.toff)).astype(np.uint64)
    tris = (sc.tris.astype(np.uint64) + base[:, None]).astype(np.uint32)
    with open(path, "wb") as f:
        f.write(np.array([len(sc.pos), len(tris)], np.uint32).tobytes())
        f.write(np.ascontiguousarray(sc.pos, np.float32).tobytes())
        f.write(np.ascontiguousarray(tris, np.uint32).tobytes())


SCENES = {
    "cornell": lambda: S.cornell(32, 32),
    "furnace": lambda: S.furnace(),
    "soup": lambda: S.soup(20000, seed=3, width=32, height=32),
    "icosphere": lambda: S.displaced_icosphere(level=5, seed=1, num_materials=8, width=32, height=32),
}


@pytest.mark.parametrize("name", list(SCENES))
def test_wide_traversal_matches_brute_force(checker, tmp_path, name):
    path = tmp_path / (name + ".bin")
    dump(SCENES[name](), path)
    r = subprocess.run([str(checker), str(path), "8000", "11"], capture_output=True, text=True, timeout=600)
    res = json.loads(r.stdout)
    assert r.returncode == 0, res
    assert res["ok"] == 1 and res["bad_t"] == 0 and res["bad_tri"] == 0 and res["bad_any"] == 0
    assert res["bad_levels"] == 0
    assert res["wide_depth"] <= 32
    # an eight-wide node replaces about three binary levels
    assert res["wide_nodes"] * 3 < res["binary_nodes"] or res["binary_nodes"] < 64


def test_grid_floor_ceil_is_exact(tmp_path):
    """The eight-wide quantization's plane arithmetic (single precision, TwoSum difference) gives
    the exact floor and ceiling of (v - org) / 2^e, checked with rational arithmetic on random
    planes, planes on grid lines, one ulp beside them, and subnormals beside large origins."""
    import ctypes as C
    import subprocess
    from fractions import Fraction
    lib_path = tmp_path / "gfc.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-o", str(lib_path),
                    f"-I{CSRC}", os.path.join(ROOT, "tests", "cpp", "grid_floor_ceil.cpp")], check=True)
    lib = C.CDLL(str(lib_path))
    rng = np.random.default_rng(5)
    n = 60000
    e = rng.integers(-40, 40, n)
    step = np.ldexp(np.float32(1), e).astype(np.float32)
    org = (rng.integers(-3000, 3000, n) * step * rng.choice([1, 3, 64], n)).astype(np.float32)
    k = rng.integers(0, 254, n)
    v = (org.astype(np.float64) + k * step.astype(np.float64)).astype(np.float32)
    kind = rng.integers(0, 5, n)
    v = np.where(kind == 1, np.nextafter(v, np.float32(-np.inf)), v)
    v = np.where(kind == 2, np.nextafter(v, np.float32(np.inf)), v)
    v = np.where(kind == 3, (v * rng.uniform(0.9, 1.1, n)).astype(np.float32), v)
    v = np.where(kind == 4, np.float32(1.4e-45) * rng.choice([-1, 1], n), v).astype(np.float32)
    inv = np.ldexp(np.float32(1), -e).astype(np.float32)
    fl = np.zeros(n, np.float32)
    cl = np.zeros(n, np.float32)
    f = np.ctypeslib.as_ctypes
    lib.grid_floor_ceil(f(v), f(org), f(inv), C.c_int(n), f(fl), f(cl))
    for i in range(n):
        q = (Fraction(float(v[i])) - Fraction(float(org[i]))) * Fraction(float(inv[i]))
        fq = q.numerator // q.denominator
        cq = -((-q.numerator) // q.denominator)
        assert (fl[i], cl[i]) == (fq, cq), (v[i], org[i], e[i], fl[i], cl[i], fq, cq)


def test_build_flags_keep_exact_float_arithmetic():
    """The device copy of the exact plane arithmetic (bvh_boxes.h) is compiled by nvcc; its
    exactness needs FMA contraction off, no flush-to-zero and IEEE division and square root. The
    build refuses flags that break that."""
    import pytest

    from x3dcore2_gb300 import build as B
    B.check_exact_flags()
    for extra in (["--use_fast_math"], ["-ftz=true"], ["--prec-div=false"]):
        with pytest.raises(RuntimeError):
            B.check_exact_flags(B.NVFLAGS + extra)
    with pytest.raises(RuntimeError):
        B.check_exact_flags([f for f in B.NVFLAGS if f != "--fmad=false"])
    with pytest.raises(RuntimeError):
        B.check_exact_flags(None, B.CXXFLAGS + ["-ffast-math"])
