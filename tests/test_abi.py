"""Host-side checks that need no GPU: the C ABI library loads and exports every function
include/e8g.h declares, the generators are deterministic and valid, host helpers agree with the
oracle."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import oracle_bind as ob
from x3dcore2_gb300 import abi
from x3dcore2_gb300 import scene as S

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "e8g.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(e8g_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 25
    raw = C.CDLL(abi.LIB_PATH)
    missing = [n for n in names if not hasattr(raw, n)]
    assert not missing, missing
    assert set(names) <= set(abi.SIGNATURES), set(names) - set(abi.SIGNATURES)


def test_version_and_defaults(lib):
    assert lib.e8g_version().startswith(b"e8g")
    p = abi.RenderParams()
    lib.e8g_default_params(C.byref(p), abi.MODE_REF_LT1, 64, 32, 4)
    assert (p.rr_start, p.rr_prob, p.max_depth, p.bdpt_max_len, p.rng) == (2, 0.5, 0, 8, abi.RNG_MINSTD)
    lib.e8g_default_params(C.byref(p), abi.MODE_MIS, 64, 32, 4)
    assert p.rng == abi.RNG_PHILOX


def test_path_seed_matches_oracle(lib, oracle):
    rng = np.random.default_rng(0)
    for _ in range(200):
        s, px, k = int(rng.integers(0, 2**63)), int(rng.integers(0, 2**31)), int(rng.integers(0, 2**20))
        assert lib.e8g_path_seed(s, px, k) == oracle.o_path_seed(s, px, k)


def test_create_without_device_reports_no_device(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert lib.e8g_create(C.byref(h), None) == 9  # E8G_ERR_NO_DEVICE
    assert not h.value


def test_null_arguments_are_rejected(lib):
    assert lib.e8g_create(None, None) == 1
    assert lib.e8g_destroy(None) == 1
    assert lib.e8g_gen_scene(None, None) == 1


@pytest.mark.parametrize("kind", [abi.GEN_CORNELL, abi.GEN_DISPLACED_ICO, abi.GEN_SOUP, abi.GEN_FURNACE])
def test_generators_are_deterministic_and_valid(lib, kind):
    kw = dict(level=2, num_tris=500, num_materials=8) if kind != abi.GEN_FURNACE else dict(level=12)
    a = S.generate(kind, seed=3, width=64, height=32, **kw)
    b = S.generate(kind, seed=3, width=64, height=32, **kw)
    assert np.array_equal(a.pos, b.pos) and np.array_equal(a.tris, b.tris)
    assert a.num_lights >= 1 and a.num_tris > 0
    # triangle indices are mesh-local and in range
    for m in range(len(a.mesh_mat)):
        nv = a.voff[m + 1] - a.voff[m]
        assert np.all(a.tris[a.toff[m]:a.toff[m + 1]] < nv)
    assert np.all(np.isfinite(a.pos)) and np.all(np.abs(np.linalg.norm(a.nrm, axis=1) - 1) < 1e-4)


def test_cornell_shape(lib):
    sc = S.cornell(256, 256)
    assert sc.num_tris == 36 and sc.num_lights == 1
    light_mesh = sc.lights[0].mesh
    tri = sc.world_triangles()[sc.toff[light_mesh]:sc.toff[light_mesh + 1]]
    areas = 0.5 * np.linalg.norm(np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0]), axis=1)
    assert np.allclose(areas, 0.25 * 0.25 / 2)  # equal-area light triangles


def test_icosphere_counts(lib):
    sc = S.displaced_icosphere(level=4, num_materials=32, width=64, height=36)
    assert sc.num_tris == 20 * 4**4 + 2 + 4 * 2


def test_invalid_generator_options(lib):
    o = abi.GenOpts(kind=99)
    h = C.c_void_p()
    assert lib.e8g_gen_scene(C.byref(o), C.byref(h)) == 1
    o = abi.GenOpts(kind=abi.GEN_DISPLACED_ICO, level=11)
    assert lib.e8g_gen_scene(C.byref(o), C.byref(h)) == 1


def test_furnace_generator_matches_reference_uv_sphere(lib):
    """The generator restates uv_sphere (geometry.cpp:162-241); the fixture holds the mesh the
    reference's own uv_sphere constructor made (r 10, res 30, flipped normals)."""
    import golden_util as G
    d = G.load("uv_sphere.npz")
    sc = S.furnace(30)
    assert np.array_equal(sc.tris, d["tris"])
    assert np.allclose(sc.pos, d["pos"], atol=1e-5) and np.allclose(sc.nrm, d["nrm"], atol=1e-6)
