"""Host-side input checks (e8g_scene_validate, the checks e8g_scene_upload runs before it touches
the GPU): non-finite positions, normals, camera, material and light values, and lights that emit
no power are refused with a reason. The reference throws or produces NaN images on such input; the
C ABI returns E8G_ERR_INVALID_ARG and never starts device work. CPU only."""
import ctypes as C

import numpy as np
import pytest

from x3dcore2_gb300 import abi
from x3dcore2_gb300 import scene as S


def validate(lib, sc):
    msg = C.create_string_buffer(256)
    st = lib.e8g_scene_validate(C.byref(sc.desc), msg, len(msg))
    return st, msg.value.decode()


def rebuilt(sc, pos=None, nrm=None, mats=None, lights=None, cam=None):
    return S.Scene(sc.voff, sc.toff, sc.mesh_mat, sc.pos if pos is None else pos, sc.nrm if nrm is None else nrm,
                   sc.tris, sc.material_list() if mats is None else mats,
                   list(sc.lights[:sc.num_lights]) if lights is None else lights,
                   sc.camera if cam is None else cam)


def test_valid_scene_passes(lib):
    assert validate(lib, S.cornell(32, 32)) == (abi.E8G_OK, "")


@pytest.mark.parametrize("what", ["pos_nan", "pos_inf", "nrm_nan"])
def test_non_finite_vertices_are_refused(lib, what):
    sc = S.cornell(32, 32)
    pos, nrm = sc.pos.copy(), sc.nrm.copy()
    if what == "pos_nan":
        pos[5, 1] = np.nan
    elif what == "pos_inf":
        pos[0, 0] = np.inf
    else:
        nrm[3, 2] = np.nan
    st, msg = validate(lib, rebuilt(sc, pos=pos, nrm=nrm))
    assert st == 1 and "finite" in msg


def test_bad_camera_material_and_light_values_are_refused(lib):
    sc = S.cornell(32, 32)
    cam = abi.Camera.from_buffer_copy(sc.camera)
    cam.origin[1] = float("nan")
    assert validate(lib, rebuilt(sc, cam=cam))[0] == 1
    cam = abi.Camera.from_buffer_copy(sc.camera)
    cam.focal_len = 0.0
    assert "positive" in validate(lib, rebuilt(sc, cam=cam))[1]
    mats = sc.material_list()
    mats[1] = abi.Material.from_buffer_copy(mats[1])
    mats[1].albedo[0] = float("inf")
    assert "material" in validate(lib, rebuilt(sc, mats=mats))[1]
    lights = [abi.Light.from_buffer_copy(l) for l in sc.lights[:sc.num_lights]]
    lights[0].radiance[1] = -1.0
    assert "radiance" in validate(lib, rebuilt(sc, lights=lights))[1]
    lights[0].radiance[:] = [0.0, 0.0, 0.0]
    assert "no power" in validate(lib, rebuilt(sc, lights=lights))[1]


def test_zero_area_light_is_refused(lib):
    sc = S.cornell(32, 32)
    light_mesh = sc.lights[0].mesh
    pos = sc.pos.copy()
    v0, v1 = sc.voff[light_mesh], sc.voff[light_mesh + 1]
    pos[v0:v1] = pos[v0]  # every vertex of the light at one point
    st, msg = validate(lib, rebuilt(sc, pos=pos))
    assert st == 1 and "no power" in msg
