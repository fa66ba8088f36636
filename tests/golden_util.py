"""Loads the golden fixtures (made by tests/golden/make_golden.py from the reference)."""
import os

import numpy as np

from x3dcore2_gb300 import abi
from x3dcore2_gb300.scene import Scene

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name)))


def scene_from(d):
    mats = []
    for row in d["mats"]:
        m = abi.Material()
        m.type = int(row[0])
        m.albedo[:] = [float(x) for x in row[1:4]]
        m.roughness, m.ior_re, m.ior_im = float(row[4]), float(row[5]), float(row[6])
        m.mix0, m.mix1 = int(row[7]), int(row[8])
        m.ratio = float(row[9])
        mats.append(m)
    lights = []
    for row in d["lights"]:
        l = abi.Light()
        l.mesh = int(row[0])
        l.radiance[:] = [float(x) for x in row[1:4]]
        lights.append(l)
    c = d["cam"]
    cam = abi.Camera()
    cam.origin[:] = [float(x) for x in c[0:3]]
    cam.rot[:] = [float(x) for x in c[3:12]]
    cam.sensor_size, cam.focal_len, cam.aspect = float(c[12]), float(c[13]), float(c[14])
    return Scene(d["voff"], d["toff"], d["mesh_mat"], d["pos"], d["nrm"], d["tris"], mats, lights, cam)
