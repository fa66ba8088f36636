"""The stand-alone scene generators (oracle/libe8scenegen.so), which the host-side timing of the
reference uses so that its process never maps the GPU library, produce the same scenes as the GPU
library's generators, byte for byte. CPU only."""
import numpy as np

import oracle_bind as ob
from x3dcore2_gb300 import abi
from x3dcore2_gb300 import scene as S


def _same(a, b):
    assert np.array_equal(a.voff, b.voff) and np.array_equal(a.toff, b.toff)
    assert np.array_equal(a.mesh_mat, b.mesh_mat)
    for x, y in ((a.pos, b.pos), (a.nrm, b.nrm)):
        assert np.array_equal(np.asarray(x).view(np.uint32), np.asarray(y).view(np.uint32))
    assert np.array_equal(a.tris, b.tris)
    assert bytes(a.desc.camera) == bytes(b.desc.camera)
    assert [bytes(m) for m in a.material_list()] == [bytes(m) for m in b.material_list()]
    assert [bytes(l) for l in a.lights[:a.num_lights]] == [bytes(l) for l in b.lights[:b.num_lights]]


def test_standalone_generators_equal_the_library_ones(lib):
    g = ob.scenegen()
    _same(S.displaced_icosphere(level=4, seed=1, num_materials=512, width=1920, height=1080, lib=g),
          S.displaced_icosphere(level=4, seed=1, num_materials=512, width=1920, height=1080))
    _same(S.cornell(256, 256, lib=g), S.cornell(256, 256))
    _same(S.soup(5000, seed=7, width=128, height=128, lib=g), S.soup(5000, seed=7, width=128, height=128))
    _same(S.generate(abi.GEN_FURNACE, level=12, lib=g), S.furnace(12))
