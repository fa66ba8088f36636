"""Wavefront OBJ ingest (e8g_obj_load / e8g_obj_parse) against the reference's own loader
(wavefront_obj::load_geometry, resource.cpp:137-255): golden fixtures made by the compiled
reference, and, where the reference sources exist, the live reference on seeded random files and
on the reference's own test data (testdata/cornellbox, loaded by tst_renderer.cpp:62-90).
Every array must match bit for bit; every file the reference rejects must be rejected."""
import os

import numpy as np
import pytest

import golden_util as G
import obj_cases as OC
import oracle_bind as ob
from x3dcore2_gb300 import scene as S
from x3dcore2_gb300.abi import E8GError

REF_TESTDATA = ob.reference_testdata("cornellbox")


def mine(text):
    try:
        return S.load_obj(text=text)
    except E8GError as e:
        return str(e)


def same_mesh(m, r):
    return (np.array_equal(m.pos.view(np.uint32), r["pos"].reshape(-1, 3).view(np.uint32))
            and np.array_equal(m.nrm.view(np.uint32), r["nrm"].reshape(-1, 3).view(np.uint32))
            and np.array_equal(m.uv.view(np.uint32), r["uv"].reshape(-1, 2).view(np.uint32))
            and np.array_equal(m.tris, r["tris"].reshape(-1, 3)))


def test_obj_loader_matches_reference_golden(lib):
    d = G.load("obj.npz")
    texts = OC.unpack_texts(d["text"], d["text_off"])
    pv = pt = 0
    for i, (name, text) in enumerate(zip(d["names"], texts)):
        got = mine(text)
        if not d["ok"][i]:
            assert isinstance(got, str), name
            continue
        nv, nt = int(d["nv"][i]), int(d["nt"][i])
        r = {"pos": d["pos"][3 * pv:3 * (pv + nv)], "nrm": d["nrm"][3 * pv:3 * (pv + nv)],
             "uv": d["uv"][2 * pv:2 * (pv + nv)], "tris": d["tris"][3 * pt:3 * (pt + nt)]}
        pv, pt = pv + nv, pt + nt
        assert not isinstance(got, str), (name, got)
        assert same_mesh(got, r), name


def test_obj_loader_refuses_what_the_reference_reads_out_of_bounds(lib):
    for name, text in OC.UNDEFINED_IN_REFERENCE.items():
        got = mine(text)
        assert isinstance(got, str) and "texcoord and normal" in got, name


def test_obj_load_from_file_equals_parse(lib, tmp_path):
    p = tmp_path / "quad.obj"
    p.write_bytes(OC.QUAD.encode())
    a, b = S.load_obj(path=p), S.load_obj(text=OC.QUAD)
    assert np.array_equal(a.pos, b.pos) and np.array_equal(a.tris, b.tris)
    with pytest.raises(E8GError, match="cannot open"):
        S.load_obj(path=tmp_path / "missing.obj")


def test_obj_loader_matches_live_reference_random(lib, reference, tmp_path):
    rng = np.random.default_rng(77)
    loaded = 0
    for k in range(400):
        text = OC.random_obj(rng, lines=int(rng.integers(4, 40)))
        got = mine(text)
        if isinstance(got, str) and "texcoord and normal" in got:
            continue  # undefined in the reference
        p = tmp_path / f"r{k}.obj"
        p.write_bytes(text.encode())
        r = ob.ref_obj_load(p, reference)
        assert isinstance(got, str) == isinstance(r, str), (k, got, r, text)
        if not isinstance(r, str):
            assert same_mesh(got, r), (k, text)
            loaded += 1
    assert loaded >= 40


@pytest.mark.skipif(REF_TESTDATA is None, reason="reference test data not on this machine")
def test_obj_loader_matches_live_reference_on_its_test_data(lib, reference):
    names = sorted(f for f in os.listdir(REF_TESTDATA) if f.endswith(".obj"))
    assert len(names) == 8
    for n in names:
        path = os.path.join(REF_TESTDATA, n)
        r = ob.ref_obj_load(path, reference)
        assert isinstance(r, dict), (n, r)
        assert same_mesh(S.load_obj(path=path), r), n
