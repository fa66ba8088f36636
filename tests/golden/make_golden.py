"""Generates the golden fixtures in this directory from the reference itself.

Runs only where the reference sources exist (the oracle Makefile compiles them, unmodified, into
oracle/_ref/libe8ref.so). Every fixture stores its scene arrays too, so consumers never depend on
regenerating geometry bit for bit on another machine.

    python tests/golden/make_golden.py              # every fixture
    python tests/golden/make_golden.py renderer     # only the named ones
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from x3dcore2_gb300 import abi, scene as S  # noqa: E402
import oracle_bind as ob  # noqa: E402

MODES = {"uni": abi.MODE_REF_UNI, "lt1": abi.MODE_REF_LT1, "bdpt": abi.MODE_REF_BDPT,
         "direct": abi.MODE_REF_DIRECT, "normal": abi.MODE_NORMAL, "position": abi.MODE_POSITION,
         "lt2": abi.MODE_REF_LT2}


def scene_arrays(sc):
    mats = np.array([[m.type, *m.albedo, m.roughness, m.ior_re, m.ior_im, m.mix0, m.mix1, m.ratio]
                     for m in sc.material_list()], np.float64)
    lights = np.array([[sc.lights[i].mesh, *sc.lights[i].radiance] for i in range(sc.num_lights)],
                      np.float64)
    cam = np.array(list(sc.camera.origin) + list(sc.camera.rot) +
                   [sc.camera.sensor_size, sc.camera.focal_len, sc.camera.aspect], np.float32)
    return dict(voff=sc.voff, toff=sc.toff, mesh_mat=sc.mesh_mat, pos=sc.pos, nrm=sc.nrm, tris=sc.tris,
                mats=mats, lights=lights, cam=cam)


def paths_fixture(name, sc, w, h, npaths, seed, modes, rng_seed=0):
    ref = ob.RefScene(sc)
    rng = np.random.default_rng(rng_seed)
    px = rng.integers(0, w * h, npaths).astype(np.uint32)
    samples = np.arange(npaths, dtype=np.uint32)
    seeds = np.array([ob.oracle().o_path_seed(seed, int(p), int(k)) for p, k in zip(px, samples)], np.uint32)
    out = dict(scene_arrays(sc), width=np.uint32(w), height=np.uint32(h), seed=np.uint64(seed), pixels=px,
               samples=samples, seeds=seeds)
    for mname in modes:
        out["rad_" + mname] = ref.render_paths(MODES[mname], w, h, px, seeds)
    rays = ref.camera_rays(w, h)
    hits = ref.trace_closest(rays)
    out.update(rays=rays, hit_t=hits["t"], hit_mesh=hits["mesh"], hit_tri=hits["tri"],
               hit_normal=hits["normal"], hit_vertex=hits["vertex"])
    np.savez_compressed(os.path.join(HERE, name), **out)
    print(name, {k: v.shape for k, v in out.items() if hasattr(v, "shape")})


def mixture_scene():
    """The Cornell room with the reference's composite materials on its surfaces: a wall without a
    material (the fail-safe Lambert, material.cpp:54-76), mixtures (mat_mixture, :78-106) of a
    Lambert wall with a GGX metal and of that metal with a rough Oren-Nayar, and a plain metal
    box."""
    sc = S.cornell(64, 48)
    mats = sc.material_list() + [
        S.material(abi.MAT_COOK_TORR, (0.8, 0.7, 0.5), 0.3, (2.5, 0.0)),     # 4
        S.material(abi.MAT_OREN_NAYAR, (0.4, 0.6, 0.8), 0.2),                # 5
        S.material(abi.MAT_MIXTURE, mix=(4, 5), ratio=0.35),                 # 6
        S.material(abi.MAT_MIXTURE, mix=(0, 4), ratio=0.7),                  # 7
    ]
    mm = np.array(sc.mesh_mat, np.int32).copy()
    mm[1], mm[2], mm[5], mm[6] = -1, 7, 6, 4
    return S.Scene(sc.voff, sc.toff, mm, sc.pos, sc.nrm, sc.tris, mats, list(sc.lights[:sc.num_lights]),
                   sc.camera)


def bsdf_fixture():
    # tst_material.cpp:28-179: cook_torr(0.787, r 0.2/0.25, ior 2.93) and oren_nayar(sigma 0.078)
    mats = [S.material(abi.MAT_COOK_TORR, (0.787, 0.787, 0.787), 0.25, (2.93, 0.0)),
            S.material(abi.MAT_COOK_TORR, (0.787, 0.787, 0.787), 0.2, (2.93, 0.0)),
            S.material(abi.MAT_OREN_NAYAR, (0.725, 0.710, 0.680), 0.078),
            S.material(abi.MAT_MIXTURE, mix=(0, 2), ratio=0.3),
            S.material(abi.MAT_FAIL_SAFE)]
    sc = S.cornell(8, 8)
    sc = sc.with_materials(mats)
    ref = ob.RefScene(sc)
    n = np.array([0.0, 0.0, 1.0], np.float32)
    o = np.array([0.57735026, 0.57735026, 0.57735026], np.float32)  # (1,1,1).normalize()
    out = dict(scene_arrays(sc), n=n, o=o)
    for mi in range(len(mats)):
        d, p = ref.bsdf_sample(mi, 13, n, o, 1000)
        out[f"dirs_{mi}"] = d
        out[f"pdf_{mi}"] = p
        ev = np.array([ref.bsdf_eval(mi, n, o, dd) for dd in d[:200]], np.float32)
        out[f"eval_{mi}"] = ev
    # special-case vectors of tst_material.cpp:142-144
    i = np.array([0.983719, 0.0456052, 0.173832], np.float32)
    oo = np.array([0.687788, 0.361631, 0.629421], np.float32)
    nn = np.array([0.687654, 0.361558, 0.62961], np.float32)
    out["special"] = np.array([ref.bsdf_eval(mi, nn, oo, i) for mi in range(len(mats))], np.float32)
    out["special_vecs"] = np.stack([i, oo, nn])
    np.savez_compressed(os.path.join(HERE, "bsdf.npz"), **out)
    print("bsdf.npz")


def draws_fixture():
    r = ob.reference()
    seeds = [0, 1, 13, 12345, 2147483646, 4294967295]
    out = {}
    for s in seeds:
        a = np.zeros(64, np.float32)
        r.r_minstd_draws(s, 64, ob.ptr(a))
        out[f"seed_{s}"] = a
    np.savez_compressed(os.path.join(HERE, "draws.npz"), **out)
    print("draws.npz")


def uv_sphere_fixture():
    r = ob.reference()
    nt = r.r_uv_sphere(10.0, 30, 1, None, None, None)
    nv = (30 - 2) * 30 + 2
    pos = np.zeros((nv, 3), np.float32)
    nrm = np.zeros((nv, 3), np.float32)
    tris = np.zeros((nt, 3), np.uint32)
    r.r_uv_sphere(10.0, 30, 1, ob.ptr(pos), ob.ptr(nrm), ob.ptr(tris))
    np.savez_compressed(os.path.join(HERE, "uv_sphere.npz"), pos=pos, nrm=nrm, tris=tris)
    print("uv_sphere.npz")


def renderer_fixture():
    """pt_image_renderer::render with one thread (one sampling task, stream seed 33), with and
    without the firefly clamp, on the Cornell fixture's scene."""
    import golden_util as G
    sc = G.scene_from(G.load("cornell.npz"))
    ref = ob.RefScene(sc)
    w, h, spp = 64, 48, 4
    out = dict(scene_arrays(sc), width=np.uint32(w), height=np.uint32(h), spp=np.uint32(spp))
    for mname in ("lt1", "uni"):
        for ff in (0, 1):
            img, _, taken = ref.render(MODES[mname], w, h, spp, 1, firefly=bool(ff))
            assert taken == spp
            out[f"img_{mname}_ff{ff}"] = img
    np.savez_compressed(os.path.join(HERE, "renderer.npz"), **out)
    print("renderer.npz")


def composite_fixture():
    """The reference's compositors (compositor.cpp:29-98) on a seeded float image with negative,
    all-zero and above-one values: clamp and ACES, auto exposure and a fixed one."""
    rng = np.random.default_rng(3)
    img = np.abs(rng.lognormal(-1.0, 1.2, (37, 53, 4))).astype(np.float32)
    img[..., 3] = rng.uniform(0.0, 1.2, (37, 53)).astype(np.float32)
    img[0, 0] = 0.0
    img[1, 1, :3] = -0.3
    ref = ob.reference()
    out = {"image": img}
    for tm, tname in ((abi.TONEMAP_CLAMP, "clamp"), (abi.TONEMAP_ACES, "aces")):
        for auto in (True, False):
            out[f"{tname}_{'auto' if auto else 'fixed'}"] = ob.composite(img, tm, auto, 0.8, lib=ref)
    np.savez_compressed(os.path.join(HERE, "composite.npz"), **out)
    print("composite.npz")


def transform_matrices():
    """Row-major 4x4 matrices for trimesh::transform: identity, a rigid motion, scale with shear,
    a projective matrix (w != 1) and one whose |det| <= 1e-5 (the reference throws)."""
    rng = np.random.default_rng(21)
    c, s = np.cos(0.7), np.sin(0.7)
    rigid = np.array([[c, 0, s, 0.3], [0, 1, 0, -1.2], [-s, 0, c, 2.5], [0, 0, 0, 1]])
    shear = np.array([[1.7, 0.4, 0.0, -0.5], [0.1, 0.6, 0.3, 0.2], [0.0, -0.2, 2.2, 1.1], [0, 0, 0, 1]])
    proj = np.eye(4) + rng.normal(0, 0.2, (4, 4))
    tiny = np.diag([0.02, 0.02, 0.02, 1.0])
    return np.stack([np.eye(4), rigid, shear, proj, tiny]).astype(np.float32)


def transform_fixture():
    """trimesh::transform (geometry.cpp:76-87) by the compiled reference: positions and normals."""
    rng = np.random.default_rng(22)
    pos = rng.uniform(-3, 3, (64, 3)).astype(np.float32)
    nrm = rng.normal(0, 1, (64, 3))
    nrm = (nrm / np.linalg.norm(nrm, axis=1, keepdims=True)).astype(np.float32)
    mats = transform_matrices()
    ref = ob.reference()
    out = {"pos": pos, "nrm": nrm, "mats": mats, "ok": np.zeros(len(mats), np.int32),
           "pos_out": np.zeros((len(mats), 64, 3), np.float32), "nrm_out": np.zeros((len(mats), 64, 3), np.float32)}
    for k, m in enumerate(mats):
        r = ob.transform_mesh(m, pos, nrm, lib=ref)
        if r is not None:
            out["ok"][k] = 1
            out["pos_out"][k], out["nrm_out"][k] = r
    np.savez_compressed(os.path.join(HERE, "transform.npz"), **out)
    print("transform.npz")


def obj_fixture():
    """wavefront_obj::load_geometry (resource.cpp:137-255) by the compiled reference on the
    hand-written cases of obj_cases.py and 64 seeded random files: vertex, normal, texcoord and
    triangle arrays, or a failure flag where the reference throws."""
    import tempfile
    import obj_cases as OC
    names = list(OC.CASES)
    texts = [OC.CASES[n] for n in names]
    rng = np.random.default_rng(31)
    for k in range(64):
        names.append(f"random{k}")
        texts.append(OC.random_obj(rng))
    ref = ob.reference()
    ok = np.zeros(len(texts), np.int32)
    nv = np.zeros(len(texts), np.int64)
    nt = np.zeros(len(texts), np.int64)
    arrays = {"pos": [], "nrm": [], "uv": [], "tris": []}
    with tempfile.TemporaryDirectory() as d:
        for i, t in enumerate(texts):
            path = os.path.join(d, f"case{i}.obj")
            with open(path, "wb") as f:
                f.write(t.encode())
            r = ob.ref_obj_load(path, ref)
            if isinstance(r, dict):
                ok[i] = 1
                nv[i], nt[i] = len(r["pos"]), len(r["tris"])
                for k in arrays:
                    arrays[k].append(r[k].reshape(-1))
    data, off = OC.pack_texts(texts)
    out = {"names": np.array(names), "text": data, "text_off": off, "ok": ok, "nv": nv, "nt": nt}
    for k, v in arrays.items():
        out[k] = np.concatenate(v) if v else np.zeros(0)
    np.savez_compressed(os.path.join(HERE, "obj.npz"), **out)
    print("obj.npz", int(ok.sum()), "of", len(ok), "load")


def main(only=()):
    subprocess.run(["make", "-s", "-C", ob.ORACLE_DIR, "all", "ref"], check=True)
    all_modes = list(MODES)
    jobs = {
        "draws": draws_fixture,
        "uv_sphere": uv_sphere_fixture,
        "bsdf": bsdf_fixture,
        "cornell": lambda: paths_fixture("cornell.npz", S.cornell(64, 48), 64, 48, 512, 7, all_modes),
        "furnace": lambda: paths_fixture("furnace.npz", S.furnace(), 32, 32, 256, 11,
                                         ["uni", "lt1", "bdpt", "direct", "lt2"]),
        "ico": lambda: paths_fixture("ico.npz", S.displaced_icosphere(level=3, seed=5, num_materials=16,
                                                                      width=48, height=27),
                                     48, 27, 384, 3, ["uni", "lt1", "bdpt", "direct", "lt2"]),
        "soup": lambda: paths_fixture("soup.npz", S.soup(3000, seed=2, width=40, height=40), 40, 40, 256, 9,
                                      ["lt1", "bdpt", "direct", "lt2"]),
        "mixture": lambda: paths_fixture("mixture.npz", mixture_scene(), 64, 48, 768, 13, all_modes, rng_seed=4),
        "renderer": renderer_fixture,  # reads cornell.npz, so it runs after it
        "composite": composite_fixture,
        "transform": transform_fixture,
        "obj": obj_fixture,
    }
    for name, fn in jobs.items():
        if not only or name in only:
            fn()


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))
