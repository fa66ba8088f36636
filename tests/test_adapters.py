"""The reference-side adapters (x3dcore2_gb300/adapters/e8g_corelib.*) compile against corelib's
headers, and a scene built from corelib objects and packed through them is the scene the
reference renders: the oracle fed the packed description reproduces the reference's own
unidirect_lt1 and bidirect_mis radiance bit for bit. Needs the reference sources (not present on
the GPU host)."""
import os
import subprocess

import pytest

import oracle_bind as ob

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_adapters_pack_the_reference_scene(tmp_path, reference, oracle, lib):
    import platform
    if platform.machine() not in ("x86_64", "AMD64"):
        pytest.skip("bit-exact check is defined on the machine that built the reference")
    exe = tmp_path / "adapter_pack_check"
    src = os.path.join(ROOT, "tests", "cpp", "adapter_pack_check.cpp")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", src,
           os.path.join(ROOT, "x3dcore2_gb300", "adapters", "e8g_corelib.cpp"),
           f"-I{os.path.join(ROOT, 'include')}", f"-I{os.path.join(ROOT, 'x3dcore2_gb300', 'adapters')}",
           f"-I{ob.ORACLE_DIR}", f"-I{ob.reference_src()}", f"-I{os.path.join(ob.ORACLE_DIR, 'qt_stub')}",
           ob.REF_LIB, ob.ORACLE_LIB, os.path.join(ROOT, "x3dcore2_gb300", "libe8g.so"),
           f"-Wl,-rpath,{os.path.dirname(ob.REF_LIB)}:{ob.ORACLE_DIR}:{os.path.join(ROOT, 'x3dcore2_gb300')}",
           "-lpthread", "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("OK"), r.stdout + r.stderr


@pytest.mark.gpu
def test_adapters_render_on_the_gpu(tmp_path, reference, oracle, lib):
    """gpu_image_renderer::render and gpu_path_tracer::sample run on the GPU behind corelib's own
    interfaces (renderer.h:57-59, pathtracer.h:59-63): images equal e8g_render's and the oracle's,
    a frame after a mesh moved equals the oracle's image of the moved scene (the adapter uploads the
    mesh and refits), and per-path radiance equals the reference's own tracers. Builds against the
    reference headers (checkout or shipped copy) and links the reference compiled here."""
    exe = tmp_path / "adapter_gpu_check"
    src = os.path.join(ROOT, "tests", "cpp", "adapter_gpu_check.cpp")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", src,
           os.path.join(ROOT, "x3dcore2_gb300", "adapters", "e8g_corelib.cpp"),
           f"-I{os.path.join(ROOT, 'include')}", f"-I{os.path.join(ROOT, 'x3dcore2_gb300', 'adapters')}",
           f"-I{ob.ORACLE_DIR}", f"-I{ob.reference_src()}", f"-I{os.path.join(ob.ORACLE_DIR, 'qt_stub')}",
           ob.REF_LIB, ob.ORACLE_LIB, os.path.join(ROOT, "x3dcore2_gb300", "libe8g.so"),
           f"-Wl,-rpath,{os.path.dirname(ob.REF_LIB)}:{ob.ORACLE_DIR}:{os.path.join(ROOT, 'x3dcore2_gb300')}",
           "-lpthread", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0 and r.stdout.rstrip().endswith("OK"), r.stdout + r.stderr
