"""Builds the in-tree native library x3dcore2_gb300/libe8g.so for sm_103a.

Host C++ (scene generators, packer, BVH builder) is compiled with g++; the CUDA translation
units with nvcc for compute_103a/sm_103a only. Float-sensitive code is built with FMA contraction
off (-ffp-contract=off on the host, --fmad=false on the device) so results follow the reference's
operation order. Objects are rebuilt only when a source or header changed.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libe8g.so")
# The bounds-checked debug build (-DE8G_CHECKS): device checks of every index a kernel reads
# through record the first failure in a check word that the host reads after each call.
BUILD_CHECKS = os.path.join(HERE, "_build_checks")
LIB_CHECKS = os.path.join(HERE, "libe8g_checks.so")
ROOT = os.path.dirname(HERE)

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
CXXFLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-pthread", "-Wall", "-Wextra",
            f"-I{os.path.join(ROOT, 'include')}"]
NVFLAGS = ["-std=c++17", "-O3", ARCH, "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
           "-Xptxas", "-warn-spills", f"-I{os.path.join(ROOT, 'include')}"]


# The exact single-precision arithmetic of the tree boxes (bvh_boxes.h: the TwoSum plane
# differences and power-of-two scalings that make device refits equal host builds byte for byte)
# and the reference's operation order in the bit-exact modes hold only without FMA contraction,
# without flush-to-zero and without approximate division or square root. Nothing in the device
# code can detect these flags, so the build refuses to run with them.
_FORBIDDEN_NVFLAGS = ("--use_fast_math", "-use_fast_math", "--ftz=true", "-ftz=true", "--prec-div=false",
                      "-prec-div=false", "--prec-sqrt=false", "-prec-sqrt=false", "--fmad=true", "-fmad=true")


def check_exact_flags(nvflags=None, cxxflags=None):
    """Raises if the flags would break the exact arithmetic the trees and bit-exact modes need."""
    nv = NVFLAGS if nvflags is None else nvflags
    cx = CXXFLAGS if cxxflags is None else cxxflags
    bad = [f for f in nv if f in _FORBIDDEN_NVFLAGS]
    if "--fmad=false" not in nv:
        bad.append("missing --fmad=false")
    if "-ffp-contract=off" not in cx or any(f in cx for f in ("-ffast-math", "-Ofast")):
        bad.append("host flags need -ffp-contract=off and no fast math")
    if bad:
        raise RuntimeError("build flags break exact float arithmetic: " + ", ".join(bad))


def _nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stderr


def build(verbose=False, jobs=None, checks=False):
    """Builds libe8g.so (or, with checks, the bounds-checked debug library libe8g_checks.so) and
    returns its path."""
    check_exact_flags()
    build_dir, lib = (BUILD_CHECKS, LIB_CHECKS) if checks else (BUILD, LIB)
    nvflags = NVFLAGS + (["-DE8G_CHECKS"] if checks else [])
    os.makedirs(build_dir, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        [os.path.join(ROOT, "include", "e8g.h")]
    nvcc = _nvcc()
    tasks = []
    objs = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cpp"))):
        obj = os.path.join(build_dir, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            tasks.append(["g++"] + CXXFLAGS + ["-c", src, "-o", obj])
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(build_dir, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            tasks.append([nvcc] + nvflags + ["-c", src, "-o", obj])
    if tasks:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(tasks), os.cpu_count() or 4)) as ex:
            for err in ex.map(_compile, tasks):
                if verbose and err:
                    sys.stderr.write(err)
    if tasks or not os.path.exists(lib):
        tmp = lib + ".tmp"
        _compile([nvcc, ARCH, "-shared", "-o", tmp] + objs + ["-lpthread"])
        os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    build(verbose=True)
    print(LIB)
