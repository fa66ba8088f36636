"""Benchmark of the per-pixel path integral on one GB300 (or N, one process per GPU).

Workload (default): the large procedural scene — icosphere level 8 (1,310,720 triangles)
displaced by seeded 3-octave value noise (amplitude 0.05) on a 2-triangle ground plane with 4
quad area lights, 512 materials (albedo U[0.1,0.9]^3, roughness U[0.05,0.8], odd ones GGX metals
with F0 U[0.5,1)) — rendered at 1920x1080, 64 spp, max depth 8, Russian roulette from depth 3,
fp32, with the product estimator (next-event estimation + BSDF sampling, power-heuristic MIS,
Philox streams). A step is one full render of that frame.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line. `value` is paths/s over the device-resident render; `e2e` is the same
metric through the public C ABI call with the image read back to pinned host memory each step.
The reference arm (--impl reference) times the reference's own CPU tracer (pt_image_renderer with
unidirect_lt1, compiled from its unmodified sources with its release flags) on the host cores, on
the same scene and camera at a quarter of the resolution in each axis (pixels spread uniformly over
the frame); the scene comes from the stand-alone generator library, so that process never maps the
GPU library. Where the reference sources are absent it times the oracle's C restatement instead.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "paths/s at fixed relMSE, plain vs wavefront-batched; adjoint/forward time"
# The workload both arms name in `config` (identical dicts). What each arm computes per path is in
# its own top-level "estimator" object.
WORKLOAD = dict(workload="displaced_icosphere_l8_1080p_64spp", triangles=1310730, width=1920,
                height=1080, spp=64, materials=512, lights=4,
                l2="GPU arm: flushed between timed steps (256 MB write); host arm: not applicable")
GPU_ESTIMATOR = dict(name="nee+bsdf power-heuristic MIS (E8G_MODE_MIS)", max_depth=8, rr_start=3, rr_prob=0.5,
                     rng="philox4x32-10")
REF_ESTIMATOR = dict(name="unidirect_lt1 (the reference's direct-lighting tracer: NEE + BSDF continuation, no MIS)",
                     max_depth=None, rr_start=2, rr_prob=0.5, rng="minstd, one stream per thread",
                     note="the reference has no MIS tracer and no depth cap; its paths are shorter than the GPU "
                          "arm's (see the GPU line's like_for_like leg for the GPU on this estimator)")
# The host arms' sample of the frame: the same scene and camera at a quarter of the resolution in
# each axis, so its pixels are spread uniformly over the whole 1920x1080 view (sky included).
REF_SAMPLE_W, REF_SAMPLE_H = 480, 270
# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) from the ncu captures summarised in
# profiles/, one kernel per capture. Eight-wide tree + wavefront: one steady-state launch of each
# wavefront kernel in a tuned configuration of the benchmark (2^24 slots, 2 bounces per graph,
# threshold 8, shading shape 6; the headline launch list and the wavefront kernels' summaries
# under profiles/): 3.822 GB per trace launch and 5.76 GB per shading phase (completion kernel +
# shading kernel) at 16 launches for the frame's 192.3 M rays, kept as bytes per ray of the frame
# (318.0 and 479.2) and scaled to the run's own rays per launch, since the tuner may pick another
# slot pool. SAH pairs + megakernel: one 480x270, 8-spp launch of k_mega, 217.1 B per path (the
# megakernel's summary under profiles/), scaled by the frame's paths.
TRAFFIC = {("wide", "wavefront"): {"kernel_per_ray": 318.0, "shade_per_ray": 479.2},
           ("sah", "megakernel"): {"kernel_per_path": 217.1}}
INTEGRATORS = {"megakernel": 0, "wavefront": 1, "plain": 2}  # E8G_INTEGRATOR_*


def l2_read_peak(ctx):
    """The L2 read bandwidth of this GPU (GB/s, best of three) from the library's own streaming
    kernel over a 64 MiB buffer (e8g_l2_read_bandwidth)."""
    from x3dcore2_gb300 import abi
    lib = abi.load()
    best = 0.0
    for _ in range(3):
        v = C.c_double()
        abi.check(lib.e8g_l2_read_bandwidth(ctx.h, 64 << 20, 20, C.byref(v)), ctx.h, "e8g_l2_read_bandwidth")
        best = max(best, v.value)
    return best


def read_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    except OSError:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def make_scene(small):
    from x3dcore2_gb300 import scene as S
    if small:
        return S.displaced_icosphere(level=5, seed=1, num_materials=512, width=320, height=180), 320, 180, 8
    return (S.displaced_icosphere(level=8, seed=1, num_materials=512, width=1920, height=1080), 1920, 1080, 64)


def ref_scene_host(small):
    """The benchmark scene built by the stand-alone generator library (oracle/libe8scenegen.so, the
    same source as the GPU library's generators): the host arms never map the GPU library."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_bind as ob
    from x3dcore2_gb300 import scene as S
    g = ob.scenegen()
    if small:
        return S.displaced_icosphere(level=5, seed=1, num_materials=512, width=320, height=180, lib=g)
    return S.displaced_icosphere(level=8, seed=1, num_materials=512, width=1920, height=1080, lib=g)


def ref_tracer(scene):
    """(render(spp) -> (seconds, paths), kind, description) for the reference's CPU tracer on the
    host cores: the reference compiled from its own sources with its release flags
    (oracle/_ref/libe8ref_timing.so, pt_image_renderer::render with unidirect_lt1 and every host
    thread) when its sources are present, else the oracle's C restatement of the same estimator
    with the reference's policy (RR from depth 2, no depth cap)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_bind as ob
    from x3dcore2_gb300 import abi
    threads = os.cpu_count() or 1
    w, h = REF_SAMPLE_W, REF_SAMPLE_H
    if not os.path.exists(ob.REF_TIMING_LIB) and ob.reference_src() is not None:
        subprocess.run(["make", "-s", "-j2", "-C", ob.ORACLE_DIR, "ref"], check=True)
    if os.path.exists(ob.REF_TIMING_LIB):
        rs = ob.RefScene(scene, timing=True)

        def render(spp):
            _, secs, taken = rs.render(abi.MODE_REF_LT1, w, h, spp, threads)
            return secs, w * h * taken
        return render, "reference", threads, (
            f"{w}x{h} frame of the same scene and camera (pixels spread uniformly over the 1920x1080 view), "
            f"the reference's pt_image_renderer::render with unidirect_lt1, compiled from its unmodified sources "
            f"with -Ofast -flto native, {threads} threads")
    osc = ob.OracleScene(scene)

    def render_port(spp):
        t = time.perf_counter()
        osc.render(abi.MODE_REF_LT1, w, h, spp, seed=1, policy=ob.REF_POLICY, threads=threads)
        return time.perf_counter() - t, w * h * spp
    return render_port, "port", threads, (
        f"{w}x{h} frame of the same scene and camera (pixels spread uniformly over the 1920x1080 view), "
        f"unidirect_lt1 restated by the oracle (reference sources absent), {threads} threads")


def cpu_sample(scene, budget_s):
    """The reference's CPU tracer timed on the host cores over about budget_s seconds (see
    ref_tracer), plus the oracle's restatement on the same sample for a few seconds where the
    reference itself ran. Returns the cpu_baseline object."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_bind as ob
    from x3dcore2_gb300 import abi
    render, kind, threads, sample = ref_tracer(scene)
    spp = threads
    render(spp)  # warm-up (thread pool, page faults)
    secs = paths = 0
    while secs < budget_s:
        dt, n = render(spp)
        secs += dt
        paths += n
    out = {"value": paths / secs, "unit": "paths/s", "cores": threads, "kind": kind,
           "sample": f"{sample}; {paths} paths in {secs:.1f} s"}
    if kind == "reference":
        osc = ob.OracleScene(scene)
        t = time.perf_counter()
        n = 0
        while time.perf_counter() - t < min(budget_s, 6.0):
            osc.render(abi.MODE_REF_LT1, REF_SAMPLE_W, REF_SAMPLE_H, threads, seed=1 + n, policy=ob.REF_POLICY,
                       threads=threads)
            n += 1
        out["port_value"] = REF_SAMPLE_W * REF_SAMPLE_H * threads * n / (time.perf_counter() - t)
        out["port_note"] = "the oracle's C restatement of unidirect_lt1 on the same sample (-O2, no fast-math)"
    return out


def reference_commit_s(scene):
    """Seconds of the reference's own tree build (its path space's commit) for the benchmark scene,
    restated by the oracle on one thread."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_bind as ob
    t0 = time.time()
    ob.OracleScene(scene)
    return time.time() - t0


def like_for_like_leg(ctx, w, h, spp, d_img, stream):
    """The GPU on the host arm's estimator: E8G_MODE_REF_LT1 (unidirect_lt1 step for step, minstd
    streams) with the reference's own policy (Russian roulette from depth 2 at p = 0.5, no depth cap)
    over the whole benchmark frame, plain and megakernel (the wavefront runs MIS only) on both fast
    trees. Device time per frame, L2 flushed between frames. Leaves the SAH pairs built."""
    import torch
    from x3dcore2_gb300 import abi
    from x3dcore2_gb300.core import default_params
    p = default_params(abi.MODE_REF_LT1, w, h, spp, seed=1)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    out = {"mode": "E8G_MODE_REF_LT1", "policy": {"max_depth": p.max_depth, "rr_start": p.rr_start,
                                                  "rr_prob": p.rr_prob}, "width": w, "height": h, "spp": spp}
    best = 0.0
    for lay, code in (("wide", abi.BVH_WIDE), ("sah", abi.BVH_SAH)):
        ctx.build_bvh(layout=code)
        for integ in ("plain", "megakernel"):
            p.integrator = INTEGRATORS[integ]
            for _ in range(2):
                ctx.render_dev(p, d_img.data_ptr(), stream.cuda_stream)
            ms = []
            for _ in range(3):
                flush.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                ctx.render_dev(p, d_img.data_ptr(), stream.cuda_stream)
                b.record(stream)
                b.synchronize()
                ms.append(a.elapsed_time(b))
            v = w * h * spp / (statistics.mean(ms) / 1e3)
            out[f"{lay}/{integ}"] = {"ms": statistics.mean(ms), "paths_per_s": v}
            best = max(best, v)
    out["best_paths_per_s"] = best
    del flush
    return out


def quality_leg(ctx, p, img64, results):
    """relMSE of the timed frame against a 4096-spp reference of the same estimator rendered with
    independent streams (epsilon 1e-2 in the denominator). relMSE falls as 1/spp, so the spp that
    reaches relMSE 1e-3 and each integrator's time to get there follow from the paths/s: every
    integrator renders the same paths, so they reach it with the same spp."""
    import ctypes as C
    import numpy as np
    from x3dcore2_gb300 import abi
    q = abi.RenderParams.from_buffer_copy(p)
    q.spp, q.seed, q.sample_offset = 4096, 4242, 0
    q.integrator = abi.INTEGRATOR_MEGAKERNEL
    ref = ctx.render(q)[..., :3].astype(np.float64)
    img = img64[..., :3].astype(np.float64)
    rel = float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))
    spp_needed = p.spp * rel / 1e-3
    paths_needed = spp_needed * p.width * p.height
    return {"reference_spp": 4096, "relmse": rel, "relmse_spp": p.spp, "spp_for_relmse_1e-3": spp_needed,
            "seconds_to_relmse_1e-3": {f"{k[0]}/{k[1]}": paths_needed / r["paths_per_s"]
                                       for k, r in results.items()}}


def cornell_leg(ctx, threads, cpu_budget_s=6.0):
    """The small configuration: the Cornell room (two rotated boxes, a 0.25 x 0.25 ceiling light of
    radiance (17, 12, 4); 36 triangles) at 256x256, 16 spp, depth 5, SAH pairs. The reference's
    direct-lighting estimator (E8G_MODE_REF_LT1: unidirect_lt1 with the depth cap; the wavefront
    runs MIS only, so plain and megakernel) and MIS (the three integrators). Per estimator: GPU
    paths/s from the kernel time, relMSE of the 16-spp frame against a 4096-spp frame of the same
    estimator with independent streams (epsilon 1e-2), and the oracle's restatement of
    unidirect_lt1 on the host cores rendering the whole frame."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import numpy as np
    from x3dcore2_gb300 import abi
    from x3dcore2_gb300 import scene as S
    from x3dcore2_gb300.core import default_params
    w = h = 256
    spp = 16
    sc = S.cornell(w, h)
    ctx.upload(sc, layout=abi.BVH_SAH)
    out = {"width": w, "height": h, "spp": spp, "max_depth": 5, "triangles": int(sc.desc.mesh_tri_offset[sc.desc.num_meshes])}
    for name, mode, integs in (("ref_lt1", abi.MODE_REF_LT1, ("plain", "megakernel")),
                               ("mis", abi.MODE_MIS, ("plain", "megakernel", "wavefront"))):
        p = default_params(mode, w, h, spp, seed=1, max_depth=5)
        if mode == abi.MODE_REF_LT1:
            lt1 = p
        row = {}
        for integ in integs:
            p.integrator = INTEGRATORS[integ]
            for _ in range(3):
                ctx.render(p)
            ms = []
            for _ in range(20):
                img = ctx.render(p)
                ms.append(ctx.stats()["kernel_ms"])
            row[integ] = {"kernel_ms": statistics.mean(ms), "paths_per_s": w * h * spp / (statistics.mean(ms) / 1e3)}
        q = abi.RenderParams.from_buffer_copy(p)
        q.spp, q.seed, q.integrator = 4096, 4242, abi.INTEGRATOR_MEGAKERNEL
        ref = ctx.render(q)[..., :3].astype(np.float64)
        rel = float(np.mean((img[..., :3].astype(np.float64) - ref) ** 2 / (ref ** 2 + 1e-2)))
        row["relmse"] = rel
        row["spp_for_relmse_1e-3"] = spp * rel / 1e-3
        out[name] = row
    import oracle_bind as ob
    osc = ob.OracleScene(sc)
    pol = ob.OPolicy(lt1.max_depth, lt1.rr_start, lt1.rr_prob, 8)  # the GPU frame's depth cap and roulette
    n_spp, paths, secs = 1, 0, 0.0
    while secs < cpu_budget_s:
        t = time.time()
        osc.render(abi.MODE_REF_LT1, w, h, n_spp, seed=1, policy=pol, threads=threads)
        secs += time.time() - t
        paths += w * h * n_spp
        n_spp *= 2
    out["cpu_oracle"] = {"paths_per_s": paths / secs, "threads": threads, "kind": "port",
                         "sample": f"whole {w}x{h} frame, unidirect_lt1 restated (oracle), {paths // (w * h)} spp"}
    return out


def bdpt_leg(ctx, w=1280, h=720, spp=32):
    """Bidirectional MIS on the benchmark scene (still uploaded) at 1280x720, subpaths of at most 6
    vertices, 32 spp: power-heuristic weights (E8G_MODE_BDPT_POWER) one thread per path
    (`power`) and in the split form (`power_split`: a subpath kernel and a connection kernel per
    chunk of paths, E8G_INTEGRATOR_WAVEFRONT), and the reference's uniform weights
    (E8G_MODE_REF_BDPT). Per form the traversal roofline of its kernels: algorithmic bytes from
    the counted run (node bytes per node box fetched + 48 B per triangle tested) over the
    integrator's device time, against the measured HBM copy bandwidth."""
    from x3dcore2_gb300 import abi
    from x3dcore2_gb300.core import default_params
    peak, _ = read_peaks()
    st = ctx.bvh_stats()
    node_bytes = st["node_bytes"] // max(st["num_nodes"], 1)
    out = {"width": w, "height": h, "spp": spp, "max_subpath": 6, "node_bytes": node_bytes,
           "tree": {0: "sah", 1: "reference", 2: "wide", 3: "linear"}.get(st.get("layout", -1), "?")}
    for name, mode, kern, integ in (("power", abi.MODE_BDPT_POWER, "k_bdpt_power", abi.INTEGRATOR_MEGAKERNEL),
                                    ("power_split", abi.MODE_BDPT_POWER, "k_bdw_walk + k_bdw_eval + trace kernels",
                                     abi.INTEGRATOR_WAVEFRONT),
                                    ("uniform", abi.MODE_REF_BDPT, "k_bdpt_ref", abi.INTEGRATOR_MEGAKERNEL)):
        p = default_params(mode, w, h, spp, seed=1, bdpt_max_len=6)
        p.integrator = integ
        ctx.render(p)
        ms = []
        for _ in range(2):
            ctx.render(p)
            ms.append(ctx.stats()["kernel_ms"])
        kms = statistics.mean(ms)
        c = ctx.count_traversal(p)
        alg = node_bytes * c["nodes"] + 48 * c["tris"]
        out[name] = {"kernel_ms": kms, "paths_per_s": w * h * spp / (kms / 1000.0),
                     "roofline": {"kernel": kern, "rays": c["rays"], "nodes": c["nodes"], "tris": c["tris"],
                                  "algorithmic_bytes": alg, "achieved_gbs": alg / (kms / 1e3) / 1e9,
                                  "frac": alg / (kms / 1e3) / 1e9 / peak}}
    return out


def batch_leg(ctx, seed=1):
    """64 independent scenes in one call: seeded random soups in an enclosing box, triangles
    log-uniform in [1k, 500k], resolution from {128, 256, 512, 1024}^2, spp from {4, 16, 64}, max
    depth 4-10, GGX roughness U[0.02, 1]. The many-scene wavefront (eight-wide trees, shared
    slots, graph-captured bounce loop) and the many-scene megakernel (SAH pairs, one persistent
    launch), against rendering the 64 scenes one call at a time (device time of each call)."""
    import numpy as np
    from x3dcore2_gb300 import abi
    from x3dcore2_gb300 import scene as S
    from x3dcore2_gb300.core import default_params, render_batch
    rng = np.random.default_rng(seed)
    scenes, params = [], []
    for k in range(64):
        ntri = int(np.exp(rng.uniform(np.log(1000), np.log(500000))))
        res = int(rng.choice([128, 256, 512, 1024]))
        spp = int(rng.choice([4, 16, 64]))
        depth = int(rng.integers(4, 11))
        scenes.append(S.soup(ntri, seed=1000 + k, width=res, height=res, roughness_lo=0.02, roughness_hi=1.0))
        params.append(default_params(abi.MODE_MIS, res, res, spp, seed=k + 1, max_depth=depth, rr_start=3))
    paths = sum(p.width * p.height * p.spp for p in params)
    out = {"scenes": 64, "paths": paths, "triangles": int(sum(s.num_tris for s in scenes))}
    for name, integ in (("wavefront", abi.INTEGRATOR_WAVEFRONT), ("megakernel", abi.INTEGRATOR_MEGAKERNEL)):
        for p in params:
            p.integrator = integ
        render_batch(ctx, scenes, params)  # warm-up
        _, st = render_batch(ctx, scenes, params)
        out[name] = {"ms": st["ms"], "paths_per_s": paths / (st["ms"] / 1000.0), "launches": st["launches"]}
    sep_ms = 0.0
    for sc, p in zip(scenes, params):
        p.integrator = abi.INTEGRATOR_MEGAKERNEL
        ctx.upload(sc)
        ctx.render(p)
        sep_ms += ctx.stats()["ms"]
    out["separate"] = {"ms": sep_ms, "paths_per_s": paths / (sep_ms / 1000.0),
                       "note": "one e8g_render per scene, SAH pairs, megakernel"}
    return out


def adjoint_leg(ctx):
    """Differentiable render: displaced icosphere level 7 (327,680 triangles), 256 materials,
    512x512, 32 spp, max depth 6; forward render vs path-replay backward of an L2 loss."""
    import numpy as np
    from x3dcore2_gb300 import abi
    from x3dcore2_gb300 import scene as S
    from x3dcore2_gb300.core import default_params
    sc = S.displaced_icosphere(level=7, seed=5, num_materials=256, width=512, height=512)
    ctx.upload(sc)
    p = default_params(abi.MODE_MIS, 512, 512, 32, seed=1, max_depth=6, rr_start=3)
    fwd, bwd = [], []
    dl = np.ones((512, 512, 3), np.float32)
    for k in range(4):
        ctx.forward(p)
        f = ctx.stats()["ms"]
        ctx.backward(dl)
        b = ctx.stats()["ms"]
        if k:
            fwd.append(f)
            bwd.append(b)
    return {"triangles": sc.num_tris, "materials": 256, "forward_ms": statistics.mean(fwd),
            "backward_ms": statistics.mean(bwd), "ratio": statistics.mean(bwd) / statistics.mean(fwd)}


def adjoint_fd_leg(ctx, spps=(1024, 4096, 16384)):
    """How the gap between the path-replay roughness gradient and central finite differences
    (h = 1e-3, common random numbers) shrinks with the sample count, on the differentiable
    configuration (level-7 displaced icosphere, 256 materials, 512x512, depth 6): the replayed
    gradient holds each sampled GGX direction fixed and differentiates the path's weight, the
    finite differences move the directions with the roughness, so the two agree in expectation
    and differ by sampling noise. The four largest roughness entries at the smallest count are
    followed at every count. Images for the differences are summed in float64 from 64-sample
    chunks of the same streams."""
    import numpy as np
    import torch
    from x3dcore2_gb300 import abi
    from x3dcore2_gb300 import scene as S
    from x3dcore2_gb300.core import default_params
    W = H = 512
    sc = S.displaced_icosphere(level=7, seed=5, num_materials=256, width=W, height=H)
    ctx.upload(sc)
    base = sc.material_list()
    rng = np.random.default_rng(3)
    pert = []
    for m in base:
        q = abi.Material.from_buffer_copy(m)
        if q.type in (abi.MAT_OREN_NAYAR, abi.MAT_COOK_TORR):
            q.albedo[:] = list(np.clip(np.array(list(m.albedo)) + rng.normal(0, 0.05, 3), 0.05, 0.95))
        if q.type == abi.MAT_COOK_TORR:
            q.roughness = float(np.clip(m.roughness + rng.normal(0, 0.05), 0.05, 1.0))
        pert.append(q)
    ctx.set_materials(pert)
    tgt = torch.from_numpy(ctx.render(default_params(abi.MODE_MIS, W, H, 64, seed=2, max_depth=6, rr_start=3))
                           [..., :3].astype(np.float64)).cuda()
    stream = torch.cuda.current_stream()
    buf = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")

    def image(mats, spp, chunk=64):
        ctx.set_materials(mats)
        q = default_params(abi.MODE_MIS, W, H, chunk, seed=1, max_depth=6, rr_start=3)
        acc = torch.zeros((H, W, 3), dtype=torch.float64, device="cuda")
        for k in range(spp // chunk):
            q.sample_offset = k * chunk
            ctx.render_dev(q, buf.data_ptr(), stream.cuda_stream)
            acc += buf[..., :3].double()
        return acc / (spp // chunk)

    metal = [m for m in range(len(base)) if base[m].type == abi.MAT_COOK_TORR]
    out, entries = {"h": 1e-3, "spp": {}}, None
    for spp in spps:
        t0 = time.time()
        img = image(base, spp)
        ctx.set_materials(base)
        ctx.forward(default_params(abi.MODE_MIS, W, H, spp, seed=1, max_depth=6, rr_start=3))
        _, dr = ctx.backward((2 * (img - tgt)).float().cpu().numpy())
        if entries is None:
            entries = sorted(metal, key=lambda m: -abs(dr[m]))[:4]
        rows = []
        for m in entries:
            plus = [abi.Material.from_buffer_copy(x) for x in base]
            minus = [abi.Material.from_buffer_copy(x) for x in base]
            plus[m].roughness += 1e-3
            minus[m].roughness -= 1e-3
            lp = float(((image(plus, spp) - tgt) ** 2).sum())
            lm = float(((image(minus, spp) - tgt) ** 2).sum())
            fd = (lp - lm) / 2e-3
            rows.append({"material": m, "fd": fd, "adjoint": float(dr[m]), "rel_gap": abs(float(dr[m]) - fd) / abs(fd)})
        out["spp"][spp] = {"entries": rows, "max_rel_gap": max(r["rel_gap"] for r in rows),
                           "mean_rel_gap": sum(r["rel_gap"] for r in rows) / len(rows), "seconds": time.time() - t0}
    ctx.set_materials(base)
    return out


def update_leg(ctx, scene):
    """Incremental commit on the benchmark scene (the 1.3 M-triangle displaced icosphere): the
    big mesh rotated on the device (trimesh::transform) and the tree refitted, against a full host
    rebuild; new host vertices of that mesh uploaded (dirty-only) and refitted; and the frame rate
    after a refit and after a rebuild (a refitted tree traverses slower as geometry moves)."""
    import numpy as np
    from x3dcore2_gb300 import abi
    from x3dcore2_gb300.core import default_params
    big = int(np.argmax(np.diff(scene.toff)))
    v0, v1 = int(scene.voff[big]), int(scene.voff[big + 1])
    c, s = np.cos(0.2), np.sin(0.2)
    rot = np.array([[c, 0, s, 0], [0, 1, 0, 0], [-s, 0, c, 0], [0, 0, 0, 1]], np.float32)
    p = default_params(abi.MODE_MIS, 1920, 1080, 4, seed=3, max_depth=8, rr_start=3)
    nt, nv = scene.num_tris, len(scene.pos)
    out = {"triangles": nt, "vertices": nv, "mesh_vertices": v1 - v0}
    moved = (scene.pos[v0:v1] * np.float32(1.001)).astype(np.float32)
    for name, lay in (("sah", abi.BVH_SAH), ("wide", abi.BVH_WIDE)):
        ctx.upload(scene, layout=lay)
        st0 = ctx.bvh_stats()
        nn = st0["num_nodes"]
        xf_wall, refit_dev = [], []
        for k in range(6):
            t0 = time.perf_counter()
            ctx.transform_mesh(big, rot if k % 2 == 0 else np.eye(4, dtype=np.float32))
            st = ctx.commit(abi.COMMIT_REFIT)
            if k >= 2:
                xf_wall.append((time.perf_counter() - t0) * 1e3)
                refit_dev.append(st["build_ms"])
        up_wall = []
        for k in range(4):
            t0 = time.perf_counter()
            ctx.update_mesh(big, moved if k % 2 == 0 else scene.pos[v0:v1])
            ctx.commit(abi.COMMIT_REFIT)
            if k >= 1:
                up_wall.append((time.perf_counter() - t0) * 1e3)
        ctx.transform_mesh(big, rot)
        ctx.commit(abi.COMMIT_REFIT)
        fr_refit = []
        for k in range(3):
            ctx.render(p)
            fr_refit.append(ctx.stats()["ms"])
        t0 = time.perf_counter()
        ctx.commit(abi.COMMIT_REBUILD)
        rebuild_wall = (time.perf_counter() - t0) * 1e3
        fr_rebuild = []
        for k in range(3):
            ctx.render(p)
            fr_rebuild.append(ctx.stats()["ms"])
        # the device builder: a rebuild from the device's vertices, and the frame on its tree
        ctx.upload(scene, layout=lay, builder=abi.BUILDER_DEVICE)
        dev_build = []
        for k in range(4):
            ctx.transform_mesh(big, rot if k % 2 == 0 else np.eye(4, dtype=np.float32))
            t0 = time.perf_counter()
            st = ctx.commit(abi.COMMIT_REBUILD)
            if k:
                dev_build.append((time.perf_counter() - t0) * 1e3)
        dev_layout = st["layout"]
        fr_dev = []
        for k in range(3):
            ctx.render(p)
            fr_dev.append(ctx.stats()["ms"])
        refit_ms = statistics.median(refit_dev)
        if lay == abi.BVH_SAH:  # per refit: triangle records, leaf walks, node boxes, vertex reduction
            alg = nt * (16 + 48 + 48) + nt * (4 + 16 + 48) + nn * 64 + (nn // 2) * 64 + nv * 16
        else:
            alg = nt * (16 + 48 + 48) + nt * (4 + 16 + 48) + nn * (96 + 32 + 8 * 32) + nv * 16
        paths = p.width * p.height * p.spp
        out[name] = {
            "nodes": nn, "host_build_ms": st0["build_ms"], "rebuild_commit_ms": rebuild_wall,
            "refit_device_ms": refit_ms, "transform_commit_wall_ms": statistics.median(xf_wall),
            "update_commit_wall_ms": statistics.median(up_wall),
            "refit_algorithmic_bytes": alg, "refit_gbs": alg / (refit_ms * 1e-3) / 1e9,
            "paths_per_s_after_refit": paths / (statistics.median(fr_refit) * 1e-3),
            "paths_per_s_after_rebuild": paths / (statistics.median(fr_rebuild) * 1e-3),
            "device_rebuild_commit_ms": statistics.median(dev_build), "device_build_layout": dev_layout,
            "paths_per_s_device_tree": paths / (statistics.median(fr_dev) * 1e-3),
        }
    ctx.upload(scene)
    return out


def obj_leg():
    """OBJ ingest: a displaced icosphere of level 7 (327,680 triangles) written as OBJ text with
    v/vt/vn/f lines and read back with the reference loader's rules (e8g_obj_parse)."""
    import numpy as np
    from x3dcore2_gb300 import scene as S
    sc = S.displaced_icosphere(level=7, seed=5, num_materials=4, width=64, height=64)
    big = int(np.argmax(np.diff(sc.toff)))
    pos = sc.pos[sc.voff[big]:sc.voff[big + 1]]
    nrm = sc.nrm[sc.voff[big]:sc.voff[big + 1]]
    tri = sc.tris[sc.toff[big]:sc.toff[big + 1]].astype(np.int64) + 1
    lines = ["v %.6f %.6f %.6f" % tuple(v) for v in pos.tolist()]
    lines += ["vn %.6f %.6f %.6f" % tuple(v) for v in nrm.tolist()]
    lines.append("vt 0 0")
    lines += ["f %d/1/%d %d/1/%d %d/1/%d" % (a, a, b, b, c, c) for a, b, c in tri.tolist()]
    text = ("\n".join(lines) + "\n").encode()
    ms = []
    for _ in range(3):
        t0 = time.perf_counter()
        m = S.load_obj(text=text)
        ms.append((time.perf_counter() - t0) * 1e3)
    assert len(m.tris) == len(tri)
    best = min(ms)
    return {"triangles": len(tri), "vertices": len(pos), "bytes": len(text), "ms": best,
            "mb_per_s": len(text) / (best * 1e-3) / 1e6, "threads": 1}


def run_leg(args):
    """One extra leg alone (for profiling it): prints {"leg": name, ...}."""
    from x3dcore2_gb300.core import Context
    if args.leg == "obj":
        print(json.dumps({"leg": "obj", **obj_leg()}))
        return
    from x3dcore2_gb300 import abi
    ctx = Context(0)
    scene, _, _, _ = make_scene(args.small)
    LAYOUTS = {"sah": abi.BVH_SAH, "wide": abi.BVH_WIDE, "reference": abi.BVH_REFERENCE}
    ctx.upload(scene, layout=LAYOUTS[args.layout] if args.layout else abi.BVH_SAH)
    bw, bh = (int(x) for x in args.res.lower().split("x")) if args.res else (1280, 720)
    fn = {"bdpt": lambda: bdpt_leg(ctx, bw, bh, args.spp or 32), "batch": lambda: batch_leg(ctx), "adjoint": lambda: adjoint_leg(ctx),
          "update": lambda: update_leg(ctx, scene), "adjoint_fd": lambda: adjoint_fd_leg(ctx),
          "cornell": lambda: cornell_leg(ctx, os.cpu_count() or 1)}[args.leg]
    print(json.dumps({"leg": args.leg, **fn()}))
    ctx.close()


def mapped_repo_libraries():
    """The shared libraries of this working tree mapped into this process (Linux /proc)."""
    try:
        with open("/proc/self/maps") as f:
            paths = {ln.split()[-1] for ln in f if ln.rstrip().endswith(".so")}
    except OSError:
        return None
    return sorted(os.path.relpath(x, ROOT) for x in paths if x.startswith(ROOT + os.sep))


def run_reference_arm(args):
    """The reference's own CPU tracer on the host cores (see ref_tracer): one step renders the
    host sample of the frame at two samples per host thread. Never maps the GPU library."""
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_bind as ob
    subprocess.run(["make", "-s", "-C", ob.ORACLE_DIR, "all", "gen"], check=True)
    scene = ref_scene_host(args.small)
    render, kind, threads, sample = ref_tracer(scene)
    spp = 2 * threads  # about 0.75 s of the reference per step on 16 Grace cores
    for _ in range(args.warmup):
        render(spp)
    secs = paths = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        dt, n = render(spp)
        secs += dt
        paths += n
    wall = time.perf_counter() - t0
    v = paths / secs
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "paths/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs * 1000 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded procedural scene)", "config": dict(WORKLOAD),
            "estimator": REF_ESTIMATOR,
            "cpu_baseline": {"value": v, "unit": "paths/s", "cores": threads, "kind": kind,
                             "sample": f"{sample}; {paths // args.steps} paths per step, {secs:.1f} s timed "
                                       f"({wall:.1f} s wall)"},
            "e2e": {"value": v, "unit": "paths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "mapped_repo_libraries": mapped_repo_libraries()}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="e8g")
    ap.add_argument("--integrator", default="all", choices=["plain", "megakernel", "wavefront", "all"],
                    help="plain: one thread per path (the baseline kernel); all: time the three")
    ap.add_argument("--small", action="store_true", help="reduced scene for quick checks (not a bench line)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--res", default=None, help="WxH override, e.g. 480x270 (profiling a smaller launch)")
    ap.add_argument("--spp", type=int, default=None, help="spp override (profiling)")
    ap.add_argument("--layout", default=None, choices=["sah", "wide", "reference"],
                    help="BVH layout (default: the library's default)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the quality, BDPT, batch and adjoint legs")
    ap.add_argument("--no-tune", action="store_true", help="wavefront with the library defaults (profiling)")
    ap.add_argument("--wf-config", default=None,
                    help="CAPACITY,BOUNCES,THRESHOLD[,SHADE]: a fixed wavefront configuration (and shading "
                         "shape) instead of tuning (profiling)")
    ap.add_argument("--leg", default=None, choices=["bdpt", "batch", "adjoint", "adjoint_fd", "update", "obj", "cornell"],
                    help="run one extra leg alone on the benchmark scene and print its JSON (not a bench line)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.leg:
        return run_leg(args)
    if args.warmup < 3:
        args.warmup = 3

    import numpy as np
    import torch
    from x3dcore2_gb300 import abi
    from x3dcore2_gb300.core import Context, default_params

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    integrators = ["plain", "megakernel", "wavefront"] if args.integrator == "all" else [args.integrator]
    scene, w, h, spp = make_scene(args.small)
    if args.res:
        w, h = (int(x) for x in args.res.lower().split("x"))
        scene.camera.aspect = w / h
        scene.desc.camera = scene.camera
    if args.spp:
        spp = args.spp
    ctx = Context(local)
    LAYOUTS = {"sah": abi.BVH_SAH, "wide": abi.BVH_WIDE, "reference": abi.BVH_REFERENCE}
    layouts = [args.layout] if args.layout else ["sah", "wide"]
    ctx.upload(scene, build=False)
    p = default_params(abi.MODE_MIS, w, h, spp, seed=1, max_depth=8, rr_start=3, rr_prob=0.5,
                       sample_offset=rank * spp)
    stream = torch.cuda.current_stream()
    d_img = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # > 129 MB L2
    h_img = torch.empty((h, w, 4), dtype=torch.float32, pin_memory=True)
    lib = abi.load()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def build(lay):
        t0 = time.time()
        ctx.build_bvh(layout=LAYOUTS[lay])
        return time.time() - t0

    def tune_wavefront():
        r = abi.TuneResult()
        pw = default_params(abi.MODE_MIS, w, h, spp, seed=1, max_depth=8, rr_start=3, rr_prob=0.5)
        abi.check(lib.e8g_wavefront_tune(ctx.h, C.byref(pw), C.byref(r)), ctx.h, "e8g_wavefront_tune")
        return {"capacity": r.capacity, "bounces_per_graph": r.bounces_per_graph, "threshold": r.threshold,
                "shade_variant": r.shade_variant, "shade_ms": [round(r.shade_ms[i], 3) for i in range(r.num_shade)],
                "concurrent": r.concurrent, "concurrent_ms": [round(r.concurrent_ms[0], 3), round(r.concurrent_ms[1], 3)],
                "candidates": [[r.cand_capacity[i], r.cand_bounces[i], r.cand_threshold[i], round(r.cand_ms[i], 3)]
                               for i in range(r.num_candidates)]}

    results, tunes, trees = {}, {}, {}
    # the wavefront records CUDA events around its trace and shading kernels in every bounce graph
    # (the per-kernel times of the roofline); the other integrators run one kernel each
    ctx.set_kernel_timing(True)
    clocks = ClockSampler(local)
    clocks.start()
    for lay in layouts:
        commit_s = build(lay)
        st = ctx.bvh_stats()
        trees[lay] = {"nodes": st["num_nodes"], "node_bytes": st["node_bytes"], "depth": st["max_depth"],
                      "build_s": round(commit_s, 3)}
        if "wavefront" in integrators and args.wf_config:
            cfg = [int(x) for x in args.wf_config.split(",")]
            abi.check(lib.e8g_wavefront_set(ctx.h, cfg[0], cfg[1], cfg[2]), ctx.h, "e8g_wavefront_set")
            if len(cfg) > 3:
                abi.check(lib.e8g_wavefront_set_shade(ctx.h, cfg[3]), ctx.h, "e8g_wavefront_set_shade")
        elif "wavefront" in integrators and not args.no_tune:
            tunes[lay] = tune_wavefront()
        for integ in integrators:
            p.integrator = INTEGRATORS[integ]
            for _ in range(args.warmup):
                ctx.render_dev(p, d_img.data_ptr(), stream.cuda_stream)
            barrier()
            starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
            ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
            kernel_ms, launches, trace_ms, shade_ms, trace_launches = [], 0, [], [], 0
            for k in range(args.steps):
                flush.zero_()  # L2 flush between timed steps (outside the event pair)
                starts[k].record(stream)
                ctx.render_dev(p, d_img.data_ptr(), stream.cuda_stream)
                ends[k].record(stream)
                st = ctx.stats()
                kernel_ms.append(st["kernel_ms"])
                trace_ms.append(st["trace_ms"])
                shade_ms.append(st["shade_ms"])
                trace_launches += st["trace_launches"]
                launches += st["launches"]
            barrier()
            total_ms = sum(s_.elapsed_time(e_) for s_, e_ in zip(starts, ends))
            if world > 1:
                t = torch.tensor([total_ms], device="cuda")
                torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
                total_ms = float(t.item())
            results[(lay, integ)] = dict(ms_per_step=total_ms / args.steps, kernel_ms=statistics.mean(kernel_ms),
                                         launches=launches)
            if integ == "wavefront":
                results[(lay, integ)].update(trace_ms=statistics.mean(trace_ms), shade_ms=statistics.mean(shade_ms),
                                             trace_launches_per_step=trace_launches / args.steps)
    clk = clocks.stop()
    paths_per_step = w * h * spp
    for r in results.values():
        r["paths_per_s"] = paths_per_step * world / (r["ms_per_step"] / 1000.0)
    best = max(results, key=lambda k: results[k]["paths_per_s"])
    best_lay, best_integ = best
    value = results[best]["paths_per_s"]
    ms_per_step = results[best]["ms_per_step"]
    launches = results[best]["launches"]
    img64 = d_img.cpu().numpy()  # the last timed frame (every combination renders the same paths)
    if best_lay != layouts[-1]:  # back to the best tree (and its wavefront tuning)
        build(best_lay)
        if best_integ == "wavefront" and not args.no_tune and not args.wf_config:
            tunes[best_lay] = tune_wavefront()
    bvh = ctx.bvh_stats()
    p.integrator = INTEGRATORS[best_integ]

    # traversal counts for the roofline: instrumented megakernel run on the same tree (the same
    # paths, rays and node visits as every integrator)
    pc = default_params(abi.MODE_MIS, w, h, spp, seed=1, max_depth=8, rr_start=3, rr_prob=0.5)
    counts = ctx.count_traversal(pc)

    # end to end through the public call: host buffer, image read back every step (two untimed
    # calls first: the calls before them rendered other configurations)
    e2e_ms = []
    for k in range(0 if args.no_e2e else 2):
        abi.check(lib.e8g_render(ctx.h, C.byref(p), C.c_void_p(h_img.data_ptr())), ctx.h, "e8g_render")
    for k in range(0 if args.no_e2e else max(3, min(args.steps, 5))):
        barrier()
        t = time.perf_counter()
        abi.check(lib.e8g_render(ctx.h, C.byref(p), C.c_void_p(h_img.data_ptr())), ctx.h, "e8g_render")
        e2e_ms.append((time.perf_counter() - t) * 1000)
    if not e2e_ms:
        e2e_ms = [float("nan")]
    e2e_value = paths_per_step * world / (statistics.mean(e2e_ms) / 1000.0)

    peak, peak_kind = read_peaks()
    l2_peak = l2_read_peak(ctx)
    rb = results[best]
    loop_ms = rb["kernel_ms"]  # the integrator's whole device time per frame (first hits and resolve excluded)
    node_bytes = bvh["node_bytes"] // max(bvh["num_nodes"], 1)  # 32 (binary node) or 96 (wide node)
    alg_bytes = node_bytes * counts["nodes"] + 48 * counts["tris"]
    tr = TRAFFIC.get(best, {})
    if best_integ == "wavefront":
        # the dominant kernel is the trace kernel: every traversal byte is fetched there
        dom_ms, dom_launches = rb["trace_ms"], rb["trace_launches_per_step"]
        dom_name = ("k_wf_trace_wide_both (extension and shadow rays of a bounce, eight-wide tree)" if best_lay == "wide"
                    else "k_wf_trace_dyn (extension and shadow rays, SAH pairs)")
    else:
        dom_ms, dom_launches = loop_ms, 1
        dom_name = {"plain": "k_plain (baseline per-path kernel)", "megakernel": "k_mega (megakernel)"}[best_integ]
    achieved = alg_bytes / (dom_ms / 1000.0) / 1e9
    achieved_loop = alg_bytes / (loop_ms / 1000.0) / 1e9
    shade_traffic = None
    if "kernel_per_ray" in tr:
        traffic = tr["kernel_per_ray"] * counts["rays"] / dom_launches
        shade_traffic = tr["shade_per_ray"] * counts["rays"] / dom_launches
    elif "kernel_per_path" in tr:
        traffic = tr["kernel_per_path"] * paths_per_step / dom_launches
    else:
        traffic = None
    commit_s = trees[best_lay]["build_s"]

    line = {
        "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
        "config": dict(WORKLOAD),
        "estimator": GPU_ESTIMATOR,
        "detail": dict(integrator=best_integ, bvh_layout=best_lay,
                       integrators={f"{k[0]}/{k[1]}": {kk: (round(vv, 4) if isinstance(vv, float) else vv)
                                                       for kk, vv in r.items()} for k, r in results.items()},
                       trees=trees, wavefront_tune={k: {kk: v for kk, v in t.items() if kk != "candidates"}
                                                    for k, t in tunes.items()},
                       small=args.small, bvh_nodes=bvh["num_nodes"], bvh_build_ms=bvh["build_ms"],
                       commit_s=round(commit_s, 3)),
        "e2e": {"value": e2e_value, "unit": "paths/s", "ms_per_step": statistics.mean(e2e_ms),
                "h2d_bytes_per_step": C.sizeof(abi.RenderParams),
                "d2h_bytes_per_step": w * h * 16},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                     "kernel": dom_name, "kernel_ms_per_step": dom_ms, "launches_per_step": dom_launches,
                     "algorithmic_bytes_per_launch": alg_bytes / dom_launches,
                     "avg_launch_ms": dom_ms / dom_launches,
                     "l2_peak": l2_peak, "frac_l2": achieved / l2_peak if l2_peak else None,
                     "node_bytes": node_bytes, "algorithmic_bytes_per_step": alg_bytes, "rays": counts["rays"],
                     "nodes": counts["nodes"], "tris": counts["tris"],
                     "traffic_note": "DRAM bytes per launch of this kernel: the DRAM bytes per ray of steady-state "
                                     "launches captured with ncu in a tuned configuration (profiles/, one kernel, three "
                                     "launches) times this run's rays per launch"},
        "roofline_loop": {"achieved": achieved_loop, "unit": "GB/s", "frac": achieved_loop / peak,
                          "frac_l2": achieved_loop / l2_peak if l2_peak else None, "loop_ms_per_step": loop_ms,
                          "trace_ms_per_step": rb.get("trace_ms"), "shade_ms_per_step": rb.get("shade_ms"),
                          "shade_traffic_per_launch": shade_traffic,
                          "note": "the same algorithmic bytes over the integrator's whole device time per frame "
                                  "(shading included)"},
        "gpu_launches": launches,
        "clocks": clk,
    }
    if rank == 0 and not args.no_extras and world == 1:
        line["like_for_like"] = like_for_like_leg(ctx, w, h, spp, d_img, stream)
        build(best_lay)
        line["quality"] = quality_leg(ctx, p, img64, results)
        line["bdpt"] = bdpt_leg(ctx)
        line["batch"] = batch_leg(ctx)
        line["adjoint"] = adjoint_leg(ctx)
        line["update"] = update_leg(ctx, scene)
        line["obj_ingest"] = obj_leg()
        line["cornell"] = cornell_leg(ctx, os.cpu_count() or 1)
    if rank == 0 and not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_sample(scene, args.cpu_budget)
        if "update" in line:
            # the reference rebuilds its whole tree on every commit (pathspace.cpp:292-328)
            line["update"]["reference_commit_ms"] = {"value": reference_commit_s(scene) * 1e3, "kind": "port",
                                                     "threads": 1,
                                                     "note": "the reference's tree build restated (oracle), one thread"}
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
