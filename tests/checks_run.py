"""Runs the workloads of the checked-build test through whichever library E8G_LIBRARY names and
prints one JSON line: the status of every call and the images, so that the test can compare the
bounds-checked build with the normal one. Run by tests/test_gpu_checks.py in a child process."""
import json
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from x3dcore2_gb300 import abi  # noqa: E402
from x3dcore2_gb300 import scene as S  # noqa: E402
from x3dcore2_gb300.core import Context, default_params, render_batch  # noqa: E402


def main(out_path):
    results = {"library": abi.LIB_PATH, "calls": [], "images": {}}
    scenes = {"cornell": S.cornell(64, 48), "soup": S.soup(20000, seed=3, width=64, height=48),
              "ico": S.displaced_icosphere(level=5, seed=2, num_materials=32, width=64, height=48)}
    modes = {"lt1": abi.MODE_REF_LT1, "uni": abi.MODE_REF_UNI, "mis": abi.MODE_MIS, "bdpt": abi.MODE_REF_BDPT,
             "bdpt_power": abi.MODE_BDPT_POWER, "lt2": abi.MODE_REF_LT2, "direct": abi.MODE_REF_DIRECT}
    layouts = {"sah": abi.BVH_SAH, "wide": abi.BVH_WIDE, "reference": abi.BVH_REFERENCE, "linear": abi.BVH_LINEAR}
    with Context(0) as ctx:
        for sname, sc in scenes.items():
            for lname, lay in layouts.items():
                if lname == "linear" and sname != "cornell":
                    continue
                ctx.upload(sc, layout=lay)
                for mname, mode in modes.items():
                    integs = [abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_PLAIN]
                    if mode == abi.MODE_MIS:
                        integs.append(abi.INTEGRATOR_WAVEFRONT)
                    for integ in integs:
                        key = f"{sname}/{lname}/{mname}/{integ}"
                        p = default_params(mode, 64, 48, 4, seed=5, max_depth=8 if mode == abi.MODE_MIS else 0,
                                           integrator=integ, bdpt_max_len=6)
                        try:
                            img = ctx.render(p)
                            results["images"][key] = img[..., :3].tolist()
                            results["calls"].append([key, "OK"])
                        except abi.E8GError as e:
                            results["calls"].append([key, str(e)])
                rays = ctx.camera_rays(64, 48)
                try:
                    ctx.trace_closest(rays)
                    results["calls"].append([f"{sname}/{lname}/trace", "OK"])
                except abi.E8GError as e:
                    results["calls"].append([f"{sname}/{lname}/trace", str(e)])
        # the many-scene batch, both forms
        batch = [S.soup(2000 + 3000 * k, seed=k, width=32, height=32) for k in range(4)]
        for integ in (abi.INTEGRATOR_WAVEFRONT, abi.INTEGRATOR_MEGAKERNEL):
            params = [default_params(abi.MODE_MIS, 32, 32, 4, seed=k + 1, max_depth=6, integrator=integ)
                      for k in range(4)]
            try:
                render_batch(ctx, batch, params)
                results["calls"].append([f"batch/{integ}", "OK"])
            except abi.E8GError as e:
                results["calls"].append([f"batch/{integ}", str(e)])
    with open(out_path, "w") as f:
        json.dump(results, f)


if __name__ == "__main__":
    main(sys.argv[1])
