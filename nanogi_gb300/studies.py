"""Measurement studies beyond the throughput line of bench.py.

    python -m nanogi_gb300.studies convergence [--ref-spp 8192]

convergence: time to reach 1% relative RMSE against an FP64 reference, for the tuned path
(FP32 shading) and the plain path (FP64 shading and path state), `pt` on the Cornell-box
workload at 256 x 256 with max path length 8.

* Reference: the plain FP64 GPU path running `ptdirect` at --ref-spp samples per pixel. On
  a scene without specular surfaces or point lights, pt and ptdirect estimate the same
  image (every path of <= 8 vertices ending on the light), and ptdirect's variance is far
  lower. The reference's own noise is measured by rendering it as two independent halves
  (disjoint sample ranges) and is subtracted in quadrature from every error below.
* For each path and each spp in a doubling ladder the film's rel-RMSE
  sqrt(sum (x - ref)^2 / sum ref^2) is measured with its render time (CUDA events inside the
  library); since Monte-Carlo error falls as spp^-1/2, spp_1% = spp * (err / 0.01)^2 from the
  largest measured rung, and time_1% = spp_1% x (seconds per spp).
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def rel_rmse(a, b) -> float:
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


def _render(ng, scene, renderer, precision, spp, w, h, m, seed, offset=0):
    r = ng.Renderer(renderer=renderer, num_samples=w * h * spp, max_num_vertices=m, width=w, height=h, seed=seed,
                    sample_offset=offset, precision=precision)
    t0 = time.perf_counter()
    film = r.render(scene)
    wall = time.perf_counter() - t0
    return film, r.last_stats["render_ms"] / 1e3, wall


def convergence(ref_spp: int = 8192, w: int = 256, h: int = 256, m: int = 8, max_ladder_spp: int = 4096):
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen

    d = tempfile.mkdtemp(prefix="ngi_cornell_")
    path = scenegen.write_scene(scenegen.cornell_box(), d)
    scene = ng.Scene.load(path, w / h)
    scene.build()
    half = ref_spp // 2
    ra, ta, _ = _render(ng, scene, "ptdirect", "fp64", half, w, h, m, seed=1001, offset=0)
    rb, tb, _ = _render(ng, scene, "ptdirect", "fp64", half, w, h, m, seed=1001, offset=w * h * half)
    ref = 0.5 * (ra + rb)
    # two independent halves: rel-RMSE(a, b) = sqrt(2) sigma_half; sigma_ref = sigma_half / sqrt(2)
    sigma_ref = rel_rmse(ra, rb) / 2.0
    out = {"workload": f"cornell_box 36 tris, {w}x{h}, pt, max length {m}",
           "reference": {"renderer": "ptdirect", "precision": "fp64", "spp": ref_spp, "seconds": ta + tb,
                         "rel_noise": sigma_ref},
           "paths": {}}
    for precision in ("fp32", "fp64"):
        rungs = []
        spp = 16
        seed = 7
        while spp <= max_ladder_spp:
            film, sec, wall = _render(ng, scene, "pt", precision, spp, w, h, m, seed=seed, offset=0)
            err = rel_rmse(film, ref)
            err_c = math.sqrt(max(err * err - sigma_ref * sigma_ref, 0.0))
            rungs.append({"spp": spp, "seconds": sec, "wall_seconds": wall, "rel_rmse": err, "rel_rmse_corrected": err_c})
            if err_c < 0.01 or sec > 20.0:
                break
            spp *= 2
        last = rungs[-1]
        spp_1 = last["spp"] * (last["rel_rmse_corrected"] / 0.01) ** 2
        sec_per_spp = last["seconds"] / last["spp"]
        out["paths"][precision] = {"rungs": rungs, "spp_to_1pct": spp_1, "seconds_to_1pct": spp_1 * sec_per_spp,
                                   "seconds_per_spp": sec_per_spp}
    out["speedup_fp32_over_fp64"] = out["paths"]["fp64"]["seconds_to_1pct"] / out["paths"]["fp32"]["seconds_to_1pct"]
    scene.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("study", choices=["convergence"])
    ap.add_argument("--ref-spp", type=int, default=8192)
    ap.add_argument("--max-ladder-spp", type=int, default=4096)
    a = ap.parse_args()
    if a.study == "convergence":
        print(json.dumps(convergence(a.ref_spp, max_ladder_spp=a.max_ladder_spp)), flush=True)


if __name__ == "__main__":
    main()
