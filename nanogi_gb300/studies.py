"""Measurement studies beyond the throughput line of bench.py.

    python -m nanogi_gb300.studies convergence [--ref-spp 65536]
    python -m nanogi_gb300.studies adjoint
    python -m nanogi_gb300.studies batch
    python -m nanogi_gb300.studies precision [--ref-spp 1024]
    python -m nanogi_gb300.studies fp32-error --workload terrain|batch|inverse [--spp 256] [--ref-spp 1024]

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


def convergence(ref_spp: int = 65536, w: int = 256, h: int = 256, m: int = 8, max_ladder_spp: int = 4096):
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


def precision(ref_spp: int = 1024, w: int = 1024, h: int = 1024, m: int = 32, num_triangles: int = 10_000_000,
              max_rung_seconds: float = 20.0, bias_spp: int = 256):
    """FP32-vs-FP64 study on the precision interior (scenegen.precision_interior): ~10M long
    thin triangles, coordinates 1e-3..1e3, one small emitter seen only through bounces;
    `ptdirect`, w x h, max path length m.

    * Reference ("FP64 oracle"): the plain path -- FP64 shading, path state and film -- with
      scaled ray offsets at ref_spp, rendered as two independent halves whose difference gives
      its own noise, subtracted in quadrature from every error below.
    * time to 1% rel-RMSE for the tuned FP32 path and the plain FP64 path (both scaled
      offsets), extrapolated from a doubling spp ladder as in `convergence`.
    * bias: FP32 (scaled offsets) and both paths with the reference's absolute tmin = 1e-4
      against the FP64 reference, on 16 x 16-pixel block means, where noise averages out.
    """
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen

    t0 = time.perf_counter()
    desc = scenegen.precision_interior(num_triangles=num_triangles)
    gen_s = time.perf_counter() - t0
    d = tempfile.mkdtemp(prefix="ngi_precision_")
    path = scenegen.write_scene(desc, d, write_meshes=False)
    t0 = time.perf_counter()
    scene = ng.Scene.load_with_meshes(path, w / h, scenegen.memory_meshes(desc))
    load_s = time.perf_counter() - t0
    del desc
    t0 = time.perf_counter()
    scene.build()
    build_s = time.perf_counter() - t0
    info = scene.info()

    def render(precision, spp, seed, offset=0, ray_offset="scaled"):
        r = ng.Renderer(renderer="ptdirect", num_samples=w * h * spp, max_num_vertices=m, width=w, height=h,
                        seed=seed, sample_offset=offset, precision=precision, ray_offset=ray_offset)
        f = r.render(scene)
        st = r.last_stats
        return f, st["render_ms"] / 1e3, st

    half = ref_spp // 2
    ra, ta, sta = render("fp64", half, 2024)
    rb, tb, _ = render("fp64", half, 2024, offset=w * h * half)
    ref = 0.5 * (ra + rb)
    sigma_ref = rel_rmse(ra, rb) / 2.0
    out = {"workload": f"precision_interior {info['num_triangles']} tris, {w}x{h}, ptdirect, max length {m}",
           "scene": {"generate_seconds": gen_s, "load_seconds": load_s, "build_seconds": build_s,
                     "bvh_nodes": info["bvh_nodes"], "bound_min": list(info["bound_min"]),
                     "bound_max": list(info["bound_max"])},
           "reference": {"precision": "fp64", "ray_offset": "scaled", "spp": ref_spp, "seconds": ta + tb,
                         "rel_noise": sigma_ref,
                         "mrays_per_s": (sta["extension_rays"] + sta["shadow_rays"]) / ta / 1e6},
           "paths": {}}
    for precision in ("fp32", "fp64"):
        rungs = []
        spp = 16
        while True:
            film, sec, st = render(precision, spp, 77)
            err = rel_rmse(film, ref)
            err_c = math.sqrt(max(err * err - sigma_ref * sigma_ref, 0.0))
            rungs.append({"spp": spp, "seconds": sec, "rel_rmse": err, "rel_rmse_corrected": err_c,
                          "mrays_per_s": (st["extension_rays"] + st["shadow_rays"]) / sec / 1e6,
                          "msamples_per_s": w * h * spp / sec / 1e6})
            if err_c < 0.01 or sec * 2 > max_rung_seconds or spp >= ref_spp:
                break
            spp *= 2
        last = rungs[-1]
        spp_1 = last["spp"] * (last["rel_rmse_corrected"] / 0.01) ** 2
        sec_per_spp = last["seconds"] / last["spp"]
        out["paths"][precision] = {"rungs": rungs, "spp_to_1pct": spp_1, "seconds_to_1pct": spp_1 * sec_per_spp,
                                   "seconds_per_spp": sec_per_spp}
    out["speedup_fp32_over_fp64"] = out["paths"]["fp64"]["seconds_to_1pct"] / out["paths"]["fp32"]["seconds_to_1pct"]

    def blocks(x, b=16):
        y = x.sum(2)
        return y[: h // b * b, : w // b * b].reshape(h // b, b, w // b, b).mean((1, 3))

    rb_ref = blocks(ref)
    bias = {}
    for precision, mode in (("fp32", "scaled"), ("fp32", "reference"), ("fp64", "reference")):
        film, sec, _ = render(precision, bias_spp, 501, ray_offset=mode)
        bias[f"{precision}/{mode}"] = {"spp": bias_spp, "image_mean_ratio": float(film.sum() / ref.sum()),
                                       "block_rel_rmse": rel_rmse(blocks(film), rb_ref),
                                       "rel_rmse": rel_rmse(film, ref)}
    film, _, _ = render("fp64", bias_spp, 501)
    bias["fp64/scaled (noise floor)"] = {"spp": bias_spp, "image_mean_ratio": float(film.sum() / ref.sum()),
                                        "block_rel_rmse": rel_rmse(blocks(film), rb_ref), "rel_rmse": rel_rmse(film, ref)}
    out["bias_vs_reference"] = bias
    r = ng.Renderer(renderer="ptdirect", num_samples=w * h * 16, max_num_vertices=m, width=w, height=h, seed=9,
                    ray_offset="scaled", flags=ng.capi.KERNEL_TIMING | ng.capi.TRAVERSAL_COUNTERS)
    r.render(scene)
    st = r.last_stats
    out["traversal_fp32_16spp"] = {
        "extend_nodes_per_ray": st["extend_nodes"] / max(st["extension_rays"], 1),
        "extend_tris_per_ray": st["extend_tris"] / max(st["extension_rays"], 1),
        "shadow_nodes_per_ray": st["shadow_nodes"] / max(st["shadow_rays"], 1),
        "shadow_tris_per_ray": st["shadow_tris"] / max(st["shadow_rays"], 1),
        "logic_ms": st["logic_ms"], "extend_ms": st["extend_ms"], "shadow_ms": st["shadow_ms"]}
    scene.close()
    return out


def adjoint_cost(w: int = 512, h: int = 512, spp: int = 64, m: int = 8, repeats: int = 3, descent_steps: int = 8):
    """Inverse-rendering workload: time of the path-replay backward pass over the forward pass
    (ptdirect, FP32 shading), plus a few steps of gradient descent on the L2 image loss."""
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen

    d = tempfile.mkdtemp(prefix="ngi_inverse_")
    scene = ng.Scene.load(scenegen.write_scene(scenegen.inverse_box(seed=5, emitter_seed=7), d + "/a"), w / h)
    hidden = ng.Scene.load(scenegen.write_scene(scenegen.inverse_box(seed=6, emitter_seed=8), d + "/b"), w / h)
    ha, he = hidden.parameters()
    hidden.close()
    scene.build()
    r = ng.Renderer(renderer="ptdirect", num_samples=w * h * spp, max_num_vertices=m, width=w, height=h, seed=3)
    ta, te = scene.parameters()
    scene.set_parameters(ha, he)
    target = r.render(scene).copy()
    scene.set_parameters(ta, te)
    fwd, bwd = [], []
    img = None
    for _ in range(repeats + 1):
        t0 = time.perf_counter()
        img = r.render(scene)
        fwd.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        r.backward(scene, 2.0 * (img - target))
        bwd.append(time.perf_counter() - t0)
    fwd, bwd = fwd[1:], bwd[1:]
    mats = [i for i, p in enumerate(scene.parameters()[0]) if p.any()]
    losses = []
    a, e = ta.copy(), te.copy()
    for step in range(descent_steps):
        scene.set_parameters(a, e)
        img = r.render(scene)
        losses.append(float(((img - target) ** 2).sum()))
        ga, ge = r.backward(scene, 2.0 * (img - target))
        lr = 0.02 / max(np.abs(ga).max(), 1e-30)
        a = np.clip(a - lr * ga, 0.0, 1.0)
    scene.set_parameters(ta, te)
    err0 = float(np.abs(ta[mats] - ha[mats]).mean())
    err1 = float(np.abs(a[mats] - ha[mats]).mean())
    scene.close()
    return {"workload": f"inverse_box 64 diffuse groups + 2 emitters, {w}x{h}, ptdirect, {spp} spp, max length {m}",
            "forward_seconds": float(np.median(fwd)), "backward_seconds": float(np.median(bwd)),
            "grad_over_fwd": float(np.median(bwd) / np.median(fwd)), "descent_losses": losses,
            "albedo_mean_abs_error_before": err0, "albedo_mean_abs_error_after": err1}


def batch(num_jobs: int = 256):
    """Batched renders: `num_jobs` independent jobs (the batch workload of scenegen.batch_jobs)
    through one persistent wave replayed from one CUDA graph, after autotuning, against the
    same jobs rendered one after another through ngi_render."""
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen

    pool, jobs = scenegen.batch_jobs(num_jobs=num_jobs)
    d = tempfile.mkdtemp(prefix="ngi_batch_")
    paths = scenegen.write_batch(pool, jobs, d)
    t0 = time.perf_counter()
    scenes = [ng.Scene.load(p, 1.0) for p in paths]
    for sc in scenes:
        sc.build()
    load_s = time.perf_counter() - t0
    work = [(sc, ng.Renderer(renderer=j["renderer"], num_samples=j["res"] * j["res"] * j["spp"],
                             max_num_vertices=j["max_vertices"], width=j["res"], height=j["res"], seed=j["seed"]))
            for sc, j in zip(scenes, jobs)]
    ng.render_batch(work[:8])  # warm the batch kernels
    t0 = time.perf_counter()
    films, st = ng.render_batch(work, autotune=True)
    batch_wall = time.perf_counter() - t0
    rays = st["extension_rays"] + st["shadow_rays"]
    seq_ms, seq_rays = 0.0, 0
    scenes[0].release_buffers()  # the batch's wave
    t0 = time.perf_counter()
    for sc, r in work:
        r.render(sc)
        seq_ms += r.last_stats["render_ms"]
        seq_rays += r.last_stats["extension_rays"] + r.last_stats["shadow_rays"]
        sc.release_buffers()  # 256 handles would otherwise keep 256 waves
    seq_wall = time.perf_counter() - t0
    out = {"workload": f"{num_jobs} jobs, res {{64,128,256,512}}^2, tris log-U[1k,200k] "
                       f"(mean {np.mean([j['triangles'] for j in jobs]):.0f}), spp log-U[16,1024], max length U[4,24], ptdirect",
           "samples": st["samples"], "load_and_build_seconds": load_s,
           "batch": {"device_ms": st["render_ms"], "wall_seconds": batch_wall, "autotune_ms": st["autotune_ms"],
                     "trials": st["trials"], "mrays_per_s": rays / (st["render_ms"] / 1e3) / 1e6,
                     "msamples_per_s": st["samples"] / (st["render_ms"] / 1e3) / 1e6,
                     "config": {"wave_size": st["wave_size"], "trace_refill": st["trace_refill"],
                                "iterations_per_graph": st["iterations_per_graph"]}},
           "one_by_one": {"device_ms": seq_ms, "wall_seconds": seq_wall, "mrays_per_s": seq_rays / (seq_ms / 1e3) / 1e6},
           "speedup_device": seq_ms / st["render_ms"], "speedup_wall": seq_wall / batch_wall}
    for sc in scenes:
        sc.close()
    return out


def _blocks(x, b=16):
    h, w = x.shape[:2]
    y = x.sum(2)
    return y[: h // b * b, : w // b * b].reshape(h // b, b, w // b, b).mean((1, 3))


def _fp32_error(render, spp: int, ref_spp: int, blocks: int = 16):
    """Error of the tuned FP32 path against an FP64 reference, with the noise taken out.

    `render(precision, spp, seed, offset)` returns a normalised film. The reference is FP64 at
    ref_spp in two independent halves (their difference gives its noise). FP32 and a second,
    independent FP64 film are rendered at `spp`; on `blocks` x `blocks`-pixel block means
    (where the per-pixel noise averages out) the FP64 film's error is the noise floor, and
    the FP32 error beyond it, taken out in quadrature, is the bias FP32 adds."""
    half = ref_spp // 2
    ra = render("fp64", half, 9001, 0)
    rb = render("fp64", half, 9001, half)
    ref = 0.5 * (ra + rb)
    sigma_ref_block = rel_rmse(_blocks(ra, blocks), _blocks(rb, blocks)) / 2.0
    f32 = render("fp32", spp, 9101, 0)
    f64 = render("fp64", spp, 9201, 0)
    e32 = rel_rmse(_blocks(f32, blocks), _blocks(ref, blocks))
    e64 = rel_rmse(_blocks(f64, blocks), _blocks(ref, blocks))
    return {"spp": spp, "ref_spp": ref_spp, "block": blocks,
            "block_rel_rmse_fp32": e32, "block_rel_rmse_fp64": e64, "reference_block_noise": sigma_ref_block,
            "fp32_bias_beyond_noise": math.sqrt(max(e32 * e32 - e64 * e64, 0.0)),
            "image_mean_ratio_fp32": float(f32.sum() / ref.sum()), "image_mean_ratio_fp64": float(f64.sum() / ref.sum()),
            "pixel_rel_rmse_fp32": rel_rmse(f32, ref), "pixel_rel_rmse_fp64": rel_rmse(f64, ref)}


def fp32_error(workload: str, spp: int = 256, ref_spp: int = 1024):
    """FP32-against-FP64 error of one configuration (see _fp32_error):
    terrain -- ptdirect 1920 x 1080, max length 16 (the headline workload);
    batch   -- 16 jobs of the batched workload (each at its own resolution, path length and
               materials; spp per job = `spp`), errors averaged over the jobs;
    inverse -- the inverse-rendering box, ptdirect 512 x 512, max length 8, plus the relative
               difference of the FP32 and FP64 path-replay gradients on the same paths."""
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen

    d = tempfile.mkdtemp(prefix="ngi_fp32err_")
    if workload == "terrain":
        w, h, m = 1920, 1080, 16
        scene = ng.Scene.load(scenegen.write_scene(scenegen.terrain_scene(), d), w / h)

        def render(precision, n, seed, offset):
            return ng.Renderer(renderer="ptdirect", num_samples=w * h * n, max_num_vertices=m, width=w, height=h,
                               seed=seed, sample_offset=w * h * offset, precision=precision).render(scene).copy()

        out = {"workload": f"terrain_scene, {w}x{h}, ptdirect, max length {m}", **_fp32_error(render, spp, ref_spp)}
        scene.close()
        return out
    if workload == "inverse":
        w, h, m = 512, 512, 8
        scene = ng.Scene.load(scenegen.write_scene(scenegen.inverse_box(seed=5, emitter_seed=7), d), w / h)

        def render(precision, n, seed, offset):
            return ng.Renderer(renderer="ptdirect", num_samples=w * h * n, max_num_vertices=m, width=w, height=h,
                               seed=seed, sample_offset=w * h * offset, precision=precision).render(scene).copy()

        out = {"workload": f"inverse_box, {w}x{h}, ptdirect, max length {m}", **_fp32_error(render, spp, ref_spp)}
        # gradients of the same paths in both precisions (L2 loss against a zero image)
        grads = {}
        for precision in ("fp32", "fp64"):
            r = ng.Renderer(renderer="ptdirect", num_samples=w * h * 64, max_num_vertices=m, width=w, height=h, seed=3,
                            precision=precision)
            img = r.render(scene)
            grads[precision] = r.backward(scene, 2.0 * img)[0]
        out["gradient_rel_diff_fp32_vs_fp64"] = rel_rmse(grads["fp32"], grads["fp64"])
        scene.close()
        return out
    if workload == "batch":
        pool, jobs = scenegen.batch_jobs(num_jobs=16)
        paths = scenegen.write_batch(pool, jobs, d)
        per_job = []
        for path, j in zip(paths, jobs):
            res = j["res"]
            scene = ng.Scene.load(path, 1.0)

            def render(precision, n, seed, offset, scene=scene, res=res, j=j):
                return ng.Renderer(renderer="ptdirect", num_samples=res * res * n, max_num_vertices=j["max_vertices"],
                                   width=res, height=res, seed=seed, sample_offset=res * res * offset,
                                   precision=precision).render(scene).copy()

            e = _fp32_error(render, spp, ref_spp, blocks=8 if res < 128 else 16)
            e["res"], e["max_vertices"], e["triangles"] = res, j["max_vertices"], j["triangles"]
            per_job.append(e)
            scene.close()
        keys = ("block_rel_rmse_fp32", "block_rel_rmse_fp64", "fp32_bias_beyond_noise", "image_mean_ratio_fp32")
        return {"workload": "16 jobs of the batched workload, ptdirect", "jobs": per_job,
                "mean": {k: float(np.mean([e[k] for e in per_job])) for k in keys},
                "max_bias_beyond_noise": float(max(e["fp32_bias_beyond_noise"] for e in per_job))}
    raise ValueError(workload)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("study", choices=["convergence", "adjoint", "batch", "precision", "fp32-error"])
    ap.add_argument("--workload", default="terrain", choices=["terrain", "batch", "inverse"])
    ap.add_argument("--spp", type=int, default=256)
    ap.add_argument("--triangles", type=int, default=10_000_000)
    ap.add_argument("--res", type=int, default=1024)
    ap.add_argument("--ref-spp", type=int, default=None)
    ap.add_argument("--max-ladder-spp", type=int, default=4096)
    a = ap.parse_args()
    if a.study == "convergence":
        print(json.dumps(convergence(a.ref_spp or 65536, max_ladder_spp=a.max_ladder_spp)), flush=True)
    elif a.study == "adjoint":
        print(json.dumps(adjoint_cost()), flush=True)
    elif a.study == "batch":
        print(json.dumps(batch()), flush=True)
    elif a.study == "precision":
        print(json.dumps(precision(a.ref_spp or 1024, a.res, a.res, num_triangles=a.triangles)), flush=True)
    elif a.study == "fp32-error":
        print(json.dumps(fp32_error(a.workload, a.spp, a.ref_spp or 1024)), flush=True)


if __name__ == "__main__":
    main()
