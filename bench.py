#!/usr/bin/env python3
"""Benchmark of the GB300 `ptdirect` path tracer on the ~1.55 M-triangle terrain workload.

`--workload cornell` (pt, 256 x 256, max length 8, 64 spp per step) and `--workload interior`
(the ~10M-triangle precision interior, ptdirect, 1024 x 1024, max length 32) measure the other
single-GPU configurations the same way.

Workload: procedural 512 x 512 fBm terrain + 200 level-4 icospheres (diffuse / glossy /
mirror / glass) + 4 quad lights, 1920 x 1080, max path length 16, `ptdirect` (the
configuration the headline metric is quoted on). A step renders `--spp-per-step` samples
per pixel of the full frame; the default 16 steps x 16 spp make the configuration's 256 spp.

Reported (one JSON line on rank 0):
  value      Mrays/s (extension rays, camera rays included, + shadow rays) over the timed
             steps, inputs resident in HBM, film accumulated on the device
  e2e        the same metric through the C ABI's host-buffer entry point ngi_render: params
             in, normalised film copied to pinned host memory every step
  roofline   the dominant traversal kernel's algorithmic bytes per launch / its CUDA-event
             duration, against the measured HBM copy bandwidth
  roofline_logic  the same for the path-logic kernels (shading + regeneration) of an iteration
  time_to_1pct  the metric's second part: seconds to rel-RMSE 1% against an FP64 reference for
             the tuned (FP32 shading) and the plain (FP64 shading and path state) GPU path, pt on
             the 256 x 256 Cornell box at max length 8, from two spp rungs each and the spp^-1/2
             fit (reference: FP64 at 16,384 spp in two halves, its noise subtracted)
  adjoint    the metric's third part: path-replay backward time over forward time (ptdirect,
             512 x 512, 64 spp, 64 diffuse material groups)
  interior   Mrays/s on the ~10M-triangle precision interior (ptdirect 1024 x 1024, max length 32),
             the configuration whose BVH and triangles exceed L2
  cpu_baseline  the CPU oracle (the reference's algorithm restated, FP64, mt19937 stream)
             on this host's cores over a bounded sample of the same workload
`--impl reference` times that CPU implementation alone, with all host threads.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mrays/s & time to rel-RMSE 1% vs FP64 ref: tuned vs plain GPU pt; grad/fwd cost"
L2_FLUSH_BYTES = 256 << 20  # larger than the 129 MB L2

# The headline workload and the other single-GPU configurations of the metric. Only
# `terrain` is the default bench line; the others are measured on request.
WORKLOADS = {
    "terrain": dict(make="terrain_scene", width=1920, height=1080, m=16, renderer="ptdirect", spp_per_step=16,
                    label="terrain_scene: 512x512 fBm terrain + 200 level-4 icospheres + 4 quad lights"),
    "cornell": dict(make="cornell_box", width=256, height=256, m=8, renderer="pt", spp_per_step=64,
                    label="cornell_box: 5 walls + 2 boxes + 1 quad light"),
    "interior": dict(make="precision_interior", width=1024, height=1024, m=32, renderer="ptdirect", spp_per_step=16,
                     label="precision_interior: ~10M long thin triangles, coordinates 1e-3..1e3, 1 hidden emitter",
                     memory=True),
}
WORKLOAD = "terrain"
WIDTH, HEIGHT, MAX_VERTICES, RENDERER = 1920, 1080, 16, "ptdirect"


def configure(args):
    global WORKLOAD, WIDTH, HEIGHT, MAX_VERTICES, RENDERER
    w = WORKLOADS[args.workload]
    WORKLOAD = args.workload
    WIDTH, HEIGHT, MAX_VERTICES, RENDERER = w["width"], w["height"], w["m"], w["renderer"]
    if args.spp_per_step <= 0:
        args.spp_per_step = w["spp_per_step"]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=16)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="terrain", choices=sorted(WORKLOADS))
    ap.add_argument("--spp-per-step", type=int, default=0, help="0 = the workload's default")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--trace-all-rays", action="store_true",
                    help="also trace the ptdirect extension rays whose hit cannot score (as the reference does)")
    ap.add_argument("--e2e-steps", type=int, default=4)
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU-baseline sample duration")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the time-to-1% and adjoint measurements")
    ap.add_argument("--scene-dir", default=None)
    ap.add_argument("--wave-size", type=int, default=0, help="path slots (0 = library default)")
    ap.add_argument("--trace-refill", type=int, default=0, help="traversal refill threshold (0 = default)")
    ap.add_argument("--iterations-per-graph", type=int, default=0, help="wave iterations per CUDA graph (0 = default)")
    args = ap.parse_args()
    configure(args)
    return args


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_desc():
    from nanogi_gb300 import scenegen

    return getattr(scenegen, WORKLOADS[WORKLOAD]["make"])()


def load_scene(scene_dir: str | None):
    """The workload's scene description and the loaded scene (through the YAML loader; meshes
    of the large interior come from memory instead of OBJ text)."""
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen

    desc = make_desc()
    d = Path(scene_dir) if scene_dir else Path(tempfile.mkdtemp(prefix=f"ngi_{WORKLOAD}_"))
    if WORKLOADS[WORKLOAD].get("memory"):
        path = scenegen.write_scene(desc, d, write_meshes=False)
        return desc, ng.Scene.load_with_meshes(path, WIDTH / HEIGHT, scenegen.memory_meshes(desc))
    path = d / "scene.yml"
    if not path.exists():
        scenegen.write_scene(desc, d)
    return desc, ng.Scene.load(path, WIDTH / HEIGHT)


class ClockSampler:
    """nvidia-smi clock / throttle-reason sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.index)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            p = [x.strip() for x in l.split(",")]
            if len(p) < 8:
                continue
            try:
                sm.append(float(p[0]))
                smax.append(float(p[1]))
            except ValueError:
                continue
            for n, v in zip(names, p[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic():
    """DRAM bytes as a fraction of the traversal kernel's algorithmic bytes, from the committed
    ncu summaries of the terrain workload: the full-size measurement when present, else the
    small case's (an upper bound for the full-size launch)."""
    import re

    if WORKLOAD != "terrain":
        return None
    for name in ("k_trace_terrain_dram_1080p.md", "k_trace_terrain_small.md"):
        p = ROOT / "profiles" / name
        if p.exists():
            m = re.search(r"^dram_fraction_of_algorithmic:\s*([0-9.]+)", p.read_text(), re.M)
            if m:
                return float(m.group(1))
    return None


def cpu_baseline(desc, spp_rays_hint, seconds, threads=0):
    """Times the oracle (reference algorithm, FP64, mt19937 stream) on this host."""
    from oracle.oracle import OracleScene

    ora = OracleScene.from_desc(desc, WIDTH / HEIGHT)
    # Calibrate: every render pays a fixed cost (per-thread W*H films, as the reference's
    # Context::film does) plus a per-sample cost; size the timed sample to ~`seconds`.
    times = []
    for n_cal in (100_000, 400_000):
        ora.render(RENDERER, num_samples=n_cal, max_vertices=MAX_VERTICES, width=WIDTH, height=HEIGHT, seed=1,
                   rng_mode="reference", threads=threads, grain=1000)
        times.append(ora.last_stats["seconds"])
    per_sample = max((times[1] - times[0]) / 300_000, 1e-9)
    fixed = max(times[0] - 100_000 * per_sample, 0.0)
    n = int(min(max((seconds - fixed) / per_sample, 400_000), 2e9))
    ora.render(RENDERER, num_samples=n, max_vertices=MAX_VERTICES, width=WIDTH, height=HEIGHT, seed=2,
               rng_mode="reference", threads=threads, grain=10000)
    st = ora.last_stats
    rays = st["extension_rays"] + st["shadow_rays"]
    return {"value": rays / st["seconds"] / 1e6, "unit": "Mrays/s", "cores": int(st["threads"]), "kind": "port",
            "sample": f"{n} samples of the {WIDTH}x{HEIGHT} {RENDERER} frame ({rays} rays, {st['seconds']:.1f} s)",
            "msamples_per_s": n / st["seconds"] / 1e6}


# Algorithmic bytes of the path-logic kernels (FP32 path state), per unit of work:
# * a shaded slot (ptdirect shading half, one per traced extension ray): reads its queue entry
#   (4), hit record (16), ray origin and direction (32), throughput (16), pixel (4), sample id
#   (8), vertex count (4), the hit triangle's vertices (48) and shading normals (48) = 180 B;
#   writes the next ray (32), throughput (16), vertex count (4), state (1) and a queue entry (4) = 57 B;
# * a started sample (regeneration half): reads its queue entry (4); writes ray (32),
#   throughput (16), pixel (4), sample id (8), vertex count (4), state (1), queue entry (4) = 73 B;
# * a shadow ray appended (next-event estimation, either half): origin, direction,
#   contribution, pixel = 52 B.
# Materials, lights and the emitter CDF are a few KB that stay in L1/L2 and are not counted.
LOGIC_BYTES_SHADED, LOGIC_BYTES_STARTED, LOGIC_BYTES_SHADOW = 180 + 57, 4 + 69, 52


def roofline_logic(st_t, st_c, peak):
    launches = max(st_t["logic_launches"], 1)
    alg = (LOGIC_BYTES_SHADED * st_c["extension_rays"] + LOGIC_BYTES_STARTED * st_c["camera_rays"]
           + LOGIC_BYTES_SHADOW * st_c["shadow_rays"])
    per_launch_ms = st_t["logic_ms"] / launches
    achieved = alg / launches / (per_launch_ms / 1e3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None, "kernel": "k_logic (shading + regeneration, one iteration)",
            "algorithmic_bytes_per_launch": alg / launches, "avg_launch_ms": per_launch_ms,
            "bytes_per_unit": {"shaded_slot": LOGIC_BYTES_SHADED, "started_sample": LOGIC_BYTES_STARTED,
                               "shadow_ray": LOGIC_BYTES_SHADOW}}


def _fit_spp_to_1pct(rungs):
    """Least-squares fit of log(err) = log(c) - a log(spp) over the rungs (a = 1/2 for Monte
    Carlo noise), and spp at 1% from the fit with a = 1/2 held fixed (c from the rungs)."""
    x = np.log([r["spp"] for r in rungs])
    y = np.log([max(r["rel_rmse_corrected"], 1e-12) for r in rungs])
    slope = float(np.polyfit(x, y, 1)[0]) if len(rungs) > 1 else float("nan")
    logc = float(np.mean(y + 0.5 * x))  # c with the exponent -1/2
    return {"fitted_exponent": slope, "c_at_half": float(np.exp(logc)),
            "spp_to_1pct": float((np.exp(logc) / 0.01) ** 2)}


def time_to_1pct(ng, ref_spp=16384, rungs=(256, 1024), w=256, h=256, m=8):
    """Seconds to rel-RMSE 1% for the tuned (fp32) and plain (fp64) GPU pt on the Cornell box."""
    from nanogi_gb300 import scenegen

    d = tempfile.mkdtemp(prefix="ngi_cornell_")
    scene = ng.Scene.load(scenegen.write_scene(scenegen.cornell_box(), d), w / h)
    scene.build()

    def render(renderer, precision, spp, seed, offset=0):
        r = ng.Renderer(renderer=renderer, num_samples=w * h * spp, max_num_vertices=m, width=w, height=h,
                        seed=seed, sample_offset=offset, precision=precision)
        f = r.render(scene).copy()
        return f, r.last_stats["render_ms"] / 1e3

    def rel(a, b):
        return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))

    # FP64 reference: ptdirect (same image as pt on this scene: area light, no specular surfaces,
    # lower variance), two independent halves; their difference gives the reference's own noise
    half = ref_spp // 2
    ra, ta = render("ptdirect", "fp64", half, 1001)
    rb, tb = render("ptdirect", "fp64", half, 1001, offset=w * h * half)
    ref = 0.5 * (ra + rb)
    sigma_ref = rel(ra, rb) / 2.0
    out = {"workload": f"cornell_box 36 tris, {w}x{h}, pt, max length {m}",
           "reference": {"renderer": "ptdirect", "precision": "fp64", "spp": ref_spp, "seconds": ta + tb,
                         "rel_noise": sigma_ref}}
    # warm every kernel form the rungs use (a pt render whose samples fit in one wave runs the queued
    # kernels, a longer one the fused kernel), in both precisions
    for precision in ("fp32", "fp64"):
        for spp in rungs:
            render("pt", precision, spp, 3)
    for precision in ("fp32", "fp64"):
        rs = []
        for spp in rungs:
            film, sec = render("pt", precision, spp, 7)
            err = rel(film, ref)
            rs.append({"spp": spp, "seconds": sec, "rel_rmse": err,
                       "rel_rmse_corrected": float(np.sqrt(max(err * err - sigma_ref * sigma_ref, 0.0)))})
        fit = _fit_spp_to_1pct(rs)
        sec_per_spp = rs[-1]["seconds"] / rs[-1]["spp"]
        out[precision] = {"rungs": rs, "fit": fit, "seconds_per_spp": sec_per_spp,
                          "seconds": fit["spp_to_1pct"] * sec_per_spp}
    out["fp64_over_fp32"] = out["fp64"]["seconds"] / out["fp32"]["seconds"]
    scene.close()
    return out


def adjoint_cost(ng, w=512, h=512, spp=64, m=8, repeats=5):
    """Device time of the path-replay backward pass over the forward pass (ngi_render_backward
    against ngi_render with the same parameters)."""
    from nanogi_gb300 import scenegen

    d = tempfile.mkdtemp(prefix="ngi_inverse_")
    scene = ng.Scene.load(scenegen.write_scene(scenegen.inverse_box(seed=5, emitter_seed=7), d), w / h)
    scene.build()
    r = ng.Renderer(renderer="ptdirect", num_samples=w * h * spp, max_num_vertices=m, width=w, height=h, seed=3)
    target = np.zeros((h, w, 3))
    fwd, bwd = [], []
    for k in range(repeats + 1):
        img = r.render(scene)
        fwd.append(r.last_stats["render_ms"])
        r.backward(scene, 2.0 * (img - target))
        bwd.append(r.last_stats["render_ms"])
    fwd, bwd = float(np.median(fwd[1:])), float(np.median(bwd[1:]))
    scene.close()
    return {"workload": f"inverse_box 64 diffuse groups + 2 emitters, {w}x{h}, ptdirect, {spp} spp, max length {m}",
            "forward_ms": fwd, "backward_ms": bwd, "adjoint_over_forward": bwd / fwd}


def interior_throughput(ng, steps=4, spp=16, w=1024, h=1024, m=32):
    """Mrays/s and Msamples/s of the ~10M-triangle precision interior (ptdirect, FP32 shading,
    scaled ray offsets), device time of `steps` renders of `spp` samples per pixel each."""
    from nanogi_gb300 import scenegen

    t0 = time.perf_counter()
    desc = scenegen.precision_interior()
    d = tempfile.mkdtemp(prefix="ngi_interior_")
    scene = ng.Scene.load_with_meshes(scenegen.write_scene(desc, d, write_meshes=False), w / h,
                                      scenegen.memory_meshes(desc))
    del desc
    scene.build()
    setup_s = time.perf_counter() - t0
    info = scene.info()

    def render(offset, flags=0):
        r = ng.Renderer(renderer="ptdirect", num_samples=w * h * spp, max_num_vertices=m, width=w, height=h, seed=77,
                        sample_offset=offset, precision="fp32", ray_offset="scaled", flags=flags)
        r.render(scene)
        return r.last_stats

    render(0)
    ms = rays = samples = 0
    for i in range(steps):
        st = render((i + 1) * w * h * spp)
        ms += st["render_ms"]
        rays += st["extension_rays"] + st["shadow_rays"]
        samples += st["camera_rays"]
    st = render(0, flags=ng.capi.TRAVERSAL_COUNTERS)
    scene.close()
    return {"workload": f"precision_interior {info['num_triangles']} tris, {w}x{h}, ptdirect, max length {m}, "
                        f"{spp} spp per step, scaled ray offsets",
            "mrays_per_s": rays / (ms / 1e3) / 1e6, "msamples_per_s": samples / (ms / 1e3) / 1e6,
            "steps": steps, "ms_per_step": ms / steps, "bvh_build_ms": info["bvh_build_ms"],
            "bvh_bytes": info["bvh_bytes"], "setup_seconds": setup_s,
            "nodes_per_extension_ray": st["extend_nodes"] / max(st["extension_rays"], 1),
            "tris_per_extension_ray": st["extend_tris"] / max(st["extension_rays"], 1)}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    desc = make_desc()
    from oracle.oracle import OracleScene

    ora = OracleScene.from_desc(desc, WIDTH / HEIGHT)
    # ~2 s of work per step on 16 cores: large enough that the per-thread film set-up the reference
    # also pays (one W x H film per thread, src/nanogi.cpp:298) does not dominate
    default_step = {"terrain": WIDTH * HEIGHT * 4, "cornell": WIDTH * HEIGHT * 64, "interior": 2_000_000}[WORKLOAD]
    n_step = int(os.environ.get("NGI_REF_SAMPLES_PER_STEP", str(default_step)))
    for i in range(args.warmup):
        ora.render(RENDERER, num_samples=n_step // 4, max_vertices=MAX_VERTICES, width=WIDTH, height=HEIGHT,
                   seed=100 + i, rng_mode="reference", grain=1000)
    rays = 0
    samples = 0
    secs = 0.0
    threads = 0
    for i in range(args.steps):
        ora.render(RENDERER, num_samples=n_step, max_vertices=MAX_VERTICES, width=WIDTH, height=HEIGHT, seed=200 + i,
                   rng_mode="reference", grain=1000, sample_offset=i * n_step)
        st = ora.last_stats
        rays += st["extension_rays"] + st["shadow_rays"]
        samples += st["camera_rays"]
        secs += st["seconds"]
        threads = st["threads"]
    value = rays / secs / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{WORKLOADS[WORKLOAD]['label']}, {WIDTH}x{HEIGHT}, {RENDERER}, max length "
                               f"{MAX_VERTICES}", "samples_per_step": n_step},
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} x {n_step} samples of the {WIDTH}x{HEIGHT} frame"},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "msamples_per_s": samples / secs / 1e6, "rays_per_sample": rays / max(samples, 1),
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch

    import nanogi_gb300 as ng
    from nanogi_gb300 import capi

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    desc, scene = load_scene(args.scene_dir)
    scene.build()
    info = scene.info()

    spp = args.spp_per_step
    n_step = WIDTH * HEIGHT * spp
    film = torch.zeros((HEIGHT, WIDTH, 3), dtype=torch.float64, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()  # the zero-fills above must land before the render stream uses them
    # One dedicated stream: the render kernels, the L2 flush and the timing events all run on it.
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)

    base_flags = capi.TRACE_ALL_RAYS if args.trace_all_rays else 0

    def render_step(offset, flags=0):
        r = ng.Renderer(renderer=RENDERER, num_samples=n_step, max_num_vertices=MAX_VERTICES, width=WIDTH,
                        height=HEIGHT, seed=1234 + rank, sample_offset=offset, precision=args.precision,
                        flags=flags | base_flags,
                        wave_size=args.wave_size, trace_refill=args.trace_refill,
                        iterations_per_graph=args.iterations_per_graph)
        r.render_device(scene, film.data_ptr(), stream.cuda_stream)
        return r.last_stats

    # rank r renders its own sample range: weak scaling, no data-path collective
    base = rank * (args.warmup + args.steps) * n_step
    for i in range(args.warmup):
        flush.zero_()
        render_step(base + i * n_step)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    totals = dict(rays=0, samples=0, launches=0)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        torch.cuda.synchronize()
        # the library runs pt with the queued kernels when the render's samples fit in one wave; a
        # queued wave that holds every sample runs regeneration in its first iteration only
        fits = n_step <= 1 << 25 if args.wave_size == 0 else args.wave_size >= n_step
        queued = RENDERER == "ptdirect" or (RENDERER == "pt" and fits)
        one_pass = queued and fits
        ev0.record(stream)
        for i in range(args.steps):
            flush.zero_()
            st = render_step(base + (args.warmup + i) * n_step)
            totals["rays"] += st["extension_rays"] + st["shadow_rays"]
            totals["samples"] += st["camera_rays"]
            # queued kernels (ptdirect, and pt renders whose samples fit in one wave): counter reset,
            # shading, regeneration and traversal per iteration (regeneration in the first iteration
            # only when the wave holds every sample), plus the wave's initial regeneration queue; the
            # fused pt kernel: path logic and traversal; both: the wave-end launch that runs the last
            # paths to their end
            if queued:
                totals["launches"] += (3 * st["iterations"] + 2) if one_pass else (4 * st["iterations"] + 1)
            else:
                totals["launches"] += 2 * st["iterations"]
            totals["launches"] += 1 if st["finish_paths"] > 0 else 0
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    if world > 1:
        t = torch.tensor([ms, totals["rays"], totals["samples"]], dtype=torch.float64, device=dev)
        mx = t[:1].clone()
        torch.distributed.all_reduce(mx, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.all_reduce(t[1:], op=torch.distributed.ReduceOp.SUM)
        ms = float(mx.item())
        all_rays, all_samples = float(t[1].item()), float(t[2].item())
        # one film exchange per job: sum of every rank's samples (outside the timed region)
        torch.distributed.all_reduce(film)
    else:
        all_rays, all_samples = float(totals["rays"]), float(totals["samples"])
    value = all_rays / (ms / 1e3) / 1e6

    # ---- per-kernel timing and traversal counters (separate, untimed renders) ----
    st_t = render_step(base, flags=capi.KERNEL_TIMING)
    st_c = render_step(base, flags=capi.TRAVERSAL_COUNTERS)
    ext_bytes = st_c["extension_rays"] * (32 + 16) + 80 * st_c["extend_nodes"] + 48 * st_c["extend_tris"]
    sh_bytes = st_c["shadow_rays"] * (32 + 4) + 80 * st_c["shadow_nodes"] + 48 * st_c["shadow_tris"]
    launches = st_t["extend_launches"]
    if st_t["shadow_launches"] == 0 and st_c["shadow_rays"] > 0:
        # one traversal launch per iteration traces both queues (no separate shadow launch to time)
        kern = {"k_logic": st_t["logic_ms"], "k_trace<extension+shadow>": st_t["extend_ms"]}
        top, alg_bytes = "k_trace<extension+shadow>", ext_bytes + sh_bytes
        rays_k = st_c["extension_rays"] + st_c["shadow_rays"]
    else:
        kern = {"k_logic": st_t["logic_ms"], "k_trace<extension>": st_t["extend_ms"],
                "k_trace<shadow>": st_t["shadow_ms"]}
        top = max(["k_trace<extension>", "k_trace<shadow>"], key=lambda k: kern[k])
        alg_bytes = ext_bytes if top == "k_trace<extension>" else sh_bytes
        rays_k = st_c["extension_rays"] if top == "k_trace<extension>" else st_c["shadow_rays"]
    per_launch_bytes = alg_bytes / max(launches, 1)
    per_launch_ms = kern[top] / max(launches, 1)
    achieved = per_launch_bytes / (per_launch_ms / 1e3) / 1e9
    peak, peak_kind = measured_peak()
    frac_dram = ncu_traffic()
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": frac_dram * per_launch_bytes if frac_dram else None,
                "traffic_source": ("not measured in this run: the DRAM share of the algorithmic bytes from the "
                                   "committed ncu capture of this kernel on this workload, times this run's "
                                   "algorithmic bytes per launch") if frac_dram else None,
                "binding_limit": "instruction issue (the BVH is L2-resident; DRAM carries a small share of "
                                 "these bytes)",
                "kernel": top,
                "peak_source": peak_kind, "algorithmic_bytes_per_launch": per_launch_bytes,
                "avg_launch_ms": per_launch_ms, "algorithmic_bytes_counter_render": alg_bytes,
                "timed_launches": launches,
                "nodes_per_ray": st_c["extend_nodes"] / max(st_c["extension_rays"], 1),
                "tris_per_ray": st_c["extend_tris"] / max(st_c["extension_rays"], 1),
                "traced_rays_per_launch": rays_k / max(launches, 1),
                "kernel_ms_share": {k: v / max(sum(kern.values()), 1e-9) for k, v in kern.items()}}

    rl_logic = roofline_logic(st_t, st_c, peak)

    # ---- end to end through the host-buffer C ABI entry point ----
    host_film = torch.empty((HEIGHT, WIDTH, 3), dtype=torch.float64, pin_memory=True).numpy()
    r_e2e = ng.Renderer(renderer=RENDERER, num_samples=n_step, max_num_vertices=MAX_VERTICES, width=WIDTH,
                        height=HEIGHT, seed=99 + rank, precision=args.precision, wave_size=args.wave_size,
                        trace_refill=args.trace_refill, iterations_per_graph=args.iterations_per_graph,
                        flags=base_flags)
    r_e2e.render(scene, host_film)  # warm the host-film path
    torch.cuda.synchronize()
    e_rays = 0
    e_samples = 0
    t0 = time.perf_counter()
    for i in range(args.e2e_steps):
        r_e2e.sample_offset = (i + 1) * n_step
        r_e2e.render(scene, host_film)
        e_rays += r_e2e.last_stats["extension_rays"] + r_e2e.last_stats["shadow_rays"]
        e_samples += r_e2e.last_stats["camera_rays"]
    e_sec = time.perf_counter() - t0
    e2e = {"value": e_rays / e_sec / 1e6, "unit": "Mrays/s", "msamples_per_s": e_samples / e_sec / 1e6,
           "h2d_bytes_per_step": ctypes_sizeof_params(), "d2h_bytes_per_step": WIDTH * HEIGHT * 3 * 8,
           "steps": args.e2e_steps}
    scene.release_buffers()  # the measurements below render other scenes

    extras = {}
    if rank == 0 and world == 1 and not args.no_extras:
        torch.cuda.set_stream(torch.cuda.default_stream(dev))
        extras["time_to_1pct"] = time_to_1pct(ng)
        extras["adjoint"] = adjoint_cost(ng)
        if WORKLOAD == "terrain":
            extras["interior"] = interior_throughput(ng)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(desc, None, args.cpu_seconds)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if args.precision == "fp32" else "f64", "data": "synthetic",
            "config": {"workload": f"{WORKLOADS[WORKLOAD]['label']}, {info['num_triangles']} tris, {WIDTH}x{HEIGHT}, "
                                   f"{RENDERER}, max length {MAX_VERTICES}, {spp} spp per step",
                       "spp_total": spp * args.steps,
                       "precision": f"{args.precision} shading, fp64 film", "l2": "flushed between steps (256 MB write)",
                       "parallelism": f"replicas x{world}, disjoint sample ranges",
                       "rays": ("every ray the reference traces" if args.trace_all_rays or RENDERER != "ptdirect" else
                                "traced rays; ptdirect extension rays whose hit Russian roulette ends are not traced "
                                "(same film; --trace-all-rays traces them)")},
            "msamples_per_s": all_samples / (ms / 1e3) / 1e6,
            "rays_per_sample": all_rays / max(all_samples, 1),
            "bvh_build_ms": info["bvh_build_ms"], "bvh_bytes": info["bvh_bytes"],
            "roofline": roofline, "roofline_logic": rl_logic, "e2e": e2e, "gpu_launches": totals["launches"],
            "clocks": clocks.summary(),
        }
        if extras:
            t1 = extras["time_to_1pct"]
            line["time_to_1pct_s"] = {"fp32": t1["fp32"]["seconds"], "fp64": t1["fp64"]["seconds"],
                                      "fp64_over_fp32": t1["fp64_over_fp32"], "workload": t1["workload"]}
            line["adjoint_over_forward"] = extras["adjoint"]["adjoint_over_forward"]
            if "interior" in extras:
                line["interior_mrays_per_s"] = extras["interior"]["mrays_per_s"]
            line["extras"] = extras
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)
    scene.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def ctypes_sizeof_params():
    import ctypes

    from nanogi_gb300.capi import RenderParams

    return ctypes.sizeof(RenderParams)


if __name__ == "__main__":
    main()
