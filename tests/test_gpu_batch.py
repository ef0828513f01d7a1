"""Batched renders (ngi_render_batch): many independent jobs through one persistent wave.

Every job of a batch traces the Philox paths it traces when rendered alone with the same
parameters -- and that the oracle traces for it (ProcessSample_PT / _PTDirect,
src/nanogi.cpp:446-802) -- whatever the mix of scenes, renderers, resolutions, sample counts and path
lengths, with and without the autotuner:
* plain FP64 path: the films are equal up to the FP64 summation order (1e-9);
* tuned FP32 path: the batch and single-job kernels are separate compilations, so FP32
  rounding can differ in the last bit and send a few grazing paths elsewhere; the films
  agree to that level (rel-RMSE 1e-4).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch_scenes(native_lib, tmp_path_factory):
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen

    pool, jobs = scenegen.batch_jobs(num_jobs=10, seed=2000, pool_size=40, max_tris=20_000)
    paths = scenegen.write_batch(pool, jobs, tmp_path_factory.mktemp("batch"))
    scenes = [ng.Scene.load(p, 1.0) for p in paths]
    cornell = ng.Scene.load(scenegen.write_scene(scenegen.cornell_box(), tmp_path_factory.mktemp("cb")), 1.0)
    yield scenes, jobs, cornell, pool
    for s in scenes:
        s.close()
    cornell.close()


def _jobs(batch_scenes, scale=1, precision="fp32"):
    import nanogi_gb300 as ng

    scenes, jobs, cornell, _ = batch_scenes
    out = []
    for k, (s, j) in enumerate(zip(scenes, jobs)):
        res = max(8, j["res"] // 8)
        spp = max(1, j["spp"] // 16) * scale
        out.append((s, ng.Renderer(renderer="pt" if k % 3 == 0 else "ptdirect", num_samples=res * res * spp + k,
                                   max_num_vertices=j["max_vertices"], width=res, height=res, seed=j["seed"],
                                   precision=precision)))
    # the same scene twice, different resolutions / renderers
    out.append((cornell, ng.Renderer(renderer="pt", num_samples=16 * 12 * 40, max_num_vertices=8, width=16, height=12,
                                     seed=5, precision=precision)))
    out.append((cornell, ng.Renderer(renderer="ptdirect", num_samples=24 * 24 * 8, max_num_vertices=-1, width=24,
                                     height=24, seed=6, precision=precision)))
    return out


def _same(f, ref, precision):
    if precision == "fp64":
        return np.allclose(f, ref, rtol=1e-9, atol=1e-12)
    denom = max(float((ref ** 2).sum()), 1e-300)
    return float(((f - ref) ** 2).sum()) / denom < 1e-8  # rel-RMSE < 1e-4


@pytest.mark.parametrize("autotune,precision", [(False, "fp64"), (True, "fp64"), (False, "fp32"), (True, "fp32")])
def test_batch_equals_individual_renders(batch_scenes, autotune, precision):
    import nanogi_gb300 as ng

    jobs = _jobs(batch_scenes, precision=precision)
    films, st = ng.render_batch(jobs, autotune=autotune, autotune_fraction=0.05)
    assert st["samples"] == sum(r.num_samples for _, r in jobs)
    if autotune:
        assert st["trials"] >= 3
    for (scene, r), f in zip(jobs, films):
        ref = r.render(scene)
        assert _same(f, ref, precision), (r.renderer, r.width, r.num_samples)
        assert r.last_stats["camera_rays"] == r.num_samples


def test_batch_small_wave_and_options(batch_scenes):
    import nanogi_gb300 as ng

    jobs = _jobs(batch_scenes, precision="fp64")[:4]
    films, st = ng.render_batch(jobs, wave_size=512, trace_refill=4, iterations_per_graph=2)
    assert st["wave_size"] == 512 and st["trace_refill"] == 4 and st["iterations_per_graph"] == 2
    for (scene, r), f in zip(jobs, films):
        assert np.allclose(f, r.render(scene), rtol=1e-9, atol=1e-12)


def test_batch_rejects_mixed_precision_and_bad_jobs(batch_scenes):
    import nanogi_gb300 as ng

    jobs = _jobs(batch_scenes)[:2]
    jobs[1][1].precision = "fp64"
    with pytest.raises(ng.NanogiError):
        ng.render_batch(jobs)
    jobs[1][1].precision = "fp32"
    jobs[1][1].width = 0
    with pytest.raises(ng.NanogiError) as e:
        ng.render_batch(jobs)
    assert "job 1" in str(e.value)
    films, st = ng.render_batch([])
    assert films == [] and st["samples"] == 0


def test_batch_jobs_replay_the_oracle(batch_scenes):
    """Three jobs of one FP64 batch (different scenes, renderers, sizes and path lengths)
    against the oracle replaying the same Philox paths."""
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen
    from oracle.oracle import OracleScene

    from conftest import rel_rmse

    scenes, jobs, _, pool = batch_scenes
    picked = []
    for k in range(3):
        res = 12 + 4 * k
        r = ng.Renderer(renderer="pt" if k == 0 else "ptdirect", num_samples=res * res * 6 + k,
                        max_num_vertices=jobs[k]["max_vertices"], width=res, height=res, seed=jobs[k]["seed"],
                        precision="fp64")
        picked.append((scenes[k], r))
    films, st = ng.render_batch(picked)
    assert st["samples"] == sum(r.num_samples for _, r in picked)
    for k, ((_, r), f) in enumerate(zip(picked, films)):
        ora = OracleScene.from_desc(scenegen.batch_job_desc(pool, jobs[k]), 1.0)
        ref = ora.render(r.renderer, num_samples=r.num_samples, max_vertices=r.max_num_vertices, width=r.width,
                         height=r.height, seed=r.seed, rng_mode="replay", use_bvh=True)
        err = rel_rmse(f, ref)
        print(f"job {k} ({r.renderer}, {r.width}x{r.height}, M={r.max_num_vertices}): rel-RMSE {err:.3e}")
        assert float(ref.sum()) > 0
        assert err < 1e-6
        ora.close()
