"""bdpt on the GPU (ProcessSample_BDPT, src/nanogi.cpp:1133-1194; include/nanogi/bdpt.hpp).

* The plain FP64 path replays the oracle's subpaths (same Philox numbers) and evaluates the
  same strategies with power-heuristic MIS on the Cornell box, the area-sensor box (t = 0
  strategies), the material box (glossy, mirror, glass, point and directional lights) and the
  textured box, with both ray-offset modes.
* The tuned FP32 path agrees in expectation with the oracle's reference-mode (mt19937) renders.
* bdpt estimates the same image as pt where both see every path (area lights only).
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_rmse

pytestmark = pytest.mark.gpu


def _r(**kw):
    import nanogi_gb300 as ng

    return ng.Renderer(renderer="bdpt", **kw)


@pytest.mark.parametrize("workload", ["cornell_box", "area_sensor_box", "material_box", "textured_box"])
@pytest.mark.parametrize("offset", ["reference", "scaled"])
def test_fp64_bdpt_replays_the_oracle(native_lib, tmp_path, workload, offset):
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen
    from oracle.oracle import OracleScene

    desc = scenegen.WORKLOADS[workload]()
    W = H = 12
    n = W * H * 8
    scene = ng.Scene.load(scenegen.write_scene(desc, tmp_path), 1.0)
    f = _r(num_samples=n, max_num_vertices=6, width=W, height=H, seed=17, precision="fp64",
           ray_offset=offset).render(scene)
    ref = OracleScene.from_desc(desc, 1.0).render("bdpt", num_samples=n, max_vertices=6, width=W, height=H,
                                                  seed=17, rng_mode="replay", use_bvh=False, ray_offset=offset)
    assert ref.sum() > 0
    assert rel_rmse(f, ref) < 1e-6, (workload, offset)


def test_fp32_bdpt_matches_reference_sampling(native_lib, cornell):
    import nanogi_gb300 as ng
    from oracle.oracle import OracleScene

    desc, path = cornell
    W = H = 8
    n = W * H * 2048
    scene = ng.Scene.load(path, 1.0)
    g = np.stack([_r(num_samples=n, max_num_vertices=8, width=W, height=H, seed=40 + k).render(scene)
                  for k in range(4)])
    o = OracleScene.from_desc(desc, 1.0)
    r = np.stack([o.render("bdpt", num_samples=n, max_vertices=8, width=W, height=H, seed=60 + k,
                           rng_mode="reference") for k in range(4)])
    assert abs(g.sum() / r.sum() - 1) < 0.02
    se = np.sqrt(g.var(0, ddof=1) / 4 + r.var(0, ddof=1) / 4)
    ok = se > 0
    z = (g.mean(0) - r.mean(0))[ok] / se[ok]
    # Welch z with 3+3 degrees of freedom has heavy tails: allow a few pixels past 4
    assert abs(z.mean()) < 0.5 and (np.abs(z) > 4).mean() < 0.07


def test_bdpt_and_pt_estimate_the_same_image(native_lib, tmp_path):
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen

    desc = scenegen.material_box(with_point=False, with_directional=False)
    scene = ng.Scene.load(scenegen.write_scene(desc, tmp_path), 1.0)
    W = H = 16
    n = W * H * 4096
    pt = ng.Renderer(renderer="pt", num_samples=n, max_num_vertices=8, width=W, height=H, seed=1).render(scene)
    pt2 = ng.Renderer(renderer="pt", num_samples=n, max_num_vertices=8, width=W, height=H, seed=2).render(scene)
    b = _r(num_samples=n, max_num_vertices=8, width=W, height=H, seed=3).render(scene)
    assert abs(b.sum() / pt.sum() - 1) < 0.02
    assert rel_rmse(b, pt) < 1.5 * rel_rmse(pt2, pt)


def test_bdpt_unbounded_length_and_small_waves(native_lib, cornell):
    desc, path = cornell
    import nanogi_gb300 as ng

    scene = ng.Scene.load(path, 1.0)
    W = H = 8
    a = _r(num_samples=W * H * 64, max_num_vertices=-1, width=W, height=H, seed=5).render(scene)
    b = _r(num_samples=W * H * 64, max_num_vertices=-1, width=W, height=H, seed=5, wave_size=256).render(scene)
    assert a.sum() > 0 and np.allclose(a, b, rtol=1e-9, atol=1e-12)
    one = _r(num_samples=64, max_num_vertices=1, width=W, height=H, seed=5).render(scene)
    assert not one.any()
