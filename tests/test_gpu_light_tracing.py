"""lt / ltdirect on the GPU (ProcessSample_LT / _LTDirect, src/nanogi.cpp:804-1131).

* The plain FP64 path replays the oracle's light paths (same Philox numbers) on the Cornell
  box (pinhole, ltdirect), the area-sensor box (lt and ltdirect) and the material box
  (glossy, mirror and glass surfaces, point and directional lights).
* The tuned FP32 path agrees in expectation with the oracle in reference mode.
* Entry points that run camera paths only refuse the light tracers.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_rmse

pytestmark = pytest.mark.gpu


def _render(scene, renderer, n, W, H, seed, precision="fp64", m=8, **kw):
    import nanogi_gb300 as ng

    return ng.Renderer(renderer=renderer, num_samples=n, max_num_vertices=m, width=W, height=H, seed=seed,
                       precision=precision, **kw).render(scene)


@pytest.mark.parametrize("workload,renderers", [("cornell_box", ["ltdirect"]),
                                                ("area_sensor_box", ["lt", "ltdirect"]),
                                                ("material_box", ["ltdirect"])])
def test_fp64_light_paths_replay_the_oracle(native_lib, tmp_path, workload, renderers):
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen
    from oracle.oracle import OracleScene

    desc = scenegen.WORKLOADS[workload]()
    W = H = 16
    scene = ng.Scene.load(scenegen.write_scene(desc, tmp_path), W / H)
    ora = OracleScene.from_desc(desc, W / H)
    for renderer in renderers:
        for offset in ("reference", "scaled"):
            n = W * H * 16
            f = _render(scene, renderer, n, W, H, 6, ray_offset=offset)
            ref = ora.render(renderer, num_samples=n, max_vertices=8, width=W, height=H, seed=6, rng_mode="replay",
                             use_bvh=False, ray_offset=offset)
            assert ref.sum() > 0, (workload, renderer)
            assert rel_rmse(f, ref) < 1e-6, (workload, renderer, offset)


@pytest.mark.parametrize("renderer", ["lt", "ltdirect"])
def test_fp32_light_paths_match_reference_sampling(native_lib, tmp_path, renderer):
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen
    from oracle.oracle import OracleScene

    desc = scenegen.area_sensor_box()
    W = H = 8
    scene = ng.Scene.load(scenegen.write_scene(desc, tmp_path), 1.0)
    n = W * H * 8192
    g = np.stack([_render(scene, renderer, n, W, H, 10 + k, precision="fp32", m=-1) for k in range(4)])
    o = OracleScene.from_desc(desc, 1.0)
    r = np.stack([o.render(renderer, num_samples=n, max_vertices=-1, width=W, height=H, seed=20 + k,
                           rng_mode="reference") for k in range(4)])
    assert abs(g.sum() / r.sum() - 1) < 0.02
    se = np.sqrt(g.var(0, ddof=1) / 4 + r.var(0, ddof=1) / 4)
    ok = se > 0
    z = (g.mean(0) - r.mean(0))[ok] / se[ok]
    # Welch z with 3+3 degrees of freedom has heavy tails: allow a few pixels past 4
    assert abs(z.mean()) < 0.5 and (np.abs(z) > 4).mean() < 0.07


def test_light_tracers_are_refused_where_unsupported(native_lib, cornell):
    import nanogi_gb300 as ng

    desc, path = cornell
    scene = ng.Scene.load(path, 1.0)
    r = ng.Renderer(renderer="ltdirect", num_samples=64, max_num_vertices=8, width=8, height=8)
    with pytest.raises(ng.NanogiError) as e:
        r.backward(scene, np.zeros((8, 8, 3)))
    assert e.value.status == 7
    with pytest.raises(ng.NanogiError) as e:
        ng.render_batch([(scene, r)])
    assert e.value.status == 7
