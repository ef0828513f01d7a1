"""GPU parity against the CPU oracle, through the C ABI.

* Traversal: ngi_intersect / ngi_visible against the oracle's FP32 brute-force nearest hit
  (the Embree query of Scene::Intersect, rt.hpp:2162-2189). Primitive ids bit-exact on
  rays whose nearest hit is not a tie; hit distances within 1e-5 relative.
* Rendering: the plain FP64 GPU path replays the oracle's Philox paths exactly (same
  sample -> same path); the tuned FP32 path is checked with a tolerance.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import T_REL_TOL, check_hits, rel_rmse

pytestmark = pytest.mark.gpu


def _random_rays(n, lo, hi, rng, tmin=1e-4):
    o = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = o
    rays[:, 3] = tmin
    rays[:, 4:7] = d.astype(np.float32)
    rays[:, 7] = np.float32(3.4e38)
    return rays


def _load(desc, tmp_path, aspect=1.0):
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen
    from oracle.oracle import OracleScene

    path = scenegen.write_scene(desc, tmp_path)
    return ng.Scene.load(path, aspect), OracleScene.from_desc(desc, aspect)


def test_intersect_cornell_bit_exact(native_lib, cornell, tmp_path):
    from nanogi_gb300 import scenegen

    scene, ora = _load(scenegen.cornell_box(), tmp_path)
    rng = np.random.default_rng(1)
    rays = _random_rays(200_000, -0.2, 1.2, rng)
    check_hits(scene.intersect(rays), ora.intersect(rays, use_bvh=False), "cornell")
    info = scene.info()
    assert info["device_ready"] == 1 and info["bvh_nodes"] >= 1


def test_intersect_sphere_field_bit_exact(native_lib, tmp_path):
    from nanogi_gb300 import scenegen

    desc = scenegen.sphere_field(num_spheres=30, grid=64, level=3)
    scene, ora = _load(desc, tmp_path)
    rng = np.random.default_rng(2)
    rays = _random_rays(20_000, -8.0, 8.0, rng)
    gpu = scene.intersect(rays)
    check_hits(gpu, ora.intersect(rays, use_bvh=False), "sphere_field/brute")
    rays2 = _random_rays(200_000, -8.0, 8.0, rng)
    check_hits(scene.intersect(rays2), ora.intersect(rays2, use_bvh=True), "sphere_field/bvh")


def test_intersect_edge_cases(native_lib, tmp_path):
    from nanogi_gb300 import scenegen

    scene, ora = _load(scenegen.cornell_box(), tmp_path)
    rays = []
    # axis-aligned directions (zero components), rays along wall planes, tmin/tmax clamps
    for d in [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]:
        for o in [(0.5, 0.5, 0.5), (0.0, 0.5, 0.5), (0.25, 0.25, 0.25), (0.5, 0.0, 0.5)]:
            rays.append([*o, 1e-4, *d, 3.4e38])
            rays.append([*o, 0.0, *d, 0.3])
    rays.append([0.5, 0.5, 0.5, 10.0, 0, 1, 0, 3.4e38])  # tmin beyond every hit
    rays = np.array(rays, np.float32)
    gp, gt, _ = scene.intersect(rays)
    op, ot, _ = ora.intersect(rays, use_bvh=False)
    assert ((gp < 0) == (op < 0)).all()
    hit = gp >= 0
    assert np.allclose(gt[hit], ot[hit], rtol=T_REL_TOL, atol=0)
    assert gp[-1] == -1
    empty = scene.intersect(np.zeros((0, 8), np.float32))
    assert empty[0].shape == (0,)


def test_visible_matches_oracle(native_lib, tmp_path):
    from nanogi_gb300 import scenegen

    scene, ora = _load(scenegen.cornell_box(), tmp_path)
    rng = np.random.default_rng(3)
    pairs = rng.uniform(0.0, 1.0, (50_000, 6))
    g = scene.visible(pairs)
    o = ora.visible(pairs, use_bvh=False)
    assert (g == o).mean() > 0.9999
    assert 0.05 < g.mean() < 0.95


@pytest.mark.parametrize("renderer", ["pt", "ptdirect"])
def test_render_fp64_replays_oracle_cornell(native_lib, cornell, renderer):
    import nanogi_gb300 as ng
    from oracle.oracle import OracleScene

    desc, path = cornell
    W, H, spp = 24, 20, 8
    scene = ng.Scene.load(path, W / H)
    r = ng.Renderer(renderer=renderer, num_samples=W * H * spp, max_num_vertices=8, width=W, height=H, seed=11,
                    precision="fp64")
    film = r.render(scene)
    ref = OracleScene.from_desc(desc, W / H).render(renderer, num_samples=W * H * spp, max_vertices=8, width=W,
                                                    height=H, seed=11, rng_mode="replay", use_bvh=False)
    assert rel_rmse(film, ref) < 1e-6
    close = np.isclose(film, ref, rtol=1e-9, atol=1e-12)
    assert close.mean() > 0.995
    st = r.last_stats
    assert st["camera_rays"] == W * H * spp
    assert st["nonfinite"] == 0


@pytest.mark.parametrize("renderer", ["pt", "ptdirect"])
def test_render_fp64_replays_oracle_materials(native_lib, tmp_path, renderer):
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen
    from oracle.oracle import OracleScene

    desc = scenegen.material_box()
    W, H, spp = 20, 20, 16
    path = scenegen.write_scene(desc, tmp_path)
    scene = ng.Scene.load(path, W / H)
    film = ng.Renderer(renderer=renderer, num_samples=W * H * spp, max_num_vertices=10, width=W, height=H, seed=5,
                       precision="fp64").render(scene)
    ref = OracleScene.from_desc(desc, W / H).render(renderer, num_samples=W * H * spp, max_vertices=10, width=W,
                                                    height=H, seed=5, rng_mode="replay", use_bvh=False)
    assert rel_rmse(film, ref) < 1e-4
    assert np.isclose(film, ref, rtol=1e-8, atol=1e-12).mean() > 0.98


@pytest.mark.parametrize("renderer", ["pt", "ptdirect"])
def test_render_fp32_close_to_oracle(native_lib, cornell, renderer):
    import nanogi_gb300 as ng
    from oracle.oracle import OracleScene

    desc, path = cornell
    W, H, spp = 24, 24, 32
    scene = ng.Scene.load(path, W / H)
    film = ng.Renderer(renderer=renderer, num_samples=W * H * spp, max_num_vertices=8, width=W, height=H, seed=3,
                       precision="fp32").render(scene)
    ref = OracleScene.from_desc(desc, W / H).render(renderer, num_samples=W * H * spp, max_vertices=8, width=W,
                                                    height=H, seed=3, rng_mode="replay", use_bvh=False)
    # same Philox paths, FP32 shading: paths agree except where rounding flips a decision
    assert rel_rmse(film, ref) < 2e-3
