"""GPU parity with the oracle on the scenes the throughput is measured on (through the C ABI).

The headline workload is the 1.55M-triangle terrain (512 x 512 fBm height field, 200 level-4
icospheres with diffuse / glossy / mirror / glass materials, 4 quad lights), rendered with
ptdirect at max length 16. The precision workload is the interior of long thin triangles whose
coordinates span 1e-3..1e3, here cut to 1M triangles so the oracle builds its BVH in seconds.

* Traversal (Scene::Intersect, rt.hpp:2162-2189): about a million camera, random and
  second-bounce rays per scene through ngi_intersect against the oracle's BVH, and a subset
  against the oracle's brute force (every triangle tested), which also pins the oracle's BVH.
  Primitive ids bit-exact on every ray that is not a tie, hit distances bit-identical.
* Rendering (ProcessSample_PTDirect, nanogi.cpp:609-802): the plain FP64 GPU path replays the
  oracle's Philox paths on the terrain; the tuned FP32 path is statistically equal, pixel by
  pixel, to the oracle's reference-mode renders (std::mt19937 stream, uniform raster
  positions) on the terrain and on the material box (every BSDF and light type).
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import assert_same_expectation, bounce_rays, camera_rays, check_hits, rel_rmse

pytestmark = pytest.mark.gpu

TERRAIN_ASPECT = 16 / 9


def _load_memory(desc, tmp_path, aspect):
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen

    path = scenegen.write_scene(desc, tmp_path, write_meshes=False)
    return ng.Scene.load_with_meshes(path, aspect, scenegen.memory_meshes(desc))


@pytest.fixture(scope="module")
def terrain(native_lib, tmp_path_factory):
    from nanogi_gb300 import scenegen
    from oracle.oracle import OracleScene

    desc = scenegen.terrain_scene()
    scene = _load_memory(desc, tmp_path_factory.mktemp("terrain"), TERRAIN_ASPECT)
    scene.build()
    ora = OracleScene.from_desc(desc, TERRAIN_ASPECT)
    yield desc, scene, ora
    scene.close()
    ora.close()


@pytest.fixture(scope="module")
def interior(native_lib, tmp_path_factory):
    from nanogi_gb300 import scenegen
    from oracle.oracle import OracleScene

    desc = scenegen.precision_interior(num_triangles=1_000_000)
    scene = _load_memory(desc, tmp_path_factory.mktemp("interior"), 1.0)
    scene.build()
    ora = OracleScene.from_desc(desc, 1.0)
    yield desc, scene, ora
    scene.close()
    ora.close()


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


def _ray_set(desc, ora, aspect, lo, hi, n_camera, n_random, seed):
    """Camera rays, random rays inside [lo, hi] and second-bounce rays off the camera hits."""
    rng = np.random.default_rng(seed)
    cam = camera_rays(desc, n_camera, aspect, rng)
    p, t, _ = ora.intersect(cam, use_bvh=True)
    bounce = bounce_rays(cam, p, t, rng)
    return {"camera": cam, "random": _random_rays(n_random, lo, hi, rng), "bounce": bounce}


def _check_scene(desc, scene, ora, aspect, lo, hi, n_camera, n_random, n_brute, seed):
    sets = _ray_set(desc, ora, aspect, lo, hi, n_camera, n_random, seed)
    total = 0
    for name, rays in sets.items():
        hits, ties = check_hits(scene.intersect(rays), ora.intersect(rays, use_bvh=True), f"{name}/bvh", rays=rays)
        total += len(rays)
        print(f"{name}: {len(rays)} rays, {hits} hits, {ties} ties")
    assert total >= 1_000_000
    # a subset against the brute force: every triangle tested, no acceleration structure
    rng = np.random.default_rng(seed + 1)
    sub = np.concatenate([r[rng.choice(len(r), n_brute // 3, replace=False)] for r in sets.values()])
    brute = ora.intersect(sub, use_bvh=False)
    check_hits(scene.intersect(sub), brute, "subset/brute", rays=sub)
    check_hits(ora.intersect(sub, use_bvh=True), brute, "oracle-bvh/brute", min_exact=1.0, rays=sub)


def test_intersect_terrain_full_scale(terrain):
    desc, scene, ora = terrain
    assert scene.info()["num_triangles"] == 1_546_250
    _check_scene(desc, scene, ora, TERRAIN_ASPECT, (-8.0, 0.0, -8.0), (8.0, 3.0, 8.0), 500_000, 300_000, 2048, 21)


def test_intersect_precision_interior_1m(interior):
    desc, scene, ora = interior
    assert scene.info()["num_triangles"] >= 1_000_000
    # random origins where the furniture and the finest floor tiles are (coordinates 1e-3..3)
    _check_scene(desc, scene, ora, 1.0, (-3.0, 0.0, -3.0), (3.0, 3.0, 3.0), 500_000, 300_000, 1536, 22)


def test_render_fp64_replays_oracle_terrain(terrain):
    import nanogi_gb300 as ng

    desc, scene, ora = terrain
    W, H, spp = 64, 36, 4
    film = ng.Renderer(renderer="ptdirect", num_samples=W * H * spp, max_num_vertices=16, width=W, height=H, seed=5,
                       precision="fp64").render(scene)
    ref = ora.render("ptdirect", num_samples=W * H * spp, max_vertices=16, width=W, height=H, seed=5,
                     rng_mode="replay", use_bvh=True)
    err = rel_rmse(film, ref)
    close = np.isclose(film, ref, rtol=1e-9, atol=1e-12).mean()
    print(f"terrain fp64 replay: rel-RMSE {err:.3e}, {close:.5f} of film values within 1e-9")
    assert float(ref.sum()) > 0
    assert err < 1e-6
    assert close > 0.995


def _z_parity(render_gpu, render_oracle, label, K=8):
    g = np.stack([render_gpu(100 + k) for k in range(K)])
    o = np.stack([render_oracle(200 + k) for k in range(K)])
    assert_same_expectation(g, o, label)


def test_fp32_statistical_parity_terrain(terrain):
    import nanogi_gb300 as ng

    desc, scene, ora = terrain
    W, H, spp = 48, 27, 128
    _z_parity(lambda s: ng.Renderer(renderer="ptdirect", num_samples=W * H * spp, max_num_vertices=16, width=W,
                                    height=H, seed=s, precision="fp32").render(scene),
              lambda s: ora.render("ptdirect", num_samples=W * H * spp, max_vertices=16, width=W, height=H, seed=s,
                                   rng_mode="reference", use_bvh=True), "terrain ptdirect")


@pytest.mark.parametrize("renderer", ["pt", "ptdirect"])
def test_fp32_statistical_parity_material_box(native_lib, tmp_path, renderer):
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen
    from oracle.oracle import OracleScene

    desc = scenegen.material_box()
    W, H, spp = 16, 16, 64
    scene = ng.Scene.load(scenegen.write_scene(desc, tmp_path), W / H)
    ora = OracleScene.from_desc(desc, W / H)
    _z_parity(lambda s: ng.Renderer(renderer=renderer, num_samples=W * H * spp, max_num_vertices=10, width=W,
                                    height=H, seed=s, precision="fp32").render(scene),
              lambda s: ora.render(renderer, num_samples=W * H * spp, max_vertices=10, width=W, height=H, seed=s,
                                   rng_mode="reference", use_bvh=True), f"material box {renderer}")
    scene.close()
