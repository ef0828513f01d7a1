"""GPU edge cases and statistical parity with the reference's own sampling (through the C ABI).

* Statistical parity: the tuned FP32 GPU path (Philox, pixel-stratified) against the oracle in
  reference mode (std::mt19937 per thread, uniform whole-image raster samples as in
  rt.hpp:735). Same expectation, different random numbers: per-pixel Welch z-scores over
  independent seeds must look like noise.
* Edge cases the reference's loop structure implies: max vertices 1 and 2, sample counts
  that are not a multiple of the pixel count, 1x1 films, empty scenes, sharded sample
  ranges, wave sizes and graph lengths that must not change the result.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import assert_same_expectation, rel_rmse

pytestmark = pytest.mark.gpu


def _scene(path, aspect):
    import nanogi_gb300 as ng

    return ng.Scene.load(path, aspect)


def _r(**kw):
    import nanogi_gb300 as ng

    return ng.Renderer(**kw)


@pytest.mark.parametrize("renderer", ["pt", "ptdirect"])
def test_statistical_parity_with_reference_sampling(native_lib, cornell, renderer):
    from oracle.oracle import OracleScene

    desc, path = cornell
    W, H, spp, K = 16, 16, 64, 8
    scene = _scene(path, W / H)
    ora = OracleScene.from_desc(desc, W / H)
    g = np.stack([_r(renderer=renderer, num_samples=W * H * spp, max_num_vertices=8, width=W, height=H,
                     seed=100 + k).render(scene) for k in range(K)])
    o = np.stack([ora.render(renderer, num_samples=W * H * spp, max_vertices=8, width=W, height=H, seed=200 + k,
                             rng_mode="reference") for k in range(K)])
    assert_same_expectation(g, o, f"cornell {renderer}")


@pytest.mark.parametrize("renderer", ["pt", "ptdirect"])
def test_max_vertices_one_and_two(native_lib, cornell, renderer):
    from oracle.oracle import OracleScene

    desc, path = cornell
    W, H = 12, 12
    scene = _scene(path, W / H)
    f1 = _r(renderer=renderer, num_samples=W * H * 4, max_num_vertices=1, width=W, height=H, seed=3).render(scene)
    assert not f1.any()  # the loop ends before the first vertex does anything
    f2 = _r(renderer=renderer, num_samples=W * H * 64, max_num_vertices=2, width=W, height=H, seed=3,
            precision="fp64").render(scene)
    ref = OracleScene.from_desc(desc, W / H).render(renderer, num_samples=W * H * 64, max_vertices=2, width=W,
                                                    height=H, seed=3, rng_mode="replay", use_bvh=False)
    assert rel_rmse(f2, ref) < 1e-9
    assert f2.any()  # the light is visible from the camera


@pytest.mark.parametrize("W,H,N", [(1, 1, 50), (3, 2, 7), (5, 4, 19), (8, 8, 64 * 3 + 5)])
def test_odd_sizes_replay_the_oracle(native_lib, cornell, W, H, N):
    from oracle.oracle import OracleScene

    desc, path = cornell
    scene = _scene(path, W / H)
    for renderer in ("pt", "ptdirect"):
        f = _r(renderer=renderer, num_samples=N, max_num_vertices=6, width=W, height=H, seed=9,
               precision="fp64").render(scene)
        ref = OracleScene.from_desc(desc, W / H).render(renderer, num_samples=N, max_vertices=6, width=W, height=H,
                                                        seed=9, rng_mode="replay", use_bvh=False)
        assert np.allclose(f, ref, rtol=1e-9, atol=1e-12), (renderer, W, H, N)


def test_uniform_raster_mode_replays_the_oracle(native_lib, cornell):
    from oracle.oracle import OracleScene

    desc, path = cornell
    W, H = 10, 10
    scene = _scene(path, W / H)
    f = _r(renderer="ptdirect", num_samples=W * H * 8, max_num_vertices=6, width=W, height=H, seed=4,
           precision="fp64", raster="uniform").render(scene)
    ref = OracleScene.from_desc(desc, W / H).render("ptdirect", num_samples=W * H * 8, max_vertices=6, width=W,
                                                    height=H, seed=4, rng_mode="replay", raster="uniform",
                                                    use_bvh=False)
    assert np.allclose(f, ref, rtol=1e-9, atol=1e-12)


def test_sample_ranges_add_up(native_lib, cornell):
    """film(0..k) + film(k..N) = film(0..N) for k on a whole pass (raw sums)."""
    desc, path = cornell
    W, H = 8, 6
    scene = _scene(path, W / H)
    wh = W * H
    N, k = wh * 10, wh * 4

    def raw(off, n):
        f = _r(renderer="ptdirect", num_samples=n, max_num_vertices=8, width=W, height=H, seed=21, sample_offset=off,
               precision="fp64").render(scene)
        return f * (n / wh)

    whole = raw(0, N)
    parts = raw(0, k) + raw(k, N - k)
    assert np.allclose(parts, whole, rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("knobs", [dict(wave_size=256), dict(wave_size=4096, iterations_per_graph=1),
                                   dict(wave_size=1 << 20, iterations_per_graph=16), dict(trace_refill=1),
                                   dict(trace_refill=32)])
def test_launch_shape_does_not_change_the_film(native_lib, cornell, knobs):
    desc, path = cornell
    W, H = 16, 16
    scene = _scene(path, W / H)
    base = _r(renderer="ptdirect", num_samples=W * H * 16, max_num_vertices=8, width=W, height=H, seed=8).render(scene)
    other = _r(renderer="ptdirect", num_samples=W * H * 16, max_num_vertices=8, width=W, height=H, seed=8,
               **knobs).render(scene)
    assert np.allclose(other, base, rtol=1e-9, atol=1e-12)


def test_pt_fused_and_queued_kernels_render_the_same_film(native_lib, cornell):
    """pt renders whose samples all fit in one wave run the queued shading and regeneration kernels;
    a wave smaller than the sample count keeps the fused kernel. Same paths, same film."""
    desc, path = cornell
    W, H = 16, 16
    scene = _scene(path, W / H)
    kw = dict(renderer="pt", num_samples=W * H * 32, max_num_vertices=8, width=W, height=H, seed=12)
    queued = _r(**kw).render(scene)
    fused = _r(wave_size=2048, **kw).render(scene)
    assert queued.sum() > 0
    np.testing.assert_allclose(queued, fused, rtol=1e-9, atol=1e-12)


def test_empty_and_lightless_scenes(native_lib, tmp_path):
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen

    s = scenegen.SceneDesc()
    s.primitives.append(scenegen.pinhole((0, 0, 5), (0, 0, 0), (0, 1, 0), 40))
    path = scenegen.write_scene(s, tmp_path / "empty")
    scene = ng.Scene.load(path, 1.0)
    f = _r(renderer="pt", num_samples=64, max_num_vertices=8, width=8, height=8).render(scene)
    assert not f.any()
    assert scene.info()["bvh_nodes"] == 0
    with pytest.raises(ng.NanogiError) as e:
        _r(renderer="ptdirect", num_samples=64, max_num_vertices=8, width=8, height=8).render(scene)
    assert e.value.status == 7
    # geometry but no light: pt renders black
    c = scenegen.cornell_box()
    c.primitives = [p for p in c.primitives if "L" not in p.type]
    scene2 = ng.Scene.load(scenegen.write_scene(c, tmp_path / "dark"), 1.0)
    f2 = _r(renderer="pt", num_samples=64 * 8, max_num_vertices=8, width=8, height=8).render(scene2)
    assert not f2.any()


def test_zero_samples_and_no_sensor(native_lib, tmp_path, cornell):
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen

    _, path = cornell
    scene = ng.Scene.load(path, 1.0)
    f = _r(renderer="pt", num_samples=0, max_num_vertices=8, width=4, height=4).render(scene)
    assert not f.any()
    c = scenegen.cornell_box()
    c.primitives = [p for p in c.primitives if "E" not in p.type]
    s2 = ng.Scene.load(scenegen.write_scene(c, tmp_path / "nocam"), 1.0)
    with pytest.raises(ng.NanogiError) as e:
        _r(renderer="pt", num_samples=16, width=4, height=4).render(s2)
    assert e.value.status == 1


def test_area_sensor_replays_the_oracle(native_lib, tmp_path):
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen
    from oracle.oracle import OracleScene

    desc = scenegen.area_sensor_box()
    W = H = 12
    scene = ng.Scene.load(scenegen.write_scene(desc, tmp_path), 1.0)
    for renderer in ("pt", "ptdirect"):
        f = _r(renderer=renderer, num_samples=W * H * 16, max_num_vertices=-1, width=W, height=H, seed=25,
               precision="fp64").render(scene)
        ref = OracleScene.from_desc(desc, 1.0).render(renderer, num_samples=W * H * 16, max_vertices=-1, width=W,
                                                      height=H, seed=25, rng_mode="replay", use_bvh=False)
        assert rel_rmse(f, ref) < 1e-6, renderer


def test_gpu_matches_committed_golden_films(native_lib, tmp_path):
    """The plain FP64 GPU path reproduces the oracle's committed golden films."""
    import json
    from pathlib import Path

    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen

    golden = Path(__file__).resolve().parent / "golden"
    meta = json.loads((golden / "films.json").read_text())
    for case in meta["cases"]:
        desc = scenegen.WORKLOADS[case["scene"]]()
        d = tmp_path / case["file"].replace(".npy", "")
        scene = ng.Scene.load(scenegen.write_scene(desc, d), case["width"] / case["height"])
        f = _r(renderer=case["renderer"], num_samples=case["num_samples"], max_num_vertices=case["max_vertices"],
               width=case["width"], height=case["height"], seed=case["seed"], precision="fp64").render(scene)
        ref = np.load(golden / case["file"])
        assert rel_rmse(f, ref) < 1e-4, case["file"]
        scene.close()


@pytest.mark.parametrize("scale", [1e-3, 1.0, 1e3])
def test_scaled_ray_offsets_replay_the_oracle(native_lib, tmp_path, scale):
    """ray_offset="scaled": the FP64 path replays the oracle's scaled-offset render of the Cornell
    box at 1e-3, 1 and 1e3 scene units, and the FP32 path gives the same image at every scale."""
    from nanogi_gb300 import scenegen
    from oracle.oracle import OracleScene

    W = H = 16
    n = W * H * 32
    desc = scenegen.transformed(scenegen.cornell_box(), scale)
    scene = _scene(scenegen.write_scene(desc, tmp_path), 1.0)
    f64 = _r(renderer="ptdirect", num_samples=n, max_num_vertices=8, width=W, height=H, seed=12, precision="fp64",
             ray_offset="scaled").render(scene)
    ref = OracleScene.from_desc(desc, 1.0).render("ptdirect", num_samples=n, max_vertices=8, width=W, height=H,
                                                  seed=12, rng_mode="replay", use_bvh=False, ray_offset="scaled")
    assert rel_rmse(f64, ref) < 1e-6
    unit = OracleScene.from_desc(scenegen.cornell_box(), 1.0).render(
        "ptdirect", num_samples=n, max_vertices=8, width=W, height=H, seed=12, rng_mode="replay", use_bvh=False,
        ray_offset="scaled")
    f32 = _r(renderer="ptdirect", num_samples=n, max_num_vertices=8, width=W, height=H, seed=12,
             ray_offset="scaled").render(scene)
    assert rel_rmse(f32, unit) < 1e-3


@pytest.mark.parametrize("renderer", ["pt", "ptdirect"])
def test_instrumented_renders_count_the_same_paths(native_lib, cornell, renderer):
    """Kernel timing and traversal counters change how a render is launched and observed, never
    what it computes: the film and every path count match the plain render of the same samples.
    The plain render also hands its last paths to the wave-end kernel, the others do not.
    The counts themselves are summed per block in shared memory, so they are checked against what
    the sample count implies."""
    from nanogi_gb300 import capi

    desc, path = cornell
    W, H, spp = 32, 32, 16
    scene = _scene(path, W / H)
    runs = {}
    for flags in (0, capi.KERNEL_TIMING, capi.TRAVERSAL_COUNTERS):
        r = _r(renderer=renderer, num_samples=W * H * spp, max_num_vertices=8, width=W, height=H, seed=7,
               wave_size=4096, flags=flags)
        film = r.render(scene)
        runs[flags] = (film, dict(r.last_stats))
    film0, st0 = runs[0]
    assert st0["camera_rays"] == W * H * spp
    if renderer == "pt":
        assert st0["extension_rays"] >= st0["camera_rays"]
    else:
        # ptdirect does not trace toward a hit that Russian roulette or the length limit ends
        assert 0 < st0["extension_rays"] < st0["camera_rays"]
    assert st0["film_contributions"] > 0
    if renderer == "ptdirect":
        assert st0["shadow_rays"] > 0
    for flags, (film, st) in runs.items():
        np.testing.assert_allclose(film, film0, rtol=1e-9, atol=1e-12)
        # (iterations differ: graph launches run whole groups of iterations, timed runs stop at the last)
        for k in ("camera_rays", "extension_rays", "shadow_rays", "film_contributions"):
            assert st[k] == st0[k], (flags, k)
    # the plain render ends with the wave-end launch (one thread per remaining path); the timed
    # one drains through the wavefront kernels alone, and both films are equal
    assert 0 < st0["finish_paths"] <= 4096
    assert runs[capi.KERNEL_TIMING][1]["finish_paths"] == 0
    assert runs[capi.TRAVERSAL_COUNTERS][1]["finish_paths"] == 0
    st_t = runs[capi.KERNEL_TIMING][1]
    assert st_t["logic_launches"] == st_t["extend_launches"] == st_t["iterations"]
    assert st_t["shadow_launches"] == 0  # one traversal launch traces both queues
    assert st_t["logic_ms"] > 0 and st_t["extend_ms"] > 0 and st_t["shadow_ms"] == 0
    st_c = runs[capi.TRAVERSAL_COUNTERS][1]
    assert st_c["extend_nodes"] >= st_c["extension_rays"] > 0
    assert st_c["extend_tris"] > 0
    if renderer == "ptdirect":
        assert st_c["shadow_nodes"] > 0


@pytest.mark.parametrize("renderer", ["ptdirect", "ltdirect"])
def test_untraced_dead_rays_leave_the_film_unchanged(native_lib, cornell, renderer):
    """Skipping the extension rays whose hit Russian roulette or the length limit ends changes the
    rays traced, never the film: the default render equals the one that traces every ray."""
    from nanogi_gb300 import capi

    desc, path = cornell
    W, H, spp = 24, 24, 32
    scene = _scene(path, W / H)
    films, stats = [], []
    for flags in (0, capi.TRACE_ALL_RAYS):
        for m in (8, 3):
            r = _r(renderer=renderer, num_samples=W * H * spp, max_num_vertices=m, width=W, height=H, seed=11,
                   wave_size=8192, flags=flags)
            films.append(r.render(scene))
            stats.append(dict(r.last_stats))
    for k in range(2):
        np.testing.assert_allclose(films[k], films[k + 2], rtol=1e-9, atol=1e-12)
        assert stats[k]["film_contributions"] == stats[k + 2]["film_contributions"]
        assert stats[k]["shadow_rays"] == stats[k + 2]["shadow_rays"]
        assert stats[k]["extension_rays"] < stats[k + 2]["extension_rays"]
    if renderer == "ptdirect":
        # with every ray traced, each sample traces its camera ray
        assert stats[2]["extension_rays"] >= W * H * spp


def test_release_buffers_between_renders(native_lib, cornell):
    """A handle that released its render buffers renders the same film again (it allocates anew)."""
    desc, path = cornell
    W, H = 16, 16
    scene = _scene(path, W / H)
    r = _r(renderer="ptdirect", num_samples=W * H * 16, max_num_vertices=6, width=W, height=H, seed=5)
    a = r.render(scene)
    scene.release_buffers()
    scene.release_buffers()  # releasing twice is harmless
    b = r.render(scene)
    np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-12)
