"""Textured albedo (TexR, rt.hpp:157-270) on the GPU.

The plain FP64 path replays the oracle on a box whose walls carry PNG, PPM, BMP and PFM
textures with tiled, negative uvs, and a glossy box with a textured G.R; the oracle takes the
texels from the arrays the files were written from, so the product's decoders are checked
too. The adjoint refuses textured scenes.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_rmse

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def textured(native_lib, tmp_path_factory):
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen
    from oracle.oracle import OracleScene

    desc = scenegen.textured_box()
    scene = ng.Scene.load(scenegen.write_scene(desc, tmp_path_factory.mktemp("tex")), 1.0)
    yield desc, scene, OracleScene.from_desc(desc, 1.0)
    scene.close()


@pytest.mark.parametrize("renderer", ["pt", "ptdirect", "ltdirect"])
def test_fp64_textured_paths_replay_the_oracle(textured, renderer):
    import nanogi_gb300 as ng

    desc, scene, ora = textured
    W = H = 16
    n = W * H * 16
    f = ng.Renderer(renderer=renderer, num_samples=n, max_num_vertices=8, width=W, height=H, seed=14,
                    precision="fp64").render(scene)
    ref = ora.render(renderer, num_samples=n, max_vertices=8, width=W, height=H, seed=14, rng_mode="replay",
                     use_bvh=False)
    assert ref.sum() > 0
    assert rel_rmse(f, ref) < 1e-6


def test_fp32_textured_matches_in_expectation(textured):
    import nanogi_gb300 as ng

    desc, scene, ora = textured
    W = H = 16
    n = W * H * 256
    f = ng.Renderer(renderer="ptdirect", num_samples=n, max_num_vertices=8, width=W, height=H, seed=15).render(scene)
    ref = ora.render("ptdirect", num_samples=n, max_vertices=8, width=W, height=H, seed=15, rng_mode="replay",
                     use_bvh=False)
    assert rel_rmse(f, ref) < 2e-3


def test_adjoint_refuses_textures(textured):
    import nanogi_gb300 as ng

    _, scene, _ = textured
    r = ng.Renderer(renderer="ptdirect", num_samples=64, max_num_vertices=6, width=8, height=8)
    with pytest.raises(ng.NanogiError) as e:
        r.backward(scene, np.zeros((8, 8, 3)))
    assert e.value.status == 7
