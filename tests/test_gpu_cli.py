"""The nanogi command line on the GPU: renderer names, the time budget and progress images
(src/nanogi.cpp:356-404, 2000-2023), and that its film is the library's film for the same
parameters (`-n` is the total number of samples, nanogi.cpp:2006)."""
from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent


@pytest.mark.parametrize("renderer,ext", [("pt", ".hdr"), ("ptdirect", ".exr"), ("ltdirect", ".png"), ("bdpt", ".pfm")])
def test_cli_renders_every_format(native_lib, cornell, tmp_path, renderer, ext):
    _, path = cornell
    out = tmp_path / "out" / f"img{ext}"
    cli = ROOT / "nanogi_gb300" / "_build" / "nanogi"
    r = subprocess.run([str(cli), renderer, str(path), str(out), "16", "12", "-n", "20000", "-m", "6", "--seed", "3"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert out.stat().st_size > 0


def test_cli_time_budget_writes_progress_images(native_lib, cornell, tmp_path):
    import nanogi_gb300 as ng

    _, path = cornell
    cli = ROOT / "nanogi_gb300" / "_build" / "nanogi"
    fmt = str(tmp_path / "progress" / "{{count}}.hdr")
    out = tmp_path / "final.hdr"
    r = subprocess.run([str(cli), "ptdirect", str(path), str(out), "32", "32", "-t", "1.0", "-m", "6",
                        "--progress-image-update-interval", "0.2", "--progress-image-update-format", fmt],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    images = sorted((tmp_path / "progress").glob("*.hdr"))
    assert len(images) >= 2
    assert images[0].name == "0000000001.hdr"
    last = ng.load_hdr(images[-1], 32, 32)
    final = ng.load_hdr(out, 32, 32)
    assert last.mean() > 0 and abs(last.mean() / final.mean() - 1) < 0.2


@pytest.mark.parametrize("renderer", ["pt", "ptdirect"])
def test_cli_film_matches_the_library(native_lib, cornell, tmp_path, renderer):
    import nanogi_gb300 as ng

    _, path = cornell
    W, H, N = 16, 12, 16 * 12 * 20 + 7
    out = tmp_path / "film.pfm"
    cli = ROOT / "nanogi_gb300" / "_build" / "nanogi"
    r = subprocess.run([str(cli), renderer, str(path), str(out), str(W), str(H), "-n", str(N), "-m", "6", "--seed",
                        "3", "--precision", "fp64"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    cli_film = ng.load_texture(out)[::-1].astype(np.float64)  # PFM rows read top first; film row 0 = bottom
    scene = ng.Scene.load(path, W / H)
    lib_film = ng.Renderer(renderer=renderer, num_samples=N, max_num_vertices=6, width=W, height=H, seed=3,
                           precision="fp64").render(scene)
    scene.close()
    assert float(lib_film.sum()) > 0
    # the .pfm holds float32: the same film to float rounding
    assert np.allclose(cli_film, lib_film.astype(np.float32).astype(np.float64), rtol=1e-6, atol=1e-7)
