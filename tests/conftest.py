"""Shared fixtures. GPU tests are marked `gpu`; everything else runs on a CPU-only host."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def native_lib():
    """Builds (incrementally) and loads libnanogi.so."""
    from nanogi_gb300.build import build_library

    build_library()
    import nanogi_gb300 as ng

    return ng.load_library()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle.oracle import lib

    return lib()


@pytest.fixture(scope="session")
def cornell(tmp_path_factory):
    """The Cornell-box workload on disk plus its in-memory description."""
    from nanogi_gb300 import scenegen

    desc = scenegen.cornell_box()
    d = tmp_path_factory.mktemp("cornell")
    path = scenegen.write_scene(desc, d)
    return desc, path


def rel_rmse(a: np.ndarray, b: np.ndarray) -> float:
    return float(np.sqrt(((a - b) ** 2).sum() / max((b ** 2).sum(), 1e-300)))


def welch_z(gpu_films: np.ndarray, oracle_films: np.ndarray):
    """Per-pixel Welch z-scores of the mean of K independent GPU films against the mean of K
    independent oracle films (same expectation, different random numbers), over the pixels
    where either side has variance, and the same z-score for the image sum (every film's
    total, one value per film). Returns (per-value z, image-sum z, ratio of the mean sums)."""
    K1, K2 = len(gpu_films), len(oracle_films)
    mg, mo = gpu_films.mean(0), oracle_films.mean(0)
    se = np.sqrt(gpu_films.var(0, ddof=1) / K1 + oracle_films.var(0, ddof=1) / K2)
    ok = se > 0
    sg, so = gpu_films.reshape(K1, -1).sum(1), oracle_films.reshape(K2, -1).sum(1)
    se_sum = np.sqrt(sg.var(ddof=1) / K1 + so.var(ddof=1) / K2)
    z_sum = float((sg.mean() - so.mean()) / se_sum) if se_sum > 0 else 0.0
    return (mg[ok] - mo[ok]) / se[ok], z_sum, float(sg.mean() / max(so.mean(), 1e-300))


def assert_same_expectation(gpu_films: np.ndarray, oracle_films: np.ndarray, label: str = "") -> None:
    """GPU and oracle films estimate the same image: the per-value z-scores look like noise
    (mean near 0, few beyond 4) and the image sums agree within 4 standard errors."""
    z, z_sum, ratio = welch_z(gpu_films, oracle_films)
    print(f"{label}: z mean {z.mean():+.3f}, |z|>4 share {(np.abs(z) > 4).mean():.4f}, image-sum z {z_sum:+.2f}, "
          f"ratio {ratio:.4f}")
    assert abs(z.mean()) < 0.15, (label, z.mean())
    assert (np.abs(z) > 4.0).mean() < 0.01, label
    assert abs(z_sum) < 4.0, (label, z_sum)


def camera_rays(desc, n: int, aspect: float, rng, tmin: float = 1e-4) -> np.ndarray:
    """n rays (ox, oy, oz, tmin, dx, dy, dz, tmax) from the scene's pinhole eye through uniform
    raster positions of its vertical field of view: the directions a camera pass traces."""
    cam = None
    for p in desc.primitives:
        if "E" in p.type and p.params["E"]["type"] == "pinhole":
            cam = p.params["E"]["pinhole"]
    eye = np.asarray(cam["view"]["eye"], np.float64)
    fwd = np.asarray(cam["view"]["center"], np.float64) - eye
    fwd /= np.linalg.norm(fwd)
    right = np.cross(fwd, np.asarray(cam["view"]["up"], np.float64))
    right /= np.linalg.norm(right)
    up = np.cross(right, fwd)
    th = np.tan(np.radians(cam["perspective"]["fov"]) / 2)
    r = rng.uniform(0.0, 1.0, (n, 2))
    d = fwd + ((2 * r[:, :1] - 1) * th * aspect) * right + ((2 * r[:, 1:] - 1) * th) * up
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = eye.astype(np.float32)
    rays[:, 3] = tmin
    rays[:, 4:7] = d.astype(np.float32)
    rays[:, 7] = np.float32(3.4e38)
    return rays


def bounce_rays(rays: np.ndarray, prim: np.ndarray, t: np.ndarray, rng, tmin: float = 1e-4) -> np.ndarray:
    """Second-bounce rays: from the hit points of `rays` (where prim >= 0) in uniform random
    directions, as extension rays leave a surface."""
    hit = prim >= 0
    o = rays[hit, 0:3].astype(np.float64) + rays[hit, 4:7].astype(np.float64) * t[hit, None].astype(np.float64)
    d = rng.normal(size=o.shape)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    out = np.zeros((len(o), 8), np.float32)
    out[:, 0:3] = o.astype(np.float32)
    out[:, 3] = tmin
    out[:, 4:7] = d.astype(np.float32)
    out[:, 7] = np.float32(3.4e38)
    return out


T_REL_TOL = 1e-5  # hit-distance tolerance
# Two coplanar or touching triangles at a ray's hit return distances that differ by the rounding
# of the watertight test, which scales with the coordinates of the vertices and the ray origin, not
# with the distance: for a ray leaving a floor 1.5 mm below it, at coordinates near 3, that is a
# relative difference of about 2e-5. With the rays given, a tie may also differ by this many units
# of those coordinates' magnitude (a few FP32 ulps).
T_COORD_TOL = 4e-7


def check_hits(gpu, ora, label, max_tie_share=0.01, min_exact=0.999, rays=None):
    """First hits of the GPU traversal against the oracle's for the same rays.

    Hit / miss agree and primitive ids are bit-exact, except on ties: rays whose two answers lie
    at the same distance to within T_REL_TOL (or, given the rays, within T_COORD_TOL of the
    magnitude of the ray origin and hit point coordinates): coincident surfaces, such as a box
    standing on a floor, two overlapping coplanar triangles or two triangles sharing the edge the
    ray hits, where the watertight test's rounding or the traversal order picks one of them. Ties
    must stay below `max_tie_share`. Hit distances are within T_REL_TOL everywhere and
    bit-identical on at least `min_exact` of the rays where the ids agree; barycentrics agree to
    1e-6 there. Returns (hit rays compared, ties)."""
    gp, gt, guv = gpu
    op, ot, ouv = ora
    miss_agree = (gp < 0) == (op < 0)
    assert miss_agree.mean() > 0.9999, f"{label}: hit/miss disagree on {(~miss_agree).sum()} rays"
    both = (gp >= 0) & (op >= 0)
    same = gp[both] == op[both]
    tie = ~same
    diff = np.abs(gt[both].astype(np.float64) - ot[both])
    rel = diff / np.maximum(np.abs(ot[both]), 1e-30)
    tie_window = T_REL_TOL * np.abs(ot[both]).astype(np.float64)
    if rays is not None:
        r = np.asarray(rays, np.float64)[both]
        hit = r[:, 0:3] + r[:, 4:7] * ot[both, None].astype(np.float64)
        coord = np.maximum(np.abs(r[:, 0:3]).max(1), np.abs(hit).max(1))
        tie_window = np.maximum(tie_window, T_COORD_TOL * coord)
    bad = tie & (diff > tie_window)
    assert not bad.any(), (f"{label}: {bad.sum()} rays hit different primitives at different distances, e.g. "
                           f"gpu t={gt[both][bad][:3]} oracle t={ot[both][bad][:3]}")
    assert tie.mean() <= max_tie_share, f"{label}: {tie.sum()} of {both.sum()} rays resolve a tie differently"
    assert rel[same].max(initial=0.0) <= T_REL_TOL, f"{label}: max rel t error {rel[same].max()}"
    exact = (gt[both][same] == ot[both][same]).mean() if same.any() else 1.0
    assert exact >= min_exact, f"{label}: only {exact:.6f} of hit distances are bit-identical"
    if same.any():
        assert np.abs(guv[both][same] - ouv[both][same]).max() <= 1e-6
    return int(both.sum()), int(tie.sum())
