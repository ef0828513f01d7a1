"""Path-replay adjoint (ngi_render_backward) against finite differences.

Workload: the inverse-rendering box -- 64 diffuse material groups and 2 emitters -- rendered
with `ptdirect` (and `pt`). Loss = sum over the film of (render - target)^2, the target
rendered with hidden parameters. Gradients w.r.t. every albedo and emitter radiance are
checked against central finite differences (h = 1e-3) with common random numbers:
  * on the GPU forward path itself (same Philox paths for +h and -h);
  * on the CPU oracle's forward path (the reference algorithm restated), the finite-difference
    gradient "from the reference renderer".
Only the test harness wraps the ABI pair in a torch.autograd.Function.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

H_FD = 1e-3
W = H = 24
SPP = 16
M = 8


@pytest.fixture(scope="module")
def inverse_setup(native_lib, tmp_path_factory):
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen

    desc = scenegen.inverse_box(seed=5, emitter_seed=7)
    hidden = scenegen.inverse_box(seed=6, emitter_seed=8)
    d = tmp_path_factory.mktemp("inverse")
    scene = ng.Scene.load(scenegen.write_scene(desc, d), W / H)
    theta_a, theta_e = scene.parameters()
    hid = ng.Scene.load(scenegen.write_scene(hidden, tmp_path_factory.mktemp("hidden")), W / H)
    ha, he = hid.parameters()
    hid.close()
    yield scene, desc, (theta_a, theta_e), (ha, he)
    scene.close()


def _renderer(renderer, precision, seed=31):
    import nanogi_gb300 as ng

    return ng.Renderer(renderer=renderer, num_samples=W * H * SPP, max_num_vertices=M, width=W, height=H, seed=seed,
                       precision=precision)


def _loss_and_grad(scene, r, target):
    img = r.render(scene)
    loss = float(((img - target) ** 2).sum())
    ga, ge = r.backward(scene, 2.0 * (img - target))
    return img, loss, ga, ge


def _fd(scene, r, target, base_a, base_e, which, idx):
    a, e = base_a.copy(), base_e.copy()
    arr = a if which == "a" else e
    v0 = arr.flat[idx]
    out = []
    for s in (+1, -1):
        arr.flat[idx] = v0 + s * H_FD
        scene.set_parameters(a, e)
        img = r.render(scene)
        out.append(float(((img - target) ** 2).sum()))
    arr.flat[idx] = v0
    scene.set_parameters(a, e)
    return (out[0] - out[1]) / (2 * H_FD)


def _compare(ad, fd, label):
    ad, fd = np.asarray(ad), np.asarray(fd)
    big = np.abs(fd) > 1e-3 * np.abs(fd).max()
    rel = np.abs(ad[big] - fd[big]) / np.abs(fd[big])
    assert rel.max() < 1e-2, f"{label}: max rel err {rel.max():.3e}"
    cos = float(ad @ fd / (np.linalg.norm(ad) * np.linalg.norm(fd)))
    assert cos > 0.9999, f"{label}: cosine {cos}"


@pytest.mark.parametrize("renderer,precision", [("ptdirect", "fp32"), ("pt", "fp32"), ("ptdirect", "fp64")])
def test_adjoint_matches_central_differences(inverse_setup, renderer, precision):
    scene, desc, (ta, te), (ha, he) = inverse_setup
    r = _renderer(renderer, precision)
    scene.set_parameters(ha, he)
    target = _renderer(renderer, precision, seed=77).render(scene)
    scene.set_parameters(ta, te)
    img, loss, ga, ge = _loss_and_grad(scene, r, target)
    assert loss > 0
    mats = [i for i, p in enumerate(desc.primitives) if p.type == ["D"]]
    lights = [i for i, p in enumerate(desc.primitives) if "L" in p.type]
    assert len(mats) == 64 and len(lights) == 2
    ad, fd = [], []
    for m in mats:
        for c in range(3):
            ad.append(ga[m, c])
            fd.append(_fd(scene, r, target, ta, te, "a", 3 * m + c))
    for l in lights:
        for c in range(3):
            ad.append(ge[l, c])
            fd.append(_fd(scene, r, target, ta, te, "e", 3 * l + c))
    _compare(ad, fd, f"{renderer}/{precision}")
    # primitives that are not parameters get no gradient
    assert not ga[lights].any() and not ge[mats].any()


def test_adjoint_matches_oracle_finite_differences(inverse_setup):
    """FD gradient of the reference algorithm (the oracle, same Philox paths) vs the GPU adjoint."""
    import copy

    from nanogi_gb300 import scenegen
    from oracle.oracle import OracleScene

    scene, desc, (ta, te), (ha, he) = inverse_setup
    w = h = 12
    spp = 8
    kw = dict(num_samples=w * h * spp, max_vertices=M, width=w, height=h, seed=41, rng_mode="replay", use_bvh=False)

    def ora_render(d):
        return OracleScene.from_desc(d, 1.0).render("ptdirect", **kw)

    hidden = scenegen.inverse_box(seed=6, emitter_seed=8)
    target = ora_render(hidden)
    import nanogi_gb300 as ng

    r = ng.Renderer(renderer="ptdirect", num_samples=w * h * spp, max_num_vertices=M, width=w, height=h, seed=41,
                    precision="fp64")
    scene.set_parameters(ta, te)
    img = r.render(scene)
    ga, ge = r.backward(scene, 2.0 * (img - target))
    checks = [(10, 0), (20, 1), (33, 2), (50, 0), (64, 1)]  # (primitive, channel) of D groups
    for prim, c in checks:
        vals = []
        for s in (+1, -1):
            d2 = copy.deepcopy(desc)
            d2.primitives[prim].params["D"]["R"][c] += s * H_FD
            f = ora_render(d2)
            vals.append(float(((f - target) ** 2).sum()))
        fd = (vals[0] - vals[1]) / (2 * H_FD)
        assert abs(ga[prim, c] - fd) <= 1e-2 * abs(fd) + 1e-9, (prim, c, ga[prim, c], fd)
    for prim in (0, 1):
        for c in range(3):
            vals = []
            for s in (+1, -1):
                d2 = copy.deepcopy(desc)
                d2.primitives[prim].params["L"]["area"]["Le"][c] += s * H_FD
                vals.append(float(((ora_render(d2) - target) ** 2).sum()))
            fd = (vals[0] - vals[1]) / (2 * H_FD)
            assert abs(ge[prim, c] - fd) <= 1e-2 * abs(fd) + 1e-9, (prim, c, ge[prim, c], fd)


def test_torch_autograd_wrapper(inverse_setup):
    """forward/backward pair wrapped as a torch.autograd.Function (test harness only)."""
    import torch

    scene, desc, (ta, te), (ha, he) = inverse_setup
    r = _renderer("ptdirect", "fp32")

    class Render(torch.autograd.Function):
        @staticmethod
        def forward(ctx, albedo, emission):
            scene.set_parameters(albedo.detach().numpy(), emission.detach().numpy())
            return torch.from_numpy(r.render(scene).copy())

        @staticmethod
        def backward(ctx, grad):
            ga, ge = r.backward(scene, grad.contiguous().numpy())
            return torch.from_numpy(ga), torch.from_numpy(ge)

    scene.set_parameters(ha, he)
    target = torch.from_numpy(r.render(scene).copy())
    a = torch.tensor(ta, requires_grad=True)
    e = torch.tensor(te, requires_grad=True)
    loss = ((Render.apply(a, e) - target) ** 2).sum()
    loss.backward()
    scene.set_parameters(ta, te)
    img = r.render(scene)
    ga, ge = r.backward(scene, 2.0 * (img - target.numpy()))
    # gradients are summed per block in FP32 in atomic order: two replays agree to ~1e-6
    assert np.allclose(a.grad.numpy(), ga, rtol=1e-4, atol=1e-6 * np.abs(ga).max())
    assert np.allclose(e.grad.numpy(), ge, rtol=1e-4, atol=1e-6 * np.abs(ge).max())
    # one gradient step lowers the loss
    with torch.no_grad():
        a2 = (a - 1e-4 * a.grad / a.grad.abs().max()).clamp(0.0, 1.0)
    loss2 = ((Render.apply(a2, e.detach()) - target) ** 2).sum()
    assert float(loss2.detach()) < float(loss.detach())
    scene.set_parameters(ta, te)


def test_backward_rejects_unbounded_paths(inverse_setup):
    import nanogi_gb300 as ng

    scene, *_ = inverse_setup
    r = ng.Renderer(renderer="ptdirect", num_samples=64, max_num_vertices=-1, width=8, height=8)
    with pytest.raises(ng.NanogiError) as e:
        r.backward(scene, np.zeros((8, 8, 3)))
    assert e.value.status == 7
