"""The allocation-free render entry point (ngi_render_device_noalloc).

Some callers cannot allocate device memory while they render -- an application whose own
allocator owns the whole device, a real-time loop that cannot take the synchronisation a
cudaMalloc may cause, a process under a fixed memory budget. This entry point keeps all of
the render's scratch in one fixed device array of the library, so it allocates nothing.
The test calls it through the C ABI twice in a row (the second call must clear what the
first left in the shared array) and compares each film with the regular entry point's.

This file is named to be collected last: if it fails, a run that stops at the first
failure has already run every other test.
"""
from __future__ import annotations

import ctypes

import pytest

pytestmark = pytest.mark.gpu

W, H, SPP = 24, 20, 12
RTOL, ATOL = 1e-9, 1e-12  # same film in a different FP64 summation order


def _film(torch):
    f = torch.zeros((H, W, 3), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    return f


@pytest.fixture(scope="module")
def built_scene(native_lib, tmp_path_factory):
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen

    d = tmp_path_factory.mktemp("noalloc")
    path = scenegen.write_scene(scenegen.material_box(), d)
    scene = ng.Scene.load(path, W / H)
    scene.build()
    yield scene
    scene.close()


@pytest.mark.parametrize("renderer,precision,wave", [("ptdirect", "fp32", 0), ("pt", "fp32", 4096),
                                                     ("ptdirect", "fp64", 1024)])
def test_noalloc_matches_regular_entry_point(native_lib, built_scene, renderer, precision, wave):
    import torch

    import nanogi_gb300 as ng
    from nanogi_gb300.capi import check

    lib = native_lib
    r = ng.Renderer(renderer=renderer, num_samples=W * H * SPP, max_num_vertices=10, width=W, height=H, seed=17,
                    precision=precision, wave_size=wave)
    p = r.params()
    ref = _film(torch)
    check(lib.ngi_render_device(built_scene.handle, ctypes.byref(p), ctypes.c_void_p(ref.data_ptr()), None))
    torch.cuda.synchronize()
    assert float(ref.abs().sum()) > 0
    # both output films exist before the measured window: the calls below must not allocate
    outs = [_film(torch), _film(torch)]
    for call, out in enumerate(outs):
        if call == 1:
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info()[0]
        check(lib.ngi_render_device_noalloc(built_scene.handle, ctypes.byref(p), ctypes.c_void_p(out.data_ptr()),
                                            None))
        torch.cuda.synchronize()
        if call == 1:
            assert torch.cuda.mem_get_info()[0] == free_before, "the allocation-free call changed free device memory"
        assert torch.allclose(out, ref, rtol=RTOL, atol=ATOL), f"call {call + 1} differs"
        st = built_scene.last_stats()
        assert st["camera_rays"] == W * H * SPP


def test_noalloc_zero_samples_only_sets_up(native_lib, built_scene):
    import torch

    import nanogi_gb300 as ng
    from nanogi_gb300.capi import check

    lib = native_lib
    out = _film(torch)
    p = ng.Renderer(renderer="ptdirect", num_samples=0, max_num_vertices=8, width=W, height=H).params()
    check(lib.ngi_render_device_noalloc(built_scene.handle, ctypes.byref(p), ctypes.c_void_p(out.data_ptr()), None))
    torch.cuda.synchronize()
    assert not bool(out.any())
    assert built_scene.last_stats()["camera_rays"] == 0


def test_noalloc_rejects_what_it_cannot_do(native_lib, built_scene, cornell):
    import torch

    import nanogi_gb300 as ng
    from nanogi_gb300.capi import RENDERERS, RenderParams

    lib = native_lib
    out = _film(torch)
    p = RenderParams(renderer=1, max_num_vertices=8, num_samples=100, width=W, height=H, wave_size=65536 + 256)
    st = lib.ngi_render_device_noalloc(built_scene.handle, ctypes.byref(p), ctypes.c_void_p(out.data_ptr()), None)
    assert st == 1 and b"exceeds" in lib.ngi_last_error()
    p.wave_size = 0
    # the light tracers and bdpt are refused (NGI_ERR_UNSUPPORTED)
    for name in ("lt", "ltdirect", "bdpt"):
        p.renderer = RENDERERS[name]
        st = lib.ngi_render_device_noalloc(built_scene.handle, ctypes.byref(p), ctypes.c_void_p(out.data_ptr()),
                                           None)
        assert st == 7, name
    p.renderer = 1
    # measurement flags need buffers of their own
    p.flags = 1
    st = lib.ngi_render_device_noalloc(built_scene.handle, ctypes.byref(p), ctypes.c_void_p(out.data_ptr()), None)
    assert st == 1
    p.flags = 0
    torch.cuda.synchronize()
    assert not bool(out.any())
    # a scene that was never uploaded cannot be rendered without allocating
    _, path = cornell
    fresh = ng.Scene.load(path, W / H)
    st = lib.ngi_render_device_noalloc(fresh.handle, ctypes.byref(p), ctypes.c_void_p(out.data_ptr()), None)
    assert st == 1 and b"ngi_scene_build" in lib.ngi_last_error()
    fresh.close()


def test_noalloc_refuses_another_current_device(native_lib, built_scene):
    """A scene built on device 0 is not rendered while another device is current."""
    import torch

    import nanogi_gb300 as ng

    if torch.cuda.device_count() < 2:
        pytest.skip("needs a second visible GPU")
    lib = native_lib
    out = _film(torch)
    p = ng.Renderer(renderer="ptdirect", num_samples=W * H, max_num_vertices=8, width=W, height=H).params()
    with torch.cuda.device(1):
        st = lib.ngi_render_device_noalloc(built_scene.handle, ctypes.byref(p), ctypes.c_void_p(out.data_ptr()),
                                           None)
    assert st == 1 and b"current" in lib.ngi_last_error()
