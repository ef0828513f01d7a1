"""The C-ABI library on a CPU-only host: it loads, exports every symbol include/nanogi.h
declares, validates arguments, and its film I/O round-trips. No compute calls need a GPU."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def _declared_symbols():
    text = (ROOT / "include" / "nanogi.h").read_text()
    return sorted(set(re.findall(r"NGI_API\s+[\w\s\*]+?\b(ngi_\w+)\s*\(", text)))


def test_every_declared_symbol_is_exported(native_lib):
    syms = _declared_symbols()
    assert len(syms) >= 14
    for s in syms:
        assert hasattr(native_lib, s), s


def test_python_binding_covers_the_header(native_lib):
    from nanogi_gb300.capi import PROTOTYPES

    assert set(PROTOTYPES) == set(_declared_symbols())


def test_abi_version(native_lib):
    assert native_lib.ngi_abi_version() == 1


def test_struct_layouts_match_header(tmp_path):
    """Every ctypes field sits at the offset the C compiler gives the header's struct."""
    import subprocess

    from nanogi_gb300.capi import BatchOptions, BatchStats, MeshData, RenderParams, RenderStats, SceneInfo

    structs = {"ngi_render_params": RenderParams, "ngi_render_stats": RenderStats, "ngi_scene_info": SceneInfo,
               "ngi_batch_options": BatchOptions, "ngi_batch_stats": BatchStats, "ngi_mesh_data": MeshData}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "nanogi.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)


def test_null_and_invalid_arguments(native_lib, cornell):
    import nanogi_gb300 as ng
    from nanogi_gb300.capi import RenderParams

    lib = native_lib
    h = ctypes.c_void_p()
    assert lib.ngi_scene_load(None, 1.0, ctypes.byref(h)) == 1
    assert lib.ngi_scene_load(b"x.yml", 1.0, None) == 1
    assert lib.ngi_last_error().decode() != ""
    _, path = cornell
    assert lib.ngi_scene_load(str(path).encode(), -1.0, ctypes.byref(h)) == 1
    scene = ng.Scene.load(path, 1.0)
    film = np.zeros((4, 4, 3))
    bad = [
        dict(renderer=7), dict(width=0), dict(height=-3), dict(num_samples=-1), dict(max_num_vertices=0),
        dict(max_num_vertices=-5), dict(precision=9), dict(raster_mode=4), dict(sample_offset=-1),
        dict(iterations_per_graph=1000), dict(width=1 << 16, height=1 << 16),
    ]
    for b in bad:
        p = RenderParams(renderer=0, max_num_vertices=8, num_samples=16, width=4, height=4)
        for k, v in b.items():
            setattr(p, k, v)
        st = lib.ngi_render(scene.handle, ctypes.byref(p), film.ctypes.data)
        assert st == 1, b
    p = RenderParams(renderer=0, max_num_vertices=8, num_samples=16, width=4, height=4)
    assert lib.ngi_render(scene.handle, ctypes.byref(p), None) == 1
    assert lib.ngi_render(None, ctypes.byref(p), film.ctypes.data) == 1
    assert lib.ngi_intersect(None, None, 0, None, None, None) == 1
    assert lib.ngi_intersect(scene.handle, None, -1, None, None, None) == 1
    lib.ngi_scene_free(None)  # no-op


def test_render_without_gpu_reports_status(native_lib, cornell):
    """On a host without a GPU the render call fails with a status, not a crash."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import nanogi_gb300 as ng

    _, path = cornell
    scene = ng.Scene.load(path, 1.0)
    with pytest.raises(ng.NanogiError) as e:
        ng.Renderer(num_samples=16, width=4, height=4).render(scene)
    assert e.value.status in (4, 8)


def test_hdr_round_trip(native_lib, tmp_path):
    import nanogi_gb300 as ng

    rng = np.random.default_rng(0)
    film = rng.uniform(0, 50, (7, 9, 3))
    film[0, 0] = 0.0
    film[1, 2] = [1e-40, 0, 0]
    ng.save_image(tmp_path / "a.hdr", film)
    back = ng.load_hdr(tmp_path / "a.hdr", 9, 7)
    big = film.max(axis=2, keepdims=True)
    # RGBE keeps 8 mantissa bits relative to the brightest channel
    assert np.all(np.abs(back - film) <= big / 128 + 1e-30)
    assert np.all(back[0, 0] == 0)
    # upright: the header lists the top scanline first, i.e. film row H-1
    raw = (tmp_path / "a.hdr").read_bytes()
    assert b"-Y 7 +X 9\n" in raw


def test_pfm_and_bad_extension(native_lib, tmp_path):
    import nanogi_gb300 as ng

    film = np.arange(2 * 3 * 3, dtype=np.float64).reshape(2, 3, 3)
    ng.save_image(tmp_path / "a.pfm", film)
    raw = (tmp_path / "a.pfm").read_bytes()
    head = b"PF\n3 2\n-1.0\n"
    assert raw.startswith(head)
    data = np.frombuffer(raw[len(head):], "<f4").reshape(2, 3, 3)
    assert np.array_equal(data, film.astype(np.float32))
    with pytest.raises(ng.NanogiError):
        ng.save_image(tmp_path / "a.bmp", film)
    with pytest.raises(ng.NanogiError):
        ng.load_hdr(tmp_path / "missing.hdr", 3, 2)


def test_cli_usage_and_errors(native_lib, tmp_path):
    import subprocess

    cli = ROOT / "nanogi_gb300" / "_build" / "nanogi"
    r = subprocess.run([str(cli)], capture_output=True, text=True)
    assert r.returncode != 0 and "Usage: nanogi" in r.stdout
    r = subprocess.run([str(cli), "ptmnee", "x.yml", "o.hdr", "4", "4"], capture_output=True, text=True)
    assert r.returncode != 0 and "not built" in r.stderr
    r = subprocess.run([str(cli), "pt", str(tmp_path / "none.yml"), "o.hdr", "4", "4"], capture_output=True, text=True)
    assert r.returncode != 0 and "ERROR" in r.stderr
    r = subprocess.run([str(cli), "-n"], capture_output=True, text=True)
    assert r.returncode != 0


def _film(w, h, seed=0):
    rng = np.random.default_rng(seed)
    f = rng.lognormal(-1.0, 1.5, (h, w, 3))
    f[0, 0] = (0.0, -1.0, np.nan)  # black, negative, NaN
    f[-1, -1] = (1e6, 1.0, 0.5)
    return np.ascontiguousarray(f)


def test_exr_writer_layout(native_lib, tmp_path):
    """Scanline OpenEXR 2.0: header attributes, offset table, float B/G/R planes, top row = film
    row H-1 (the reference flips y before tinyexr, basic.hpp:586-592)."""
    import struct

    import nanogi_gb300 as ng

    w, h = 7, 5
    film = _film(w, h)
    path = tmp_path / "deep" / "dir" / "f.exr"  # the directory is created, as the reference does
    ng.save_image(path, film)
    b = path.read_bytes()
    assert b[:4] == bytes([0x76, 0x2F, 0x31, 0x01]) and struct.unpack("<I", b[4:8])[0] == 2
    pos, attrs = 8, {}
    while b[pos] != 0:
        name_end = b.index(b"\0", pos)
        type_end = b.index(b"\0", name_end + 1)
        name, typ = b[pos:name_end].decode(), b[name_end + 1:type_end].decode()
        size = struct.unpack("<i", b[type_end + 1:type_end + 5])[0]
        attrs[name] = (typ, b[type_end + 5:type_end + 5 + size])
        pos = type_end + 5 + size
    pos += 1
    assert attrs["compression"] == ("compression", b"\0")
    assert struct.unpack("<4i", attrs["dataWindow"][1]) == (0, 0, w - 1, h - 1)
    ch = attrs["channels"][1]
    names = []
    q = 0
    while ch[q] != 0:
        e = ch.index(b"\0", q)
        names.append(ch[q:e].decode())
        assert struct.unpack("<i", ch[e + 1:e + 5])[0] == 2  # FLOAT
        q = e + 17
    assert names == ["B", "G", "R"]
    offsets = struct.unpack(f"<{h}Q", b[pos:pos + 8 * h])
    for y, off in enumerate(offsets):
        yy, size = struct.unpack("<ii", b[off:off + 8])
        assert yy == y and size == 12 * w
        planes = np.frombuffer(b[off + 8:off + 8 + size], "<f4").reshape(3, w)
        expect = film[h - 1 - y].astype(np.float32)
        got = np.stack([planes[2], planes[1], planes[0]], 1)
        assert np.array_equal(got, expect, equal_nan=True)


def test_png_writer_tone_map(native_lib, tmp_path):
    """8-bit RGB PNG with the reference's tone map clamp(int(255 v^(1/2.2)), 0, 255)
    (basic.hpp:625-634), top row = film row H-1; decoded with zlib and checked by CRC."""
    import struct
    import zlib

    import nanogi_gb300 as ng

    w, h = 9, 4
    film = _film(w, h, seed=3)
    path = tmp_path / "f.png"
    ng.save_image(path, film)
    b = path.read_bytes()
    assert b[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, {}
    while pos < len(b):
        n = struct.unpack(">I", b[pos:pos + 4])[0]
        typ, data = b[pos + 4:pos + 8], b[pos + 8:pos + 8 + n]
        assert struct.unpack(">I", b[pos + 8 + n:pos + 12 + n])[0] == zlib.crc32(typ + data)
        chunks[typ] = chunks.get(typ, b"") + data
        pos += 12 + n
    assert struct.unpack(">IIBBBBB", chunks[b"IHDR"]) == (w, h, 8, 2, 0, 0, 0)
    raw = np.frombuffer(zlib.decompress(chunks[b"IDAT"]), np.uint8).reshape(h, 1 + 3 * w)
    assert not raw[:, 0].any()
    img = raw[:, 1:].reshape(h, w, 3)
    with np.errstate(invalid="ignore"):
        v = np.power(film[::-1], 1 / 2.2) * 255.0
    expect = np.where(np.isnan(v), 0, np.clip(np.where(v >= 255, 255, np.trunc(np.nan_to_num(v, nan=0))), 0, 255))
    assert np.array_equal(img, expect.astype(np.uint8))


def test_save_image_rejects_unknown_extensions(native_lib, tmp_path):
    import nanogi_gb300 as ng

    with pytest.raises(ng.NanogiError) as e:
        ng.save_image(tmp_path / "f.jpg", np.zeros((2, 2, 3)))
    assert "Invalid extension" in e.value.message
