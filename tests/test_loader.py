"""Scene loading through the C ABI on a CPU-only host (Scene::Load, rt.hpp:1519-2154).

The flattened arrays the product builds from YAML + OBJ files must equal the in-memory
description the files were written from, and malformed inputs must come back as status
codes with a message -- never an abort.
"""
from __future__ import annotations

import numpy as np
import pytest


def _load(native_lib, path, aspect=1.0):
    import nanogi_gb300 as ng

    return ng.Scene.load(path, aspect)


@pytest.mark.parametrize("workload", ["cornell_box", "material_box", "area_sensor_box"])
def test_flattened_arrays_match_description(native_lib, tmp_path, workload):
    from nanogi_gb300 import scenegen
    from oracle.oracle import flatten

    desc = scenegen.WORKLOADS[workload]()
    path = scenegen.write_scene(desc, tmp_path)
    s = _load(native_lib, path)
    info = s.info()
    _, pos, nrm, uv = flatten([(p.type, p.params, p.mesh) for p in desc.primitives])
    assert info["num_triangles"] == len(pos)
    assert info["num_primitives"] == len(desc.primitives)
    assert info["num_lights"] == sum("L" in p.type for p in desc.primitives)
    assert info["sensor_index"] == max(i for i, p in enumerate(desc.primitives) if "E" in p.type)
    P, N, U, prim = s.triangles()
    assert np.array_equal(P.reshape(-1, 9), pos)  # float32 round trip through the OBJ text
    assert np.array_equal(N.reshape(-1, 9), nrm)
    assert np.array_equal(U.reshape(-1, 6), uv)
    counts = np.bincount(prim, minlength=len(desc.primitives))
    for i, p in enumerate(desc.primitives):
        assert counts[i] == (len(p.mesh.faces) if p.mesh is not None else 0)
    lo = pos.reshape(-1, 3).min(0)
    hi = pos.reshape(-1, 3).max(0)
    assert np.allclose(info["bound_min"], lo) and np.allclose(info["bound_max"], hi)


def _write(tmp_path, yaml_text, objs=None):
    for name, text in (objs or {}).items():
        (tmp_path / name).write_text(text)
    p = tmp_path / "scene.yml"
    p.write_text(yaml_text)
    return p


QUAD_OBJ = """# quad with normals
o q
v 0 0 0
v 1 0 0
v 1 0 1
v 0 0 1
vn 0 1 0
f 1//1 4//1 3//1 2//1
"""

CAMERA = """
    - type: [E]
      params:
        E:
          type: pinhole
          pinhole:
            We: [1, 1, 1]
            view:
              eye: [0.5, 2, 0.5]   # comment after a value
              center: [0.5, 0, 0.5]
              up: [0, 0, -1]
            perspective:
              fov: 45
"""


def test_yaml_subset_and_quad_triangulation(native_lib, tmp_path):
    yaml = """# leading comment
version: 4
scene:
  primitives:
    - type: ["L", 'D']
      mesh:
        path: "quad.obj"
      params:
        L:
          type: area
          area:
            Le: [1.5, 2, 3e0]
        D:
          R: [0, 0, 0]
""" + CAMERA
    s = _load(native_lib, _write(tmp_path, yaml, {"quad.obj": QUAD_OBJ}))
    info = s.info()
    assert info["num_triangles"] == 2 and info["num_lights"] == 1 and info["sensor_type"] == 1
    P, N, _, prim = s.triangles()
    # fan triangulation from the first corner: (1,4,3), (1,3,2)
    assert np.array_equal(P[0], np.array([[0, 0, 0], [0, 0, 1], [1, 0, 1]], np.float32))
    assert np.array_equal(P[1], np.array([[0, 0, 0], [1, 0, 1], [1, 0, 0]], np.float32))
    assert np.all(N[..., 1] == 1.0)


def test_obj_index_forms_and_generated_normals(native_lib, tmp_path):
    obj = """v 0 0 0
v 1 0 0
v 0 1 0
vt 0 0
vt 1 0
vt 0 1
f -3/1 -2/2 -1/3
o second_object_is_ignored
v 5 5 5
f 1 2 4
"""
    yaml = """version: 5
scene:
  primitives:
    - type: [D]
      mesh:
        path: 'tri.obj'
        postprocess:
          generate_normals: true
      params:
        D:
          R: [0.5, 0.5, 0.5]
""" + CAMERA
    s = _load(native_lib, _write(tmp_path, yaml, {"tri.obj": obj}))
    P, N, U, _ = s.triangles()
    assert P.shape == (1, 3, 3)
    assert np.allclose(N[0], [[0, 0, 1]] * 3)          # flat normal of the face
    assert np.allclose(U[0], [[0, 0], [1, 0], [0, 1]])


@pytest.mark.parametrize("case,status", [
    ("version: 2\nscene:\n  primitives: []\n", "NGI_ERR_PARSE"),
    ("version: 5\nscene:\n  primitives:\n    - type: [L, E]\n      params: {}\n", "NGI_ERR_PARSE"),
    ("version: 5\nscene:\n  primitives:\n    - type: [X]\n      params: {}\n", "NGI_ERR_PARSE"),
    ("version: 5\nscene:\n  primitives:\n    - type: [L]\n      params:\n        L:\n          type: area\n"
     "          area:\n            Le: [1, 1, 1]\n", "NGI_ERR_PARSE"),            # area light without mesh
    ("version: 5\nscene:\n  primitives:\n    - type: [D]\n      mesh:\n        path: missing.obj\n"
     "      params:\n        D:\n          R: [1, 1, 1]\n", "NGI_ERR_IO"),
    ("version: 5\nscene:\n  primitives:\n    - type: [D]\n      mesh:\n        path: quad.obj\n"
     "      params:\n        D:\n          TexR: missing.png\n", "NGI_ERR_IO"),
    ("version: 5\nscene:\n  primitives:\n    - type: [D]\n      mesh:\n        path: quad.obj\n"
     "      params:\n        D:\n          R: [1, 1]\n", "NGI_ERR_PARSE"),
    ("version: 5\nscene:\n  primitives:\n    - type: [D\n", "NGI_ERR_PARSE"),
    ("version: five\n", "NGI_ERR_PARSE"),
])
def test_malformed_scenes_return_status(native_lib, tmp_path, case, status):
    import nanogi_gb300 as ng

    p = _write(tmp_path, case, {"quad.obj": QUAD_OBJ})
    with pytest.raises(ng.NanogiError) as e:
        ng.Scene.load(p, 1.0)
    assert str(e.value).startswith(status), str(e.value)


def test_missing_scene_file(native_lib, tmp_path):
    import nanogi_gb300 as ng

    with pytest.raises(ng.NanogiError) as e:
        ng.Scene.load(tmp_path / "nope.yml", 1.0)
    assert e.value.status == 2


def test_malformed_obj(native_lib, tmp_path):
    import nanogi_gb300 as ng

    yaml = "version: 5\nscene:\n  primitives:\n    - type: [D]\n      mesh:\n        path: bad.obj\n" \
           "      params:\n        D:\n          R: [1, 1, 1]\n"
    for bad in ["v 0 0 0\nf 1 2 3\n", "v 0 0\n", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 0\n", "# nothing\n"]:
        p = _write(tmp_path, yaml, {"bad.obj": bad})
        with pytest.raises(ng.NanogiError) as e:
            ng.Scene.load(p, 1.0)
        assert e.value.status == 3, (bad, str(e.value))


def test_directional_light_post_configuration(native_lib, tmp_path):
    """Scene-bound dependent light parameters exist only after loading (rt.hpp:2059-2079)."""
    from nanogi_gb300 import scenegen

    desc = scenegen.material_box()
    path = scenegen.write_scene(desc, tmp_path)
    s = _load(native_lib, path)
    info = s.info()
    assert info["num_lights"] == 3
    assert info["bound_min"] == pytest.approx([0, 0, 0], abs=1e-6)
    assert info["bound_max"] == pytest.approx([1, 1, 1], abs=1e-6)


@pytest.mark.parametrize("workload", ["cornell_box", "material_box"])
def test_memory_meshes_match_obj_files(native_lib, tmp_path, workload):
    """ngi_scene_load_with_meshes flattens caller-held meshes exactly like their OBJ files."""
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen

    desc = scenegen.WORKLOADS[workload]()
    a = _load(native_lib, scenegen.write_scene(desc, tmp_path / "files"))
    b = ng.Scene.load_with_meshes(scenegen.write_scene(desc, tmp_path / "mem", write_meshes=False), 1.0,
                                  scenegen.memory_meshes(desc))
    for x, y in zip(a.triangles(), b.triangles()):
        assert np.array_equal(x, y)
    ia, ib = a.info(), b.info()
    for k in ("num_triangles", "num_primitives", "num_lights", "sensor_index", "bound_min", "bound_max"):
        assert np.array_equal(np.asarray(ia[k]), np.asarray(ib[k])), k


def test_memory_mesh_flat_normals_and_errors(native_lib, tmp_path):
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen

    desc = scenegen.cornell_box()
    path = scenegen.write_scene(desc, tmp_path, write_meshes=False)
    mm = {k: (v[0], v[1], None, v[3]) for k, v in scenegen.memory_meshes(desc).items()}
    s = ng.Scene.load_with_meshes(path, 1.0, mm)
    P, N, _, _ = s.triangles()
    P, N = P.reshape(-1, 3, 3).astype(np.float64), N.reshape(-1, 3, 3)
    n = np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 0])
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    assert np.allclose(N, n[:, None, :], atol=1e-6)
    bad = dict(mm)
    k0 = next(iter(bad))
    faces = bad[k0][1].copy()
    faces[0, 0] = len(bad[k0][0])
    bad[k0] = (bad[k0][0], faces)
    with pytest.raises(ng.NanogiError) as e:
        ng.Scene.load_with_meshes(path, 1.0, bad)
    assert e.value.status == 1 and "out of range" in e.value.message
    # a mesh missing from memory falls back to its (absent) file: an I/O error
    del mm[k0]
    with pytest.raises(ng.NanogiError):
        ng.Scene.load_with_meshes(path, 1.0, mm)


@pytest.mark.parametrize("ext", [".png", ".ppm", ".bmp", ".pfm"])
def test_texture_decoders_round_trip(native_lib, tmp_path, ext):
    """TexR images decode to the texels they were written from (8-bit as v/255), top row first."""
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen

    rng = np.random.default_rng(len(ext))
    img = (rng.integers(0, 256, (13, 17, 3)) / np.float32(255.0)).astype(np.float32)
    if ext == ".pfm":
        img = rng.uniform(-1, 4, (13, 17, 3)).astype(np.float32)
    path = tmp_path / f"t{ext}"
    scenegen.write_texture(path, img)
    got = ng.load_texture(path)
    assert got.shape == img.shape
    assert np.array_equal(got, img)


def test_png_decoder_handles_rgba_stored_blocks_and_bad_files(native_lib, tmp_path):
    import struct
    import zlib

    import nanogi_gb300 as ng

    def png(w, h, ctype, raw, level=9, depth=8):
        def chunk(t, d):
            return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d))
        return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0))
                + chunk(b"IDAT", zlib.compress(raw, level)) + chunk(b"IEND", b""))

    rng = np.random.default_rng(5)
    rgba = rng.integers(0, 256, (6, 4, 4), dtype=np.uint8)
    raw = b"".join(b"\x00" + rgba[y].tobytes() for y in range(6))
    for level in (0, 1, 9):  # stored, fixed and dynamic Huffman blocks
        p = tmp_path / f"a{level}.png"
        p.write_bytes(png(4, 6, 6, raw, level))
        got = ng.load_texture(p)
        assert np.array_equal(got, rgba[:, :, :3].astype(np.float32) / np.float32(255.0))
    gray = tmp_path / "g.png"
    gray.write_bytes(png(4, 6, 0, b"".join(b"\x00" + bytes(4) for _ in range(6))))
    with pytest.raises(ng.NanogiError) as e:
        ng.load_texture(gray)
    assert e.value.status == 7  # the reference accepts 24/32-bit bitmaps only
    bad = tmp_path / "bad.png"
    bad.write_bytes(png(4, 6, 2, b"\x00" * 10))
    with pytest.raises(ng.NanogiError):
        ng.load_texture(bad)
    with pytest.raises(ng.NanogiError):
        ng.load_texture(tmp_path / "missing.png")


def test_textured_scene_loads(native_lib, tmp_path):
    import nanogi_gb300 as ng
    from nanogi_gb300 import scenegen

    desc = scenegen.textured_box()
    s = ng.Scene.load(scenegen.write_scene(desc, tmp_path), 1.0)
    assert s.info()["num_primitives"] == len(desc.primitives)
    (tmp_path / "left.ppm").unlink()
    with pytest.raises(ng.NanogiError):
        ng.Scene.load(tmp_path / "scene.yml", 1.0)
