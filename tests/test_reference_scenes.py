"""The reference's own example scenes load unchanged (CPU; no GPU needed).

nanogi ships two scene files with its job scripts (utils/runc/data/scene.yml and
utils/runc/data/cornelbox/scene.yml, schema version 5, OBJ meshes with quads and `f v//vn`
faces). They carry no expected images, so they pin only the loader: every primitive's
triangles, the light and sensor, and the scene bounds are compared with a plain parse of the
OBJ files (polygons split as fans from their first vertex, as the loader documents).

The files are read where the reference tree lies (the NGI_REFERENCE_ROOT environment
variable); the tests are skipped when it is unset or the tree is absent. The last test checks
that tests/golden/reference_scenes.npz, the fixture the GPU tests render these scenes from,
still holds exactly what the loader reads from the reference's files.
"""
from __future__ import annotations

import os
from pathlib import Path

import numpy as np
import pytest

REF = Path(os.environ["NGI_REFERENCE_ROOT"]) if os.environ.get("NGI_REFERENCE_ROOT") else None
SCENE_FILES = {
    "runc": Path("utils") / "runc" / "data" / "scene.yml",
    "cornelbox": Path("utils") / "runc" / "data" / "cornelbox" / "scene.yml",
}


def _scene_file(name: str) -> Path:
    if REF is None:
        pytest.skip("NGI_REFERENCE_ROOT is not set")
    yml = REF / SCENE_FILES[name]
    if not yml.exists():
        pytest.skip("the reference's example scenes are not present under NGI_REFERENCE_ROOT")
    return yml


def _obj_triangles(path: Path) -> np.ndarray:
    """Fan-triangulated faces of an OBJ file as (n, 3, 3) float32 positions."""
    verts, tris = [], []
    for line in path.read_text().splitlines():
        parts = line.split()
        if not parts:
            continue
        if parts[0] == "v":
            verts.append([float(x) for x in parts[1:4]])
        elif parts[0] == "f":
            idx = []
            for tok in parts[1:]:
                i = int(tok.split("/")[0])
                idx.append(i - 1 if i > 0 else len(verts) + i)
            for k in range(1, len(idx) - 1):
                tris.append([verts[idx[0]], verts[idx[k]], verts[idx[k + 1]]])
    return np.asarray(tris, np.float32).reshape(-1, 3, 3)


def _mesh_paths(yml: Path) -> list[Path | None]:
    """Mesh file of each primitive in file order (None for a primitive without a mesh)."""
    out: list[Path | None] = []
    for line in yml.read_text().splitlines():
        s = line.strip()
        if s.startswith("- type:"):
            out.append(None)
        elif s.startswith("path:") and out:
            out[-1] = yml.parent / s.split(":", 1)[1].strip().strip("'\"")
    return out


def _tri_key(t: np.ndarray) -> tuple:
    """Order-independent key of one triangle: its three vertices, sorted."""
    return tuple(sorted(tuple(float(c) for c in v) for v in t))


@pytest.mark.parametrize("name", sorted(SCENE_FILES))
def test_reference_example_scene_loads_unchanged(native_lib, name):
    yml = _scene_file(name)
    import nanogi_gb300 as ng

    meshes = _mesh_paths(yml)
    scene = ng.Scene.load(str(yml), 1.0)
    info = scene.info()
    pos, _, _, prim = scene.triangles()
    scene.close()

    assert info["num_primitives"] == len(meshes)
    text = yml.read_text()
    assert info["num_lights"] == text.count("type: [L")
    assert info["sensor_index"] == len(meshes) - 1  # the camera is the last primitive in both files
    expect_all = []
    for i, mp in enumerate(meshes):
        got = pos[prim == i]
        if mp is None:
            assert len(got) == 0
            continue
        want = _obj_triangles(mp)
        expect_all.append(want)
        assert len(got) == len(want), (name, mp.name)
        assert sorted(_tri_key(t) for t in got) == sorted(_tri_key(t) for t in want), (name, mp.name)
    allv = np.concatenate(expect_all).reshape(-1, 3)
    assert np.allclose(info["bound_min"], allv.min(0)) and np.allclose(info["bound_max"], allv.max(0))


@pytest.mark.parametrize("name", sorted(SCENE_FILES))
def test_fixture_matches_the_reference_scene(native_lib, name):
    """tests/golden/reference_scenes.npz holds the scene the loader reads from the reference."""
    import json
    import sys

    yml = _scene_file(name)
    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    from make_reference_scenes import scene_arrays

    prims, pos, nrm, prim = scene_arrays(yml)
    d = np.load(Path(__file__).resolve().parent / "golden" / "reference_scenes.npz")
    assert json.loads(bytes(d[f"{name}_prims"]).decode()) == prims
    assert np.array_equal(d[f"{name}_pos"], pos)
    assert np.array_equal(d[f"{name}_nrm"], nrm)
    assert np.array_equal(d[f"{name}_prim"], prim)
