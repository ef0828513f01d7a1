"""Writes tests/golden/reference_scenes.npz from the reference's two example scenes.

nanogi ships two scene files with its job scripts: utils/runc/data/scene.yml (an area light,
a glossy conductor sphere, a diffuse sphere, a Fresnel dielectric sphere and two planes, seen
by a pinhole camera) and utils/runc/data/cornelbox/scene.yml (the Cornell box at millimetre
scale). They are the only scene inputs the reference itself holds. This script reads them where
the reference tree lies (NGI_REFERENCE_ROOT, required) through this library's own CPU loader
(ngi_scene_load: YAML v5 + OBJ, fan triangulation, no GPU needed) and stores what a render
needs: per primitive its type list and parameters (parsed from the YAML here), and the
flattened triangles with their normals. The GPU tests rebuild each scene from the fixture and
render it on the GPU and in the oracle, so they run where the reference tree is absent.

    NGI_REFERENCE_ROOT=<reference checkout> python tests/golden/make_reference_scenes.py
"""
from __future__ import annotations

import json
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

SCENES = {
    "runc": Path("utils") / "runc" / "data" / "scene.yml",
    "cornelbox": Path("utils") / "runc" / "data" / "cornelbox" / "scene.yml",
}


def _scalar(text: str):
    t = text.strip()
    if t.startswith("[") and t.endswith("]"):
        inner = t[1:-1].strip()
        return [_scalar(x) for x in inner.split(",")] if inner else []
    if len(t) >= 2 and t[0] == t[-1] and t[0] in "'\"":
        return t[1:-1]
    for conv in (int, float):
        try:
            return conv(t)
        except ValueError:
            pass
    return t


def parse_yaml(text: str):
    """The block-YAML subset the scene files use: nested mappings, sequences of mappings, flow
    lists of scalars, quoted or bare scalars and whole-line '#' comments."""
    lines = []
    for raw in text.splitlines():
        s = raw.rstrip()
        if s.strip() and not s.strip().startswith("#"):
            lines.append((len(s) - len(s.lstrip(" ")), s.strip()))

    def block(i: int, indent: int):
        if lines[i][1].startswith("- "):
            seq = []
            while i < len(lines) and lines[i][0] == indent and lines[i][1].startswith("- "):
                # "- key: value" opens a mapping whose keys sit two columns further in
                lines[i] = (indent + 2, lines[i][1][2:])
                item, i = block(i, indent + 2)
                seq.append(item)
            return seq, i
        out = {}
        while i < len(lines) and lines[i][0] == indent:
            key, _, rest = lines[i][1].partition(":")
            if rest.strip():
                out[key.strip()] = _scalar(rest)
                i += 1
            else:
                out[key.strip()], i = block(i + 1, lines[i + 1][0])
        return out, i

    value, _ = block(0, lines[0][0])
    return value


def scene_arrays(yml: Path):
    import nanogi_gb300 as ng

    doc = parse_yaml(yml.read_text())
    prims = [{"type": p["type"], "params": p.get("params", {})} for p in doc["scene"]["primitives"]]
    scene = ng.Scene.load(yml, 1.0)
    pos, nrm, _, prim = scene.triangles()
    scene.close()
    return prims, pos, nrm, prim


def main() -> None:
    root = os.environ.get("NGI_REFERENCE_ROOT")
    if not root:
        raise SystemExit("set NGI_REFERENCE_ROOT to the reference checkout")
    out = {}
    for name, rel in SCENES.items():
        prims, pos, nrm, prim = scene_arrays(Path(root) / rel)
        out[f"{name}_prims"] = np.frombuffer(json.dumps(prims).encode(), np.uint8)
        out[f"{name}_pos"] = pos.astype(np.float32)
        out[f"{name}_nrm"] = nrm.astype(np.float32)
        out[f"{name}_prim"] = prim.astype(np.int32)
        print(f"{name}: {len(prims)} primitives, {len(pos)} triangles")
    np.savez_compressed(HERE / "reference_scenes.npz", **out)


if __name__ == "__main__":
    main()
