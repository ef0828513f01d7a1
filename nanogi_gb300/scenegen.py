"""Seeded synthetic scenes in nanogi's scene format (YAML version 5 + one OBJ per primitive).

Every scene is first built in memory as a ``SceneDesc`` (float32 vertex arrays exactly as
they are written to the OBJ files, plus the per-primitive parameters of schema.yml), then
written to disk. Tests hand the same in-memory description to the CPU oracle, so the
product's YAML/OBJ loader is checked against data it never parsed.

Workloads (sizes from the benchmark configurations):
* ``cornell_box``   -- open unit box, 5 wall quads, two rotated boxes, 0.25 x 0.25 ceiling
                       light of radiance (17, 12, 4): 36 triangles.
* ``terrain_scene`` -- 512 x 512 fBm height field (seeded value noise, 6 octaves), 200
                       level-4 icospheres (5120 triangles each) of log-uniform radius
                       0.05-1 with diffuse / glossy / mirror / glass materials drawn
                       uniformly, 4 quad lights of radiance U[5, 20]: ~1.55 M triangles.
"""
from __future__ import annotations

import copy
import math
import os
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

# Conductor constants used for every glossy (G) material: published optical constants of
# gold at (650, 550, 450) nm.
GOLD_ETA = (0.14, 0.129, 0.1585)
GOLD_K = (4.58625, 3.348125, 2.329375)


@dataclass
class Mesh:
    positions: np.ndarray          # (V, 3) float32
    normals: np.ndarray            # (V, 3) float32
    faces: np.ndarray              # (F, 3) int64, 0-based
    uvs: np.ndarray | None = None  # (V, 2) float32


@dataclass
class Primitive:
    type: list[str]
    params: dict
    mesh: Mesh | None = None
    name: str = "prim"


@dataclass
class SceneDesc:
    primitives: list[Primitive] = field(default_factory=list)
    # TexR images by file name: (H, W, 3) float32, row 0 = the image's top row. 8-bit formats
    # hold multiples of 1/255 so the file stores them exactly.
    textures: dict = field(default_factory=dict)

    @property
    def num_triangles(self) -> int:
        return sum(len(p.mesh.faces) for p in self.primitives if p.mesh is not None)


# ---- mesh helpers ------------------------------------------------------------------------------
def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).astype(np.float32))


def quad(p0, p1, p2, p3, normal) -> Mesh:
    """Quad p0-p1-p2-p3 (counter-clockwise seen from `normal`) as two triangles."""
    P = _f32([p0, p1, p2, p3])
    N = _f32([normal] * 4)
    F = np.array([[0, 1, 2], [0, 2, 3]], np.int64)
    return Mesh(P, N, F, _f32([[0, 0], [1, 0], [1, 1], [0, 1]]))


def box(center, size, angle_deg) -> Mesh:
    """Axis-aligned box rotated about +y, 6 faces x 2 triangles, outward flat normals."""
    cx, cy, cz = center
    sx, sy, sz = size
    a = math.radians(angle_deg)
    ca, sa = math.cos(a), math.sin(a)

    def tr(x, y, z):
        return (cx + ca * x + sa * z, cy + y, cz - sa * x + ca * z)

    def rn(nx, ny, nz):
        return (ca * nx + sa * nz, ny, -sa * nx + ca * nz)

    hx, hy, hz = sx / 2, sy / 2, sz / 2
    faces = [
        ((-hx, -hy, hz), (hx, -hy, hz), (hx, hy, hz), (-hx, hy, hz), (0, 0, 1)),
        ((hx, -hy, -hz), (-hx, -hy, -hz), (-hx, hy, -hz), (hx, hy, -hz), (0, 0, -1)),
        ((hx, -hy, hz), (hx, -hy, -hz), (hx, hy, -hz), (hx, hy, hz), (1, 0, 0)),
        ((-hx, -hy, -hz), (-hx, -hy, hz), (-hx, hy, hz), (-hx, hy, -hz), (-1, 0, 0)),
        ((-hx, hy, hz), (hx, hy, hz), (hx, hy, -hz), (-hx, hy, -hz), (0, 1, 0)),
        ((-hx, -hy, -hz), (hx, -hy, -hz), (hx, -hy, hz), (-hx, -hy, hz), (0, -1, 0)),
    ]
    P, N, F = [], [], []
    for q0, q1, q2, q3, n in faces:
        b = len(P)
        P += [tr(*q0), tr(*q1), tr(*q2), tr(*q3)]
        N += [rn(*n)] * 4
        F += [[b, b + 1, b + 2], [b, b + 2, b + 3]]
    return Mesh(_f32(P), _f32(N), np.array(F, np.int64))


def icosphere(level: int) -> tuple[np.ndarray, np.ndarray]:
    """Unit icosphere: (V, 3) float64 vertices, (F, 3) faces, outward winding."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, np.float64) / np.linalg.norm(p) for p in v]
    faces = list(f)
    for _ in range(level):
        cache: dict[tuple[int, int], int] = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.array(verts), np.array(faces, np.int64)


_ICO_CACHE: dict[int, tuple[np.ndarray, np.ndarray]] = {}


def sphere_mesh(center, radius, level=4) -> Mesh:
    if level not in _ICO_CACHE:
        _ICO_CACHE[level] = icosphere(level)
    V, F = _ICO_CACHE[level]
    P = _f32(V * radius + np.asarray(center, np.float64))
    return Mesh(P, _f32(V), F.copy())


# ---- materials -------------------------------------------------------------------------------------
def diffuse(r) -> tuple[list[str], dict]:
    return ["D"], {"D": {"R": [float(x) for x in r]}}


def glossy(r, roughness) -> tuple[list[str], dict]:
    return ["G"], {"G": {"R": [float(x) for x in r], "Eta": list(GOLD_ETA), "K": list(GOLD_K),
                         "Roughness": float(roughness)}}


def mirror(r=(1.0, 1.0, 1.0)) -> tuple[list[str], dict]:
    return ["S"], {"S": {"type": "reflection", "reflection": {"R": [float(x) for x in r]}}}


def glass(eta2=1.5, r=(1.0, 1.0, 1.0)) -> tuple[list[str], dict]:
    return ["S"], {"S": {"type": "fresnel", "fresnel": {"R": [float(x) for x in r], "eta1": 1.0, "eta2": float(eta2)}}}


def area_light(le) -> tuple[list[str], dict]:
    # Light primitives carry a black diffuse BSDF, as the reference's own scenes do: a pure
    # [L] primitive reaches assert(0) in SampleDirection after a hit (rt.hpp:909).
    return ["L", "D"], {"L": {"type": "area", "area": {"Le": [float(x) for x in le]}}, "D": {"R": [0.0, 0.0, 0.0]}}


def pinhole(eye, center, up, fov) -> Primitive:
    return Primitive(["E"], {"E": {"type": "pinhole", "pinhole": {
        "We": [1.0, 1.0, 1.0], "view": {"eye": [float(x) for x in eye], "center": [float(x) for x in center],
                                         "up": [float(x) for x in up]},
        "perspective": {"fov": float(fov)}}}}, None, "camera")


def phong_to_beckmann(n: float) -> float:
    """Beckmann roughness matching a Phong lobe exponent (Walter et al. 2007): sqrt(2/(n+2))."""
    return math.sqrt(2.0 / (n + 2.0))


def transformed(desc: SceneDesc, scale: float, offset=(0.0, 0.0, 0.0)) -> SceneDesc:
    """The scene scaled by `scale` about the origin and moved by `offset`: mesh positions and
    pinhole eye/center. Radiance is unchanged, so every image of the scene is unchanged."""
    d = copy.deepcopy(desc)
    off = np.asarray(offset, np.float64)
    for p in d.primitives:
        if p.mesh is not None:
            p.mesh.positions = _f32(p.mesh.positions.astype(np.float64) * scale + off)
        if "E" in p.type and p.params["E"]["type"] == "pinhole":
            v = p.params["E"]["pinhole"]["view"]
            v["eye"] = [float(x) for x in np.asarray(v["eye"], np.float64) * scale + off]
            v["center"] = [float(x) for x in np.asarray(v["center"], np.float64) * scale + off]
    return d


# ---- workloads -------------------------------------------------------------------------------------
def cornell_box(light_le=(17.0, 12.0, 4.0)) -> SceneDesc:
    """Open unit box [0,1]^3 (front face z=1 open), camera outside looking in -z."""
    s = SceneDesc()
    grey, red, green = (0.73, 0.73, 0.73), (0.63, 0.065, 0.05), (0.14, 0.45, 0.09)
    walls = [
        ("floor", quad((0, 0, 1), (1, 0, 1), (1, 0, 0), (0, 0, 0), (0, 1, 0)), grey),
        ("ceiling", quad((0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1), (0, -1, 0)), grey),
        ("back", quad((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1)), grey),
        ("left", quad((0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1), (1, 0, 0)), red),
        ("right", quad((1, 0, 1), (1, 1, 1), (1, 1, 0), (1, 0, 0), (-1, 0, 0)), green),
    ]
    lt, lp = area_light(light_le)
    h = 1.0 - 1e-3
    s.primitives.append(Primitive(lt, lp, quad((0.375, h, 0.375), (0.625, h, 0.375), (0.625, h, 0.625),
                                                (0.375, h, 0.625), (0, -1, 0)), "light"))
    for name, m, col in walls:
        t, p = diffuse(col)
        s.primitives.append(Primitive(t, p, m, name))
    t, p = diffuse(grey)
    s.primitives.append(Primitive(t, p, box((0.33, 0.3, 0.37), (0.3, 0.6, 0.3), 15.0), "tallbox"))
    s.primitives.append(Primitive(list(t), dict(p), box((0.68, 0.15, 0.65), (0.3, 0.3, 0.3), -18.0), "shortbox"))
    s.primitives.append(pinhole((0.5, 0.5, 2.4), (0.5, 0.5, 0.0), (0, 1, 0), 36.0))
    return s


def _value_noise_fbm(x: np.ndarray, z: np.ndarray, seed: int, octaves: int = 6) -> np.ndarray:
    """Fractional Brownian motion of seeded value noise (smoothstep-interpolated lattice)."""
    rng = np.random.default_rng(seed)
    out = np.zeros_like(x)
    amp, freq, norm = 1.0, 1.0, 0.0
    for _ in range(octaves):
        lat = rng.random((257, 257)) * 2.0 - 1.0
        gx, gz = x * freq, z * freq
        ix, iz = np.floor(gx).astype(np.int64), np.floor(gz).astype(np.int64)
        fx, fz = gx - ix, gz - iz
        sx, sz = fx * fx * (3 - 2 * fx), fz * fz * (3 - 2 * fz)
        ix, iz = ix % 256, iz % 256
        v00, v10 = lat[ix, iz], lat[ix + 1, iz]
        v01, v11 = lat[ix, iz + 1], lat[ix + 1, iz + 1]
        out += amp * ((v00 * (1 - sx) + v10 * sx) * (1 - sz) + (v01 * (1 - sx) + v11 * sx) * sz)
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return out / norm


def terrain_mesh(grid: int = 512, extent: float = 16.0, height: float = 1.5, seed: int = 2) -> tuple[Mesh, callable]:
    xs = np.linspace(-extent / 2, extent / 2, grid)
    X, Z = np.meshgrid(xs, xs, indexing="ij")
    base = 0.35  # lattice frequency in cells per scene unit
    H = height * _value_noise_fbm((X + extent) * base, (Z + extent) * base, seed)
    P = np.stack([X, H, Z], -1).reshape(-1, 3)
    # vertex normals from central differences of the height field
    dx = xs[1] - xs[0]
    gx = np.gradient(H, dx, axis=0)
    gz = np.gradient(H, dx, axis=1)
    Nn = np.stack([-gx, np.ones_like(H), -gz], -1)
    Nn /= np.linalg.norm(Nn, axis=-1, keepdims=True)
    idx = np.arange(grid * grid).reshape(grid, grid)
    a, b = idx[:-1, :-1].ravel(), idx[1:, :-1].ravel()
    c, d = idx[1:, 1:].ravel(), idx[:-1, 1:].ravel()
    # winding so that cross(p2-p1, p3-p1) points up (+y)
    F = np.concatenate([np.stack([a, d, c], -1), np.stack([a, c, b], -1)])

    def height_at(x, z):
        return float(height * _value_noise_fbm(np.array([(x + extent) * base]), np.array([(z + extent) * base]), seed)[0])

    return Mesh(_f32(P), _f32(Nn.reshape(-1, 3)), F.astype(np.int64)), height_at


def terrain_scene(num_spheres: int = 200, grid: int = 512, level: int = 4, seed_terrain: int = 2,
                  seed_spheres: int = 3) -> SceneDesc:
    """The ~1.55 M-triangle ptdirect workload."""
    s = SceneDesc()
    extent = 16.0
    terrain, height_at = terrain_mesh(grid, extent, 1.5, seed_terrain)
    rng = np.random.default_rng(seed_spheres)
    lrng = np.random.default_rng(seed_spheres + 1000)
    # 4 quad lights of radiance U[5, 20] above the terrain, facing down
    for i, (lx, lz) in enumerate([(-4.0, -3.0), (4.0, -3.0), (-4.0, 4.0), (4.0, 4.0)]):
        le = lrng.uniform(5.0, 20.0, 3)
        hs, y = 0.9, 7.0
        t, p = area_light(le)
        s.primitives.append(Primitive(t, p, quad((lx - hs, y, lz - hs), (lx + hs, y, lz - hs), (lx + hs, y, lz + hs),
                                                 (lx - hs, y, lz + hs), (0, -1, 0)), f"light{i}"))
    t, p = diffuse((0.45, 0.5, 0.4))
    s.primitives.append(Primitive(t, p, terrain, "terrain"))
    for i in range(num_spheres):
        r = float(math.exp(rng.uniform(math.log(0.05), math.log(1.0))))
        x, z = rng.uniform(-extent / 2 + 1, extent / 2 - 1, 2)
        y = height_at(x, z) + r
        kind = int(rng.integers(0, 4))
        if kind == 0:
            t, p = diffuse(rng.uniform(0.1, 0.9, 3))
        elif kind == 1:
            n = float(math.exp(rng.uniform(math.log(10.0), math.log(1000.0))))
            t, p = glossy(rng.uniform(0.5, 1.0, 3), phong_to_beckmann(n))
        elif kind == 2:
            t, p = mirror((0.95, 0.95, 0.95))
        else:
            t, p = glass(1.5)
        s.primitives.append(Primitive(t, p, sphere_mesh((x, y, z), r, level), f"sphere{i}"))
    s.primitives.append(pinhole((0.0, 7.5, 13.0), (0.0, 0.0, 0.0), (0, 1, 0), 45.0))
    return s


# ---- writers --------------------------------------------------------------------------------------------
def _fmt_rows(prefix: str, a: np.ndarray) -> str:
    # '%.9g' round-trips float32 exactly
    a = np.asarray(a)
    if a.dtype.kind == "f":
        cols = [np.char.mod("%.9g", a[:, k].astype(np.float64)) for k in range(a.shape[1])]
    else:
        cols = [a[:, k].astype(str) for k in range(a.shape[1])]
    out = np.char.add(prefix, cols[0])
    for c in cols[1:]:
        out = np.char.add(np.char.add(out, " "), c)
    return "\n".join(out.tolist()) + "\n"


def write_obj(path: Path, m: Mesh, name: str) -> None:
    parts = [f"o {name}\n", _fmt_rows("v ", m.positions)]
    if m.uvs is not None:
        parts.append(_fmt_rows("vt ", m.uvs))
    parts.append(_fmt_rows("vn ", m.normals))
    f1 = (m.faces + 1).astype(np.int64)
    if m.uvs is not None:
        idx = [np.char.add(np.char.add(np.char.add(np.char.add(f1[:, k].astype(str), "/"), f1[:, k].astype(str)), "/"),
                           f1[:, k].astype(str)) for k in range(3)]
    else:
        idx = [np.char.add(np.char.add(f1[:, k].astype(str), "//"), f1[:, k].astype(str)) for k in range(3)]
    lines = np.char.add(np.char.add(np.char.add(np.char.add(np.char.add("f ", idx[0]), " "), idx[1]), " "), idx[2])
    parts.append("\n".join(lines.tolist()) + "\n")
    Path(path).write_text("".join(parts))


def _yaml_value(v, indent: int) -> str:
    pad = " " * indent
    if isinstance(v, dict):
        out = ""
        for k, x in v.items():
            if isinstance(x, dict):
                out += f"{pad}{k}:\n" + _yaml_value(x, indent + 2)
            else:
                out += f"{pad}{k}: {_yaml_scalar(x)}\n"
        return out
    return pad + _yaml_scalar(v) + "\n"


def _yaml_scalar(x) -> str:
    if isinstance(x, (list, tuple)):
        return "[" + ", ".join(_yaml_scalar(y) for y in x) + "]"
    if isinstance(x, bool):
        return "true" if x else "false"
    if isinstance(x, (int, np.integer)):
        return str(int(x))
    if isinstance(x, (float, np.floating)):
        return repr(float(x))
    return str(x)


# ---- texture files (the images TexR names) --------------------------------------------------
def _png_bytes(img8: np.ndarray) -> bytes:
    """8-bit RGB PNG; the rows cycle through the five filter types."""
    import struct
    import zlib

    h, w, _ = img8.shape
    stride = 3 * w
    prev = np.zeros(stride, np.int32)
    raw = bytearray()
    for y in range(h):
        cur = img8[y].reshape(-1).astype(np.int32)
        a = np.concatenate([np.zeros(3, np.int32), cur[:-3]])
        c = np.concatenate([np.zeros(3, np.int32), prev[:-3]])
        ft = y % 5
        if ft == 0:
            out = cur
        elif ft == 1:
            out = cur - a
        elif ft == 2:
            out = cur - prev
        elif ft == 3:
            out = cur - (a + prev) // 2
        else:
            p = a + prev - c
            pa, pb, pc = np.abs(p - a), np.abs(p - prev), np.abs(p - c)
            pred = np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, prev, c))
            out = cur - pred
        raw.append(ft)
        raw += (out % 256).astype(np.uint8).tobytes()
        prev = cur

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)

    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0))
            + chunk(b"IDAT", zlib.compress(bytes(raw), 9)) + chunk(b"IEND", b""))


def write_texture(path: Path, img: np.ndarray) -> None:
    """Writes a TexR image as .png / .ppm / .bmp (8-bit) or .pfm (float), top row first."""
    import struct

    img = np.asarray(img, np.float32)
    h, w, _ = img.shape
    ext = Path(path).suffix
    if ext == ".pfm":
        Path(path).write_bytes(f"PF\n{w} {h}\n-1.0\n".encode() + img[::-1].astype("<f4").tobytes())
        return
    img8 = np.rint(img * 255.0).astype(np.uint8)
    if ext == ".png":
        Path(path).write_bytes(_png_bytes(img8))
    elif ext == ".ppm":
        Path(path).write_bytes(f"P6\n# nanogi texture\n{w} {h}\n255\n".encode() + img8.tobytes())
    elif ext == ".bmp":
        stride = (3 * w + 3) & ~3
        rows = b"".join(img8[y, :, ::-1].tobytes() + b"\0" * (stride - 3 * w) for y in range(h - 1, -1, -1))
        header = struct.pack("<2sIHHI", b"BM", 54 + len(rows), 0, 0, 54)
        dib = struct.pack("<IiiHHIIiiII", 40, w, h, 1, 24, 0, len(rows), 2835, 2835, 0, 0)
        Path(path).write_bytes(header + dib + rows)
    else:
        raise ValueError(f"no writer for {ext}")


def _mesh_file(i: int, p: Primitive) -> str:
    return f"{i:04d}_{p.name}.obj"


def write_scene(desc: SceneDesc, directory: str | os.PathLike, name: str = "scene.yml",
                write_meshes: bool = True) -> Path:
    """Writes the YAML scene and, unless ``write_meshes`` is False, one OBJ per mesh. Without
    the OBJ files the scene loads through ``Scene.load_with_meshes(path, a, memory_meshes(desc))``."""
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    for tex_name, img in desc.textures.items():
        write_texture(d / tex_name, img)
    lines = ["version: 5", "scene:", "  primitives:"]
    for i, p in enumerate(desc.primitives):
        lines.append(f"    - type: [{', '.join(p.type)}]")
        if p.mesh is not None:
            fn = _mesh_file(i, p)
            if write_meshes:
                write_obj(d / fn, p.mesh, p.name)
            lines.append("      mesh:")
            lines.append(f"        path: '{fn}'")
        lines.append("      params:")
        lines.append(_yaml_value(p.params, 8).rstrip("\n"))
        lines.append("")
    path = d / name
    path.write_text("\n".join(lines) + "\n")
    return path


def memory_meshes(desc: SceneDesc) -> dict:
    """{mesh path in the YAML of write_scene: (positions, faces, normals, uvs)} for every mesh."""
    return {_mesh_file(i, p): (p.mesh.positions, p.mesh.faces.astype(np.uint32), p.mesh.normals, p.mesh.uvs)
            for i, p in enumerate(desc.primitives) if p.mesh is not None}


WORKLOADS = {
    "cornell_box": cornell_box,
    "terrain_scene": terrain_scene,
}


def material_box(with_point=True, with_directional=True, level=2) -> SceneDesc:
    """Cornell box holding one sphere of every BSDF (G, S reflection / refraction / fresnel)
    plus, optionally, a point light and a directional light: covers every emitter and BSDF
    branch of the path tracers in a few thousand triangles."""
    s = cornell_box()
    cam = s.primitives.pop()  # keep the camera last
    spheres = [
        ((0.25, 0.75, 0.5), 0.12, glossy((0.9, 0.8, 0.7), 0.2)),
        ((0.75, 0.75, 0.5), 0.12, mirror((0.9, 0.9, 0.9))),
        ((0.5, 0.45, 0.8), 0.1, (["S"], {"S": {"type": "refraction", "refraction": {"R": [1.0, 1.0, 1.0],
                                                                                      "eta1": 1.0, "eta2": 1.33}}})),
        ((0.5, 0.8, 0.75), 0.09, glass(1.5)),
    ]
    for i, (c, r, (t, p)) in enumerate(spheres):
        s.primitives.append(Primitive(t, p, sphere_mesh(c, r, level), f"ball{i}"))
    if with_point:
        s.primitives.append(Primitive(["L"], {"L": {"type": "point", "point": {"Le": [0.3, 0.3, 0.3],
                                                                              "position": [0.5, 0.9, 0.6]}}},
                                      None, "pointlight"))
    if with_directional:
        s.primitives.append(Primitive(["L"], {"L": {"type": "directional", "directional": {
            "Le": [1.0, 1.0, 1.0], "direction": [0.0, -1.0, 0.0]}}}, None, "sun"))
    s.primitives.append(cam)
    return s


def area_sensor_box() -> SceneDesc:
    """Cornell box seen through an area sensor: a quad with uvs just inside the open face,
    facing into the box (EType::Area, rt.hpp:1910-1929)."""
    s = cornell_box()
    s.primitives.pop()  # drop the pinhole
    m = quad((0.05, 0.05, 0.999), (0.05, 0.95, 0.999), (0.95, 0.95, 0.999), (0.05 + 0.9, 0.05, 0.999), (0, 0, -1))
    # uv = raster position: u along +x, v along +y
    m.uvs = _f32([[0, 0], [0, 1], [1, 1], [1, 0]])
    s.primitives.append(Primitive(["E"], {"E": {"type": "area", "area": {"We": [1.0, 1.0, 1.0]}}}, m, "sensor"))
    return s


def textured_box(seed: int = 12) -> SceneDesc:
    """Cornell box whose back, left and right walls and floor carry TexR albedo (PNG, PPM, BMP
    and PFM images), with uvs tiled 3x and shifted negative so that the fract wrap matters,
    plus a glossy box with a textured G.R (rt.hpp:1947-1979)."""
    rng = np.random.default_rng(seed)
    s = cornell_box()
    names = {"back": "back.png", "left": "left.ppm", "right": "right.bmp", "floor": "floor.pfm"}
    for name, fn in names.items():
        hh, ww = int(rng.integers(3, 9)), int(rng.integers(3, 9))
        img = rng.integers(10, 240, (hh, ww, 3)).astype(np.float32) / np.float32(255.0)
        if fn.endswith(".pfm"):
            img = rng.uniform(0.05, 0.9, (hh, ww, 3)).astype(np.float32)
        s.textures[fn] = img
        for p in s.primitives:
            if p.name == name:
                p.params = {"D": {"TexR": fn}}
                p.mesh.uvs = _f32(p.mesh.uvs.astype(np.float64) * 3.0 - 1.3)
    s.textures["gloss.png"] = rng.integers(30, 230, (4, 5, 3)).astype(np.float32) / np.float32(255.0)
    for p in s.primitives:
        if p.name == "shortbox":
            p.type = ["G"]
            p.params = {"G": {"TexR": "gloss.png", "Eta": list(GOLD_ETA), "K": list(GOLD_K),
                              "Roughness": phong_to_beckmann(50.0)}}
            n = len(p.mesh.positions)
            p.mesh.uvs = _f32(np.stack([np.arange(n) % 4 / 4.0 + 0.1, np.arange(n) // 4 % 4 / 4.0 + 0.1], 1))
    return s


def sphere_field(num_spheres=40, grid=96, level=3, seed=11) -> SceneDesc:
    """A small terrain_scene (same generator, fewer triangles) for traversal tests."""
    s = terrain_scene(num_spheres=num_spheres, grid=grid, level=level, seed_terrain=seed, seed_spheres=seed + 1)
    return s


WORKLOADS.update({"material_box": material_box, "area_sensor_box": area_sensor_box, "sphere_field": sphere_field,
                  "textured_box": textured_box})


def inverse_box(seed: int = 5, emitter_seed: int = 7) -> SceneDesc:
    """The inverse-rendering workload: the Cornell box split into 64 diffuse material groups
    (RGB albedo float32 U[0.05, 0.95], drawn with `seed`) lit by 2 ceiling quad emitters
    (radiance U[5, 20], drawn with `emitter_seed`). Walls are cut into tiles: the back wall
    4 x 4, the other four walls 3 x 3 each, plus the 12 faces of the two boxes = 64 groups."""
    rng = np.random.default_rng(seed)
    erng = np.random.default_rng(emitter_seed)
    s = SceneDesc()
    h = 1.0 - 1e-3
    for i, (x0, x1) in enumerate([(0.2, 0.4), (0.6, 0.8)]):
        le = erng.uniform(5.0, 20.0, 3)
        t, p = area_light(le)
        s.primitives.append(Primitive(t, p, quad((x0, h, 0.4), (x1, h, 0.4), (x1, h, 0.6), (x0, h, 0.6), (0, -1, 0)),
                                      f"emitter{i}"))

    def tiles(origin, eu, ev, n, normal, name):
        o, eu, ev = np.asarray(origin, float), np.asarray(eu, float), np.asarray(ev, float)
        out = []
        for a in range(n):
            for b in range(n):
                p0 = o + eu * (a / n) + ev * (b / n)
                p1 = o + eu * ((a + 1) / n) + ev * (b / n)
                p2 = o + eu * ((a + 1) / n) + ev * ((b + 1) / n)
                p3 = o + eu * (a / n) + ev * ((b + 1) / n)
                out.append((quad(p0, p1, p2, p3, normal), f"{name}{a}{b}"))
        return out

    groups = []
    groups += tiles((0, 0, 0), (1, 0, 0), (0, 1, 0), 4, (0, 0, 1), "back")
    groups += tiles((0, 0, 1), (1, 0, 0), (0, 0, -1), 3, (0, 1, 0), "floor")
    groups += tiles((0, 1, 0), (1, 0, 0), (0, 0, 1), 3, (0, -1, 0), "ceiling")
    groups += tiles((0, 0, 0), (0, 1, 0), (0, 0, 1), 3, (1, 0, 0), "left")
    groups += tiles((1, 0, 1), (0, 1, 0), (0, 0, -1), 3, (-1, 0, 0), "right")
    for bi, b in enumerate([box((0.33, 0.3, 0.37), (0.3, 0.6, 0.3), 15.0), box((0.68, 0.15, 0.65), (0.3, 0.3, 0.3), -18.0)]):
        for f in range(6):
            idx = np.arange(4 * f, 4 * f + 4)
            groups.append((Mesh(b.positions[idx].copy(), b.normals[idx].copy(), np.array([[0, 1, 2], [0, 2, 3]], np.int64)),
                           f"box{bi}f{f}"))
    assert len(groups) == 64
    for m, name in groups:
        r = rng.uniform(0.05, 0.95, 3).astype(np.float32).astype(np.float64)
        t, p = diffuse(r)
        s.primitives.append(Primitive(t, p, m, name))
    s.primitives.append(pinhole((0.5, 0.5, 2.4), (0.5, 0.5, 0.0), (0, 1, 0), 36.0))
    return s


WORKLOADS["inverse_box"] = inverse_box


def _sliver_face(rng, corner, eu, ev, normal, mu, sigma):
    """Rectangle corner + [0,1] eu + [0,1] ev (|eu| >= |ev|) cut across ev into strips of two
    long thin triangles each; every triangle's area is drawn log-normal(mu, sigma), the last
    strip is clipped to the rectangle. Returns (positions (V,3), faces (F,3)) in float64."""
    L = float(np.linalg.norm(eu))
    S = float(np.linalg.norm(ev))
    mean = math.exp(mu + 0.5 * sigma * sigma)
    chunks, total = [], 0.0
    while total < S:
        w = 2.0 * rng.lognormal(mu, sigma, int(1.2 * S * L / (2.0 * mean)) + 8) / L
        chunks.append(w)
        total += float(w.sum())
    cw = np.cumsum(np.concatenate(chunks))
    k = int(np.searchsorted(cw, S))
    f = np.concatenate([[0.0], np.minimum(cw[:k + 1], S)]) / S  # strip edges along ev
    n = len(f) - 1
    P = corner + f[:, None] * ev                                   # P_i on the corner edge
    Q = P + eu                                                     # Q_i on the far edge
    V = np.concatenate([P, Q])
    i = np.arange(n)
    F = np.concatenate([np.stack([i, n + 1 + i, n + 2 + i], 1), np.stack([i, n + 2 + i, i + 1], 1)])
    if np.dot(np.cross(eu, ev), normal) < 0:
        F = F[:, ::-1]
    return V, F


def precision_interior(num_triangles: int = 10_000_000, seed: int = 4, mu: float = -9.0, sigma: float = 2.5,
                       light_le: float = 4.0e4) -> SceneDesc:
    """The FP32-vs-FP64 precision workload: a furnished hall whose coordinates span 1e-3 to
    1e3 scene units, built from long thin triangles.

    * Hall: 2000 x 1000 x 2000 box (walls, ceiling), diffuse grey 0.4, facing in.
    * Floor: graded square tiling around the origin, tiles h_k / 4 wide in the ring between
      the squares of half-width h_(k-1) and h_k = 1000 / 2^(20-k): 9.5e-4 units next to the
      origin, 250 units at the walls.
    * Furniture: boxes of largest side s log-uniform in [1e-3, 2.4] (other sides s x U[0.15, 1]),
      standing on the floor at distance s x 10^U[0.25, 1.4] from the origin, aligned with the
      hall (turned by 0 or 90 degrees) except one in ten turned by U[0, 180) degrees, in 4
      diffuse albedo classes. Every face is cut into strips of two
      long thin triangles with log-normal(mu, sigma) areas, until `num_triangles` in total.
    * Light: one 0.05 x 0.05 quad emitter, 0.5 below a 60 x 60 white panel at height 3 and
      facing it, so every path reaches the camera through at least one bounce.
    """
    rng = np.random.default_rng(seed)
    s = SceneDesc()
    # hall shell (inward normals)
    H, W = 1000.0, 1000.0
    shell = [quad((-W, 0, -W), (-W, H, -W), (-W, H, W), (-W, 0, W), (1, 0, 0)),
             quad((W, 0, W), (W, H, W), (W, H, -W), (W, 0, -W), (-1, 0, 0)),
             quad((W, 0, -W), (W, H, -W), (-W, H, -W), (-W, 0, -W), (0, 0, 1)),
             quad((-W, 0, W), (-W, H, W), (W, H, W), (W, 0, W), (0, 0, -1)),
             quad((-W, H, -W), (W, H, -W), (W, H, W), (-W, H, W), (0, -1, 0))]
    t, p = diffuse((0.4, 0.4, 0.4))
    s.primitives.append(Primitive(t, p, _merge(shell), "hall"))
    # graded floor
    tiles = []
    h = [W / 2 ** (20 - k) for k in range(21)]
    for k in range(21):
        size = h[k] / 2 if k == 0 else h[k] / 4
        n = 2 if k == 0 else 8
        for a in range(n):
            for b in range(n):
                x0, z0 = -h[k] + a * size, -h[k] + b * size
                if k > 0 and -h[k - 1] <= x0 < h[k - 1] and -h[k - 1] <= z0 < h[k - 1]:
                    continue
                tiles.append(quad((x0, 0, z0 + size), (x0 + size, 0, z0 + size), (x0 + size, 0, z0), (x0, 0, z0),
                                  (0, 1, 0)))
    t, p = diffuse((0.5, 0.5, 0.5))
    s.primitives.append(Primitive(t, p, _merge(tiles), "floor"))
    # reflector panel and the light under it
    t, p = diffuse((0.8, 0.8, 0.8))
    s.primitives.append(Primitive(t, p, quad((-30, 3, -30), (30, 3, -30), (30, 3, 30), (-30, 3, 30), (0, -1, 0)),
                                  "panel"))
    lt, lp = area_light((light_le, light_le, light_le))
    lx, ly, lz, e = 0.4, 2.5, -0.6, 0.025
    s.primitives.append(Primitive(lt, lp, quad((lx - e, ly, lz + e), (lx + e, ly, lz + e), (lx + e, ly, lz - e),
                                               (lx - e, ly, lz - e), (0, 1, 0)), "light"))
    eye = np.array([3.0, 2.2, 7.0])
    # furniture
    albedo = [(0.7, 0.55, 0.35), (0.75, 0.75, 0.72), (0.35, 0.38, 0.42), (0.6, 0.2, 0.15)]
    parts = [([], []) for _ in albedo]
    count = 0
    unit_faces = [((-1, -1, 1), (1, 0, 0), (0, 1, 0), (0, 0, 1)), ((1, -1, -1), (-1, 0, 0), (0, 1, 0), (0, 0, -1)),
                  ((1, -1, 1), (0, 0, -1), (0, 1, 0), (1, 0, 0)), ((-1, -1, -1), (0, 0, 1), (0, 1, 0), (-1, 0, 0)),
                  ((-1, 1, 1), (1, 0, 0), (0, 0, -1), (0, 1, 0)), ((-1, -1, -1), (1, 0, 0), (0, 0, 1), (0, -1, 0))]
    while count < num_triangles:
        smax = 10 ** rng.uniform(-3.0, math.log10(2.4))
        dims = smax * np.concatenate([[1.0], rng.uniform(0.15, 1.0, 2)])
        dims = rng.permutation(dims)
        r = smax * 10 ** rng.uniform(0.25, 1.4)
        phi = rng.uniform(0, 2 * math.pi)
        c = np.array([r * math.cos(phi), dims[1] / 2, r * math.sin(phi)])
        if math.hypot(c[0] - eye[0], c[2] - eye[2]) < smax + 0.6:
            continue
        # furniture follows the hall's grid, except one piece in ten
        th = rng.uniform(0, math.pi) if rng.uniform() < 0.1 else 0.5 * math.pi * int(rng.integers(2))
        rot = np.array([[math.cos(th), 0, math.sin(th)], [0, 1, 0], [-math.sin(th), 0, math.cos(th)]])
        half = dims / 2
        cls = int(rng.integers(len(albedo)))
        for q0, du, dv, nn in unit_faces:
            corner = c + rot @ (np.array(q0) * half)
            eu = rot @ (np.array(du) * 2 * half)
            ev = rot @ (np.array(dv) * 2 * half)
            nrm = rot @ np.array(nn, np.float64)
            if np.linalg.norm(eu) < np.linalg.norm(ev):
                eu, ev = ev, eu
            V, F = _sliver_face(rng, corner, eu, ev, nrm, mu, sigma)
            parts[cls][0].append((V, nrm))
            parts[cls][1].append(F)
            count += len(F)
    for cls, (vs, fs) in enumerate(parts):
        if not vs:
            continue
        base = np.cumsum([0] + [len(v) for v, _ in vs[:-1]])
        P = np.concatenate([v for v, _ in vs])
        N = np.concatenate([np.broadcast_to(n, v.shape) for v, n in vs])
        F = np.concatenate([f + b for f, b in zip(fs, base)])
        t, p = diffuse(albedo[cls])
        s.primitives.append(Primitive(t, p, Mesh(_f32(P), _f32(N), F.astype(np.int64)), f"furniture{cls}"))
    s.primitives.append(pinhole(eye, (0.0, 0.2, 0.0), (0, 1, 0), 45.0))
    return s


def _merge(meshes) -> Mesh:
    base = np.cumsum([0] + [len(m.positions) for m in meshes[:-1]])
    uvs = [m.uvs if m.uvs is not None else np.zeros((len(m.positions), 2), np.float32) for m in meshes]
    return Mesh(np.concatenate([m.positions for m in meshes]), np.concatenate([m.normals for m in meshes]),
                np.concatenate([m.faces + b for m, b in zip(meshes, base)]), np.concatenate(uvs))


def batch_jobs(num_jobs: int = 256, seed: int = 1000, pool_size: int = 160, max_tris: int = 200_000):
    """The batched-render workload: `num_jobs` independent jobs, each with a resolution drawn
    uniformly from {64^2, 128^2, 256^2, 512^2}, a triangle count log-uniform in 1k..max_tris,
    spp log-uniform 16..1024, max path length uniform 4..24 and the terrain workload's material
    distribution. Each job's clutter is a random subset (seeded per job: seed + job index) of a
    shared pool of icospheres (levels 1-4) and boxes, plus a floor, 1-2 quad lights and a camera.

    Returns (primitives of the pool, list of job dicts) -- pass them to write_batch()."""
    prng = np.random.default_rng(seed - 1)
    pool = []
    for i in range(pool_size):
        kind = prng.integers(0, 5)
        c = prng.uniform(-4, 4, 3) * np.array([1.0, 0.0, 1.0]) + np.array([0.0, 0.0, 0.0])
        if kind < 4:
            level = int(kind) + 1
            r = float(np.exp(prng.uniform(np.log(0.15), np.log(0.8))))
            c[1] = r
            mesh = sphere_mesh(c, r, level)
        else:
            sz = prng.uniform(0.2, 1.2, 3)
            c[1] = sz[1] / 2
            mesh = box(c, sz, float(prng.uniform(-45, 45)))
        k = int(prng.integers(0, 4))
        if k == 0:
            t, p = diffuse(prng.uniform(0.1, 0.9, 3))
        elif k == 1:
            t, p = glossy(prng.uniform(0.5, 1.0, 3), phong_to_beckmann(float(np.exp(prng.uniform(np.log(10), np.log(1000))))))
        elif k == 2:
            t, p = mirror((0.95, 0.95, 0.95))
        else:
            t, p = glass(1.5)
        pool.append(Primitive(t, p, mesh, f"pool{i}"))
    sizes = np.array([len(p.mesh.faces) for p in pool])
    jobs = []
    for j in range(num_jobs):
        rng = np.random.default_rng(seed + j)
        res = int(rng.choice([64, 128, 256, 512]))
        target = int(np.exp(rng.uniform(np.log(1000), np.log(max_tris))))
        spp = int(np.exp(rng.uniform(np.log(16), np.log(1024))))
        m = int(rng.integers(4, 25))
        order = rng.permutation(pool_size)
        chosen, total = [], 0
        for i in order:
            if total >= target:
                break
            if total + sizes[i] > 1.5 * target and total > 0:
                continue
            chosen.append(int(i))
            total += int(sizes[i])
        nl = int(rng.integers(1, 3))
        lights = [(rng.uniform(-3, 3), rng.uniform(-3, 3), rng.uniform(5.0, 20.0, 3)) for _ in range(nl)]
        ang = rng.uniform(0, 2 * np.pi)
        eye = (9.0 * np.cos(ang), rng.uniform(3.0, 6.0), 9.0 * np.sin(ang))
        jobs.append({"res": res, "spp": spp, "max_vertices": m, "pool": chosen, "triangles": total + 2 + 2 * nl,
                     "lights": lights, "eye": eye, "renderer": "ptdirect", "seed": seed + j})
    return pool, jobs


def _batch_light(lx, lz) -> Mesh:
    return quad((lx - 0.7, 6.0, lz - 0.7), (lx + 0.7, 6.0, lz - 0.7), (lx + 0.7, 6.0, lz + 0.7), (lx - 0.7, 6.0, lz + 0.7),
                (0, -1, 0))


def _batch_floor() -> Mesh:
    return quad((-6, 0, 6), (6, 0, 6), (6, 0, -6), (-6, 0, -6), (0, 1, 0))


def batch_job_desc(pool, job) -> SceneDesc:
    """The scene of one batch job in memory, primitives in the order write_batch writes them
    (lights, floor, the job's pool subset, camera)."""
    s = SceneDesc()
    for lx, lz, le in job["lights"]:
        t, p = area_light(le)
        s.primitives.append(Primitive(t, p, _batch_light(lx, lz), "light"))
    t, p = diffuse((0.5, 0.5, 0.5))
    s.primitives.append(Primitive(t, p, _batch_floor(), "floor"))
    for i in job["pool"]:
        s.primitives.append(pool[i])
    s.primitives.append(pinhole(job["eye"], (0.0, 0.5, 0.0), (0, 1, 0), 50.0))
    return s


def write_batch(pool, jobs, directory) -> list:
    """Writes the pool's OBJ files once and one YAML per job; returns the YAML paths."""
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    files = []
    for i, p in enumerate(pool):
        fn = f"pool_{i:04d}.obj"
        if not (d / fn).exists():
            write_obj(d / fn, p.mesh, p.name)
        files.append(fn)
    if not (d / "floor.obj").exists():
        write_obj(d / "floor.obj", _batch_floor(), "floor")
    paths = []
    for j, job in enumerate(jobs):
        lines = ["version: 5", "scene:", "  primitives:"]

        def add(type_list, params, mesh_file):
            lines.append(f"    - type: [{', '.join(type_list)}]")
            if mesh_file:
                lines.append("      mesh:")
                lines.append(f"        path: '{mesh_file}'")
            lines.append("      params:")
            lines.append(_yaml_value(params, 8).rstrip("\n"))

        for k, (lx, lz, le) in enumerate(job["lights"]):
            fn = f"light_{j:04d}_{k}.obj"
            write_obj(d / fn, _batch_light(lx, lz), "light")
            t, p = area_light(le)
            add(t, p, fn)
        t, p = diffuse((0.5, 0.5, 0.5))
        add(t, p, "floor.obj")
        for i in job["pool"]:
            add(pool[i].type, pool[i].params, files[i])
        cam = pinhole(job["eye"], (0.0, 0.5, 0.0), (0, 1, 0), 50.0)
        add(cam.type, cam.params, None)
        path = d / f"job_{j:04d}.yml"
        path.write_text("\n".join(lines) + "\n")
        paths.append(path)
    return paths
