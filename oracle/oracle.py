"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, only as the
checker or the timed CPU baseline. Nothing in the product imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "ngi_oracle.cpp"
HDR = HERE / "ngi_oracle.h"
OUT = HERE / "_build"
LIB = OUT / "libngi_oracle.so"


def build_oracle() -> Path:
    """Compiles the oracle with g++ (no FMA contraction, so FP32 traversal is reproducible)."""
    OUT.mkdir(exist_ok=True)
    if LIB.exists() and LIB.stat().st_mtime >= max(SRC.stat().st_mtime, HDR.stat().st_mtime):
        return LIB
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-o", str(LIB), str(SRC)]
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + proc.stdout)
    return LIB


class PrimDesc(ctypes.Structure):
    _fields_ = [
        ("type", ctypes.c_int32), ("has_mesh", ctypes.c_int32),
        ("tri_first", ctypes.c_int64), ("tri_count", ctypes.c_int64),
        ("l_type", ctypes.c_int32), ("e_type", ctypes.c_int32),
        ("Le", ctypes.c_double * 3), ("l_position", ctypes.c_double * 3), ("l_direction", ctypes.c_double * 3),
        ("We", ctypes.c_double * 3),
        ("eye", ctypes.c_double * 3), ("center", ctypes.c_double * 3), ("up", ctypes.c_double * 3),
        ("fov_deg", ctypes.c_double),
        ("D_R", ctypes.c_double * 3),
        ("G_R", ctypes.c_double * 3), ("G_eta", ctypes.c_double * 3), ("G_k", ctypes.c_double * 3),
        ("G_roughness", ctypes.c_double),
        ("s_type", ctypes.c_int32), ("has_uv", ctypes.c_int32),
        ("S_R", ctypes.c_double * 3), ("S_eta1", ctypes.c_double), ("S_eta2", ctypes.c_double),
        ("D_tex", ctypes.c_void_p), ("D_tex_w", ctypes.c_int32), ("D_tex_h", ctypes.c_int32),
        ("G_tex", ctypes.c_void_p), ("G_tex_w", ctypes.c_int32), ("G_tex_h", ctypes.c_int32),
    ]


class RenderParams(ctypes.Structure):
    _fields_ = [
        ("renderer", ctypes.c_int32), ("max_vertices", ctypes.c_int32), ("num_samples", ctypes.c_int64),
        ("width", ctypes.c_int32), ("height", ctypes.c_int32), ("seed", ctypes.c_uint64),
        ("sample_offset", ctypes.c_int64), ("rng_mode", ctypes.c_int32), ("raster_mode", ctypes.c_int32),
        ("num_threads", ctypes.c_int32), ("use_bvh", ctypes.c_int32), ("grain_size", ctypes.c_int64),
        ("ray_offset", ctypes.c_int32), ("pad_", ctypes.c_int32),
    ]


class RenderStats(ctypes.Structure):
    _fields_ = [("camera_rays", ctypes.c_int64), ("extension_rays", ctypes.c_int64),
                ("shadow_rays", ctypes.c_int64), ("seconds", ctypes.c_double), ("threads", ctypes.c_int32),
                ("extension_misses", ctypes.c_int64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build_oracle()
        L = ctypes.CDLL(str(LIB))
        P = ctypes.POINTER
        v = ctypes.c_void_p
        L.ora_scene_create.restype = v
        L.ora_scene_create.argtypes = [P(PrimDesc), ctypes.c_int32, v, v, v, ctypes.c_int64, ctypes.c_double]
        L.ora_scene_free.argtypes = [v]
        L.ora_last_error.restype = ctypes.c_char_p
        L.ora_intersect.argtypes = [v, v, ctypes.c_int64, ctypes.c_int32, v, v, v]
        L.ora_visible.argtypes = [v, v, ctypes.c_int64, ctypes.c_int32, v]
        L.ora_render.argtypes = [v, P(RenderParams), v, P(RenderStats)]
        L.ora_philox4x32_10.argtypes = [v, v, v]
        L.ora_mt19937_nth.restype = ctypes.c_uint32
        L.ora_mt19937_nth.argtypes = [ctypes.c_uint32, ctypes.c_int64]
        L.ora_mt19937_uniform.restype = ctypes.c_double
        L.ora_mt19937_uniform.argtypes = [ctypes.c_uint32, ctypes.c_int64]
        L.ora_bsdf_sample.argtypes = [P(PrimDesc), v, v, v, v, v]
        L.ora_bsdf_eval.argtypes = [P(PrimDesc), v, v, ctypes.c_int, v, v]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


TYPE_BITS = {"D": 1, "G": 2, "S": 4, "L": 8, "E": 16}


def prim_desc(type_list, params: dict, textures=None, keep=None) -> PrimDesc:
    """PrimDesc from the schema's type list and params mapping (schema.yml:33-334).
    `textures` maps a TexR path to its texels ((H, W, 3) float32, row 0 = the image's top
    row); the arrays handed to the oracle are appended to `keep`."""
    d = PrimDesc()

    def tex(name):
        a = np.ascontiguousarray(np.asarray(textures[name], np.float32))
        keep.append(a)
        return a.ctypes.data, a.shape[1], a.shape[0]

    for t in type_list:
        d.type |= TYPE_BITS[t]

    def v3(x):
        return (ctypes.c_double * 3)(*[float(y) for y in x])

    if "L" in params and (d.type & 8):
        L = params["L"]
        kind = L["type"]
        d.l_type = {"area": 0, "point": 1, "directional": 2}[kind]
        d.Le = v3(L[kind]["Le"])
        if kind == "point":
            d.l_position = v3(L["point"]["position"])
        if kind == "directional":
            d.l_direction = v3(L["directional"]["direction"])
    if "E" in params and (d.type & 16):
        E = params["E"]
        kind = E["type"]
        d.e_type = {"area": 0, "pinhole": 1}[kind]
        d.We = v3(E[kind]["We"])
        if kind == "pinhole":
            d.eye = v3(E["pinhole"]["view"]["eye"])
            d.center = v3(E["pinhole"]["view"]["center"])
            d.up = v3(E["pinhole"]["view"]["up"])
            d.fov_deg = float(E["pinhole"]["perspective"]["fov"])
    if "D" in params and (d.type & 1):
        if "R" in params["D"]:
            d.D_R = v3(params["D"]["R"])
        else:
            d.D_tex, d.D_tex_w, d.D_tex_h = tex(params["D"]["TexR"])
    if "G" in params and (d.type & 2):
        G = params["G"]
        if "R" in G:
            d.G_R = v3(G["R"])
        else:
            d.G_tex, d.G_tex_w, d.G_tex_h = tex(G["TexR"])
        d.G_eta = v3(G["Eta"])
        d.G_k = v3(G["K"])
        d.G_roughness = float(G["Roughness"])
    if "S" in params and (d.type & 4):
        S = params["S"]
        kind = S["type"]
        d.s_type = {"reflection": 0, "refraction": 1, "fresnel": 2}[kind]
        d.S_R = v3(S[kind]["R"])
        if kind != "reflection":
            d.S_eta1 = float(S[kind]["eta1"])
            d.S_eta2 = float(S[kind]["eta2"])
    return d


def flatten(primitives, textures=None, keep=None):
    """primitives: iterable of (type_list, params, mesh-or-None) where mesh has positions,
    normals, faces, uvs. Returns (PrimDesc array, tri_pos, tri_nrm, tri_uv)."""
    descs, pos, nrm, uvs = [], [], [], []
    keep = [] if keep is None else keep
    first = 0
    for type_list, params, mesh in primitives:
        d = prim_desc(type_list, params, textures, keep)
        if mesh is not None:
            F = np.asarray(mesh.faces, np.int64)
            P = np.asarray(mesh.positions, np.float32)
            N = np.asarray(mesh.normals, np.float32)
            pos.append(P[F].reshape(-1, 9))
            nrm.append(N[F].reshape(-1, 9))
            if mesh.uvs is not None:
                uvs.append(np.asarray(mesh.uvs, np.float32)[F].reshape(-1, 6))
                d.has_uv = 1
            else:
                uvs.append(np.zeros((len(F), 6), np.float32))
            d.has_mesh = 1
            d.tri_first = first
            d.tri_count = len(F)
            first += len(F)
        descs.append(d)
    arr = (PrimDesc * len(descs))(*descs)
    cat = lambda xs, k: np.ascontiguousarray(np.concatenate(xs) if xs else np.zeros((0, k), np.float32))
    return arr, cat(pos, 9), cat(nrm, 9), cat(uvs, 6)


class OracleScene:
    def __init__(self, primitives, aspect: float, textures=None):
        self._tex_keep = []
        self.descs, self.pos, self.nrm, self.uv = flatten(primitives, textures, self._tex_keep)
        h = lib().ora_scene_create(self.descs, len(self.descs), _p(self.pos), _p(self.nrm), _p(self.uv),
                                   len(self.pos), float(aspect))
        if not h:
            raise RuntimeError(lib().ora_last_error().decode())
        self._h = ctypes.c_void_p(h)

    @classmethod
    def from_desc(cls, desc, aspect: float) -> "OracleScene":
        return cls([(p.type, p.params, p.mesh) for p in desc.primitives], aspect, getattr(desc, "textures", None))

    def close(self):
        if self._h:
            lib().ora_scene_free(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_triangles(self) -> int:
        return len(self.pos)

    def intersect(self, rays: np.ndarray, use_bvh: bool = False):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = rays.shape[0]
        prim = np.empty(n, np.int32)
        t = np.empty(n, np.float32)
        uv = np.empty((n, 2), np.float32)
        lib().ora_intersect(self._h, _p(rays), n, int(use_bvh), _p(prim), _p(t), _p(uv))
        return prim, t, uv

    def visible(self, pairs: np.ndarray, use_bvh: bool = True) -> np.ndarray:
        pairs = np.ascontiguousarray(pairs, np.float64).reshape(-1, 6)
        out = np.empty(pairs.shape[0], np.uint8)
        lib().ora_visible(self._h, _p(pairs), pairs.shape[0], int(use_bvh), _p(out))
        return out.astype(bool)

    def render(self, renderer="pt", num_samples=1000, max_vertices=-1, width=16, height=16, seed=0,
               sample_offset=0, rng_mode="replay", raster="stratified", threads=0, use_bvh=True, grain=1000,
               ray_offset="reference"):
        p = RenderParams(renderer={"pt": 0, "ptdirect": 1, "lt": 2, "ltdirect": 3, "bdpt": 4}[renderer], max_vertices=max_vertices,
                         num_samples=num_samples, width=width, height=height, seed=seed & 0xFFFFFFFFFFFFFFFF,
                         sample_offset=sample_offset, rng_mode={"reference": 0, "replay": 1}[rng_mode],
                         raster_mode={"stratified": 0, "uniform": 1}[raster], num_threads=threads,
                         use_bvh=int(use_bvh), grain_size=grain,
                         ray_offset={"reference": 0, "scaled": 1}[ray_offset])
        film = np.zeros((height, width, 3), np.float64)
        st = RenderStats()
        if lib().ora_render(self._h, ctypes.byref(p), _p(film), ctypes.byref(st)) != 0:
            raise RuntimeError(lib().ora_last_error().decode())
        self.last_stats = {k: getattr(st, k) for k, _ in RenderStats._fields_}
        return film


def philox4x32_10(ctr, key):
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    out = np.empty(4, np.uint32)
    lib().ora_philox4x32_10(_p(c), _p(k), _p(out))
    return out


def bsdf_sample(type_list, params, wi, u):
    d = prim_desc(type_list, params)
    wi = np.asarray(wi, np.float64)
    u = np.asarray(u, np.float64)
    wo = np.empty(3)
    fs = np.empty(3)
    pdf = np.empty(1)
    ok = lib().ora_bsdf_sample(ctypes.byref(d), _p(wi), _p(u), _p(wo), _p(pdf), _p(fs))
    return bool(ok), wo, float(pdf[0]), fs


def bsdf_eval(type_list, params, wi, wo, force=False):
    d = prim_desc(type_list, params)
    wi = np.asarray(wi, np.float64)
    wo = np.asarray(wo, np.float64)
    fs = np.empty(3)
    pdf = np.empty(1)
    lib().ora_bsdf_eval(ctypes.byref(d), _p(wi), _p(wo), int(force), _p(fs), _p(pdf))
    return fs, float(pdf[0])
