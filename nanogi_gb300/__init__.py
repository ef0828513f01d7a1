"""nanogi-gb300: GB300-native `pt` / `ptdirect` path tracing behind nanogi's renderer interface.

Python mirror of the reference's host API (src/nanogi.cpp, include/nanogi/rt.hpp) over
the C ABI of include/nanogi.h:

* ``Scene.load(path, aspect)``   -- Scene::Load (rt.hpp:1519)
* ``Renderer(...).render(scene)`` -- Renderer::Load + Renderer::Render (nanogi.cpp:117, 182)
* ``save_image(path, film)``     -- SaveImage (basic.hpp:506)

The film is a numpy array of shape (height, width, 3), float64, row 0 = bottom scanline,
i.e. the reference's std::vector<glm::dvec3> reshaped.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

from . import capi
from .capi import NanogiError, RenderParams, RenderStats, SceneInfo, check, load_library

__all__ = ["Scene", "Renderer", "NanogiError", "render_batch", "save_image", "load_hdr", "load_library"]


def _ptr(a: np.ndarray) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data)


class Scene:
    """A loaded scene: host arrays plus (after ``build``) the BVH and tables in HBM."""

    def __init__(self, handle: int):
        self._h = ctypes.c_void_p(handle)

    @classmethod
    def load(cls, path: str | os.PathLike, aspect: float) -> "Scene":
        lib = load_library()
        h = ctypes.c_void_p()
        check(lib.ngi_scene_load(os.fsencode(str(path)), float(aspect), ctypes.byref(h)))
        return cls(h.value)

    @classmethod
    def load_with_meshes(cls, path: str | os.PathLike, aspect: float, meshes: dict) -> "Scene":
        """Like ``load``, but a mesh path that is a key of ``meshes`` takes that mesh from memory:
        ``{path: (positions (V,3) float32, faces (F,3) uint32[, normals (V,3) float32 or None[, uvs (V,2)
        float32 or None]])}``."""
        lib = load_library()
        keep = []
        arr = (capi.MeshData * max(len(meshes), 1))()

        def opt(m, k, cols):
            return None if len(m) <= k or m[k] is None else np.ascontiguousarray(m[k], np.float32).reshape(-1, cols)

        for i, (name, m) in enumerate(meshes.items()):
            pos = np.ascontiguousarray(m[0], np.float32).reshape(-1, 3)
            faces = np.ascontiguousarray(m[1], np.uint32).reshape(-1, 3)
            nrm, uv = opt(m, 2, 3), opt(m, 3, 2)
            keep += [pos, faces, nrm, uv]
            arr[i] = capi.MeshData(os.fsencode(str(name)), pos.ctypes.data, None if nrm is None else nrm.ctypes.data,
                                   None if uv is None else uv.ctypes.data, faces.ctypes.data, pos.shape[0],
                                   faces.shape[0])
        h = ctypes.c_void_p()
        check(lib.ngi_scene_load_with_meshes(os.fsencode(str(path)), float(aspect), arr, len(meshes), ctypes.byref(h)))
        return cls(h.value)

    @property
    def handle(self) -> ctypes.c_void_p:
        if not self._h:
            raise ValueError("scene is closed")
        return self._h

    def close(self) -> None:
        if self._h:
            load_library().ngi_scene_free(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> dict:
        inf = SceneInfo()
        check(load_library().ngi_scene_get_info(self.handle, ctypes.byref(inf)))
        d = {k: getattr(inf, k) for k, _ in SceneInfo._fields_}
        d["bound_min"] = list(inf.bound_min)
        d["bound_max"] = list(inf.bound_max)
        return d

    def triangles(self):
        """Flattened host arrays: pos (n,3,3), nrm (n,3,3), uv (n,3,2) float32, prim (n,) int32."""
        n = self.info()["num_triangles"]
        pos = np.empty((n, 3, 3), np.float32)
        nrm = np.empty((n, 3, 3), np.float32)
        uv = np.empty((n, 3, 2), np.float32)
        prim = np.empty(n, np.int32)
        check(load_library().ngi_scene_get_triangles(self.handle, _ptr(pos), _ptr(nrm), _ptr(uv), _ptr(prim)))
        return pos, nrm, uv, prim

    def build(self) -> None:
        check(load_library().ngi_scene_build(self.handle))

    def release_buffers(self) -> None:
        """Frees the render buffers kept between renders; the next render allocates them again."""
        check(load_library().ngi_scene_release_buffers(self.handle))

    def intersect(self, rays: np.ndarray):
        """rays: (n, 8) float32 = ox, oy, oz, tmin, dx, dy, dz, tmax -> (prim, t, uv)."""
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        n = rays.shape[0]
        prim = np.empty(n, np.int32)
        t = np.empty(n, np.float32)
        uv = np.empty((n, 2), np.float32)
        check(load_library().ngi_intersect(self.handle, _ptr(rays), n, _ptr(prim), _ptr(t), _ptr(uv)))
        return prim, t, uv

    def visible(self, pairs: np.ndarray) -> np.ndarray:
        """pairs: (n, 6) float64 = p1, p2 -> bool array (Scene::Visible)."""
        pairs = np.ascontiguousarray(pairs, dtype=np.float64).reshape(-1, 6)
        out = np.empty(pairs.shape[0], np.uint8)
        check(load_library().ngi_visible(self.handle, _ptr(pairs), pairs.shape[0], _ptr(out)))
        return out.astype(bool)

    def parameters(self):
        """(albedo, emission): (num_primitives, 3) float64 arrays of R and Le."""
        n = self.info()["num_primitives"]
        a = np.empty((n, 3), np.float64)
        e = np.empty((n, 3), np.float64)
        check(load_library().ngi_scene_get_parameters(self.handle, _ptr(a), _ptr(e)))
        return a, e

    def set_parameters(self, albedo=None, emission=None) -> None:
        n = self.info()["num_primitives"]
        a = None if albedo is None else np.ascontiguousarray(albedo, np.float64).reshape(n, 3)
        e = None if emission is None else np.ascontiguousarray(emission, np.float64).reshape(n, 3)
        check(load_library().ngi_scene_set_parameters(self.handle, None if a is None else _ptr(a),
                                                      None if e is None else _ptr(e)))

    def last_stats(self) -> dict:
        st = RenderStats()
        check(load_library().ngi_get_render_stats(self.handle, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in RenderStats._fields_}


@dataclass
class Renderer:
    """Renderer::Params of the reference (src/nanogi.cpp:85-97) plus the GPU knobs."""

    renderer: str = "pt"
    num_samples: int = 10_000_000
    max_num_vertices: int = -1
    width: int = 1280
    height: int = 720
    seed: int = 0
    sample_offset: int = 0
    precision: str = "fp32"
    raster: str = "stratified"
    wave_size: int = 0
    iterations_per_graph: int = 0
    flags: int = 0
    trace_refill: int = 0
    ray_offset: str = "reference"
    last_stats: dict = field(default_factory=dict, repr=False)

    def params(self) -> RenderParams:
        if self.renderer not in capi.RENDERERS:
            raise NanogiError(1, f"renderer '{self.renderer}' is not one of pt, ptdirect, lt, ltdirect, bdpt")
        return RenderParams(
            renderer=capi.RENDERERS[self.renderer],
            max_num_vertices=int(self.max_num_vertices),
            num_samples=int(self.num_samples),
            width=int(self.width),
            height=int(self.height),
            seed=int(self.seed) & 0xFFFFFFFFFFFFFFFF,
            sample_offset=int(self.sample_offset),
            precision=capi.PRECISIONS[self.precision],
            raster_mode=capi.RASTER_MODES[self.raster],
            wave_size=int(self.wave_size),
            iterations_per_graph=int(self.iterations_per_graph),
            flags=int(self.flags),
            trace_refill=int(self.trace_refill),
            ray_offset=capi.RAY_OFFSETS[self.ray_offset],
        )

    def render(self, scene: Scene, film: np.ndarray | None = None) -> np.ndarray:
        """Renders into a host film (normalised by W*H/N like RenderProcess)."""
        p = self.params()
        if film is None:
            film = np.empty((self.height, self.width, 3), np.float64)
        if film.dtype != np.float64 or not film.flags.c_contiguous or film.size != 3 * self.width * self.height:
            raise ValueError("film must be a C-contiguous float64 array of width*height*3")
        check(load_library().ngi_render(scene.handle, ctypes.byref(p), _ptr(film)))
        self.last_stats = scene.last_stats()
        return film

    def backward(self, scene: Scene, d_film: np.ndarray):
        """Path-replay adjoint of render(): dLoss/dalbedo, dLoss/demission per primitive."""
        p = self.params()
        d = np.ascontiguousarray(d_film, np.float64)
        if d.size != 3 * self.width * self.height:
            raise ValueError("d_film must hold width*height*3 values")
        n = scene.info()["num_primitives"]
        ga = np.empty((n, 3), np.float64)
        ge = np.empty((n, 3), np.float64)
        check(load_library().ngi_render_backward(scene.handle, ctypes.byref(p), _ptr(d), _ptr(ga), _ptr(ge)))
        self.last_stats = scene.last_stats()
        return ga, ge

    def render_device(self, scene: Scene, d_film_ptr: int, stream: int = 0) -> None:
        """Adds raw (un-normalised) sums into a device film (e.g. a torch.cuda tensor's data_ptr)."""
        p = self.params()
        check(load_library().ngi_render_device(scene.handle, ctypes.byref(p), ctypes.c_void_p(d_film_ptr),
                                               ctypes.c_void_p(stream)))
        self.last_stats = scene.last_stats()


def render_batch(jobs, autotune: bool = False, wave_size: int = 0, trace_refill: int = 0,
                 iterations_per_graph: int = 0, autotune_fraction: float = 0.0):
    """Renders [(scene, Renderer), ...] in one persistent wave (ngi_render_batch).
    Returns (films, stats): one (H, W, 3) film per job, normalised like Renderer.render."""
    from .capi import BatchOptions, BatchStats

    n = len(jobs)
    scenes = (ctypes.c_void_p * n)(*[s.handle.value for s, _ in jobs])
    params = (RenderParams * n)(*[r.params() for _, r in jobs])
    films = [np.empty((r.height, r.width, 3), np.float64) for _, r in jobs]
    ptrs = (ctypes.c_void_p * n)(*[f.ctypes.data for f in films])
    opt = BatchOptions(autotune=int(autotune), wave_size=int(wave_size), trace_refill=int(trace_refill),
                       iterations_per_graph=int(iterations_per_graph), autotune_fraction=float(autotune_fraction))
    st = BatchStats()
    check(load_library().ngi_render_batch(scenes, params, n, ptrs, ctypes.byref(opt), ctypes.byref(st)))
    return films, {k: getattr(st, k) for k, _ in BatchStats._fields_}


def save_image(path: str | os.PathLike, film: np.ndarray) -> None:
    film = np.ascontiguousarray(film, dtype=np.float64)
    h, w = film.shape[:2]
    check(load_library().ngi_save_image(os.fsencode(str(path)), _ptr(film), w, h))


def load_hdr(path: str | os.PathLike, width: int, height: int) -> np.ndarray:
    film = np.empty((height, width, 3), np.float64)
    check(load_library().ngi_load_hdr(os.fsencode(str(path)), _ptr(film), width, height))
    return film


def load_texture(path: str | os.PathLike) -> np.ndarray:
    """A TexR image as (H, W, 3) float32, row 0 = the image's top row (Texture::Load)."""
    lib = load_library()
    w, h = ctypes.c_int32(), ctypes.c_int32()
    check(lib.ngi_load_texture(os.fsencode(str(path)), None, ctypes.byref(w), ctypes.byref(h)))
    img = np.empty((h.value, w.value, 3), np.float32)
    check(lib.ngi_load_texture(os.fsencode(str(path)), _ptr(img), ctypes.byref(w), ctypes.byref(h)))
    return img
