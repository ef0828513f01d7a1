"""ctypes binding of the C ABI declared in include/nanogi.h.

This is the binding a maintainer of the reference would add on the Python side; the
C++ side binds the same header directly. Loading fails loudly when the library has not
been built -- there is no fallback implementation.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libnanogi.so"

NGI_OK = 0
STATUS_NAMES = {
    0: "NGI_OK",
    1: "NGI_ERR_INVALID_ARGUMENT",
    2: "NGI_ERR_IO",
    3: "NGI_ERR_PARSE",
    4: "NGI_ERR_CUDA",
    5: "NGI_ERR_OUT_OF_MEMORY",
    6: "NGI_ERR_DEVICE_TIMEOUT",
    7: "NGI_ERR_UNSUPPORTED",
    8: "NGI_ERR_NO_DEVICE",
}
RENDERERS = {"pt": 0, "ptdirect": 1, "lt": 2, "ltdirect": 3, "bdpt": 4}
PRECISIONS = {"fp32": 0, "fp64": 1}
RASTER_MODES = {"stratified": 0, "uniform": 1}
RAY_OFFSETS = {"reference": 0, "scaled": 1}


class RenderParams(ctypes.Structure):
    _fields_ = [
        ("renderer", ctypes.c_int32),
        ("max_num_vertices", ctypes.c_int32),
        ("num_samples", ctypes.c_int64),
        ("width", ctypes.c_int32),
        ("height", ctypes.c_int32),
        ("seed", ctypes.c_uint64),
        ("sample_offset", ctypes.c_int64),
        ("precision", ctypes.c_int32),
        ("raster_mode", ctypes.c_int32),
        ("wave_size", ctypes.c_int32),
        ("iterations_per_graph", ctypes.c_int32),
        ("flags", ctypes.c_int32),
        ("trace_refill", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("ray_offset", ctypes.c_int32),
    ]


KERNEL_TIMING = 1
TRAVERSAL_COUNTERS = 2
TRACE_ALL_RAYS = 4


class RenderStats(ctypes.Structure):
    _fields_ = [
        ("camera_rays", ctypes.c_int64),
        ("extension_rays", ctypes.c_int64),
        ("shadow_rays", ctypes.c_int64),
        ("film_contributions", ctypes.c_int64),
        ("iterations", ctypes.c_int64),
        ("nonfinite", ctypes.c_int64),
        ("render_ms", ctypes.c_double),
        ("logic_ms", ctypes.c_double),
        ("extend_ms", ctypes.c_double),
        ("shadow_ms", ctypes.c_double),
        ("logic_launches", ctypes.c_int64),
        ("extend_launches", ctypes.c_int64),
        ("shadow_launches", ctypes.c_int64),
        ("extend_nodes", ctypes.c_int64),
        ("extend_tris", ctypes.c_int64),
        ("shadow_nodes", ctypes.c_int64),
        ("shadow_tris", ctypes.c_int64),
        ("finish_paths", ctypes.c_int64),
    ]


class SceneInfo(ctypes.Structure):
    _fields_ = [
        ("num_primitives", ctypes.c_int32),
        ("num_lights", ctypes.c_int32),
        ("sensor_index", ctypes.c_int32),
        ("sensor_type", ctypes.c_int32),
        ("num_triangles", ctypes.c_int64),
        ("num_vertices", ctypes.c_int64),
        ("bound_min", ctypes.c_double * 3),
        ("bound_max", ctypes.c_double * 3),
        ("device_ready", ctypes.c_int32),
        ("bvh_nodes", ctypes.c_int32),
        ("bvh_bytes", ctypes.c_int64),
        ("bvh_build_ms", ctypes.c_double),
    ]


class BatchOptions(ctypes.Structure):
    _fields_ = [
        ("autotune", ctypes.c_int32),
        ("wave_size", ctypes.c_int32),
        ("trace_refill", ctypes.c_int32),
        ("iterations_per_graph", ctypes.c_int32),
        ("autotune_fraction", ctypes.c_double),
    ]


class BatchStats(ctypes.Structure):
    _fields_ = [
        ("render_ms", ctypes.c_double),
        ("autotune_ms", ctypes.c_double),
        ("samples", ctypes.c_int64),
        ("extension_rays", ctypes.c_int64),
        ("shadow_rays", ctypes.c_int64),
        ("iterations", ctypes.c_int64),
        ("wave_size", ctypes.c_int32),
        ("trace_refill", ctypes.c_int32),
        ("iterations_per_graph", ctypes.c_int32),
        ("trials", ctypes.c_int32),
    ]


class MeshData(ctypes.Structure):
    _fields_ = [
        ("path", ctypes.c_char_p),
        ("positions", ctypes.c_void_p),
        ("normals", ctypes.c_void_p),
        ("texcoords", ctypes.c_void_p),
        ("faces", ctypes.c_void_p),
        ("num_vertices", ctypes.c_int64),
        ("num_triangles", ctypes.c_int64),
    ]


# name -> (restype, argtypes); every symbol include/nanogi.h declares
_P = ctypes.POINTER
PROTOTYPES = {
    "ngi_last_error": (ctypes.c_char_p, []),
    "ngi_abi_version": (ctypes.c_int32, []),
    "ngi_scene_load": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_double, _P(ctypes.c_void_p)]),
    "ngi_scene_load_with_meshes": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_double, _P(MeshData), ctypes.c_int32,
                                                  _P(ctypes.c_void_p)]),
    "ngi_scene_free": (None, [ctypes.c_void_p]),
    "ngi_scene_get_info": (ctypes.c_int, [ctypes.c_void_p, _P(SceneInfo)]),
    "ngi_scene_get_triangles": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_void_p]),
    "ngi_scene_build": (ctypes.c_int, [ctypes.c_void_p]),
    "ngi_scene_release_buffers": (ctypes.c_int, [ctypes.c_void_p]),
    "ngi_render": (ctypes.c_int, [ctypes.c_void_p, _P(RenderParams), ctypes.c_void_p]),
    "ngi_render_device": (ctypes.c_int, [ctypes.c_void_p, _P(RenderParams), ctypes.c_void_p, ctypes.c_void_p]),
    "ngi_get_render_stats": (ctypes.c_int, [ctypes.c_void_p, _P(RenderStats)]),
    "ngi_render_device_noalloc": (ctypes.c_int, [ctypes.c_void_p, _P(RenderParams), ctypes.c_void_p,
                                                 ctypes.c_void_p]),
    "ngi_render_batch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                        _P(BatchOptions), _P(BatchStats)]),
    "ngi_scene_get_parameters": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "ngi_scene_set_parameters": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "ngi_render_backward": (ctypes.c_int, [ctypes.c_void_p, _P(RenderParams), ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p]),
    "ngi_intersect": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_void_p]),
    "ngi_visible": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]),
    "ngi_save_image": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32]),
    "ngi_load_hdr": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32]),
    "ngi_load_texture": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_void_p, _P(ctypes.c_int32), _P(ctypes.c_int32)]),
}

_lib = None


class NanogiError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status
        self.message = message


def load_library(path: Path | str | None = None):
    """Loads libnanogi.so (built by nanogi_gb300.build) and declares every prototype."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(
            f"{p} is missing: build the CUDA extension first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(status: int) -> None:
    if status != NGI_OK:
        msg = load_library().ngi_last_error().decode(errors="replace")
        raise NanogiError(status, msg)
