"""ctypes binding of librmn.so (include/rmn.h).

The library is built in-tree by raym0nade_gb300/build.py. Loading fails loudly
when it is missing: there is no CPU fallback anywhere in the package.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

LIB_PATH = _build.LIB


class Material(C.Structure):
    _fields_ = [("base_color", C.c_float * 3), ("has_base", C.c_float), ("emission", C.c_float * 3),
                ("has_emission", C.c_float), ("roughness", C.c_float), ("metallic", C.c_float),
                ("has_specular", C.c_float), ("opacity", C.c_float), ("ior", C.c_float),
                ("transmitting_color", C.c_float * 3)]


class SceneDesc(C.Structure):
    _fields_ = [("num_vertices", C.c_int32), ("positions", C.c_void_p), ("normals", C.c_void_p),
                ("uvs", C.c_void_p), ("num_triangles", C.c_int32), ("indices", C.c_void_p),
                ("num_meshes", C.c_int32), ("mesh_first", C.c_void_p), ("mesh_material", C.c_void_p),
                ("num_materials", C.c_int32), ("materials", C.c_void_p), ("env_width", C.c_int32),
                ("env_height", C.c_int32), ("env_rgb", C.c_void_p), ("num_textures", C.c_int32),
                ("textures", C.c_void_p), ("material_textures", C.c_void_p)]


class PostArgs(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("exposure", C.c_float), ("focus", C.c_float),
                ("CoC", C.c_float), ("camera_position", C.c_float * 3)]


class Texture(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("channels", C.c_int32), ("texels", C.c_void_p)]


class SceneInfo(C.Structure):
    _fields_ = [("num_triangles", C.c_int32), ("num_inner_nodes", C.c_int32), ("bvh_depth", C.c_int32),
                ("heap_slots", C.c_int32), ("num_lights", C.c_int32), ("num_materials", C.c_int32),
                ("device_bytes", C.c_int64)]


class RenderArgs(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("direction", C.c_float * 3), ("up", C.c_float * 3),
                ("right", C.c_float * 3), ("accuracy", C.c_float), ("focus", C.c_float), ("CoC", C.c_float),
                ("exposure", C.c_float), ("P_Direct", C.c_float), ("width", C.c_int32), ("height", C.c_int32),
                ("spp", C.c_int32), ("threads", C.c_int32), ("max_depth", C.c_int32), ("seed", C.c_uint64),
                ("lanes_per_pixel", C.c_int32), ("slots_per_unit", C.c_int32), ("reserved", C.c_int32 * 2)]


class Image(C.Structure):
    _fields_ = [("radiance_Dd", C.c_void_p), ("radiance_Ds", C.c_void_p), ("radiance_Id", C.c_void_p),
                ("radiance_Is", C.c_void_p), ("gbuffer", C.c_void_p), ("dropped", C.c_void_p)]


class RenderProfile(C.Structure):
    _fields_ = [("primary_ms", C.c_double), ("path_ms", C.c_double), ("logic_ms", C.c_double),
                ("trace_ms", C.c_double), ("iterations", C.c_int64), ("closest_rays", C.c_uint64),
                ("shadow_rays", C.c_uint64), ("inner_visits", C.c_uint64), ("leaf_visits", C.c_uint64),
                ("triangle_tests", C.c_uint64), ("sample_slots", C.c_uint64), ("pixels", C.c_uint64)]


class BatchItem(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("args", RenderArgs), ("image", Image)]


class BatchOptions(C.Structure):
    _fields_ = [("use_graph", C.c_int32), ("pool_workers", C.c_int32), ("lanes", C.c_int32),
                ("stack_entries", C.c_int32), ("ray_order", C.c_int32), ("reserved", C.c_int32)]


class TuneResult(C.Structure):
    _fields_ = [("slots_per_unit", C.c_int32), ("pool_workers", C.c_int32), ("best_ms", C.c_double),
                ("default_ms", C.c_double), ("candidates", C.c_int32), ("lanes", C.c_int32),
                ("stack_entries", C.c_int32), ("ray_order", C.c_int32)]


class ImageDesc(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("channels", C.c_int32),
                ("bytes_per_channel", C.c_int32)]


# name -> (restype, argtypes); every declaration of include/rmn.h.
SIGNATURES = {
    "rmn_last_error": (C.c_char_p, []),
    "rmn_version": (C.c_char_p, []),
    "rmn_scene_create": (C.c_int, [C.POINTER(SceneDesc), C.POINTER(C.c_void_p)]),
    "rmn_scene_destroy": (C.c_int, [C.c_void_p]),
    "rmn_scene_info_get": (C.c_int, [C.c_void_p, C.POINTER(SceneInfo)]),
    "rmn_trace_closest": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    "rmn_trace_shadow": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    "rmn_render": (C.c_int, [C.c_void_p, C.POINTER(RenderArgs), C.POINTER(Image), C.c_void_p]),
    "rmn_release_cached_memory": (C.c_int, []),
    "rmn_adjoint": (C.c_int, [C.c_void_p, C.POINTER(RenderArgs), C.POINTER(Image), C.c_void_p, C.c_void_p,
                              C.c_void_p]),
    "rmn_render_profile_get": (C.c_int, [C.c_void_p, C.POINTER(RenderArgs), C.POINTER(Image),
                                         C.POINTER(RenderProfile), C.c_void_p]),
    "rmn_batch_create": (C.c_int, [C.POINTER(BatchItem), C.c_int32, C.POINTER(BatchOptions), C.c_void_p,
                                   C.POINTER(C.c_void_p)]),
    "rmn_batch_autotune": (C.c_int, [C.POINTER(BatchItem), C.c_int32, C.c_float, C.POINTER(TuneResult), C.c_void_p]),
    "rmn_batch_device_bytes": (C.c_int, [C.POINTER(BatchItem), C.c_int32, C.POINTER(BatchOptions),
                                         C.POINTER(C.c_int64)]),
    "rmn_batch_render": (C.c_int, [C.c_void_p, C.c_void_p]),
    "rmn_batch_update": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]),
    "rmn_batch_update_bytes": (C.c_int64, [C.c_void_p]),
    "rmn_batch_profile": (C.c_int, [C.c_void_p, C.POINTER(RenderProfile), C.c_void_p]),
    "rmn_batch_destroy": (C.c_int, [C.c_void_p]),
    "rmn_compose": (C.c_int, [C.POINTER(Image), C.c_int32, C.c_int32, C.c_float, C.c_int32, C.c_void_p,
                              C.c_void_p]),
    "rmn_compose_noalloc": (C.c_int, [C.POINTER(Image), C.c_int32, C.c_int32, C.c_float, C.c_int32, C.c_void_p,
                                      C.c_void_p]),
    "rmn_fxaa": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]),
    "rmn_post_process": (C.c_int, [C.POINTER(Image), C.POINTER(PostArgs), C.c_int32, C.c_void_p, C.c_void_p]),
    "rmn_spatial_clamp": (C.c_int, [C.POINTER(Image), C.c_int32, C.c_int32, C.c_void_p]),
    "rmn_filter": (C.c_int, [C.POINTER(Image), C.c_int32, C.c_int32, C.c_void_p]),
    "rmn_export_set": (C.c_int, [C.POINTER(Image), C.POINTER(PostArgs), C.c_void_p, C.POINTER(C.c_int32),
                                 C.c_void_p]),
    "rmn_export_tag": (C.c_char_p, [C.c_int32]),
    "rmn_save_png": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_char_p]),
    "rmn_reverse_gamma": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p]),
    "rmn_export_options": (C.c_int32, [C.c_int32]),
    "rmn_image_load": (C.c_int, [C.c_char_p, C.c_int32, C.POINTER(ImageDesc), C.c_void_p, C.c_size_t]),
    "rmn_model_read": (C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.POINTER(C.c_void_p)]),
    "rmn_model_desc": (C.c_int, [C.c_void_p, C.POINTER(SceneDesc)]),
    "rmn_model_material_name": (C.c_char_p, [C.c_void_p, C.c_int32]),
    "rmn_model_free": (C.c_int, [C.c_void_p]),
    "rmn_scene_texture_get": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(ImageDesc), C.c_void_p,
                                        C.c_size_t]),
}

_lib = None


def load(build_if_missing: bool = False) -> C.CDLL:
    """Load librmn.so; raise if it is not built (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise ImportError(f"{LIB_PATH} is not built; run `python -c 'import __graft_entry__ as g; g.build()'` "
                              "or `python raym0nade_gb300/build.py`")
        _build.build()
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib
