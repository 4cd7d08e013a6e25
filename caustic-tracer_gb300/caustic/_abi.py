"""ctypes mirror of include/caustic.h (structure layouts and constants)."""
from __future__ import annotations

import ctypes as C

PRIM_STRIDE = 16
NODE_STRIDE = 8
MAT_STRIDE = 16
MAX_LEAF_PRIMS = 4
SAH_BUCKETS = 12
PRIM_SPHERE = 0
PRIM_TRIANGLE = 1
MAT_LAMBERTIAN = 0
MAT_METAL = 1
MAT_DIELECTRIC = 2
MAT_EMISSIVE = 3
RAY_FLOATS = 8

STATUS_NAMES = {
    0: "CT_OK",
    1: "CT_ERR_INVALID_ARGUMENT",
    2: "CT_ERR_CUDA",
    3: "CT_ERR_OUT_OF_MEMORY",
    4: "CT_ERR_UNSUPPORTED",
    5: "CT_ERR_TIMEOUT",
    6: "CT_ERR_BUDGET",
    7: "CT_ERR_CANCELLED",
    8: "CT_ERR_NOT_FOUND",
}

D3 = C.c_double * 3


class ct_sky(C.Structure):
    _fields_ = [("kind", C.c_int32), ("zenith", D3), ("horizon", D3), ("strength", C.c_double)]


class ct_camera_frame(C.Structure):
    _fields_ = [
        ("origin", D3),
        ("right", D3),
        ("up", D3),
        ("forward", D3),
        ("tan_half_fov", C.c_double),
        ("aspect", C.c_double),
        ("lens_radius", C.c_double),
        ("focus_distance", C.c_double),
    ]


class ct_trace_options(C.Structure):
    _fields_ = [("max_bounces", C.c_int32), ("russian_roulette", C.c_int32), ("nee", C.c_int32)]


class ct_render_options(C.Structure):
    _fields_ = [
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("spp", C.c_int32),
        ("max_bounces", C.c_int32),
        ("russian_roulette", C.c_int32),
        ("nee", C.c_int32),
        ("seed", C.c_uint32),
    ]


class ct_packed_scene_view(C.Structure):
    _fields_ = [
        ("prims", C.POINTER(C.c_float)),
        ("prim_count", C.c_uint32),
        ("nodes", C.POINTER(C.c_float)),
        ("node_count", C.c_uint32),
        ("mats", C.POINTER(C.c_float)),
        ("mat_count", C.c_uint32),
        ("lights", C.POINTER(C.c_int32)),
        ("light_count", C.c_uint32),
        ("prim_object", C.POINTER(C.c_uint32)),
        ("sky", ct_sky),
    ]


class ct_shape(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("p", C.c_double * 9),
        ("vertices", C.POINTER(C.c_double)),
        ("vertex_count", C.c_uint32),
        ("indices", C.POINTER(C.c_uint32)),
        ("index_count", C.c_uint32),
    ]


class ct_material(C.Structure):
    _fields_ = [
        ("type", C.c_int32),
        ("color", D3),
        ("param", C.c_double),
        ("has_checker", C.c_int32),
        ("checker_color2", D3),
        ("checker_scale", C.c_double),
        ("has_emission", C.c_int32),
        ("emission", D3),
    ]


class ct_object(C.Structure):
    _fields_ = [("shape", ct_shape), ("material", ct_material)]


class ct_packed_scene(C.Structure):
    _fields_ = [("view", ct_packed_scene_view), ("order", C.POINTER(C.c_uint32))]


class ct_batch_job(C.Structure):
    _fields_ = [
        ("scene", C.c_void_p),
        ("frame", ct_camera_frame),
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("first_frame_index", C.c_uint32),
        ("passes", C.c_int32),
        ("accum", C.c_void_p),
    ]


class ct_stats(C.Structure):
    _fields_ = [
        ("kernel_ms", C.c_double),
        ("total_ms", C.c_double),
        ("rays", C.c_uint64),
        ("fp64_fallbacks", C.c_uint64),
        ("launches", C.c_uint32),
    ]


# Every entry point of include/caustic.h: name -> (restype, argtypes).
P = C.c_void_p
SIGNATURES = {
    "ct_abi_version": (C.c_int32, []),
    "ct_last_error": (C.c_char_p, []),
    "ct_pack_scene": (C.c_int, [C.POINTER(ct_object), C.c_uint32, C.POINTER(ct_sky), C.POINTER(C.POINTER(ct_packed_scene))]),
    "ct_packed_scene_free": (None, [C.POINTER(ct_packed_scene)]),
    "ct_scene_create": (C.c_int, [C.POINTER(ct_packed_scene_view), C.POINTER(P)]),
    "ct_scene_destroy": (None, [P]),
    "ct_scene_device_bytes": (C.c_uint64, [P]),
    "ct_scene_set_option": (C.c_int, [P, C.c_int32, C.c_int64]),
    "ct_scene_walk": (C.c_int32, [P]),
    "ct_trace_closest": (C.c_int, [P, P, C.c_uint32, P, P, P, P, C.POINTER(ct_stats)]),
    "ct_trace_occluded": (C.c_int, [P, P, C.c_uint32, P, C.POINTER(ct_stats)]),
    "ct_trace_closest_device": (C.c_int, [P, P, C.c_uint32, P, P, P, P, P]),
    "ct_trace_occluded_device": (C.c_int, [P, P, C.c_uint32, P, P]),
    "ct_set_traversal": (C.c_int32, [C.c_int32]),
    "ct_accumulate_pass": (C.c_int, [P, C.POINTER(ct_camera_frame), C.c_int32, C.c_int32, C.c_uint32,
                                     C.POINTER(ct_trace_options), P, C.POINTER(ct_stats)]),
    "ct_render_image": (C.c_int, [P, C.POINTER(ct_camera_frame), C.POINTER(ct_render_options), P,
                                  C.POINTER(ct_stats)]),
    "ct_accumulate_passes_device": (C.c_int, [P, C.POINTER(ct_camera_frame), C.c_int32, C.c_int32, C.c_uint32,
                                              C.c_int32, C.POINTER(ct_trace_options), P, P, P]),
    "ct_render_image_device": (C.c_int, [P, C.POINTER(ct_camera_frame), C.POINTER(ct_render_options), P, P]),
    "ct_batch_create": (C.c_int, [C.POINTER(ct_batch_job), C.c_uint32, C.POINTER(ct_trace_options), C.c_int64,
                                  C.c_int32, C.POINTER(P)]),
    "ct_batch_set_first_frames": (C.c_int, [P, C.POINTER(C.c_uint32)]),
    "ct_batch_run": (C.c_int, [P, P]),
    "ct_batch_run_direct": (C.c_int, [P, P]),
    "ct_batch_run_direct_after": (C.c_int, [P, P, P]),
    "ct_batch_info": (C.c_int, [P, C.POINTER(C.c_uint32), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                C.POINTER(C.c_int32)]),
    "ct_batch_destroy": (None, [P]),
    "ct_accumulate_pass_noalloc": (C.c_int, [P, C.POINTER(ct_camera_frame), C.c_int32, C.c_int32, C.c_uint32,
                                             C.POINTER(ct_trace_options), P, P]),
    "ct_tonemap_device": (C.c_int, [P, C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_int32, P, P]),
    "ct_ppm_device": (C.c_int, [P, C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_int32, P, C.c_uint64,
                                C.POINTER(C.c_uint64), P]),
    "ct_pick": (C.c_int, [P, C.POINTER(ct_camera_frame), C.c_uint32, P, P, P, P, P, P]),
    "ct_profile_enable": (None, [C.c_int32]),
    "ct_profile_reset": (None, []),
    "ct_profile_read": (C.c_int32, [C.POINTER(C.c_char_p), C.POINTER(C.c_double), C.POINTER(C.c_uint64), C.c_int32]),
    "ct_rng_stream": (C.c_uint32, [C.c_uint32, C.c_int32, C.c_uint64, C.c_int32, C.c_double, C.c_double,
                                   C.POINTER(C.c_double)]),
}
