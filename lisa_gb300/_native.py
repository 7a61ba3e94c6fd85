"""ctypes bindings of the C ABI declared in include/lisa_gb.h.

The shared library is built in-tree (lisa_gb300/liblisa_gb.so) by
``lisa_gb300.build``.  Importing this module never falls back to anything
else: if the library is missing, ``lib()`` raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblisa_gb.so")

LISA_OK = 0
LISA_ERR_INVALID = 1
LISA_ERR_PARSE = 2
LISA_ERR_IO = 3
LISA_ERR_CUDA = 4
LISA_ERR_OOM = 5
LISA_ERR_DEVICE = 6
LISA_ERR_UNSUPPORTED = 7
LISA_STATUS_WAIT_TIMEOUT = 16  # device status bit: a bounded tensor-core wait ran out

LISA_MODE_COMPAT = 0
LISA_MODE_GUIDED = 1
LISA_ESTIMATOR_COMPAT = 0
LISA_ESTIMATOR_PHYSICAL = 1
LISA_RNG_PER_SAMPLE = 0
LISA_RNG_PER_PIXEL = 1

GUIDE_IN = 64
GUIDE_HIDDEN = 64
GUIDE_OUT = 40
GUIDE_NUM_PARAMS = 4 * 64 * 64 + 64 * 40 + 4 * 64 + 40


class Float3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class Material(C.Structure):
    _fields_ = [("roughness", C.c_float), ("alpha", C.c_float), ("n", C.c_float),
                ("diffuse_color", Float3), ("emit", C.c_uint8), ("_pad", C.c_uint8 * 3),
                ("emission_color", Float3)]


class Camera(C.Structure):
    _fields_ = [("eye", Float3), ("look_at", Float3), ("fov", C.c_float)]


class RendererParams(C.Structure):
    _fields_ = [("vertices", C.POINTER(Float3)), ("normals", C.POINTER(Float3)),
                ("materials", C.POINTER(Material)), ("mat_indices", C.POINTER(C.c_int32)),
                ("num_vertices", C.c_int32), ("num_materials", C.c_int32),
                ("width", C.c_uint32), ("height", C.c_uint32), ("camera", Camera),
                ("num_samples", C.c_uint32), ("num_bounces", C.c_uint32),
                ("output_image", C.c_char_p)]


class Options(C.Structure):
    _fields_ = [("struct_size", C.c_uint32), ("mode", C.c_uint32), ("rng", C.c_uint32),
                ("seed", C.c_uint32), ("paths_in_flight", C.c_uint32), ("blocks_per_sm", C.c_uint32),
                ("threads_per_block", C.c_uint32), ("use_graph", C.c_uint32),
                ("stage_timing", C.c_uint32), ("accum_fp64", C.c_uint32),
                ("aperture", C.c_float), ("focal_distance", C.c_float),
                ("guide_bsdf_fraction", C.c_float), ("guide_lr", C.c_float),
                ("guide_train_batch", C.c_uint32), ("guide_train_waves", C.c_uint32),
                ("alloc_cap_bytes", C.c_uint64), ("count_traversal", C.c_uint32),
                ("guide_warmup_waves", C.c_uint32), ("guide_steps_per_wave", C.c_uint32),
                ("guide_spp_per_wave", C.c_uint32), ("refill_idle", C.c_uint32),
                ("estimator", C.c_uint32), ("bvh_lbvh_only", C.c_uint32), ("guide_min_spp", C.c_uint32),
                ("guide_max_depth", C.c_uint32), ("guide_train_steps", C.c_uint32)]


class RenderStats(C.Structure):
    _fields_ = [("rays_primary", C.c_uint64), ("rays_bounce", C.c_uint64), ("rays_shadow", C.c_uint64),
                ("paths", C.c_uint64), ("samples_total", C.c_uint64), ("ms_device", C.c_double),
                ("ms_trace", C.c_double), ("ms_shade", C.c_double), ("ms_nee", C.c_double),
                ("ms_guide", C.c_double), ("ms_other", C.c_double),
                ("launches_trace", C.c_uint32), ("launches_shade", C.c_uint32),
                ("launches_nee", C.c_uint32), ("launches_guide", C.c_uint32),
                ("launches_total", C.c_uint32), ("device_status", C.c_uint32),
                ("guide_loss", C.c_double), ("nee_vertices", C.c_uint64),
                ("node_visits_trace", C.c_uint64), ("tri_tests_trace", C.c_uint64),
                ("node_visits_nee", C.c_uint64), ("tri_tests_nee", C.c_uint64),
                ("shadow_traversals", C.c_uint64), ("ms_guide_infer", C.c_double),
                ("ms_guide_train", C.c_double), ("guide_infer_rows", C.c_uint64),
                ("guide_train_samples", C.c_uint64)]

    @property
    def rays(self) -> int:
        return int(self.rays_primary + self.rays_bounce + self.rays_shadow)

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class Tuning(C.Structure):
    _fields_ = [("struct_size", C.c_uint32), ("paths_in_flight", C.c_uint32),
                ("threads_per_block", C.c_uint32), ("blocks_per_sm", C.c_uint32),
                ("refill_idle", C.c_uint32), ("candidates", C.c_uint32), ("probe_spp", C.c_uint32),
                ("reserved", C.c_uint32), ("mrays_per_s", C.c_double), ("key", C.c_char * 160)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k not in ("struct_size", "reserved", "key")}
        d["key"] = self.key.decode()
        return d


# name -> (restype, argtypes); every symbol include/lisa_gb.h declares
_P = C.c_void_p
SIGNATURES = {
    "lisa_last_error": (C.c_char_p, []),
    "lisa_version": (C.c_char_p, []),
    "lisa_device_info": (C.c_int, [C.POINTER(C.c_int)] * 3),
    "lisa_device_cache_release": (C.c_int, [C.POINTER(C.c_uint64)]),
    "lisa_scene_parse": (C.c_int, [C.c_char_p, C.POINTER(_P)]),
    "lisa_scene_parse_string": (C.c_int, [C.c_char_p, C.c_size_t, C.c_char_p, C.POINTER(_P)]),
    "lisa_scene_params": (C.c_int, [_P, C.POINTER(RendererParams)]),
    "lisa_scene_destroy": (None, [_P]),
    "lisa_scene_create_empty": (C.c_int, [C.POINTER(_P)]),
    "lisa_scene_append_obj": (C.c_int, [_P, C.c_char_p, C.c_int32]),
    "lisa_options_default": (None, [C.POINTER(Options)]),
    "lisa_renderer_create": (C.c_int, [C.POINTER(RendererParams), C.POINTER(Options), C.POINTER(_P)]),
    "lisa_renderer_create_batch": (C.c_int, [C.POINTER(RendererParams), C.c_int32, C.POINTER(Options),
                                             C.POINTER(_P)]),
    "lisa_renderer_destroy": (None, [_P]),
    "lisa_render": (C.c_int, [_P, C.POINTER(RenderStats)]),
    "lisa_render_progressive": (C.c_int, [_P, C.c_uint32, C.POINTER(RenderStats)]),
    "lisa_reset_accumulation": (C.c_int, [_P]),
    "lisa_set_sample_offset": (C.c_int, [_P, C.c_int32, C.c_uint64]),
    "lisa_get_image": (C.c_int, [_P, C.c_int32, _P, _P, _P, _P]),
    "lisa_get_ppm_rgb8": (C.c_int, [_P, C.c_int32, _P]),
    "lisa_save_image": (C.c_int, [_P, C.c_int32, C.c_char_p]),
    "lisa_write_ppm": (C.c_int, [C.c_char_p, _P, C.c_uint32, C.c_uint32]),
    "lisa_trace_closest": (C.c_int, [_P, _P, C.c_uint32, _P, _P]),
    "lisa_trace_closest_device": (C.c_int, [_P, _P, C.c_uint32, _P, _P, _P]),
    "lisa_trace_brute_device": (C.c_int, [_P, _P, C.c_uint32, _P, _P, _P]),
    "lisa_trace_count": (C.c_int, [_P, _P, C.c_uint32, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "lisa_trace_soup_noalloc": (C.c_int, [_P, C.c_uint32, _P, C.c_uint32, _P, _P, _P]),
    "lisa_bvh_info": (C.c_int, [_P, C.c_int32, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                C.POINTER(C.c_uint32), C.POINTER(C.c_double)]),
    "lisa_autotune": (C.c_int, [_P, C.c_int32, _P, C.c_char_p, _P]),
    "lisa_tuning_apply": (None, [_P, _P]),
    "lisa_tuning_cache_lookup": (C.c_int, [C.c_char_p, C.c_char_p, _P, C.POINTER(C.c_int32)]),
    "lisa_tuning_cache_store": (C.c_int, [C.c_char_p, _P]),
    "lisa_guide_create": (C.c_int, [C.c_uint32, C.POINTER(_P)]),
    "lisa_selftest_wait_timeout": (C.c_int, [C.c_uint32, C.POINTER(C.c_uint32)]),
    "lisa_guide_destroy": (None, [_P]),
    "lisa_guide_get_params": (C.c_int, [_P, _P]),
    "lisa_guide_set_params": (C.c_int, [_P, _P]),
    "lisa_guide_forward": (C.c_int, [_P, _P, C.c_uint32, _P]),
    "lisa_guide_train_step": (C.c_int, [_P, _P, _P, _P, C.c_uint32, C.c_float, _P, _P]),
    "lisa_batch_render": (C.c_int, [_P, C.c_int32, _P, _P]),
    "lisa_guide_train_steps": (C.c_int, [_P, _P, _P, _P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_float, _P]),
    "lisa_renderer_guide": (C.c_int, [_P, C.c_int32, C.POINTER(_P)]),
}

_lib = None


class LisaError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def lib() -> C.CDLL:
    """Load liblisa_gb.so (built in-tree).  Raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(code: int) -> None:
    if code != LISA_OK:
        msg = lib().lisa_last_error()
        raise LisaError(code, msg.decode() if msg else "")


def default_options(**kw) -> Options:
    o = Options()
    lib().lisa_options_default(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise AttributeError(f"unknown option {k}")
        setattr(o, k, v)
    return o
