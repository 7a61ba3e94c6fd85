"""ORACLE -- test infrastructure only (tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py).  Nothing in lisa_gb300 imports this module.

ctypes bindings of oracle/liblisa_oracle.so, the scalar CPU restatement of
the reference estimator and closest-hit query (oracle/cpu_tracer.cc).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblisa_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")

_lib = None


class OracleMaterial(C.Structure):
    _fields_ = [("roughness", C.c_float), ("alpha", C.c_float), ("n", C.c_float),
                ("diffuse", C.c_float * 3), ("emit", C.c_uint8), ("pad", C.c_uint8 * 3),
                ("emission", C.c_float * 3)]


class OracleScene(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("normals", C.c_void_p), ("mat_indices", C.c_void_p),
                ("num_triangles", C.c_uint32), ("materials", C.c_void_p), ("num_materials", C.c_uint32),
                ("width", C.c_uint32), ("height", C.c_uint32), ("spp", C.c_uint32), ("bounces", C.c_uint32),
                ("eye", C.c_float * 3), ("look_at", C.c_float * 3), ("fov", C.c_float),
                ("rng_mode", C.c_uint32), ("seed", C.c_uint32), ("sample_base", C.c_uint64),
                ("subframe", C.c_uint32), ("estimator", C.c_uint32),
                ("lens_radius", C.c_float), ("focal_distance", C.c_float)]


def build() -> str:
    """Compile liblisa_oracle.so (gcc, -ffp-contract=off) if needed."""
    src = os.path.join(HERE, "cpu_tracer.cc")
    if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-C", HERE, "all"], check=True, capture_output=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        L.oracle_closest.argtypes = [P, C.c_uint32, P, C.c_uint32, C.c_int, C.c_int, P, P]
        L.oracle_render.argtypes = [C.POINTER(OracleScene), C.c_int, C.c_int, C.c_uint32, C.c_uint32, P, P, P]
        L.oracle_ctx_create.restype = C.c_void_p
        L.oracle_ctx_create.argtypes = [C.POINTER(OracleScene), C.c_int]
        L.oracle_ctx_destroy.argtypes = [P]
        L.oracle_ctx_render.argtypes = [P, C.POINTER(OracleScene), C.c_int, C.c_uint32, C.c_uint32, P, P, P]
        L.oracle_make_color.argtypes = [P, C.c_uint64, P]
        L.oracle_tea16.restype = C.c_uint32
        L.oracle_tea16.argtypes = [C.c_uint32, C.c_uint32]
        L.oracle_tea4.restype = C.c_uint32
        L.oracle_tea4.argtypes = [C.c_uint32, C.c_uint32]
        L.oracle_rnd.restype = C.c_float
        L.oracle_rnd.argtypes = [C.POINTER(C.c_uint32)]
        for name in ("oracle_normalize",):
            getattr(L, name).argtypes = [P, P]
        L.oracle_reflect.argtypes = [P, P, P]
        L.oracle_faceforward.argtypes = [P, P, P, P]
        L.oracle_lerp.argtypes = [P, P, C.c_float, P]
        L.oracle_fresnel.restype = C.c_float
        L.oracle_fresnel.argtypes = [C.c_float, C.c_float]
        L.oracle_refract.argtypes = [C.c_float, P, P, C.c_float, P]
        L.oracle_brdf.restype = C.c_float
        L.oracle_brdf.argtypes = [P, P]
        L.oracle_barycentric_normal.argtypes = [P, P, P, P]
        L.oracle_hemi.argtypes = [P, C.POINTER(C.c_uint32), P]
        L.oracle_uvw.argtypes = [P, P, C.c_float, C.c_uint32, C.c_uint32, P]
        _lib = L
    return _lib


def _p(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


class Scene:
    """Oracle view of a soup + camera + render settings."""

    def __init__(self, vertices, normals, mat_indices, materials, width, height, eye, look_at, fov, spp, bounces,
                 rng_mode=0, seed=0, sample_base=0, subframe=0, estimator=0, lens_radius=0.0,
                 focal_distance=0.0):
        self.v = np.ascontiguousarray(np.asarray(vertices, np.float32).reshape(-1, 9))
        self.n = np.ascontiguousarray(np.asarray(normals, np.float32).reshape(-1, 9))
        self.mi = np.ascontiguousarray(np.asarray(mat_indices, np.int32).reshape(-1))
        table = np.asarray(materials, np.float32).reshape(-1, 10)
        self.mats = (OracleMaterial * max(1, table.shape[0]))()
        for i, r in enumerate(table):
            m = self.mats[i]
            m.roughness, m.alpha, m.n = float(r[0]), float(r[1]), float(r[2])
            m.diffuse[:] = [float(r[3]), float(r[4]), float(r[5])]
            m.emit = int(r[6] != 0)
            m.emission[:] = [float(r[7]), float(r[8]), float(r[9])]
        s = OracleScene()
        s.vertices = self.v.ctypes.data
        s.normals = self.n.ctypes.data
        s.mat_indices = self.mi.ctypes.data
        s.num_triangles = self.v.shape[0]
        s.materials = C.cast(self.mats, C.c_void_p)
        s.num_materials = table.shape[0]
        s.width, s.height, s.spp, s.bounces = int(width), int(height), int(spp), int(bounces)
        s.eye[:] = [float(x) for x in eye]
        s.look_at[:] = [float(x) for x in look_at]
        s.fov = float(fov)
        s.rng_mode, s.seed, s.sample_base, s.subframe = int(rng_mode), int(seed), int(sample_base), int(subframe)
        s.estimator = int(estimator)  # 0 = the reference estimator, 1 = physically based
        s.lens_radius, s.focal_distance = float(lens_radius), float(focal_distance)  # thin lens (0 = pinhole)
        self.s = s

    @classmethod
    def from_scene(cls, scene, **kw):
        v, n, mi = scene.soup()
        args = dict(width=scene.width, height=scene.height, eye=scene.eye, look_at=scene.look_at, fov=scene.fov,
                    spp=scene.num_samples, bounces=scene.num_bounces)
        args.update(kw)
        return cls(v, n, mi, scene.material_table(), **args)

    def render(self, px0=0, px1=None, use_bvh=True, threads=0):
        """FP64 per-pixel sums over spp samples: (sum, sumsq, rays[3]).  The
        scene context (CPU BVH) is built on the first call and reused."""
        npix = self.s.width * self.s.height
        px1 = npix if px1 is None else px1
        k = px1 - px0
        s = np.zeros((max(k, 0), 3), np.float64)
        q = np.zeros((max(k, 0), 3), np.float64)
        rays = np.zeros(3, np.uint64)
        ctx = self._ctx(bool(use_bvh))
        lib().oracle_ctx_render(ctx, C.byref(self.s), int(threads), px0, px1, _p(s), _p(q), _p(rays))
        return s, q, rays

    def _ctx(self, use_bvh: bool):
        cache = self.__dict__.setdefault("_ctxs", {})
        if use_bvh not in cache:
            cache[use_bvh] = lib().oracle_ctx_create(C.byref(self.s), int(use_bvh))
        return cache[use_bvh]

    def __del__(self):
        for c in self.__dict__.get("_ctxs", {}).values():
            if c:
                lib().oracle_ctx_destroy(c)


def closest(vertices, rays, use_bvh=False, threads=0):
    v = np.ascontiguousarray(np.asarray(vertices, np.float32).reshape(-1, 9))
    r = np.ascontiguousarray(np.asarray(rays, np.float32).reshape(-1, 8))
    prim = np.empty(r.shape[0], np.int32)
    t = np.empty(r.shape[0], np.float32)
    lib().oracle_closest(_p(v), v.shape[0], _p(r), r.shape[0], int(use_bvh), int(threads), _p(prim), _p(t))
    return prim, t


def make_color(rgb):
    a = np.ascontiguousarray(np.asarray(rgb, np.float32).reshape(-1, 3))
    out = np.empty((a.shape[0], 4), np.uint8)
    lib().oracle_make_color(_p(a), a.shape[0], _p(out))
    return out


def ref_binary(name: str):
    """Path of a reference-compiled helper under oracle/_ref, or None where
    the reference sources were not available to build it."""
    p = os.path.join(REF_DIR, name)
    return p if os.path.exists(p) else None
