"""lisa_gb300 -- a GB300-native Monte Carlo path tracer with LiSA's surface.

Host mirror of the reference's interface (src/LiSA/src/main.cc:6-27):

    parser   = SceneParser("scene.rto")       # scene_parser.hh:10-13
    params   = parser.get_params()
    wrapper  = Renderer(params)               # OptixWrapper(params)
    render(wrapper, params)                   # render.hh:5 -> writes the PPM

All work happens in the native library (include/lisa_gb.h) through ctypes;
this module only marshals arguments and raises ``LisaError`` on failure.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional, Sequence

import numpy as np

from . import _native as N
from ._native import LisaError, Options, RenderStats, Tuning, default_options  # noqa: F401

__all__ = ["SceneParser", "Params", "Renderer", "Guide", "render", "display", "params_from_arrays",
           "params_from_scene", "write_ppm", "LisaError", "default_options", "autotune", "apply_tuning",
           "tuning_cache_lookup", "tuning_cache_store", "Tuning"]


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else C.c_void_p(a.ctypes.data)


class Params:
    """A RendererParams (structs.hh:90-103) plus the arrays it borrows."""

    def __init__(self, raw: N.RendererParams, keep=()):
        self.raw = raw
        self._keep = list(keep)

    # numpy views of the soup (valid while this object lives)
    @property
    def num_triangles(self) -> int:
        return self.raw.num_vertices // 3

    def vertices(self) -> np.ndarray:
        n = self.raw.num_vertices
        if n == 0:
            return np.zeros((0, 3), np.float32)
        return np.ctypeslib.as_array(C.cast(self.raw.vertices, C.POINTER(C.c_float)), (n, 3))

    def normals(self) -> np.ndarray:
        n = self.raw.num_vertices
        if n == 0:
            return np.zeros((0, 3), np.float32)
        return np.ctypeslib.as_array(C.cast(self.raw.normals, C.POINTER(C.c_float)), (n, 3))

    def mat_indices(self) -> np.ndarray:
        n = self.raw.num_vertices // 3
        if n == 0:
            return np.zeros((0,), np.int32)
        return np.ctypeslib.as_array(self.raw.mat_indices, (n,))

    def materials(self) -> List[N.Material]:
        return [self.raw.materials[i] for i in range(self.raw.num_materials)]

    def __getattr__(self, k):
        return getattr(self.raw, k)


class SceneParser:
    """Parses a .rto scene and its OBJ meshes (scene_parser.cc:35-57)."""

    def __init__(self, path: str = None, text: str = None, base_dir: str = None):
        L = N.lib()
        h = C.c_void_p()
        if text is not None:
            b = text.encode()
            N.check(L.lisa_scene_parse_string(b, len(b), base_dir.encode() if base_dir else None, C.byref(h)))
        else:
            N.check(L.lisa_scene_parse(str(path).encode(), C.byref(h)))
        self._h = h

    def get_params(self) -> Params:
        raw = N.RendererParams()
        N.check(N.lib().lisa_scene_params(self._h, C.byref(raw)))
        return Params(raw, keep=[self])

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            N.lib().lisa_scene_destroy(h)
            self._h = None


def _materials_array(table: np.ndarray):
    """(M, 10) rows: roughness, alpha, n, diffuse rgb, emit, emission rgb."""
    M = table.shape[0]
    arr = (N.Material * max(M, 1))()
    for i, r in enumerate(table):
        m = arr[i]
        m.roughness, m.alpha, m.n = float(r[0]), float(r[1]), float(r[2])
        m.diffuse_color = N.Float3(float(r[3]), float(r[4]), float(r[5]))
        m.emit = int(r[6] != 0)
        m.emission_color = N.Float3(float(r[7]), float(r[8]), float(r[9]))
    return arr


def params_from_arrays(vertices, normals, mat_indices, materials, width, height, eye, look_at, fov,
                       num_samples, num_bounces, output_image="out.ppm") -> Params:
    """Build RendererParams from in-memory arrays: vertices/normals (3T, 3)
    float32, mat_indices (T,) int32, materials (M, 10) float32 table."""
    v = np.ascontiguousarray(np.asarray(vertices, np.float32).reshape(-1, 3))
    n = np.ascontiguousarray(np.asarray(normals, np.float32).reshape(-1, 3))
    mi = np.ascontiguousarray(np.asarray(mat_indices, np.int32).reshape(-1))
    mats = _materials_array(np.asarray(materials, np.float32).reshape(-1, 10))
    raw = N.RendererParams()
    raw.vertices = C.cast(_ptr(v), C.POINTER(N.Float3))
    raw.normals = C.cast(_ptr(n), C.POINTER(N.Float3))
    raw.mat_indices = C.cast(_ptr(mi), C.POINTER(C.c_int32))
    raw.materials = C.cast(mats, C.POINTER(N.Material))
    raw.num_vertices = v.shape[0]
    raw.num_materials = len(materials)
    raw.width, raw.height = int(width), int(height)
    raw.camera = N.Camera(N.Float3(*map(float, eye)), N.Float3(*map(float, look_at)), float(fov))
    raw.num_samples, raw.num_bounces = int(num_samples), int(num_bounces)
    out = output_image.encode()
    raw.output_image = out
    return Params(raw, keep=[v, n, mi, mats, out])


def params_from_scene(scene, **override) -> Params:
    """RendererParams of a lisa_gb300.scenes.Scene (no files written)."""
    v, n, mi = scene.soup()
    kw = dict(width=scene.width, height=scene.height, eye=scene.eye, look_at=scene.look_at, fov=scene.fov,
              num_samples=scene.num_samples, num_bounces=scene.num_bounces, output_image=scene.output_image)
    kw.update(override)
    return params_from_arrays(v, n, mi, scene.material_table(), **kw)


class Renderer:
    """Scene(s) on the GPU: upload, BVH build and wavefront buffers.  The
    counterpart of OptixWrapper (optix_wrapper.hh:3-20)."""

    def __init__(self, params, options: Optional[Options] = None, **opt_kw):
        L = N.lib()
        if isinstance(params, Params):
            params = [params]
        self._params = list(params)
        arr = (N.RendererParams * len(self._params))(*[p.raw for p in self._params])
        self.options = options if options is not None else default_options(**opt_kw)
        h = C.c_void_p()
        N.check(L.lisa_renderer_create_batch(arr, len(self._params), C.byref(self.options), C.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def scene_size(self, scene: int = 0):
        p = self._params[scene].raw
        return int(p.width), int(p.height)

    def render(self) -> RenderStats:
        st = RenderStats()
        N.check(N.lib().lisa_render(self._h, C.byref(st)))
        return st

    def render_progressive(self, spp: int) -> RenderStats:
        st = RenderStats()
        N.check(N.lib().lisa_render_progressive(self._h, int(spp), C.byref(st)))
        return st

    def reset(self):
        N.check(N.lib().lisa_reset_accumulation(self._h))

    def set_sample_offset(self, first_sample: int, scene: int = 0):
        """Render the samples first_sample, first_sample+1, ... (a shard of
        a frame split over GPUs; see lisa_gb300.shard)."""
        N.check(N.lib().lisa_set_sample_offset(self._h, scene, int(first_sample)))

    def image(self, scene: int = 0, variance: bool = False, fp64: bool = False):
        """Mean radiance (h, w, 3) float32 with row 0 = bottom; optionally the
        per-pixel sample variance (FP64) and the FP64 mean."""
        w, h = self.scene_size(scene)
        rgb = np.empty((h, w, 3), np.float32)
        var = np.empty((h, w, 3), np.float64) if variance else None
        m64 = np.empty((h, w, 3), np.float64) if fp64 else None
        N.check(N.lib().lisa_get_image(self._h, scene, _ptr(rgb), None, _ptr(var), _ptr(m64)))
        out = [rgb]
        if variance:
            out.append(var)
        if fp64:
            out.append(m64)
        return out[0] if len(out) == 1 else tuple(out)

    def rgba8(self, scene: int = 0) -> np.ndarray:
        w, h = self.scene_size(scene)
        out = np.empty((h, w, 4), np.uint8)
        N.check(N.lib().lisa_get_image(self._h, scene, None, _ptr(out), None, None))
        return out

    def ppm_rgb8(self, scene: int = 0) -> np.ndarray:
        w, h = self.scene_size(scene)
        out = np.empty((h, w, 3), np.uint8)
        N.check(N.lib().lisa_get_ppm_rgb8(self._h, scene, _ptr(out)))
        return out

    def save_image(self, path: Optional[str] = None, scene: int = 0):
        N.check(N.lib().lisa_save_image(self._h, scene, path.encode() if path else None))

    def trace_closest(self, rays: np.ndarray):
        rays = np.ascontiguousarray(np.asarray(rays, np.float32).reshape(-1, 8))
        n = rays.shape[0]
        prim = np.empty(n, np.int32)
        t = np.empty(n, np.float32)
        N.check(N.lib().lisa_trace_closest(self._h, _ptr(rays), n, _ptr(prim), _ptr(t)))
        return prim, t

    def trace_count(self, rays: np.ndarray):
        rays = np.ascontiguousarray(np.asarray(rays, np.float32).reshape(-1, 8))
        v, t = C.c_uint64(), C.c_uint64()
        N.check(N.lib().lisa_trace_count(self._h, _ptr(rays), rays.shape[0], C.byref(v), C.byref(t)))
        return int(v.value), int(t.value)

    def bvh_info(self, scene: int = 0) -> dict:
        a, b, c, d = C.c_uint32(), C.c_uint32(), C.c_uint32(), C.c_double()
        N.check(N.lib().lisa_bvh_info(self._h, scene, C.byref(a), C.byref(b), C.byref(c), C.byref(d)))
        return {"nodes": a.value, "tri_slots": b.value, "depth": c.value, "build_ms": d.value}

    def guide(self, scene: int = 0) -> "Guide":
        h = C.c_void_p()
        N.check(N.lib().lisa_renderer_guide(self._h, scene, C.byref(h)))
        return Guide(handle=h, owner=self)

    def close(self):
        h = getattr(self, "_h", None)
        if h:
            N.lib().lisa_renderer_destroy(h)
            self._h = None

    def __del__(self):
        self.close()


class Guide:
    """The MLP path guide (no reference counterpart)."""

    def __init__(self, seed: int = 0, handle=None, owner=None):
        self._owner = owner
        if handle is None:
            h = C.c_void_p()
            N.check(N.lib().lisa_guide_create(int(seed), C.byref(h)))
            self._h = h
        else:
            # a renderer's network: the handle is ours to free, the network
            # stays with the renderer (kept alive through _owner)
            self._h = handle
        self._own = True

    def params(self) -> np.ndarray:
        out = np.empty(N.GUIDE_NUM_PARAMS, np.float32)
        N.check(N.lib().lisa_guide_get_params(self._h, _ptr(out)))
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(np.asarray(p, np.float32))
        assert p.size == N.GUIDE_NUM_PARAMS
        N.check(N.lib().lisa_guide_set_params(self._h, _ptr(p)))

    def forward(self, features: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(np.asarray(features, np.float32).reshape(-1, N.GUIDE_IN))
        out = np.empty((x.shape[0], N.GUIDE_OUT), np.float32)
        N.check(N.lib().lisa_guide_forward(self._h, _ptr(x), x.shape[0], _ptr(out)))
        return out

    def train_step(self, features, dirs, weights, lr: float = 0.0, want_grads: bool = True):
        x = np.ascontiguousarray(np.asarray(features, np.float32).reshape(-1, N.GUIDE_IN))
        d = np.ascontiguousarray(np.asarray(dirs, np.float32).reshape(-1, 3))
        w = np.ascontiguousarray(np.asarray(weights, np.float32).reshape(-1))
        loss = C.c_float()
        g = np.empty(N.GUIDE_NUM_PARAMS, np.float32) if want_grads else None
        N.check(N.lib().lisa_guide_train_step(self._h, _ptr(x), _ptr(d), _ptr(w), x.shape[0], float(lr),
                                              C.cast(C.byref(loss), C.c_void_p), _ptr(g)))
        return float(loss.value), g

    def train_steps(self, features, dirs, weights, chunk: int, steps: int, lr: float) -> float:
        """Adam steps on consecutive slices of `chunk` samples, in one launch
        (the same updates as train_step on each slice); the last step's loss."""
        x = np.ascontiguousarray(np.asarray(features, np.float32).reshape(-1, N.GUIDE_IN))
        d = np.ascontiguousarray(np.asarray(dirs, np.float32).reshape(-1, 3))
        w = np.ascontiguousarray(np.asarray(weights, np.float32).reshape(-1))
        loss = C.c_float()
        N.check(N.lib().lisa_guide_train_steps(self._h, _ptr(x), _ptr(d), _ptr(w), x.shape[0], int(chunk), int(steps),
                                               float(lr), C.cast(C.byref(loss), C.c_void_p)))
        return float(loss.value)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and getattr(self, "_own", False):
            N.lib().lisa_guide_destroy(h)
            self._h = None


def render(renderer: Renderer, params: Optional[Params] = None) -> RenderStats:
    """Batch render and save the PPM to params.output_image (render.cc:133-148)."""
    st = renderer.render()
    renderer.save_image(None if params is None else params.raw.output_image.decode())
    return st


def display(renderer: Renderer, params: Optional[Params] = None, spp_per_launch: int = 16) -> RenderStats:
    """Headless form of the reference's display loop (render.cc:75-131):
    progressive launches of 16 spp until num_samples, then the PPM."""
    target = int((params or renderer._params[0]).raw.num_samples)
    done, st = 0, None
    while done < target:
        st = renderer.render_progressive(spp_per_launch)
        done += spp_per_launch
    renderer.save_image(None if params is None else params.raw.output_image.decode())
    return st


def write_ppm(path: str, rgba8: np.ndarray):
    """sutil::saveImage for UNSIGNED_BYTE4 input (row 0 = bottom)."""
    a = np.ascontiguousarray(np.asarray(rgba8, np.uint8))
    h, w = a.shape[:2]
    N.check(N.lib().lisa_write_ppm(path.encode(), _ptr(a), w, h))


def autotune(params, options: Optional[Options] = None, cache: Optional[str] = None, **opt_kw) -> N.Tuning:
    """Queue and block sizes for the workload `params` (one Params or a list),
    timed on the GPU under `options` (or defaults with `opt_kw`); with
    `cache`, a JSON file answers repeated workloads.  Returns a Tuning;
    ``apply_tuning`` copies it into options."""
    if isinstance(params, Params):
        params = [params]
    params = list(params)
    arr = (N.RendererParams * len(params))(*[p.raw for p in params])
    o = options if options is not None else default_options(**opt_kw)
    t = N.Tuning()
    N.check(N.lib().lisa_autotune(arr, len(params), C.byref(o), cache.encode() if cache else None, C.byref(t)))
    return t


def apply_tuning(tuning: N.Tuning, options: Optional[Options] = None, **opt_kw) -> Options:
    o = options if options is not None else default_options(**opt_kw)
    N.lib().lisa_tuning_apply(C.byref(tuning), C.byref(o))
    return o


def tuning_cache_lookup(path: str, key: str) -> Optional[N.Tuning]:
    t, found = N.Tuning(), C.c_int32(0)
    N.check(N.lib().lisa_tuning_cache_lookup(path.encode(), key.encode(), C.byref(t), C.byref(found)))
    return t if found.value else None


def tuning_cache_store(path: str, tuning: N.Tuning) -> None:
    N.check(N.lib().lisa_tuning_cache_store(path.encode(), C.byref(tuning)))
