"""Seeded procedural scenes in LiSA's scene form (.rto grammar + OBJ meshes).

Every scene is a list of materials, a list of meshes (one material each) and
a camera, exactly the pieces LiSA's SceneParser reads
(src/LiSA/src/scene_parser.cc:35-57).  A scene can be written out as a
``.rto`` file plus one OBJ per mesh (``write_rto``), or flattened directly
into the triangle soup the parser would produce (``Scene.soup``): three
vertices and three normals per triangle in mesh order, plus one material
index per triangle (src/LiSA/src/parse_obj.cc:24-69).

Workloads:

* ``cornell_box``      -- small Cornell box: 5 walls, 0.25x0.25 ceiling
  light, a white box, a rotated dielectric box (n=1.5), a 32x16 UV sphere.
  256x256, 64 spp, 7 bounces.
* ``icosphere_box``    -- icosphere subdivided to ~1.3M triangles, displaced
  by seeded 6-octave value noise (amplitude 0.08 r), dielectric n=1.5, in the
  same box.  1024x1024, 256 spp, 8 bounces.
* ``sphere_soup``      -- 20,000 UV spheres (16x8) in a 100^3 box, radii
  log-uniform in [0.1, 2], 10% emissive.  1920x1080, 64 spp, 12 bounces.
* ``hard_indirect``    -- the icosphere box with the light shrunk to
  0.02x0.02 and hidden behind a seeded baffle quad.  1024x1024, 8 bounces.
* ``batch_scenes``     -- 64 seeded scenes of uneven size, resolution, spp
  and bounce count, each a box + displaced icosphere or a sphere soup.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field
from typing import List, Optional, Tuple

import numpy as np

# Material kinds, mirroring the three branches of the reference material
# model (structs.hh:16-52): emissive, opaque (roughness) and dielectric
# (alpha < 1, refractive index n).


@dataclass
class Material:
    name: str
    color: Tuple[float, float, float]
    alpha: float = 1.0
    roughness: Optional[float] = 1.0
    n: Optional[float] = None
    emit: bool = False
    # Emitted radiance = colour x scale.  The .rto grammar cannot express a
    # radiance above 1 (colours above 1 are divided by 255,
    # scene_parser.cc:139-143), so a scale other than 1 only reaches the
    # renderer through the C ABI (material_table); write_rto drops it.
    scale: float = 1.0

    def rto(self) -> str:
        c = self.color
        lines = [f"material {self.name} {{"]
        if self.emit:
            lines.append("  emit = true")
        lines.append(f"  color = ({_f(c[0])}, {_f(c[1])}, {_f(c[2])}, {_f(self.alpha)})")
        if not self.emit:
            if self.alpha < 1.0:
                lines.append(f"  n = {_f(self.n)}")
            else:
                lines.append(f"  roughness = {_f(self.roughness)}")
        lines.append("}")
        return "\n".join(lines)


@dataclass
class Mesh:
    name: str
    material: str
    vertices: np.ndarray  # (T, 3, 3) float32
    normals: np.ndarray   # (T, 3, 3) float32


@dataclass
class Scene:
    materials: List[Material]
    meshes: List[Mesh]
    eye: Tuple[float, float, float]
    look_at: Tuple[float, float, float]
    fov: float
    width: int
    height: int
    num_samples: int
    num_bounces: int
    output_image: str = "out.ppm"
    name: str = "scene"
    extra: dict = field(default_factory=dict)

    @property
    def num_triangles(self) -> int:
        return int(sum(m.vertices.shape[0] for m in self.meshes))

    def material_index(self) -> dict:
        idx = {}
        for m in self.materials:
            if m.name not in idx:
                idx[m.name] = len(idx)
        return idx

    def soup(self):
        """Flatten to (vertices (3T,3) f32, normals (3T,3) f32, mat_idx (T,) i32)."""
        idx = self.material_index()
        vs = [m.vertices.reshape(-1, 3) for m in self.meshes]
        ns = [m.normals.reshape(-1, 3) for m in self.meshes]
        mi = [np.full(m.vertices.shape[0], idx[m.material], np.int32) for m in self.meshes]
        return (np.ascontiguousarray(np.concatenate(vs).astype(np.float32)),
                np.ascontiguousarray(np.concatenate(ns).astype(np.float32)),
                np.ascontiguousarray(np.concatenate(mi).astype(np.int32)))

    def material_table(self) -> np.ndarray:
        """Materials in parser order as a (M, 10) float32 table:
        roughness, alpha, n, diffuse rgb, emit, emission rgb."""
        seen = set()
        rows = []
        for m in self.materials:
            if m.name in seen:
                continue
            seen.add(m.name)
            rgb = _parsed_color(m.color)
            if m.emit:
                rows.append([0.0, 1.0, 0.0, 0.0, 0.0, 0.0, 1.0, *[v * m.scale for v in rgb]])
            elif m.alpha < 1.0:
                rows.append([0.0, m.alpha, m.n, *rgb, 0.0, 0.0, 0.0, 0.0])
            else:
                rows.append([m.roughness, m.alpha, 0.0, *rgb, 0.0, 0.0, 0.0, 0.0])
        return np.asarray(rows, np.float32)


def _f(x: float) -> str:
    """Format a float so that it re-parses to the same float32 and stays
    inside the .rto float grammar ([+-]?([0-9]*[.])?[0-9]+, no exponent)."""
    x32 = float(np.float32(x))
    for digits in range(1, 40):
        s = f"{x32:.{digits}f}"
        if float(np.float32(float(s))) == x32:
            break
    if "." in s:
        s = s.rstrip("0")
        if s.endswith("."):
            s += "0"
    return s


def _parsed_color(c):
    """The reference rescales by 1/255 when any channel exceeds 1
    (scene_parser.cc:139-143)."""
    c = [np.float32(float(np.float32(float(_f(v))))) for v in c]
    if c[0] > 1 or c[1] > 1 or c[2] > 1:
        c = [np.float32(np.float64(v) / 255.0) for v in c]
    return [float(v) for v in c]


# ----------------------------------------------------------------------------
# geometry helpers


def quad(p0, p1, p2, p3, normal=None):
    """Two triangles (p0,p1,p2), (p0,p2,p3) with a flat normal."""
    p = np.asarray([p0, p1, p2, p3], np.float64)
    if normal is None:
        normal = np.cross(p[1] - p[0], p[2] - p[0])
    normal = np.asarray(normal, np.float64)
    normal = normal / np.linalg.norm(normal)
    v = np.stack([p[[0, 1, 2]], p[[0, 2, 3]]])
    n = np.broadcast_to(normal, v.shape)
    return v.astype(np.float32), np.ascontiguousarray(n).astype(np.float32)


def box(lo, hi, rot_y_deg=0.0):
    """Axis-aligned (optionally y-rotated about its centre) box: 12 triangles
    with outward flat normals."""
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    c = 0.5 * (lo + hi)
    corners = np.array([[x, y, z] for x in (lo[0], hi[0]) for y in (lo[1], hi[1]) for z in (lo[2], hi[2])])
    a = math.radians(rot_y_deg)
    R = np.array([[math.cos(a), 0, math.sin(a)], [0, 1, 0], [-math.sin(a), 0, math.cos(a)]])
    corners = (corners - c) @ R.T + c
    idx = lambda x, y, z: x * 4 + y * 2 + z  # noqa: E731
    faces = [
        (idx(0, 0, 0), idx(0, 0, 1), idx(0, 1, 1), idx(0, 1, 0), [-1, 0, 0]),
        (idx(1, 0, 0), idx(1, 1, 0), idx(1, 1, 1), idx(1, 0, 1), [1, 0, 0]),
        (idx(0, 0, 0), idx(1, 0, 0), idx(1, 0, 1), idx(0, 0, 1), [0, -1, 0]),
        (idx(0, 1, 0), idx(0, 1, 1), idx(1, 1, 1), idx(1, 1, 0), [0, 1, 0]),
        (idx(0, 0, 0), idx(0, 1, 0), idx(1, 1, 0), idx(1, 0, 0), [0, 0, -1]),
        (idx(0, 0, 1), idx(1, 0, 1), idx(1, 1, 1), idx(0, 1, 1), [0, 0, 1]),
    ]
    vs, ns = [], []
    for f in faces:
        nrm = R @ np.asarray(f[4], np.float64)
        v, n = quad(corners[f[0]], corners[f[1]], corners[f[2]], corners[f[3]], nrm)
        vs.append(v)
        ns.append(n)
    return np.concatenate(vs), np.concatenate(ns)


def uv_sphere(center, radius, n_seg, n_ring):
    """UV sphere with n_seg segments and n_ring rings, without the
    degenerate pole triangles: 2*n_seg*(n_ring-1) triangles, smooth normals."""
    th = np.linspace(0.0, math.pi, n_ring + 1)
    ph = np.linspace(0.0, 2 * math.pi, n_seg + 1)
    T, P = np.meshgrid(th, ph, indexing="ij")
    dirs = np.stack([np.sin(T) * np.cos(P), np.cos(T), np.sin(T) * np.sin(P)], -1)
    dirs[0, :] = [0, 1, 0]
    dirs[-1, :] = [0, -1, 0]
    tris = []
    for r in range(n_ring):
        for s in range(n_seg):
            a, b = (r, s), (r, s + 1)
            c, d = (r + 1, s + 1), (r + 1, s)
            if r != 0:
                tris.append((a, c, b))
            if r != n_ring - 1:
                tris.append((a, d, c))
    ia = np.array([[t[k][0] for k in range(3)] for t in tris])
    ib = np.array([[t[k][1] for k in range(3)] for t in tris])
    n = dirs[ia, ib]
    v = np.asarray(center, np.float64) + radius * n
    return v.astype(np.float32), n.astype(np.float32)


def _unit_sphere_template(n_seg, n_ring):
    v, n = uv_sphere((0, 0, 0), 1.0, n_seg, n_ring)
    return v.astype(np.float64), n.astype(np.float64)


def icosphere(level):
    """Icosphere: (vertices (V,3) f64 on the unit sphere, faces (F,3) int)."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
                  [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                  [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                  [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    for _ in range(level):
        nv = v.shape[0]
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e.sort(axis=1)
        key = e[:, 0] * nv + e[:, 1]
        uk, inv = np.unique(key, return_inverse=True)
        a, b = uk // nv, uk % nv
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        m = inv.reshape(3, -1) + nv
        m01, m12, m20 = m[0], m[1], m[2]
        v = np.concatenate([v, mid])
        f = np.concatenate([
            np.stack([f[:, 0], m01, m20], 1), np.stack([f[:, 1], m12, m01], 1),
            np.stack([f[:, 2], m20, m12], 1), np.stack([m01, m12, m20], 1)])
    return v, f


def value_noise(p, seed, octaves=6):
    """Seeded 3D value noise, ``octaves`` octaves (frequency x2, amplitude
    x0.5 each), normalised to [-1, 1]."""
    p = np.asarray(p, np.float64)
    total = np.zeros(p.shape[0])
    amp, freq, norm = 1.0, 2.0, 0.0

    def lattice(ix, iy, iz, octave):
        h = (ix.astype(np.uint64) * np.uint64(73856093)) ^ (iy.astype(np.uint64) * np.uint64(19349663)) \
            ^ (iz.astype(np.uint64) * np.uint64(83492791)) ^ np.uint64((seed * 2654435761 + octave * 97531) & 0xFFFFFFFF)
        h ^= h >> np.uint64(13)
        h *= np.uint64(0x5bd1e995)
        h ^= h >> np.uint64(15)
        return (h & np.uint64(0xFFFFFF)).astype(np.float64) / float(0xFFFFFF) * 2.0 - 1.0

    for o in range(octaves):
        q = p * freq + 1000.0
        i0 = np.floor(q).astype(np.int64)
        fr = q - i0
        s = fr * fr * (3 - 2 * fr)
        acc = 0.0
        for dx in (0, 1):
            for dy in (0, 1):
                for dz in (0, 1):
                    w = (s[:, 0] if dx else 1 - s[:, 0]) * (s[:, 1] if dy else 1 - s[:, 1]) * \
                        (s[:, 2] if dz else 1 - s[:, 2])
                    acc = acc + w * lattice(i0[:, 0] + dx, i0[:, 1] + dy, i0[:, 2] + dz, o)
        total += amp * acc
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return total / norm


def displaced_icosphere(level, center, radius, seed, amplitude=0.08):
    v, f = icosphere(level)
    d = value_noise(v, seed)
    r = radius * (1.0 + amplitude * d)
    pos = np.asarray(center, np.float64) + v * r[:, None]
    # smooth vertex normals: area-weighted face normals
    fn = np.cross(pos[f[:, 1]] - pos[f[:, 0]], pos[f[:, 2]] - pos[f[:, 0]])
    vn = np.zeros_like(pos)
    for k in range(3):
        np.add.at(vn, f[:, k], fn)
    vn /= np.linalg.norm(vn, axis=1, keepdims=True)
    return pos[f].astype(np.float32), vn[f].astype(np.float32)


# ----------------------------------------------------------------------------
# workloads


def _box_walls(light_size=0.25, light=True):
    h = 0.5
    mats = [
        Material("white", (1, 1, 1), roughness=1.0),
        Material("red", (1, 0, 0), roughness=1.0),
        Material("green", (0, 1, 0), roughness=1.0),
        Material("light", (1, 1, 1), emit=True),
    ]
    meshes = []
    v, n = quad((-h, -h, -h), (h, -h, -h), (h, -h, h), (-h, -h, h), (0, 1, 0))
    meshes.append(Mesh("floor", "white", v, n))
    v, n = quad((-h, h, -h), (-h, h, h), (h, h, h), (h, h, -h), (0, -1, 0))
    meshes.append(Mesh("ceiling", "white", v, n))
    v, n = quad((-h, -h, -h), (-h, h, -h), (h, h, -h), (h, -h, -h), (0, 0, 1))
    meshes.append(Mesh("back", "white", v, n))
    v, n = quad((-h, -h, -h), (-h, -h, h), (-h, h, h), (-h, h, -h), (1, 0, 0))
    meshes.append(Mesh("left", "red", v, n))
    v, n = quad((h, -h, -h), (h, h, -h), (h, h, h), (h, -h, h), (-1, 0, 0))
    meshes.append(Mesh("right", "green", v, n))
    if light:
        s = light_size / 2
        y = h - 1e-3
        v, n = quad((-s, y, -s), (-s, y, s), (s, y, s), (s, y, -s), (0, -1, 0))
        meshes.append(Mesh("light", "light", v, n))
    return mats, meshes


_BOX_CAMERA = dict(eye=(0.0, 0.0, 1.9), look_at=(0.0, 0.0, 0.0), fov=40.0)


def cornell_box(width=256, height=256, num_samples=64, num_bounces=7):
    mats, meshes = _box_walls()
    mats.append(Material("transparent", (1, 1, 1), alpha=0.0, roughness=None, n=1.5))
    v, n = box((-0.38, -0.5, -0.38), (-0.08, 0.1, -0.08))
    meshes.append(Mesh("large_box", "white", v, n))
    v, n = box((0.08, -0.5, -0.2), (0.33, -0.25, 0.05), rot_y_deg=30.0)
    meshes.append(Mesh("small_box", "transparent", v, n))
    v, n = uv_sphere((-0.2, -0.34, 0.22), 0.16, 32, 16)
    meshes.append(Mesh("sphere", "white", v, n))
    return Scene(mats, meshes, width=width, height=height, num_samples=num_samples,
                 num_bounces=num_bounces, name="cornell_box", **_BOX_CAMERA)


def icosphere_box(level=8, seed=1, width=1024, height=1024, num_samples=256, num_bounces=8,
                  light_size=0.25):
    mats, meshes = _box_walls(light_size=light_size)
    mats.append(Material("glass", (1, 1, 1), alpha=0.0, roughness=None, n=1.5))
    v, n = displaced_icosphere(level, (0.0, -0.18, 0.0), 0.28, seed)
    meshes.append(Mesh("icosphere", "glass", v, n))
    return Scene(mats, meshes, width=width, height=height, num_samples=num_samples,
                 num_bounces=num_bounces, name=f"icosphere_box_l{level}", **_BOX_CAMERA)


def hard_indirect(level=8, seed=3, width=1024, height=1024, num_samples=64, num_bounces=8):
    sc = icosphere_box(level=level, seed=seed, width=width, height=height, num_samples=num_samples,
                       num_bounces=num_bounces, light_size=0.02)
    rng = np.random.default_rng(seed)
    cx, cz = rng.uniform(-0.02, 0.02, 2)
    s = rng.uniform(0.06, 0.09)
    y = 0.5 - rng.uniform(0.03, 0.05)
    v, n = quad((cx - s, y, cz - s), (cx + s, y, cz - s), (cx + s, y, cz + s), (cx - s, y, cz + s),
                (0, 1, 0))
    sc.meshes.append(Mesh("baffle", "white", v, n))
    sc.name = f"hard_indirect_l{level}"
    return sc


def sphere_soup(n_spheres=20000, seed=2, width=1920, height=1080, num_samples=64, num_bounces=12,
                n_seg=16, n_ring=8, extent=100.0):
    rng = np.random.default_rng(seed)
    centers = rng.uniform(0.0, extent, (n_spheres, 3))
    radii = np.exp(rng.uniform(math.log(0.1), math.log(2.0), n_spheres))
    emissive = rng.uniform(0, 1, n_spheres) < 0.1
    le = rng.uniform(1.0, 5.0, n_spheres)
    albedo = rng.uniform(0.2, 0.9, (n_spheres, 3))
    tv, tn = _unit_sphere_template(n_seg, n_ring)
    mats, meshes = [], []
    for i in range(n_spheres):
        name = f"s{i}"
        if emissive[i]:
            mats.append(Material(name, (1.0, 1.0, 1.0), emit=True, scale=float(le[i])))
        else:
            mats.append(Material(name, tuple(albedo[i]), roughness=1.0))
        v = (centers[i] + radii[i] * tv).astype(np.float32)
        meshes.append(Mesh(name, name, v, tn.astype(np.float32)))
    return Scene(mats, meshes, eye=(50.0, 50.0, 175.0), look_at=(50.0, 50.0, 50.0), fov=40.0,
                 width=width, height=height, num_samples=num_samples, num_bounces=num_bounces,
                 name="sphere_soup")


def batch_scenes(n=64, seed=5, max_res=1024):
    """Uneven batch: each scene is a box + displaced icosphere or a sphere
    soup, with triangle count log-uniform in [1k, 500k], pixel count
    log-uniform in [128^2, max_res^2], spp in {16, 64, 256, 1024} and 4-12
    bounces."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        tris = math.exp(rng.uniform(math.log(1e3), math.log(5e5)))
        side = int(round(math.exp(rng.uniform(math.log(128), math.log(max_res)))))
        spp = int(rng.choice([16, 64, 256, 1024]))
        bounces = int(rng.integers(4, 13))
        if rng.uniform() < 0.5:
            level = int(np.clip(round(math.log(tris / 20.0, 4)), 3, 7))
            sc = icosphere_box(level=level, seed=seed * 1000 + i, width=side, height=side,
                               num_samples=spp, num_bounces=bounces)
        else:
            ns = max(4, int(tris / 224))
            sc = sphere_soup(n_spheres=ns, seed=seed * 1000 + i, width=side, height=side,
                             num_samples=spp, num_bounces=bounces, extent=100.0 * (ns / 20000) ** (1 / 3))
            ext = 100.0 * (ns / 20000) ** (1 / 3)
            sc.eye = (ext / 2, ext / 2, ext * 1.75)
            sc.look_at = (ext / 2, ext / 2, ext / 2)
        sc.name = f"batch{i:02d}_{sc.name}"
        out.append(sc)
    return out


# ----------------------------------------------------------------------------
# writers


def write_obj(path: str, vertices: np.ndarray, normals: np.ndarray) -> None:
    """OBJ with one 'v' and one 'vn' per soup corner and 'f a//a b//b c//c'
    faces (parse_obj.cc:48-57 reads v, vn and f v/vt/vn)."""
    v = vertices.reshape(-1, 3)
    nn = normals.reshape(-1, 3)
    with open(path, "w") as fh:
        fh.write("# generated by lisa_gb300.scenes\n")
        fh.write("".join(f"v {_g(a)} {_g(b)} {_g(c)}\n" for a, b, c in v.tolist()))
        fh.write("".join(f"vn {_g(a)} {_g(b)} {_g(c)}\n" for a, b, c in nn.tolist()))
        k = np.arange(1, v.shape[0] + 1).reshape(-1, 3)
        fh.write("".join(f"f {a}//{a} {b}//{b} {c}//{c}\n" for a, b, c in k.tolist()))


def _g(x: float) -> str:
    # 9 significant digits round-trip every float32
    return format(float(np.float32(x)), ".9g")


def write_rto(scene: Scene, directory: str, rto_name: Optional[str] = None,
              relative_to: Optional[str] = None) -> str:
    """Write ``scene`` as a .rto file plus one OBJ per mesh under
    ``directory``.  OBJ paths in the .rto are absolute unless
    ``relative_to`` is given (LiSA opens them relative to the working
    directory, scene_parser.cc:190-193)."""
    os.makedirs(directory, exist_ok=True)
    rto_name = rto_name or f"{scene.name}.rto"
    parts = ["/* generated by lisa_gb300.scenes */"]
    for m in scene.materials:
        parts.append(m.rto())
    for i, mesh in enumerate(scene.meshes):
        obj = os.path.join(directory, f"{scene.name}_{i:05d}_{mesh.name}.obj")
        write_obj(obj, mesh.vertices, mesh.normals)
        p = os.path.relpath(obj, relative_to) if relative_to else os.path.abspath(obj)
        parts.append(f"mesh {{\n  obj_file = {p}\n  material = {mesh.material}\n}}")
    e, la = scene.eye, scene.look_at
    parts.append("camera {\n"
                 f"  position = ({_f(e[0])}, {_f(e[1])}, {_f(e[2])})\n"
                 f"  look_at = ({_f(la[0])}, {_f(la[1])}, {_f(la[2])})\n"
                 f"  fov = {_f(scene.fov)}\n}}")
    parts.append(f"num_samples = {scene.num_samples}\nnum_bounces = {scene.num_bounces}\n")
    parts.append(f"width = {scene.width}\nheight = {scene.height}\n")
    parts.append(f"output_image = {scene.output_image}")
    path = os.path.join(directory, rto_name)
    with open(path, "w") as fh:
        fh.write("\n\n".join(parts) + "\n")
    return path
