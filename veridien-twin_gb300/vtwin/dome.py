"""Seeded synthetic dome scenes in the twin's scene layout.

These are the inputs of every test and benchmark: a hemisphere of radius 4 m (icosphere level 5, upper half),
a floor disk, a table box and two emitting ring lamps, with eight Lambertian materials drawn from the twin's
seeded generator (mulberry32, control/rng.js:4-13).  The arrays follow what gpu/scene_gpu.js:prepareScene
consumes after welding (gpu/scene_gpu.js:241-349): per static mesh its own vertex set, a mesh table with a
material index and flags (gpu/scene_gpu.js:14 MESH_FLAG), and posed bodies (one BLAS each) whose emitter meshes
form the area light (gpu/scene_gpu.js:316-343).

Lambertian materials are expressed as the twin's dielectric with ior = 1: the exact Fresnel term is then 0 for
every cosine > 0 and Fbar = 0, so f = rho/pi exactly (gpu/bsdf.js:98-117).

Also here: seeded radiosity patch sets over the same dome (centres, normals, areas, albedo, emission) for the
node-radiosity solve, and the kinematic poses of capsule instruments for the batched configuration.
"""
from __future__ import annotations

import math
import numpy as np

MESH_FLAG = {"STATIC": 1, "EMITTER": 2, "LAYER": 4, "BOARD": 8, "INSTRUMENT": 16, "SCOPE": 32, "BENCH": 64,
             "TEXTURED": 128}


def mulberry32(seed: int):
    """Uniforms in [0, 1) exactly as control/rng.js:4-13 (32-bit integer arithmetic)."""
    a = seed & 0xFFFFFFFF

    def nxt() -> float:
        nonlocal a
        a = (a + 0x6D2B79F5) & 0xFFFFFFFF
        t = a
        t = ((t ^ (t >> 15)) * (t | 1)) & 0xFFFFFFFF
        t ^= (t + (((t ^ (t >> 7)) * (t | 61)) & 0xFFFFFFFF)) & 0xFFFFFFFF
        return ((t ^ (t >> 14)) & 0xFFFFFFFF) / 4294967296.0

    return nxt


class Rng:
    """control/rng.js:15-29: uniform, int and Box-Muller normal with a cached spare."""

    def __init__(self, seed: int):
        self.u = mulberry32(seed)
        self._spare = None

    def uniform(self, lo=0.0, hi=1.0):
        return lo + (hi - lo) * self.u()

    def int(self, lo, hi):
        return lo + math.floor(self.u() * (hi - lo + 1))

    def normal(self, mu=0.0, sigma=1.0):
        if self._spare is not None:
            s = self._spare
            self._spare = None
            return mu + sigma * s
        u = 0.0
        while u <= 1e-300:
            u = self.u()
        v = self.u()
        r = math.sqrt(-2.0 * math.log(u))
        self._spare = r * math.sin(2 * math.pi * v)
        return mu + sigma * r * math.cos(2 * math.pi * v)


# ------------------------------------------------------------------------------------------------ geometry

def icosphere(level: int):
    """Unit icosphere: vertices (float64) and faces (int) after `level` 4-way splits."""
    p = (1.0 + math.sqrt(5.0)) / 2.0
    V = [(-1, p, 0), (1, p, 0), (-1, -p, 0), (1, -p, 0), (0, -1, p), (0, 1, p), (0, -1, -p), (0, 1, -p),
         (p, 0, -1), (p, 0, 1), (-p, 0, -1), (-p, 0, 1)]
    V = [np.array(v, float) / np.linalg.norm(v) for v in V]
    F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    for _ in range(level):
        cache = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = V[a] + V[b]
                V.append(m / np.linalg.norm(m))
                cache[key] = len(V) - 1
            return cache[key]

        F2 = []
        for a, b, c in F:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            F2 += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        F = F2
    return np.array(V), np.array(F, dtype=np.int64)


def _submesh(P, N, faces):
    """Own vertex set of a face subset (each static mesh is welded on its own, gpu/scene_gpu.js:274-277)."""
    used = np.unique(faces.ravel())
    remap = -np.ones(len(P), np.int64)
    remap[used] = np.arange(len(used))
    return P[used].astype(np.float32), N[used].astype(np.float32), remap[faces].astype(np.uint32)


def dome_geometry(radius=4.0, level=5):
    """The hemisphere as four azimuth-quadrant meshes, inward normals, the rim flattened onto z = 0."""
    V, F = icosphere(level)
    cen = V[F].mean(axis=1)
    keep = cen[:, 2] > 0
    F = F[keep]
    cen = cen[keep]
    P = V * radius
    P[:, 2] = np.maximum(P[:, 2], 0.0)
    N = -V.copy()
    q = np.clip(np.floor((np.arctan2(cen[:, 1], cen[:, 0]) + math.pi) / (math.pi / 2)), 0, 3).astype(int)
    return [_submesh(P, N, F[q == k]) for k in range(4)]


def floor_geometry(radius=4.0, rings=16, seg=64):
    """Polar-grid disk at z = 0 (1984 triangles): inner (r < radius/2) and outer meshes, normal +z."""
    P = [(0.0, 0.0, 0.0)]
    for j in range(1, rings + 1):
        r = radius * j / rings
        for s in range(seg):
            a = 2 * math.pi * (s + 0.5 * (j % 2)) / seg
            P.append((r * math.cos(a), r * math.sin(a), 0.0))
    P = np.array(P)
    ring = lambda j, s: 1 + (j - 1) * seg + (s % seg)
    F = [(0, ring(1, s), ring(1, s + 1)) for s in range(seg)]
    for j in range(1, rings):
        for s in range(seg):
            a, b = ring(j, s), ring(j, s + 1)
            if j % 2:
                c, d = ring(j + 1, s), ring(j + 1, s + 1)
                F += [(a, c, d), (a, d, b)]
            else:
                c, d = ring(j + 1, s - 1), ring(j + 1, s)
                F += [(a, c, d), (a, d, b)]
    F = np.array(F, np.int64)
    N = np.tile([0.0, 0.0, 1.0], (len(P), 1))
    rc = np.linalg.norm(P[F].mean(axis=1)[:, :2], axis=1)
    inner = rc < radius / 2
    return [_submesh(P, N, F[inner]), _submesh(P, N, F[~inner])]


def box_geometry(lo, hi):
    """Axis-aligned box, flat outward normals: top face (2 tris) and the other five faces (10 tris)."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    faces = {  # corner lists (counter-clockwise seen from outside) and normal
        "top": ([(x0, y0, z1), (x1, y0, z1), (x1, y1, z1), (x0, y1, z1)], (0, 0, 1)),
        "bottom": ([(x0, y0, z0), (x0, y1, z0), (x1, y1, z0), (x1, y0, z0)], (0, 0, -1)),
        "xm": ([(x0, y0, z0), (x0, y0, z1), (x0, y1, z1), (x0, y1, z0)], (-1, 0, 0)),
        "xp": ([(x1, y0, z0), (x1, y1, z0), (x1, y1, z1), (x1, y0, z1)], (1, 0, 0)),
        "ym": ([(x0, y0, z0), (x1, y0, z0), (x1, y0, z1), (x0, y0, z1)], (0, -1, 0)),
        "yp": ([(x0, y1, z0), (x0, y1, z1), (x1, y1, z1), (x1, y1, z0)], (0, 1, 0)),
    }
    out = []
    for names in (["top"], ["bottom", "xm", "xp", "ym", "yp"]):
        P, N, I = [], [], []
        for nm in names:
            cs, n = faces[nm]
            o = len(P)
            P += cs
            N += [n] * 4
            I += [(o, o + 1, o + 2), (o, o + 2, o + 3)]
        out.append((np.array(P, np.float32), np.array(N, np.float32), np.array(I, np.uint32)))
    return out


def torus_geometry(centre, R=0.35, r=0.04, nmaj=8, nmin=3):
    """Ring lamp: a torus about +z with nmaj x nmin x 2 triangles (48 by default), outward normals."""
    P, N = [], []
    for i in range(nmaj):
        a = 2 * math.pi * i / nmaj
        ca, sa = math.cos(a), math.sin(a)
        for j in range(nmin):
            b = 2 * math.pi * j / nmin
            cb, sb = math.cos(b), math.sin(b)
            n = (ca * cb, sa * cb, sb)
            P.append((centre[0] + (R + r * cb) * ca, centre[1] + (R + r * cb) * sa, centre[2] + r * sb))
            N.append(n)
    I = []
    for i in range(nmaj):
        for j in range(nmin):
            a = i * nmin + j
            b = ((i + 1) % nmaj) * nmin + j
            c = ((i + 1) % nmaj) * nmin + (j + 1) % nmin
            d = i * nmin + (j + 1) % nmin
            I += [(a, b, c), (a, c, d)]
    return np.array(P, np.float32), np.array(N, np.float32), np.array(I, np.uint32)


def capsule_geometry(radius=0.006, length=0.25, nring=20, nseg=14, ncap=8):
    """Capsule along +z from 0 to `length`, radius `radius`, 1240 triangles by default (instrument meshes)."""
    P, N = [], []
    rows = []  # (z, rho, nz)
    for k in range(ncap, 0, -1):  # bottom hemisphere rings (pole excluded)
        t = (math.pi / 2) * k / ncap
        rows.append((-radius * math.sin(t) + 0.0, radius * math.cos(t), -math.sin(t)))
    for k in range(nseg + 1):
        rows.append((length * k / nseg, radius, 0.0))
    for k in range(1, ncap + 1):
        t = (math.pi / 2) * k / ncap
        rows.append((length + radius * math.sin(t), radius * math.cos(t), math.sin(t)))
    # drop the last rows' tiny radii at the poles: add pole vertices instead
    P.append((0.0, 0.0, -radius))
    N.append((0.0, 0.0, -1.0))
    for z, rho, nz in rows:
        nr = math.sqrt(max(0.0, 1 - nz * nz))
        for s in range(nring):
            a = 2 * math.pi * s / nring
            P.append((rho * math.cos(a), rho * math.sin(a), z))
            N.append((nr * math.cos(a), nr * math.sin(a), nz))
    P.append((0.0, 0.0, length + radius))
    N.append((0.0, 0.0, 1.0))
    nrow = len(rows)
    I = []
    vid = lambda row, s: 1 + row * nring + (s % nring)
    for s in range(nring):
        I.append((0, vid(0, s + 1), vid(0, s)))
    for row in range(nrow - 1):
        for s in range(nring):
            a, b, c, d = vid(row, s), vid(row, s + 1), vid(row + 1, s + 1), vid(row + 1, s)
            I += [(a, b, c), (a, c, d)]
    top = len(P) - 1
    for s in range(nring):
        I.append((top, vid(nrow - 1, s), vid(nrow - 1, s + 1)))
    I = np.array(I, np.uint32)
    return np.array(P, np.float32), np.array(N, np.float32), I


# ------------------------------------------------------------------------------------------------ cameras

def look_at(pos, target, up=(0.0, 0.0, 1.0)):
    """T_D_C (row-major 4x4) of an OpenCV camera at `pos` looking at `target` (x right, y down, z forward),
    axes built as renderer.js overviewCamera does (gpu/renderer.js:1122-1127)."""
    pos = np.asarray(pos, float)
    z = np.asarray(target, float) - pos
    z /= np.linalg.norm(z)
    x = np.cross(z, up)
    x /= np.linalg.norm(x)
    y = np.cross(z, x)
    T = np.eye(4)
    T[:3, 0], T[:3, 1], T[:3, 2], T[:3, 3] = x, y, z, pos
    return T


def kb4_camera(name, size, fx, fy, cx, cy, k, T, alpha=0.0):
    return {"name": name, "size": [int(size[0]), int(size[1])], "fx": float(fx), "fy": float(fy), "cx": float(cx),
            "cy": float(cy), "alpha": float(alpha), "k": [float(x) for x in k], "T_D_C": np.asarray(T, float)}


# ------------------------------------------------------------------------------------------------ scenes

def lambertian(name, rho):
    return {"name": name, "metallic": 0, "rho": [float(x) for x in rho], "f0": [0.56, 0.57, 0.58],
            "roughness": 0.5, "ior": 1.0, "fbar": float("nan"), "coated": 0, "coat_ior": 1.5,
            "coat_roughness": 0.05, "tau": [1.0, 1.0, 1.0], "emitter": 0}


def emitter_material():
    """The emitter body's own material (gpu/scene_gpu.js:323): dark, glossy, flagged as the emitter."""
    m = lambertian("emitter", [0.02, 0.02, 0.02])
    m.update({"roughness": 0.05, "ior": 1.5, "emitter": 1, "no_table": 1})
    return m


def make_dome_scene(seed: int = 1, width=640, height=480, level=5, with_instruments: int = 0, tool_radius: float = 0.006):
    """Config-0 dome: ~10.2k dome + 1984 floor + 12 table + 96 lamp triangles, 8 Lambertian materials
    (rho ~ U[0.2, 0.8] per channel from mulberry32(seed)), one KB4 camera, lamps L0 = 50 W sr^-1 m^-2, p = 1.

    with_instruments > 0 adds that many 1240-triangle capsule bodies (kind 'instrument', radius `tool_radius`, length
    0.25 m), posed by set_poses."""
    rng = Rng(seed)
    mats = [lambertian(f"mat{i}", [rng.uniform(0.2, 0.8) for _ in range(3)]) for i in range(8)]
    meshes, static = [], []
    S = MESH_FLAG["STATIC"]

    def add_static(name, mat, geo):
        meshes.append({"name": name, "mat": mat, "flags": S, "build_dir": [0.0, 0.0, 1.0], "layer": [0.0, 0.0]})
        static.append((len(meshes) - 1, geo))

    for qi, g in enumerate(dome_geometry(level=level)):
        add_static(f"dome_q{qi}", qi, g)
    fin, fout = floor_geometry()
    add_static("floor_in", 4, fin)
    add_static("floor_out", 5, fout)
    top, sides = box_geometry((-1.0, -0.4, 0.0), (1.0, 0.4, 0.9))
    add_static("table_top", 6, top)
    add_static("table_sides", 7, sides)
    # bench_white: the twin always appends the bench material after the mesh materials (gpu/scene_gpu.js:245-247)
    mats.append(lambertian("bench_white", [0.5, 0.5, 0.5]))
    # the emitter body: two ring lamps, one BLAS, identity pose (kind 'scope': it carries the light)
    mats.append(emitter_material())
    em = len(mats) - 1
    lamp_meshes = []
    for li, cx in enumerate((-1.2, 1.2)):
        meshes.append({"name": f"lamp{li}", "mat": em, "flags": MESH_FLAG["EMITTER"] | MESH_FLAG["SCOPE"],
                       "build_dir": [0.0, 0.0, 1.0], "layer": [0.0, 0.0]})
        lamp_meshes.append((len(meshes) - 1, torus_geometry((cx, 0.0, 2.2))))
    bodies = [_body("lamps", "scope", lamp_meshes)]
    if with_instruments:
        steel = len(mats)
        mats.append({**lambertian("steel", [0.0, 0.0, 0.0]), "metallic": 1, "f0": [0.56, 0.57, 0.58],
                     "roughness": 0.35, "ior": 1.5})
        cap = capsule_geometry(radius=tool_radius)
        for k in range(with_instruments):
            meshes.append({"name": f"tool{k}", "mat": steel, "flags": MESH_FLAG["INSTRUMENT"],
                           "build_dir": [0.0, 0.0, 1.0], "layer": [0.0, 0.0]})
            bodies.append(_body(f"tool{k}", "instrument", [(len(meshes) - 1, cap)]))
    st = _concat_static(static)
    cam = kb4_camera("CAM1", (width, height), 300.0 * width / 640, 300.0 * width / 640,
                     (width - 1) / 2.0, (height - 1) / 2.0, (0.05, -0.01, 0.002, -0.0003),
                     look_at((0.0, -3.0, 1.5), (0.0, 0.0, 0.6)))
    emitter = {"L0": [50.0, 50.0, 50.0], "theta": [0.0, math.pi], "p": [1.0, 1.0], "axis_deg": 0.0}
    return {"static": st, "bodies": bodies, "meshes": meshes, "materials": mats, "emitter": emitter,
            "cameras": [cam]}


def disk_geometry(radius, n=24, z=0.0):
    """Flat disk at height z facing +z: a fan of n triangles about its centre."""
    P = [(0.0, 0.0, z)] + [(radius * math.cos(2 * math.pi * k / n), radius * math.sin(2 * math.pi * k / n), z) for k in range(n)]
    I = [(0, 1 + k, 1 + (k + 1) % n) for k in range(n)]
    N = [(0.0, 0.0, 1.0)] * len(P)
    return np.array(P, np.float32), np.array(N, np.float32), np.array(I, np.uint32)


def make_scope_scene(seed: int = 1, level: int = 7, n_tools: int = 6, width: int = 1280, height: int = 720, n_cams: int = 3,
                     radius: float = 0.35):
    """A dome at the scale of the twin's own (lite_nodes draws it: radius 0.35 m, 3 mm nodes at level 7, depth range
    1 m): hemisphere + floor disk + a 16 x 12 x 3 cm pad (big triangles), a scope body (kind 'scope': a 5 mm shaft
    along -z ending in a 4 mm emitting outlet at its origin that faces +z, emission profile falling to 0 at 55 deg),
    `n_tools` 2.5 mm x 0.2 m instrument capsules and `n_cams` KB4 cameras on the dome wall looking at the pad (fx
    ~ U[550, 650] at 1920 px, k_i ~ N(0, 0.02)). Poses: scope_poses."""
    rng = Rng(seed)
    mats = [lambertian(f"pla{i}", [rng.uniform(0.6, 0.9) for _ in range(3)]) for i in range(4)]
    mats.append(lambertian("floor", [0.35, 0.35, 0.38]))
    mats.append(lambertian("pad", [0.7, 0.3, 0.3]))
    meshes, static = [], []
    S = MESH_FLAG["STATIC"]

    def add_static(name, mat, geo):
        meshes.append({"name": name, "mat": mat, "flags": S, "build_dir": [0.0, 0.0, 1.0], "layer": [0.0, 0.0]})
        static.append((len(meshes) - 1, geo))

    for qi, g in enumerate(dome_geometry(radius=radius, level=level)):
        add_static(f"dome_q{qi}", qi, g)
    fin, fout = floor_geometry(radius=radius, rings=64, seg=256)
    add_static("floor_in", 4, fin)
    add_static("floor_out", 4, fout)
    top, sides = box_geometry((-0.08, -0.06, 0.0), (0.08, 0.06, 0.03))
    add_static("pad_top", 5, top)
    add_static("pad_sides", 5, sides)
    mats.append(lambertian("bench_white", [0.5, 0.5, 0.5]))
    mats.append(emitter_material())
    em = len(mats) - 1
    steel = len(mats)
    mats.append({**lambertian("steel", [0.0, 0.0, 0.0]), "metallic": 1, "f0": [0.56, 0.57, 0.58], "roughness": 0.35, "ior": 1.5})
    meshes.append({"name": "scope_shaft", "mat": steel, "flags": MESH_FLAG["SCOPE"], "build_dir": [0.0, 0.0, 1.0], "layer": [0.0, 0.0]})
    sp, sn, si = capsule_geometry(radius=0.005, length=0.3)
    sp = sp.copy()
    sp[:, 2] -= 0.3 + 0.0052
    meshes.append({"name": "scope_outlet", "mat": em, "flags": MESH_FLAG["EMITTER"] | MESH_FLAG["SCOPE"],
                   "build_dir": [0.0, 0.0, 1.0], "layer": [0.0, 0.0]})
    bodies = [_body("scope", "scope", [(len(meshes) - 2, (sp, sn, si)), (len(meshes) - 1, disk_geometry(0.004))])]
    cap = capsule_geometry(radius=0.0025, length=0.2)
    for k in range(n_tools):
        meshes.append({"name": f"tool{k}", "mat": steel, "flags": MESH_FLAG["INSTRUMENT"], "build_dir": [0.0, 0.0, 1.0],
                       "layer": [0.0, 0.0]})
        bodies.append(_body(f"tool{k}", "instrument", [(len(meshes) - 1, cap)]))
    cams = []
    for c in range(n_cams):
        a = 2 * math.pi * c / n_cams - math.pi / 2
        pos = (0.3 * math.cos(a), 0.3 * math.sin(a), 0.12)
        fx = rng.uniform(550, 650) * width / 1920.0
        fy = fx * (1 + 0.004 * (rng.u() - 0.5))
        k = [rng.normal(0, 0.02) for _ in range(4)]
        cams.append(kb4_camera(f"CAM{c + 1}", (width, height), fx, fy, (width - 1) / 2.0, (height - 1) / 2.0, k,
                               look_at(pos, (0.0, 0.0, 0.04))))
    th = [math.radians(x) for x in (0.0, 10.0, 25.0, 40.0, 50.0, 55.0)]
    emitter = {"L0": [2.0e4, 1.9e4, 1.7e4], "theta": th, "p": [1.0, 0.97, 0.75, 0.35, 0.08, 0.0], "axis_deg": 0.0}
    return {"static": _concat_static(static), "bodies": bodies, "meshes": meshes, "materials": mats, "emitter": emitter,
            "cameras": cams}


def scope_poses(n_poses=16, n_tools=6, seed=21):
    """(n_poses, 1 + n_tools, 16) column-major body transforms for make_scope_scene: the scope tip 12-18 cm above
    the pad pointing down within 20 deg of vertical, the tools rotated uniformly about points 4-12 cm above it."""
    rng = Rng(seed)
    out = np.zeros((n_poses, 1 + n_tools, 16), np.float64)
    for p in range(n_poses):
        tilt, az = math.radians(20.0) * rng.u(), 2 * math.pi * rng.u()
        d = np.array([math.sin(tilt) * math.cos(az), math.sin(tilt) * math.sin(az), -math.cos(tilt)])   # +z of the scope
        x = np.cross([0.0, 1.0, 0.0], d)
        x /= np.linalg.norm(x)
        y = np.cross(d, x)
        T = np.eye(4)
        T[:3, 0], T[:3, 1], T[:3, 2] = x, y, d
        T[:3, 3] = [rng.uniform(-0.03, 0.03), rng.uniform(-0.03, 0.03), rng.uniform(0.12, 0.18)]
        out[p, 0] = T.T.ravel()
        for t in range(n_tools):
            R = random_rotation(rng)
            T = np.eye(4)
            T[:3, :3] = R
            T[:3, 3] = [rng.uniform(-0.06, 0.06), rng.uniform(-0.06, 0.06), rng.uniform(0.04, 0.12)]
            out[p, 1 + t] = T.T.ravel()
    return out


def _body(key, kind, parts):
    P, N, I, tm = [], [], [], []
    off = 0
    for mesh_id, (p, n, i) in parts:
        P.append(p)
        N.append(n)
        I.append(i + off)
        tm.append(np.full(len(i), mesh_id, np.uint32))
        off += len(p)
    P = np.concatenate(P).astype(np.float32)
    return {"key": key, "kind": kind, "P": P, "N": np.concatenate(N).astype(np.float32),
            "I": np.concatenate(I).astype(np.uint32), "tri_mesh": np.concatenate(tm),
            "UV": np.zeros((len(P), 2), np.float32)}


def _concat_static(static):
    P, N, I, tm, vm = [], [], [], [], []
    off = 0
    for mesh_id, (p, n, i) in static:
        P.append(p)
        N.append(n)
        I.append(i + off)
        tm.append(np.full(len(i), mesh_id, np.uint32))
        vm.append(np.full(len(p), mesh_id, np.uint32))
        off += len(p)
    return {"P": np.concatenate(P).astype(np.float32), "N": np.concatenate(N).astype(np.float32),
            "I": np.concatenate(I).astype(np.uint32), "tri_mesh": np.concatenate(tm),
            "vert_mesh": np.concatenate(vm)}


def batched_cameras(seed=3, n=3, width=1920, height=1200):
    """Three KB4 tracking cameras on the dome wall looking at the table: fx ~ U[550, 650] at 1920 px wide (scaled by
    width / 1920 for other sizes, so the field of view is kept), k_i ~ N(0, 0.02) (Box-Muller of mulberry32,
    control/rng.js:19-27)."""
    rng = Rng(seed)
    cams = []
    for c in range(n):
        a = 2 * math.pi * c / n - math.pi / 2
        pos = (3.2 * math.cos(a), 3.2 * math.sin(a), 1.6)
        fx = rng.uniform(550, 650) * width / 1920.0
        fy = fx * (1 + 0.004 * (rng.u() - 0.5))
        k = [rng.normal(0, 0.02) for _ in range(4)]
        cams.append(kb4_camera(f"CAM{c + 1}", (width, height), fx, fy, (width - 1) / 2.0, (height - 1) / 2.0, k,
                               look_at(pos, (0.0, 0.0, 0.7))))
    return cams


def random_rotation(rng: Rng):
    """Uniform rotation on SO(3) from a uniform unit quaternion (Shoemake 1992)."""
    u1, u2, u3 = rng.u(), rng.u(), rng.u()
    a, b = math.sqrt(1 - u1), math.sqrt(u1)
    x, y, z, w = a * math.sin(2 * math.pi * u2), a * math.cos(2 * math.pi * u2), b * math.sin(2 * math.pi * u3), \
        b * math.cos(2 * math.pi * u3)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def instrument_poses(n_poses=64, n_tools=6, seed=11, centre=(0.0, 0.0, 1.15)):
    """Rigid poses (column-major 4x4 per body, as setPoses takes them, gpu/renderer.js:620) of `n_tools`
    capsules: rotation uniform on SO(3), translation ~ U[-0.3, 0.3] m about a point above the table."""
    rng = Rng(seed)
    out = np.zeros((n_poses, n_tools, 16), np.float64)
    for p in range(n_poses):
        for t in range(n_tools):
            R = random_rotation(rng)
            tr = np.array(centre) + np.array([rng.uniform(-0.3, 0.3) for _ in range(3)])
            T = np.eye(4)
            T[:3, :3], T[:3, 3] = R, tr
            out[p, t] = T.T.ravel()  # column-major
    return out


def batch_pose_array(tool_poses, n_fixed: int = 1) -> np.ndarray:
    """(n_poses, n_fixed + n_tools, 16) body transforms for a pose batch: the scene's leading fixed bodies (the
    lamps) at identity, then the tools' poses (instrument_poses)."""
    tp = np.asarray(tool_poses, np.float64)
    n = tp.shape[0]
    eye = np.tile(np.eye(4).T.ravel(), (n, n_fixed, 1))
    return np.ascontiguousarray(np.concatenate([eye, tp], axis=1))


# ------------------------------------------------------------------------------------------------ radiosity

def fib_hemisphere(n, radius):
    i = np.arange(n) + 0.5
    z = 1 - i / n  # uniform in z on (0, 1): uniform area on the hemisphere
    r = np.sqrt(1 - z * z)
    phi = i * math.pi * (3 - math.sqrt(5))
    d = np.stack([r * np.cos(phi), r * np.sin(phi), z], 1)
    return d * radius, -d


def fib_disk(n, radius):
    i = np.arange(n) + 0.5
    r = radius * np.sqrt(i / n)
    phi = i * math.pi * (3 - math.sqrt(5))
    return np.stack([r * np.cos(phi), r * np.sin(phi), np.zeros(n)], 1)


def dome_patches(n: int, seed: int = 2, n_lamp: int = 96):
    """N radiosity patches over the dome: `n_lamp` on the two ring lamps (the lamp triangles' centroids),
    the rest on the hemisphere, floor and table in proportion to area.  Returns dict of float32 arrays
    (centres N x 3, normals N x 3, areas N, rho N ~ U[0.1, 0.9] from mulberry32(seed)) and the lamp index list."""
    rng = Rng(seed)
    lampP, lampN, lampA = [], [], []
    per = n_lamp // 2
    for cx in (-1.2, 1.2):
        nmaj = max(1, per // 6)
        P, Nn, I = torus_geometry((cx, 0.0, 2.2), nmaj=nmaj, nmin=3)
        v0, v1, v2 = P[I[:, 0]], P[I[:, 1]], P[I[:, 2]]
        c = (v0 + v1 + v2) / 3
        cr = np.cross(v1 - v0, v2 - v0)
        a = 0.5 * np.linalg.norm(cr, axis=1)
        nn = (Nn[I[:, 0]] + Nn[I[:, 1]] + Nn[I[:, 2]])
        nn /= np.linalg.norm(nn, axis=1, keepdims=True)
        lampP.append(c)
        lampN.append(nn)
        lampA.append(a)
    lampP, lampN, lampA = np.concatenate(lampP), np.concatenate(lampN), np.concatenate(lampA)
    m = n - len(lampP)
    A_dome, A_floor = 2 * math.pi * 16.0, math.pi * 16.0 - 1.6
    A_top, A_side = 1.6, 2 * (2.0 * 0.9 + 0.8 * 0.9)
    tot = A_dome + A_floor + A_top + A_side
    n_dome = int(round(m * A_dome / tot))
    n_top = max(4, int(round(m * A_top / tot)))
    n_side = max(4, int(round(m * A_side / tot)))
    n_floor = m - n_dome - n_top - n_side
    dP, dN = fib_hemisphere(n_dome, 4.0)
    # floor: Fibonacci disk points outside the table footprint
    k = n_floor
    while True:
        fp = fib_disk(int(k * 1.05) + 16, 4.0)
        fp = fp[~((np.abs(fp[:, 0]) < 1.0) & (np.abs(fp[:, 1]) < 0.4))]
        if len(fp) >= n_floor:
            fp = fp[:n_floor]
            break
        k = int(k * 1.1) + 16
    fN = np.tile([0.0, 0.0, 1.0], (n_floor, 1))
    gx = int(math.ceil(math.sqrt(n_top * 2.5)))
    gy = int(math.ceil(n_top / gx))
    tp = np.array([(-1 + 2 * (i + 0.5) / gx, -0.4 + 0.8 * (j + 0.5) / gy, 0.9) for j in range(gy) for i in range(gx)])[:n_top]
    tN = np.tile([0.0, 0.0, 1.0], (n_top, 1))
    # table sides: perimeter parameterised, rows in z
    per_len = 2 * (2.0 + 0.8)
    ncol = int(math.ceil(math.sqrt(n_side * per_len / 0.9)))
    nrow = int(math.ceil(n_side / ncol))
    sp, sn = [], []
    for j in range(nrow):
        for i in range(ncol):
            s = per_len * (i + 0.5) / ncol
            z = 0.9 * (j + 0.5) / nrow
            if s < 2.0:
                sp.append((-1 + s, -0.4, z)); sn.append((0, -1, 0))
            elif s < 2.8:
                sp.append((1.0, -0.4 + (s - 2.0), z)); sn.append((1, 0, 0))
            elif s < 4.8:
                sp.append((1.0 - (s - 2.8), 0.4, z)); sn.append((0, 1, 0))
            else:
                sp.append((-1.0, 0.4 - (s - 4.8), z)); sn.append((-1, 0, 0))
    sp, sn = np.array(sp)[:n_side], np.array(sn, float)[:n_side]
    C = np.concatenate([lampP, dP, fp, tp, sp]).astype(np.float32)
    Nrm = np.concatenate([lampN, dN, fN, tN, sn]).astype(np.float32)
    A = np.concatenate([lampA, np.full(n_dome, A_dome / n_dome), np.full(n_floor, A_floor / n_floor),
                        np.full(n_top, A_top / n_top), np.full(n_side, A_side / n_side)]).astype(np.float32)
    rho = np.array([rng.uniform(0.1, 0.9) for _ in range(n)], np.float32)
    lamps = np.arange(len(lampP), dtype=np.int64)
    return {"centres": C, "normals": Nrm, "areas": A, "rho": rho, "lamps": lamps}


def radiosity_rhs(n: int, lamps, n_rhs: int, seed: int = 5, single_value: float = 50.0):
    """Emission right-hand sides (N x R, float32).  R = 1: E = `single_value` on every lamp node.
    R > 1: each column a random on/off mask over the lamp nodes with intensities ~ U[10, 100] (mulberry32)."""
    E = np.zeros((n, n_rhs), np.float32)
    if n_rhs == 1:
        E[lamps, 0] = single_value
        return E
    rng = Rng(seed)
    for r in range(n_rhs):
        for i in lamps:
            on = rng.u() < 0.5
            val = rng.uniform(10.0, 100.0)
            if on:
                E[i, r] = val
        if not E[:, r].any():
            E[lamps[0], r] = 50.0
    return E
