"""Seeded procedural scenes for the render hot path, emitted as OBJ text that
loads through the reference's loader (Mesh.load_with_materials).

    room_sphere()          1280x736 interactive scene: a 10-triangle box room
                           (open front), a UV sphere of 4,960 triangles on the
                           floor and a 2-triangle emissive ceiling quad
    displaced_icosphere()  ray-cast isolation: an icosphere of subdivision 6
                           (81,920 triangles) displaced radially by
                           0.05 x value noise (seed 7) inside the same room
    random_walk_tube()     a tube of 256 radial segments along a seeded random
                           walk (seed 11), about 870k triangles, in the room
    spheres_and_boxes()    one of the uneven-instance scenes: spheres and boxes
                           up to a triangle budget (seed from the caller)

Materials follow the reference's indoor scene (main.rs:72-79). Coordinates: y
up, the camera looks down -z from in front of the open side of the room.
"""

import math

import numpy as np

from . import SMaterial

ROOM_LO = np.array([-2.0, 0.0, -4.0])
ROOM_HI = np.array([2.0, 2.5, 0.0])


def reference_materials():
    """The name -> SMaterial map of main.rs:72-79 (textures not shipped)."""
    M = SMaterial
    return {
        "baseboard": M.with_glossiness(M.white(), 4),
        "ceiling": M.with_glossiness(M.white(), 1),
        "fauteuil": M.diffuse(1.0, 0.1, 0.4),
        "floor": M.with_texture(M.with_glossiness(M.diffuse(0.569, 0.494, 0.345), 4), 1),
        "glass": M.sky(),
        "wall": M.with_glossiness(M.diffuse(0.65, 0.7, 0.9), 1),
        "wood_light": M.with_texture(M.with_glossiness(M.diffuse(0.6, 0.533, 0.455), 3), 2),
    }


class ObjWriter:
    """Collects vertices, faces and materials; emits OBJ text for the loader,
    or the triangle array (n x 16 words, cvx_triangle) that loading that text
    gives, without the text round trip for large meshes. Vertices are rounded
    to float32 on entry, which is what the text's %.9g round-trips to."""

    def __init__(self):
        self.lines = []
        self.nv = 0
        self.nvt = 0
        self.verts = []
        self.texs = []
        self.blocks = []  # (faces (k x 3, global 0-based), tex faces or None, material name)
        self.mat = None

    def material(self, name):
        self.lines.append("usemtl %s" % name)
        self.mat = name

    def vertices(self, v):
        v = np.asarray(v, dtype=np.float32)
        base = self.nv
        self.verts.append(v)
        self.nv += v.shape[0]
        return base

    def tex_coords(self, t):
        t = np.asarray(t, dtype=np.float32)
        base = self.nvt
        self.texs.append(t)
        self.nvt += t.shape[0]
        return base

    def faces(self, f, base, tbase=None):
        f = np.asarray(f, dtype=np.int64)
        self.blocks.append((f + base, None if tbase is None else f + tbase, self.mat))
        self.lines.append(("faces", len(self.blocks) - 1))

    def text(self):
        verts = np.concatenate(self.verts) if self.verts else np.zeros((0, 3), np.float32)
        texs = np.concatenate(self.texs) if self.texs else np.zeros((0, 2), np.float32)
        out = ["v %.9g %.9g %.9g" % tuple(r) for r in verts.tolist()]
        out += ["vt %.9g %.9g" % tuple(r) for r in texs.tolist()]
        for item in self.lines:
            if isinstance(item, tuple):
                f, tf, _ = self.blocks[item[1]]
                if tf is None:
                    out.extend("f %d %d %d" % tuple(r) for r in (f + 1).tolist())
                else:
                    out.extend("f %d/%d %d/%d %d/%d" % (a, x, b, y, c, z)
                               for (a, b, c), (x, y, z) in zip((f + 1).tolist(), (tf + 1).tolist()))
            else:
                out.append(item)
        return "\n".join(out) + "\n"

    def triangles(self, materials):
        """The cvx_triangle array (n x 16 uint32) in face order."""
        verts = np.concatenate(self.verts).astype(np.float32)
        texs = np.concatenate(self.texs).astype(np.float32) if self.texs else np.zeros((0, 2), np.float32)
        parts = []
        for f, tf, mat in self.blocks:
            t = np.zeros((f.shape[0], 16), np.float32)
            t[:, 0:9] = verts[f].reshape(-1, 9)
            if tf is not None:
                t[:, 9:15] = texs[tf].reshape(-1, 6)
            u = t.view(np.uint32)
            u[:, 15] = materials[mat] if mat is not None else SMaterial.white()
            parts.append(u)
        return np.concatenate(parts)


def _room(w, lo=ROOM_LO, hi=ROOM_HI, floor_tex=True):
    """Box room of 10 triangles: floor, ceiling, back, left and right walls."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    quads = {
        "floor": [(x0, y0, z1), (x1, y0, z1), (x1, y0, z0), (x0, y0, z0)],
        "ceiling": [(x0, y1, z0), (x1, y1, z0), (x1, y1, z1), (x0, y1, z1)],
        "wall": [(x0, y0, z0), (x1, y0, z0), (x1, y1, z0), (x0, y1, z0),   # back
                 (x0, y0, z1), (x0, y0, z0), (x0, y1, z0), (x0, y1, z1),   # left
                 (x1, y0, z0), (x1, y0, z1), (x1, y1, z1), (x1, y1, z0)],  # right
    }
    for name, pts in quads.items():
        w.material(name)
        for q in range(len(pts) // 4):
            base = w.vertices(pts[4 * q:4 * q + 4])
            if name == "floor" and floor_tex:
                tb = w.tex_coords([(0, 0), (4, 0), (4, 4), (0, 4)])
                w.faces([(0, 1, 2), (0, 2, 3)], base, tb)
            else:
                w.faces([(0, 1, 2), (0, 2, 3)], base)


def _ceiling_light(w, y=None, cx=0.0, cz=-2.0, half=0.5):
    y = ROOM_HI[1] - 0.01 if y is None else y
    w.material("glass")
    base = w.vertices([(cx - half, y, cz - half), (cx + half, y, cz - half), (cx + half, y, cz + half),
                       (cx - half, y, cz + half)])
    w.faces([(0, 2, 1), (0, 3, 2)], base)


def uv_sphere(center, radius, segments, rings):
    """UV sphere with 2*S*(R-1) triangles: pole caps as triangles, bands as quads."""
    th = math.pi * np.arange(1, rings)[:, None] / rings
    ph = 2.0 * math.pi * np.arange(segments)[None, :] / segments
    ring_pts = np.stack([radius * np.sin(th) * np.cos(ph), np.broadcast_to(radius * np.cos(th), (rings - 1, segments)),
                         radius * np.sin(th) * np.sin(ph)], -1).reshape(-1, 3)
    verts = np.concatenate([[[0.0, radius, 0.0]], ring_pts, [[0.0, -radius, 0.0]]]) + np.asarray(center)
    s = np.arange(segments)
    ring = lambda r, k: 1 + (r - 1) * segments + (k % segments)
    top = np.stack([np.zeros(segments, np.int64), ring(1, s + 1), ring(1, s)], 1)
    r = np.arange(1, rings - 1)[:, None]
    a, b, c, d = ring(r, s[None, :]), ring(r, s[None, :] + 1), ring(r + 1, s[None, :] + 1), ring(r + 1, s[None, :])
    band = np.stack([np.stack([a, b, c], -1), np.stack([a, c, d], -1)], 2).reshape(-1, 3)
    south = verts.shape[0] - 1
    bottom = np.stack([np.full(segments, south, np.int64), ring(rings - 1, s), ring(rings - 1, s + 1)], 1)
    return verts, np.concatenate([top, band, bottom])


def _emit(w, obj):
    mats = reference_materials()
    return (w.text(), mats) if obj else (w.triangles(mats), mats)


def room_sphere(obj=True):
    """1280x736 interactive scene: 10 + 4,960 + 2 triangles. Returns (OBJ text,
    materials), or (triangle array, materials) when obj is false."""
    w = ObjWriter()
    _room(w)
    w.material("fauteuil")
    v, f = uv_sphere((0.0, 0.5, -2.0), 0.5, 80, 32)
    w.faces(f, w.vertices(v))
    _ceiling_light(w)
    return _emit(w, obj)


def _splitmix64(x):
    x = (x + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    return x ^ (x >> 31)


def value_noise(p, seed, freq=3.0):
    """Trilinear value noise in [-1, 1] with smoothstep weights; lattice
    values hashed from integer coordinates and the seed (splitmix64)."""
    p = np.asarray(p, dtype=np.float64) * freq
    i0 = np.floor(p).astype(np.int64)
    f = p - i0
    f = f * f * (3.0 - 2.0 * f)

    def lattice(ix, iy, iz):
        h = (ix.astype(np.uint64) * np.uint64(0x8DA6B343) ^ iy.astype(np.uint64) * np.uint64(0xD8163841)
             ^ iz.astype(np.uint64) * np.uint64(0xCB1AB31F) ^ np.uint64(seed * 0x9E3779B1))
        with np.errstate(over="ignore"):
            h = h + np.uint64(0x9E3779B97F4A7C15)
            h = (h ^ (h >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            h = (h ^ (h >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            h = h ^ (h >> np.uint64(31))
        return (h >> np.uint64(11)).astype(np.float64) / float(1 << 53) * 2.0 - 1.0

    out = 0.0
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                wgt = ((f[:, 0] if dx else 1 - f[:, 0]) * (f[:, 1] if dy else 1 - f[:, 1])
                       * (f[:, 2] if dz else 1 - f[:, 2]))
                out = out + wgt * lattice(i0[:, 0] + dx, i0[:, 1] + dy, i0[:, 2] + dz)
    return out


def icosphere(subdivisions):
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
                  (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)], dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
                  (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
                  (6, 2, 10), (8, 6, 7), (9, 8, 1)], dtype=np.int64)
    for _ in range(subdivisions):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        key = np.sort(e, axis=1)
        uniq, inv = np.unique(key[:, 0] * v.shape[0] + key[:, 1], return_inverse=True)
        a, b = uniq // v.shape[0], uniq % v.shape[0]
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        m = inv.reshape(3, -1) + v.shape[0]
        v = np.concatenate([v, mid])
        m01, m12, m20 = m
        f = np.concatenate([np.stack([f[:, 0], m01, m20], 1), np.stack([f[:, 1], m12, m01], 1),
                            np.stack([f[:, 2], m20, m12], 1), np.stack([m01, m12, m20], 1)])
    return v, f


def displaced_icosphere(subdivisions=6, seed=7, center=(0.0, 1.1, -2.0), radius=0.8, obj=True, light=False):
    """Icosphere of 20*4^s triangles displaced by 0.05 * value_noise(seed) in
    the room; with `light`, plus the 2-triangle ceiling light."""
    d, f = icosphere(subdivisions)
    r = radius + 0.05 * value_noise(d, seed)
    v = d * r[:, None] + np.asarray(center)
    w = ObjWriter()
    _room(w)
    w.material("wall")
    w.faces(f, w.vertices(v))
    if light:  # the ray-cast workload has none; rendering it needs one
        _ceiling_light(w)
    return _emit(w, obj)


def random_rays(n, seed=7, lo=ROOM_LO, hi=ROOM_HI):
    """n rays: origins uniform in the room box, directions uniform on S^2 (float32)."""
    rng = np.random.default_rng(seed)
    o = lo + (hi - lo) * rng.random((n, 3))
    z = rng.uniform(-1.0, 1.0, n)
    ph = rng.uniform(0.0, 2.0 * math.pi, n)
    s = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    d = np.stack([s * np.cos(ph), s * np.sin(ph), z], 1)
    return o.astype(np.float32), d.astype(np.float32)


def random_walk_tube(segments=256, rings=1700, seed=11, radius=0.04, obj=True):
    """A tube of `segments` radial segments around a random-walk centre line of
    `rings` rings (2*segments*(rings-1) triangles) inside the room, plus the room
    and the ceiling light."""
    rng = np.random.default_rng(seed)
    lo, hi = ROOM_LO + 0.3, ROOM_HI - 0.3
    p = np.array([0.0, 1.2, -2.0])
    d = np.array([1.0, 0.0, 0.0])
    centers, tangents = [], []
    step = 0.02
    for _ in range(rings):
        d = d + rng.normal(0.0, 0.25, 3)
        for k in range(3):  # steer back inside the room
            if p[k] < lo[k]:
                d[k] += 0.5
            if p[k] > hi[k]:
                d[k] -= 0.5
        d /= np.linalg.norm(d)
        p = p + step * d
        centers.append(p.copy())
        tangents.append(d.copy())
    centers, tangents = np.array(centers), np.array(tangents)
    # parallel-transported frame
    n0 = np.cross(tangents[0], [0.0, 1.0, 0.0])
    if np.linalg.norm(n0) < 1e-6:
        n0 = np.cross(tangents[0], [1.0, 0.0, 0.0])
    n0 /= np.linalg.norm(n0)
    normals = [n0]
    for i in range(1, rings):
        n = normals[-1] - np.dot(normals[-1], tangents[i]) * tangents[i]
        normals.append(n / np.linalg.norm(n))
    normals = np.array(normals)
    binormals = np.cross(tangents, normals)
    ang = 2.0 * math.pi * np.arange(segments) / segments
    ring_pts = (centers[:, None, :] + radius * (np.cos(ang)[None, :, None] * normals[:, None, :]
                                                + np.sin(ang)[None, :, None] * binormals[:, None, :]))
    verts = ring_pts.reshape(-1, 3)
    r = np.arange(rings - 1)[:, None]
    s = np.arange(segments)[None, :]
    a = r * segments + s
    b = r * segments + (s + 1) % segments
    c = (r + 1) * segments + (s + 1) % segments
    dd = (r + 1) * segments + s
    faces = np.concatenate([np.stack([a, b, c], -1).reshape(-1, 3), np.stack([a, c, dd], -1).reshape(-1, 3)])
    w = ObjWriter()
    _room(w)
    w.material("wood_light")
    w.faces(faces, w.vertices(verts))
    _ceiling_light(w)
    return _emit(w, obj)


def _box(center, size):
    cx, cy, cz = center
    hx, hy, hz = np.asarray(size) / 2.0
    v = np.array([(cx + sx * hx, cy + sy * hy, cz + sz * hz) for sx in (-1, 1) for sy in (-1, 1) for sz in (-1, 1)])
    f = np.array([(0, 1, 3), (0, 3, 2), (4, 6, 7), (4, 7, 5), (0, 4, 5), (0, 5, 1), (2, 3, 7), (2, 7, 6),
                  (0, 2, 6), (0, 6, 4), (1, 5, 7), (1, 7, 3)])
    return v, f


def spheres_and_boxes(n_tris, seed, obj=True):
    """Random spheres and boxes in the room until about `n_tris` triangles,
    plus the ceiling light."""
    rng = np.random.default_rng(seed)
    w = ObjWriter()
    w.material("wall")
    total = 0
    mats = ["wall", "fauteuil", "baseboard", "wood_light"]
    while total < n_tris - 2:
        left = n_tris - 2 - total
        c = ROOM_LO + 0.4 + (ROOM_HI - ROOM_LO - 0.8) * rng.random(3)
        w.material(mats[int(rng.integers(len(mats)))])
        if left < 60 or rng.random() < 0.3:
            v, f = _box(c, 0.1 + 0.4 * rng.random(3))
        else:
            seg = int(min(max(6, rng.integers(6, 48)), max(6, left // 12)))
            rings = max(3, min(seg // 2 + 1, left // (2 * seg) + 1))
            v, f = uv_sphere(c, 0.05 + 0.3 * rng.random(), seg, rings)
        w.faces(f, w.vertices(v))
        total += f.shape[0]
    _ceiling_light(w)
    return _emit(w, obj)


def look_at_quaternion(eye, target):
    """Unit quaternion (a, b, c, d) rotating the camera's -z view axis onto
    target - eye with +y kept up, for rotate() (quaternion.rs:110-153)."""
    fwd = np.asarray(target, dtype=np.float64) - np.asarray(eye, dtype=np.float64)
    fwd /= np.linalg.norm(fwd)
    up = np.array([0.0, 1.0, 0.0])
    right = np.cross(fwd, up)
    if np.linalg.norm(right) < 1e-9:
        right = np.array([1.0, 0.0, 0.0])
    right /= np.linalg.norm(right)
    true_up = np.cross(right, fwd)
    m = np.stack([right, true_up, -fwd], 1)  # columns: camera x, y, z in world space
    tr = np.trace(m)
    if tr > 0:
        s = math.sqrt(tr + 1.0) * 2
        q = (0.25 * s, (m[2, 1] - m[1, 2]) / s, (m[0, 2] - m[2, 0]) / s, (m[1, 0] - m[0, 1]) / s)
    elif m[0, 0] > m[1, 1] and m[0, 0] > m[2, 2]:
        s = math.sqrt(1.0 + m[0, 0] - m[1, 1] - m[2, 2]) * 2
        q = ((m[2, 1] - m[1, 2]) / s, 0.25 * s, (m[0, 1] + m[1, 0]) / s, (m[0, 2] + m[2, 0]) / s)
    elif m[1, 1] > m[2, 2]:
        s = math.sqrt(1.0 + m[1, 1] - m[0, 0] - m[2, 2]) * 2
        q = ((m[0, 2] - m[2, 0]) / s, (m[0, 1] + m[1, 0]) / s, 0.25 * s, (m[1, 2] + m[2, 1]) / s)
    else:
        s = math.sqrt(1.0 + m[2, 2] - m[0, 0] - m[1, 1]) * 2
        q = ((m[1, 0] - m[0, 1]) / s, (m[0, 2] + m[2, 0]) / s, (m[1, 2] + m[2, 1]) / s, 0.25 * s)
    q = np.array(q)
    return q / np.linalg.norm(q)


DEFAULT_EYE = (0.0, 1.2, 1.6)
DEFAULT_TARGET = (0.0, 1.0, -2.0)


def default_camera(camera, eye=DEFAULT_EYE, target=DEFAULT_TARGET):
    """Places a Camera (still, no motion blur) at `eye` looking at `target`."""
    camera.set_position(eye, (0.0, 0.0, 0.0))
    camera.set_orientation(look_at_quaternion(eye, target), (0.0, 0.0, 0.0, 0.0))
    return camera
