"""ctypes front end of liboracle.so (convector_oracle.cpp).

ORACLE / TEST INFRASTRUCTURE: only tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py use this module, as the checker. The product
(convector_gb300) never imports it.
"""

import ctypes
import os

import numpy as np

from . import build as _build

_L = None

P, U32, I32, F32, U64 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int32, ctypes.c_float, ctypes.c_uint64

RNG_PATCH, RNG_GROUP = 0, 1
# classes of orc_classify: why two traversals' nearest hits of a ray differ
SAME, TIE, GRAZING, UNCLASSIFIED = 0, 1, 2, 3
TRAVERSE_PACKET, TRAVERSE_SINGLE, BRUTE_FORCE = 0, 1, 2


def lib():
    global _L
    if _L is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        sig = {
            "orc_scene_new": (P, [P, U32, P, U32, P, U32, ctypes.c_int]),
            "orc_scene_free": (None, [P]),
            "orc_intersect": (None, [P, P, P, P, P, P, P, U32, F32, ctypes.c_int, P, P, P, P, P, P, ctypes.c_int]),
            "orc_classify": (None, [P, P, P, P, P, P, P, U32, F32, P, P, P, P, P, ctypes.c_int]),
            "orc_scene_work": (None, [P, P]),
            "orc_bvh_build": (P, [P, U32]),
            "orc_bvh_num_nodes": (U32, [P]),
            "orc_bvh_num_triangles": (U32, [P]),
            "orc_bvh_copy": (None, [P, P, P, P]),
            "orc_bvh_stats": (None, [P, P, P, P]),
            "orc_bvh_free": (None, [P]),
            "orc_render": (U64, [P, P, U32, U32, U32, ctypes.c_int, ctypes.c_int, P, P, P, P, ctypes.c_int,
                                 ctypes.c_int]),
            "orc_render_patches": (U64, [P, P, U32, U32, U32, ctypes.c_int, U32, P, U32, P, P, P, P,
                                         ctypes.c_int]),
            "orc_display_new": (P, [U32, U32, P, P, U32, U32]),
            "orc_display_free": (None, [P]),
            "orc_display_frame": (None, [P, P, P, ctypes.c_int, ctypes.c_int, P]),
            "orc_resolve": (None, [P, U32, U32, U32, P]),
            "orc_rcp": (F32, [F32]), "orc_rsqrt": (F32, [F32]), "orc_recip_precise": (F32, [F32]),
            "orc_sin": (F32, [F32]), "orc_cos": (F32, [F32]), "orc_acos": (F32, [F32]),
            "orc_acos_fast": (F32, [F32]), "orc_cvtps": (I32, [F32]),
            "orc_fma3": (F32, [ctypes.c_int, F32, F32, F32]), "orc_abs": (F32, [F32]),
            "orc_any_sign_bit_positive_masked": (ctypes.c_int, [P, P]),
            "orc_rng_draws": (None, [U32, U32, U32, U32, P]),
            "orc_rng_samples": (None, [U32, U32, U32, ctypes.c_int, U32, P]),
            "orc_rotate_hemisphere": (None, [P, P, P]),
            "orc_quat_rotate": (None, [P, P, P]),
            "orc_quat_interpolate": (None, [P, P, F32, P]),
            "orc_aabb_intersect": (ctypes.c_int, [P, P, P, P, P]),
            "orc_triangle_intersect": (ctypes.c_int, [P, P, P, F32, P]),
            "orc_intersect_direct": (ctypes.c_int, [P, P, P, P]),
            "orc_camera_ray": (None, [P, F32, F32, F32, P]),
            "orc_sky_intensity": (None, [P, P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _L = L
    return _L


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def f32(*v):
    return np.ascontiguousarray(np.array(v, dtype=np.float32).ravel())


def default_threads():
    return max(1, os.cpu_count() or 1)


class OracleScene:
    """The hot path's scene: BVH-order triangles (n x 16 words) and nodes (n x 8 words)."""

    def __init__(self, triangles, nodes, general_pick=True):
        self.triangles = np.ascontiguousarray(triangles).view(np.uint32).reshape(-1, 16)
        self.nodes = np.ascontiguousarray(nodes).view(np.uint32).reshape(-1, 8)
        ds = np.nonzero((self.triangles[:, 15] >> 30) & 1)[0].astype(np.uint32)
        self.ds = np.ascontiguousarray(ds)
        self._h = lib().orc_scene_new(_p(self.triangles), self.triangles.shape[0], _p(self.nodes),
                                      self.nodes.shape[0], _p(self.ds), self.ds.shape[0], int(general_pick))

    @staticmethod
    def from_bvh(bvh, general_pick=True):
        return OracleScene(bvh.triangles, bvh.nodes, general_pick)

    def intersect(self, origins, directions, far=1.0e5, mode=TRAVERSE_PACKET, nthreads=None, counters=False):
        o = np.asarray(origins, dtype=np.float32)
        d = np.asarray(directions, dtype=np.float32)
        n = o.shape[0]
        cols = [np.ascontiguousarray(o[:, k]) for k in range(3)] + [np.ascontiguousarray(d[:, k]) for k in range(3)]
        t = np.empty(n, np.float32)
        tri = np.empty(n, np.int32)
        tu = np.empty(n, np.float32)
        tv = np.empty(n, np.float32)
        na = np.zeros(n, np.uint32) if counters else None
        nt = np.zeros(n, np.uint32) if counters else None
        lib().orc_intersect(self._h, *[_p(c) for c in cols], n, far, mode, _p(t), _p(tri), _p(tu), _p(tv), _p(na),
                            _p(nt), nthreads or default_threads())
        if counters:
            return t, tri, na, nt
        return t, tri

    def classify(self, origins, directions, ta, ia, tb, ib, far=1.0e5, nthreads=None):
        """Per ray, why the results (ta, ia) and (tb, ib) of two traversals
        differ: SAME, TIE (equal t, the first tested triangle wins), GRAZING
        (the approximate-reciprocal slab test rejects a box that holds the
        nearer hit) or UNCLASSIFIED."""
        o = np.asarray(origins, dtype=np.float32)
        d = np.asarray(directions, dtype=np.float32)
        n = o.shape[0]
        cols = [np.ascontiguousarray(o[:, k]) for k in range(3)] + [np.ascontiguousarray(d[:, k]) for k in range(3)]
        arrs = [np.ascontiguousarray(ta, dtype=np.float32), np.ascontiguousarray(ia, dtype=np.int32),
                np.ascontiguousarray(tb, dtype=np.float32), np.ascontiguousarray(ib, dtype=np.int32)]
        assert all(a.shape == (n,) for a in arrs)
        cls = np.empty(n, np.uint8)
        lib().orc_classify(self._h, *[_p(c) for c in cols], n, far, *[_p(a) for a in arrs], _p(cls),
                           nthreads or default_threads())
        return cls

    def render(self, camera, width, height, frame, rng_order=RNG_GROUP, traversal=TRAVERSE_PACKET, nthreads=None,
               color=True, accum=None, debug=False):
        cam = np.ascontiguousarray(camera, dtype=np.float32)
        rgba = np.zeros((height, width), np.uint32)
        gbuf = np.zeros((height, width), np.uint32)
        col = np.zeros((height, width, 3), np.float32) if color else None
        rays = lib().orc_render(self._h, _p(cam), width, height, frame, rng_order, traversal, _p(rgba), _p(gbuf),
                                _p(col), _p(accum), nthreads or default_threads(), int(debug))
        return rgba, gbuf, col, rays

    def last_render_work(self):
        """(boxes, triangles) the single-ray traversals of the last render tested."""
        out = np.zeros(2, np.uint64)
        lib().orc_scene_work(self._h, _p(out))
        return int(out[0]), int(out[1])

    def render_patches(self, camera, width, height, frame, patch_width, origins, traversal=TRAVERSE_PACKET,
                       rgba=None, gbuf=None, accum=None, nthreads=None):
        """renderer.rs:306-362 for the listed patch origins (x, y), into the given
        full-frame buffers (rgba and gbuf uint32 [h, w], accum float32 [h, w, 3])."""
        cam = np.ascontiguousarray(camera, dtype=np.float32)
        xy = np.ascontiguousarray(np.asarray(origins, dtype=np.uint32).reshape(-1, 2))
        return lib().orc_render_patches(self._h, _p(cam), width, height, frame, traversal, patch_width, _p(xy),
                                        xy.shape[0], _p(rgba), _p(gbuf), None, _p(accum),
                                        nthreads or default_threads())

    def __del__(self):
        if getattr(self, "_h", None) and _L is not None:
            _L.orc_scene_free(self._h)
            self._h = None


class OracleBvh:
    """Bvh::build (bvh.rs:488-545) restated in bvh_oracle.cpp: nodes (n x 8
    words), BVH-order triangles (n x 16 words), the source index of each
    BVH-order triangle, and the build statistics (bvh.rs:570-583) plus depth."""

    def __init__(self, triangles):
        tris = np.ascontiguousarray(np.asarray(triangles).view(np.uint32).reshape(-1, 16))
        h = lib().orc_bvh_build(_p(tris), tris.shape[0])
        if not h:
            raise ValueError("the BVH root does not split (bvh.rs:512 asserts)")
        try:
            nn, nt = lib().orc_bvh_num_nodes(h), lib().orc_bvh_num_triangles(h)
            self.nodes = np.zeros((nn, 8), np.uint32)
            self.triangles = np.zeros((nt, 16), np.uint32)
            self.source_index = np.zeros(nt, np.uint32)
            lib().orc_bvh_copy(h, _p(self.nodes), _p(self.triangles), _p(self.source_index))
            a, r, d = ctypes.c_float(), ctypes.c_float(), ctypes.c_uint32()
            lib().orc_bvh_stats(h, ctypes.byref(a), ctypes.byref(r), ctypes.byref(d))
            self.avg_tris_per_leaf, self.avg_area_ratio, self.depth = a.value, r.value, d.value
        finally:
            lib().orc_bvh_free(h)


def resolve(accum, n):
    h, w = accum.shape[:2]
    rgba = np.zeros((h, w), np.uint32)
    lib().orc_resolve(_p(np.ascontiguousarray(accum, dtype=np.float32)), w, h, n, _p(rgba))
    return rgba


class OracleDisplay:
    """The display post-process restatement (ring of 8 frames kept inside)."""

    def __init__(self, width, height, tex1, tex2):
        self.w, self.h = width, height
        self.t1 = np.ascontiguousarray(tex1, dtype=np.uint8)
        self.t2 = np.ascontiguousarray(tex2, dtype=np.uint8)
        th, tw = self.t1.shape[:2]
        self._h = lib().orc_display_new(width, height, _p(self.t1), _p(self.t2), tw, th)

    def frame(self, rgba, gbuf, blend=True, median=True):
        out = np.zeros((self.h, self.w), np.uint32)
        a = np.ascontiguousarray(rgba, dtype=np.uint32)
        g = np.ascontiguousarray(gbuf, dtype=np.uint32)
        lib().orc_display_frame(self._h, _p(a), _p(g), int(blend), int(median), _p(out))
        return out

    def __del__(self):
        if getattr(self, "_h", None) and _L is not None:
            _L.orc_display_free(self._h)
            self._h = None
