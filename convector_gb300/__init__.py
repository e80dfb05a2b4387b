"""GB300 render hot path of ruuda/convector.

Python mirror of the reference's Rust API for the render path, over the C-ABI
in include/convector_gpu.h (libconvector_gpu.so):

    SMaterial               material.rs:74-136   32-bit material encoding
    Mesh.load_with_materials wavefront.rs:83-152  OBJ loading
    Bvh.from_meshes / build bvh.rs:488-568       binned tree-SAH build
    Scene.from_meshes       scene.rs:114-129     scene + camera
    Camera                  scene.rs:20-100
    Renderer                renderer.rs:120-410  frames, accumulation, resolve

There is no CPU fallback: every render and query runs the CUDA kernels, and
a missing or unbuilt extension raises.
"""

import ctypes
import math
import os

import numpy as np

from . import _build

__all__ = ["SMaterial", "Mesh", "Bvh", "Scene", "Camera", "Renderer", "RenderConfig", "Batch", "View", "Server", "Display",
           "CvxError", "lib", "TRIANGLE_DTYPE_WORDS", "NODE_DTYPE_WORDS"]

TRIANGLE_DTYPE_WORDS = 16  # cvx_triangle: v0 v1 v2 (9 f32), uv0..2 (6 f32), material (u32)
NODE_DTYPE_WORDS = 8       # cvx_bvh_node: origin far_ (6 f32), index, len (u32)

TRAVERSE_PACKET, TRAVERSE_SINGLE = 0, 1
REFILL_AFTER_CAMERA, REFILL_ALL, REFILL_NONE = 0, 1, 2
RNG_PATCH, RNG_GROUP = 0, 1
MODE_MEGAKERNEL, MODE_WAVEFRONT, MODE_AUTO = 0, 1, 2
HOST_ACCESS_AUTO, HOST_ACCESS_COPY = 0, 1

_LIB = None


class CvxError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("convector_gpu error %d: %s" % (status, msg))
        self.status = status


class _Camera(ctypes.Structure):
    _fields_ = [("position", ctypes.c_float * 3), ("position_delta", ctypes.c_float * 3),
                ("orientation", ctypes.c_float * 4), ("orientation_delta", ctypes.c_float * 4),
                ("screen_distance", ctypes.c_float)]


class _View(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_uint32), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("spp", ctypes.c_uint32), ("frame_base", ctypes.c_uint32), ("camera", _Camera)]


class _ServerConfig(ctypes.Structure):
    _fields_ = [("framebuffer_bytes", ctypes.c_uint64), ("max_groups", ctypes.c_uint32),
                ("traversal", ctypes.c_uint32), ("use_graph", ctypes.c_uint32), ("sequential", ctypes.c_uint32),
                ("blocks_per_sm", ctypes.c_uint32), ("refill_mode", ctypes.c_uint32),
                ("kernel_mode", ctypes.c_uint32), ("fused_blocks_per_sm", ctypes.c_uint32),
                ("wavefront_streams", ctypes.c_uint32), ("deep_single_launch", ctypes.c_uint32),
                ("max_inflight_pixels", ctypes.c_uint64), ("samples_per_wave", ctypes.c_uint32),
                ("sample_buffer_bytes", ctypes.c_uint64)]


class _Request(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_uint32), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("spp", ctypes.c_uint32), ("frame_base", ctypes.c_uint32), ("camera", _Camera)]


class _Result(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("submit_s", ctypes.c_double), ("start_s", ctypes.c_double),
                ("done_s", ctypes.c_double), ("rays", ctypes.c_uint64)]


class RenderConfig(ctypes.Structure):
    _fields_ = [("rng_order", ctypes.c_uint32), ("traversal", ctypes.c_uint32), ("mode", ctypes.c_uint32),
                ("block_size", ctypes.c_uint32), ("use_graph", ctypes.c_uint32), ("blocks_per_sm", ctypes.c_uint32),
                ("refill_mode", ctypes.c_uint32)]


def lib(build=False):
    """Loads libconvector_gpu.so (building it first when `build` is true)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.build() if build else _build.LIB
    if not os.path.exists(path):
        raise RuntimeError("libconvector_gpu.so is not built: run __graft_entry__.build() or "
                           "python -m convector_gb300._build")
    L = ctypes.CDLL(path)
    P, U32, I32, F32, SZ = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int32, ctypes.c_float, ctypes.c_size_t
    sig = {
        "cvx_last_error": (I32, [ctypes.c_char_p, SZ]),
        "cvx_device_info": (I32, [P, ctypes.c_char_p, SZ]),
        "cvx_mesh_load_obj": (I32, [ctypes.c_char_p, P, P, U32, P]),
        "cvx_mesh_parse_obj": (I32, [ctypes.c_char_p, SZ, P, P, U32, P]),
        "cvx_mesh_num_triangles": (U32, [P]),
        "cvx_mesh_destroy": (None, [P]),
        "cvx_bvh_from_meshes": (I32, [P, U32, P]),
        "cvx_bvh_build": (I32, [P, U32, P]),
        "cvx_bvh_build_device": (I32, [P, U32, P]),
        "cvx_bvh_num_nodes": (U32, [P]),
        "cvx_bvh_num_triangles": (U32, [P]),
        "cvx_bvh_copy_nodes": (None, [P, P]),
        "cvx_bvh_copy_triangles": (None, [P, P]),
        "cvx_bvh_copy_source_index": (None, [P, P]),
        "cvx_bvh_stats": (None, [P, P, P, P]),
        "cvx_bvh_destroy": (None, [P]),
        "cvx_camera_default": (None, [P]),
        "cvx_camera_set_rotation": (None, [P, F32, F32]),
        "cvx_camera_set_fov": (None, [P, F32]),
        "cvx_camera_set_interactive": (None, [P, F32, F32]),
        "cvx_renderer_set_time": (I32, [P, F32, F32]),
        "cvx_renderer_update_scene": (I32, [P]),
        "cvx_set_traversal_stack_limit": (I32, [U32]),
        "cvx_inject_allocation_failure": (I32, [I32]),
        "cvx_scene_create": (I32, [P, U32, P, U32, P]),
        "cvx_scene_from_bvh": (I32, [P, P]),
        "cvx_scene_num_direct_samples": (U32, [P]),
        "cvx_scene_set_light_pick": (I32, [P, U32]),
        "cvx_scene_set_query_launch": (I32, [P, U32]),
        "cvx_scene_set_query_stack": (I32, [P, U32]),
        "cvx_scene_set_host_access": (I32, [P, U32, P]),
        "cvx_scene_destroy": (None, [P]),
        "cvx_intersect_nearest": (I32, [P, P, P, P, P, P, P, U32, F32, U32, P, P]),
        "cvx_intersect_nearest_device": (I32, [P, P, U32, F32, U32, P, P, P, P]),
        "cvx_intersect_nearest_noalloc": (I32, [P, P, P, P, P, P, P, U32, F32, U32, P, P]),
        "cvx_renderer_create": (I32, [P, U32, U32, P, P]),
        "cvx_renderer_destroy": (None, [P]),
        "cvx_renderer_set_camera": (I32, [P, P]),
        "cvx_render_frame_u8": (I32, [P, U32, P, P]),
        "cvx_render_patches_u8": (I32, [P, U32, P, U32, U32, P, P]),
        "cvx_accumulate_patches_f32": (I32, [P, U32, P, U32, U32, P]),
        "cvx_accumulate_frame_f32": (I32, [P, U32, P]),
        "cvx_accumulate_frames_f32": (I32, [P, U32, U32, P]),
        "cvx_resolve_u8": (I32, [P, U32, P]),
        "cvx_read_accumulator": (I32, [P, P]),
        "cvx_clear_accumulator": (I32, [P]),
        "cvx_read_frame_f32": (I32, [P, P]),
        "cvx_renderer_stats": (I32, [P, P, P]),
        "cvx_renderer_count_work": (I32, [P, U32, P]),
        "cvx_batch_create": (I32, [P, U32, U32, ctypes.c_uint64, P, P]),
        "cvx_batch_render": (I32, [P, P, U32, P, P, P]),
        "cvx_batch_destroy": (None, [P]),
        "cvx_batch_set_scene_mode": (I32, [P, U32, U32]),
        "cvx_server_set_scene_mode": (I32, [P, U32, U32]),
        "cvx_server_create": (I32, [P, U32, P, P]),
        "cvx_server_submit": (I32, [P, P, P, P]),
        "cvx_server_wait": (I32, [P, ctypes.c_uint64, U32, P]),
        "cvx_server_cancel": (I32, [P, ctypes.c_uint64]),
        "cvx_server_stats": (I32, [P, P, P, P, P]),
        "cvx_server_engine_stats": (I32, [P, P, P]),
        "cvx_server_destroy": (None, [P]),
        "cvx_renderer_set_debug_view": (I32, [P, U32]),
        "cvx_display_create": (I32, [U32, U32, P, P, U32, U32, P]),
        "cvx_display_frame": (I32, [P, P, P, U32, U32, P]),
        "cvx_display_destroy": (None, [P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = L
    return L


def _check(status):
    if status != 0:
        buf = ctypes.create_string_buffer(1024)
        lib().cvx_last_error(buf, 1024)
        raise CvxError(status, buf.value.decode(errors="replace"))


def set_traversal_stack_limit(entries):
    """Lowers the traversal stack's capacity on the current device (0: the
    default 128) so that tests can run the stack-overflow status path."""
    _check(lib().cvx_set_traversal_stack_limit(int(entries)))


def inject_allocation_failure(after):
    """The library's next `after` device allocations succeed and the one after
    them fails as out of memory (CVX_ERR_CAPACITY); negative cancels."""
    _check(lib().cvx_inject_allocation_failure(int(after)))


def _ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def device_info():
    """(ordinal, name) of the device new handles of this thread belong to."""
    ordinal, name = ctypes.c_int32(), ctypes.create_string_buffer(256)
    _check(lib().cvx_device_info(ctypes.byref(ordinal), name, 256))
    return ordinal.value, name.value.decode(errors="replace")


def _host_rays(origins, directions):
    """(n, 3) float32 origin and direction arrays, each as six contiguous columns."""
    o = np.ascontiguousarray(origins, dtype=np.float32)
    d = np.ascontiguousarray(directions, dtype=np.float32)
    if o.ndim != 2 or o.shape[1] != 3 or d.shape != o.shape:
        raise ValueError("origins and directions must be (n, 3) arrays of the same n, got %s and %s"
                         % (o.shape, d.shape))
    return o.shape[0], [np.ascontiguousarray(o[:, k]) for k in range(3)] + \
        [np.ascontiguousarray(d[:, k]) for k in range(3)]


def _frame_buffer(a, height, width, name):
    """A caller's output image, written in place: it must be (height, width) C-contiguous uint32."""
    if not isinstance(a, np.ndarray) or a.dtype != np.uint32 or a.shape != (height, width) or \
            not a.flags.c_contiguous or not a.flags.writeable:
        raise ValueError("%s must be a writeable C-contiguous (%d, %d) uint32 array" % (name, height, width))
    return a


def _device_tensor(x, name, count, floating):
    """A CUDA tensor the device query reads or writes: contiguous, 4-byte
    elements of the expected kind, and at least `count` of them."""
    if not getattr(x, "is_cuda", False) or not x.is_contiguous() or x.element_size() != 4 or \
            x.dtype.is_floating_point != floating or x.numel() < count:
        raise ValueError("%s must be a contiguous CUDA tensor of at least %d 4-byte %s elements"
                         % (name, count, "float" if floating else "integer"))
    return ctypes.c_void_p(x.data_ptr())


class SMaterial:
    """The reference's 32-bit material (material.rs:10-31, 84-136)."""

    @staticmethod
    def sky():
        return 0xC0000000

    @staticmethod
    def diffuse(r, g, b):
        def q(c):  # `(c * 255.0) as u32` on f32
            v = float(np.float32(c) * np.float32(255.0))
            return 0 if not v > 0 else min(int(v), 0xFFFFFFFF)
        return ((q(b) << 16) | (q(g) << 8) | q(r)) & 0xFFFFFFFF

    @staticmethod
    def white():
        return SMaterial.diffuse(1.0, 1.0, 1.0)

    @staticmethod
    def glass():
        return 0x60000000

    @staticmethod
    def with_glossiness(mat, glossiness):
        assert 0 <= glossiness <= 6
        return ((mat & 0b11100011_11111111_11111111_11111111) | (glossiness << 26)) & 0xFFFFFFFF

    @staticmethod
    def with_texture(mat, texture_index):
        assert 0 <= texture_index <= 3
        return ((mat & 0b11111100_11111111_11111111_11111111) | (texture_index << 24)) & 0xFFFFFFFF

    @staticmethod
    def is_direct_sample(mat):
        return (mat >> 30) & 1 == 1


def _material_arrays(materials):
    materials = materials or {}
    names = list(materials.keys())
    arr_names = (ctypes.c_char_p * max(1, len(names)))(*[n.encode() for n in names])
    arr_vals = np.array([materials[n] for n in names] or [0], dtype=np.uint32)
    return arr_names, arr_vals, len(names)


class Mesh:
    """A loaded OBJ mesh (wavefront.rs:24-28)."""

    def __init__(self, handle):
        self._h = ctypes.c_void_p(handle)

    @staticmethod
    def load(path):
        return Mesh.load_with_materials(path, {})

    @staticmethod
    def load_with_materials(path, materials):
        names, vals, n = _material_arrays(materials)
        out = ctypes.c_void_p()
        _check(lib().cvx_mesh_load_obj(os.fsencode(path), names, _ptr(vals), n, ctypes.byref(out)))
        return Mesh(out.value)

    @staticmethod
    def parse(text, materials=None):
        data = text.encode() if isinstance(text, str) else bytes(text)
        names, vals, n = _material_arrays(materials)
        out = ctypes.c_void_p()
        _check(lib().cvx_mesh_parse_obj(data, len(data), names, _ptr(vals), n, ctypes.byref(out)))
        return Mesh(out.value)

    @property
    def num_triangles(self):
        return lib().cvx_mesh_num_triangles(self._h)

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value and _LIB is not None:
            _LIB.cvx_mesh_destroy(self._h)
            self._h = None


class Bvh:
    """A built BVH in the reference's node and triangle order (bvh.rs:33-42)."""

    def __init__(self, handle):
        L = lib()
        self._h = ctypes.c_void_p(handle)
        nn, nt = L.cvx_bvh_num_nodes(self._h), L.cvx_bvh_num_triangles(self._h)
        self.nodes = np.zeros((nn, NODE_DTYPE_WORDS), dtype=np.uint32)
        self.triangles = np.zeros((nt, TRIANGLE_DTYPE_WORDS), dtype=np.uint32)
        self.source_index = np.zeros(nt, dtype=np.uint32)
        L.cvx_bvh_copy_nodes(self._h, _ptr(self.nodes))
        L.cvx_bvh_copy_triangles(self._h, _ptr(self.triangles))
        L.cvx_bvh_copy_source_index(self._h, _ptr(self.source_index))
        a, b, d = ctypes.c_float(), ctypes.c_float(), ctypes.c_uint32()
        L.cvx_bvh_stats(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(d))
        self.avg_tris_per_leaf, self.avg_area_ratio, self.depth = a.value, b.value, d.value

    @staticmethod
    def from_meshes(meshes):
        arr = (ctypes.c_void_p * len(meshes))(*[m._h.value for m in meshes])
        out = ctypes.c_void_p()
        _check(lib().cvx_bvh_from_meshes(arr, len(meshes), ctypes.byref(out)))
        return Bvh(out.value)

    @staticmethod
    def build(triangles):
        tris = np.ascontiguousarray(triangles).view(np.uint32).reshape(-1, TRIANGLE_DTYPE_WORDS)
        out = ctypes.c_void_p()
        _check(lib().cvx_bvh_build(_ptr(tris), tris.shape[0], ctypes.byref(out)))
        return Bvh(out.value)

    @staticmethod
    def build_device(triangles):
        """Bvh.build on the GPU: identical nodes, triangle order and statistics."""
        tris = np.ascontiguousarray(triangles).view(np.uint32).reshape(-1, TRIANGLE_DTYPE_WORDS)
        out = ctypes.c_void_p()
        _check(lib().cvx_bvh_build_device(_ptr(tris), tris.shape[0], ctypes.byref(out)))
        return Bvh(out.value)

    @property
    def triangles_f32(self):
        return self.triangles.view(np.float32)

    @property
    def nodes_f32(self):
        return self.nodes.view(np.float32)

    @property
    def direct_sample(self):
        """Indices of direct-sample triangles in BVH order (scene.rs:117-122)."""
        return np.nonzero((self.triangles[:, 15] >> 30) & 1)[0].astype(np.uint32)

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value and _LIB is not None:
            _LIB.cvx_bvh_destroy(self._h)
            self._h = None


class Camera:
    """scene.rs:20-100; the setters compute on the host in f32 like the reference."""

    def __init__(self):
        self._c = _Camera()
        lib().cvx_camera_default(ctypes.byref(self._c))

    def set_position(self, position, delta=(0.0, 0.0, 0.0)):
        self._c.position[:] = [float(np.float32(v)) for v in position]
        self._c.position_delta[:] = [float(np.float32(v)) for v in delta]

    def set_orientation(self, orientation, delta=(0.0, 0.0, 0.0, 0.0)):
        self._c.orientation[:] = [float(np.float32(v)) for v in orientation]
        self._c.orientation_delta[:] = [float(np.float32(v)) for v in delta]

    def set_rotation(self, radians, delta=0.0):
        lib().cvx_camera_set_rotation(ctypes.byref(self._c), radians, delta)

    def set_interactive(self, time, time_delta=0.0):
        """The camera of Renderer::update_scene (renderer.rs:140-147) at `time`."""
        lib().cvx_camera_set_interactive(ctypes.byref(self._c), time, time_delta)
        return self

    def set_fov(self, fov):
        lib().cvx_camera_set_fov(ctypes.byref(self._c), fov)

    def as_array(self):
        """pos[3], pos_delta[3], q[4], dq[4], screen_distance as float32."""
        c = self._c
        return np.array(list(c.position) + list(c.position_delta) + list(c.orientation)
                        + list(c.orientation_delta) + [c.screen_distance], dtype=np.float32)


class Scene:
    """A scene resident on the GPU (scene.rs:102-129)."""

    def __init__(self, bvh, light_pick=1):
        self.bvh = bvh
        self.camera = Camera()
        out = ctypes.c_void_p()
        _check(lib().cvx_scene_create(_ptr(bvh.triangles), bvh.triangles.shape[0], _ptr(bvh.nodes),
                                      bvh.nodes.shape[0], ctypes.byref(out)))
        self._h = out
        if light_pick != 1:
            _check(lib().cvx_scene_set_light_pick(self._h, light_pick))

    @staticmethod
    def from_meshes(meshes, light_pick=1):
        return Scene(Bvh.from_meshes(meshes), light_pick=light_pick)

    def set_query_launch(self, blocks_per_sm):
        """Resident blocks per SM of the nearest-hit kernel (0: default)."""
        _check(lib().cvx_scene_set_query_launch(self._h, blocks_per_sm))

    def set_query_stack(self, shared_entries):
        """Stack entries per lane the single-ray query keeps in shared memory
        (0, 4, 8 or 12; default 8)."""
        _check(lib().cvx_scene_set_query_stack(self._h, shared_entries))

    def set_host_access(self, mode):
        """How intersect_nearest brings host rays to the device: HOST_ACCESS_AUTO
        reads them in place where the device shares the host's page tables,
        HOST_ACCESS_COPY copies them first. Returns True when calls will read in
        place."""
        in_place = ctypes.c_uint32()
        _check(lib().cvx_scene_set_host_access(self._h, mode, ctypes.byref(in_place)))
        return bool(in_place.value)

    def direct_sample_num(self):
        return lib().cvx_scene_num_direct_samples(self._h)

    def intersect_nearest(self, origins, directions, far=1.0e5, traversal=TRAVERSE_PACKET):
        """Bvh::intersect_nearest over rays (n x 3 arrays); returns (t, triangle index in BVH order)."""
        n, cols = _host_rays(origins, directions)
        t = np.empty(n, dtype=np.float32)
        tri = np.empty(n, dtype=np.int32)
        _check(lib().cvx_intersect_nearest(self._h, *[_ptr(c) for c in cols], n, far, traversal, _ptr(t), _ptr(tri)))
        return t, tri

    def intersect_nearest_noalloc(self, origins, directions, far=1.0e5, traversal=TRAVERSE_PACKET):
        """intersect_nearest without any device allocation: stages through the
        library's static 16 MiB device buffer (at most 524,288 rays per call)."""
        n, cols = _host_rays(origins, directions)
        t = np.empty(n, dtype=np.float32)
        tri = np.empty(n, dtype=np.int32)
        _check(lib().cvx_intersect_nearest_noalloc(self._h, *[_ptr(c) for c in cols], n, far, traversal, _ptr(t),
                                                   _ptr(tri)))
        return t, tri

    def intersect_nearest_device(self, rays_soa, t_out, tri_out, far=1.0e5, traversal=TRAVERSE_PACKET,
                                 counters=None, stream=None):
        """Device form over torch CUDA tensors: rays_soa is a (6, n) float32
        tensor, t_out n float32, tri_out n int32 and counters (optional) 2n
        32-bit integers."""
        if len(rays_soa.shape) != 2 or rays_soa.shape[0] != 6:
            raise ValueError("rays_soa must be a (6, n) tensor, got %s" % (tuple(rays_soa.shape),))
        n = rays_soa.shape[1]
        rays = _device_tensor(rays_soa, "rays_soa", 6 * n, True)
        t = _device_tensor(t_out, "t_out", n, True)
        tri = _device_tensor(tri_out, "tri_out", n, False)
        cnt = None if counters is None else _device_tensor(counters, "counters", 2 * n, False)
        _check(lib().cvx_intersect_nearest_device(self._h, rays, n, far, traversal, t, tri, cnt,
                                                  None if stream is None else ctypes.c_void_p(stream)))

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value and _LIB is not None:
            _LIB.cvx_scene_destroy(self._h)
            self._h = None


class Renderer:
    """renderer.rs:120-410 as whole-frame GPU calls."""

    def __init__(self, scene, width, height, rng_order=RNG_GROUP, traversal=TRAVERSE_PACKET,
                 mode=MODE_MEGAKERNEL, block_size=0, use_graph=0, blocks_per_sm=0, refill_mode=REFILL_AFTER_CAMERA):
        self.scene, self.width, self.height = scene, width, height
        self.config = RenderConfig(rng_order, traversal, mode, block_size, use_graph, blocks_per_sm, refill_mode)
        out = ctypes.c_void_p()
        _check(lib().cvx_renderer_create(scene._h, width, height, ctypes.byref(self.config), ctypes.byref(out)))
        self._h = out
        self.set_camera(scene.camera)

    def set_camera(self, camera):
        _check(lib().cvx_renderer_set_camera(self._h, ctypes.byref(camera._c)))

    def set_time(self, time, time_delta=0.0):
        """Renderer::set_time (renderer.rs:134-137)."""
        _check(lib().cvx_renderer_set_time(self._h, time, time_delta))

    def update_scene(self):
        """Renderer::update_scene (renderer.rs:140-147): moves this renderer's
        camera along the interactive path to the time set by set_time."""
        _check(lib().cvx_renderer_update_scene(self._h))

    def toggle_debug_view(self, enable=None):
        """Renderer::toggle_debug_view (renderer.rs:150-152); with an argument, sets it."""
        self.debug_view = (not getattr(self, "debug_view", False)) if enable is None else bool(enable)
        _check(lib().cvx_renderer_set_debug_view(self._h, int(self.debug_view)))

    def render_frame_u8(self, frame_number, gbuffer=True):
        rgba = np.empty((self.height, self.width), dtype=np.uint32)
        gb = np.empty((self.height, self.width), dtype=np.uint32) if gbuffer else None
        _check(lib().cvx_render_frame_u8(self._h, frame_number, _ptr(rgba), _ptr(gb)))
        return rgba, gb

    def render_patches_u8(self, patch_width, origins, frame_number, rgba=None, gbuffer=None):
        """Renderer::render_patch_u8 (renderer.rs:306-327) for every (x, y) in
        `origins`, into full-frame uint32 buffers (created when None; pixels
        outside the patches are left as they are). Returns (rgba, gbuffer)."""
        xy = np.ascontiguousarray(np.asarray(origins, dtype=np.uint32).reshape(-1, 2))
        rgba = np.zeros((self.height, self.width), np.uint32) if rgba is None else \
            _frame_buffer(rgba, self.height, self.width, "rgba")
        gbuffer = np.zeros((self.height, self.width), np.uint32) if gbuffer is None else \
            _frame_buffer(gbuffer, self.height, self.width, "gbuffer")
        _check(lib().cvx_render_patches_u8(self._h, patch_width, _ptr(xy), xy.shape[0], frame_number, _ptr(rgba),
                                           _ptr(gbuffer)))
        return rgba, gbuffer

    def accumulate_patches_f32(self, patch_width, origins, frame_number, gbuffer=None):
        """Renderer::accumulate_patch_f32 (renderer.rs:339-362) for every (x, y) in `origins`."""
        xy = np.ascontiguousarray(np.asarray(origins, dtype=np.uint32).reshape(-1, 2))
        if gbuffer is not None:
            _frame_buffer(gbuffer, self.height, self.width, "gbuffer")
        _check(lib().cvx_accumulate_patches_f32(self._h, patch_width, _ptr(xy), xy.shape[0], frame_number,
                                                _ptr(gbuffer)))
        return gbuffer

    def accumulate_frame_f32(self, frame_number, gbuffer=False):
        gb = np.empty((self.height, self.width), dtype=np.uint32) if gbuffer else None
        _check(lib().cvx_accumulate_frame_f32(self._h, frame_number, _ptr(gb)))
        return gb

    def accumulate_frames_f32(self, first_frame, n_frames, gbuffer=False):
        """accumulate_frame_f32 for frames first_frame .. first_frame +
        n_frames - 1 in one call (cvx_accumulate_frames_f32): the same bits,
        with up to 32 frames per path-refill launch for a single-launch,
        single-ray renderer in the per-group RNG order."""
        gb = np.empty((self.height, self.width), dtype=np.uint32) if gbuffer else None
        _check(lib().cvx_accumulate_frames_f32(self._h, first_frame, n_frames, _ptr(gb)))
        return gb

    def resolve_u8(self, num_samples):
        rgba = np.empty((self.height, self.width), dtype=np.uint32)
        _check(lib().cvx_resolve_u8(self._h, num_samples, _ptr(rgba)))
        return rgba

    def read_accumulator(self):
        out = np.empty((self.height, self.width, 3), dtype=np.float32)
        _check(lib().cvx_read_accumulator(self._h, _ptr(out)))
        return out

    def clear_accumulator(self):
        _check(lib().cvx_clear_accumulator(self._h))

    def read_frame_f32(self):
        out = np.empty((self.height, self.width, 3), dtype=np.float32)
        _check(lib().cvx_read_frame_f32(self._h, _ptr(out)))
        return out

    def stats(self):
        rays, ms = ctypes.c_uint64(), ctypes.c_float()
        _check(lib().cvx_renderer_stats(self._h, ctypes.byref(rays), ctypes.byref(ms)))
        return rays.value, ms.value

    def count_work(self, frame):
        """The work of frame `frame` (cvx_renderer_count_work): rays traced,
        boxes and triangles they tested, and shading steps that evaluated
        every light's PDF."""
        out = (ctypes.c_uint64 * 4)()
        _check(lib().cvx_renderer_count_work(self._h, frame, out))
        return {"rays": out[0], "boxes": out[1], "triangles": out[2], "light_shades": out[3]}

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value and _LIB is not None:
            _LIB.cvx_renderer_destroy(self._h)
            self._h = None


class Display:
    """Window::display_buffer (ui.rs:313-364) on headless device buffers: the
    gbuffer texture composite, the 8-frame blend and the XYZ median filter of
    src/gpu/*.glsl, restated as CUDA kernels. tex1/tex2: (h, w, 3) uint8 sRGB."""

    def __init__(self, width, height, tex1, tex2):
        self.width, self.height = width, height
        self._t1 = np.ascontiguousarray(tex1, dtype=np.uint8)
        self._t2 = np.ascontiguousarray(tex2, dtype=np.uint8)
        assert self._t1.shape == self._t2.shape and self._t1.shape[2] == 3
        out = ctypes.c_void_p()
        _check(lib().cvx_display_create(width, height, _ptr(self._t1), _ptr(self._t2), self._t1.shape[1],
                                        self._t1.shape[0], ctypes.byref(out)))
        self._h = out
        self.enable_blend, self.enable_median = True, True

    def display_buffer(self, rgba, gbuffer):
        out = np.empty((self.height, self.width), dtype=np.uint32)
        a = np.ascontiguousarray(rgba, dtype=np.uint32)
        g = np.ascontiguousarray(gbuffer, dtype=np.uint32)
        if a.size != self.width * self.height or g.size != self.width * self.height:
            raise ValueError("rgba and gbuffer must hold %d x %d words" % (self.height, self.width))
        _check(lib().cvx_display_frame(self._h, _ptr(a), _ptr(g), int(self.enable_blend), int(self.enable_median),
                                       _ptr(out)))
        return out

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value and _LIB is not None:
            _LIB.cvx_display_destroy(self._h)
            self._h = None


class View:
    """One image of a batch: a scene index, size, samples and camera."""

    def __init__(self, scene, width, height, spp=1, frame_base=0, camera=None):
        self.scene, self.width, self.height, self.spp, self.frame_base = scene, width, height, spp, frame_base
        self.camera = camera if camera is not None else Camera()

    def _c(self):
        return _View(self.scene, self.width, self.height, self.spp, self.frame_base, self.camera._c)


class Batch:
    """Many views of many resident scenes rendered in shared wavefronts."""

    def __init__(self, scenes, max_groups=1 << 20, max_pixels=1 << 24, traversal=TRAVERSE_SINGLE, use_graph=1,
                 blocks_per_sm=0, refill_mode=REFILL_AFTER_CAMERA, mode=MODE_AUTO):
        self.scenes = list(scenes)
        arr = (ctypes.c_void_p * len(self.scenes))(*[s._h.value for s in self.scenes])
        cfg = RenderConfig(RNG_GROUP, traversal, mode, 0, use_graph, blocks_per_sm, refill_mode)
        out = ctypes.c_void_p()
        _check(lib().cvx_batch_create(arr, len(self.scenes), max_groups, max_pixels, ctypes.byref(cfg),
                                      ctypes.byref(out)))
        self._h = out

    def render(self, views, want_images=True):
        cv = (_View * len(views))(*[v._c() for v in views])
        imgs = [np.empty((v.height, v.width), dtype=np.uint32) for v in views] if want_images else None
        ptrs = (ctypes.c_void_p * len(views))(*[im.ctypes.data for im in imgs]) if want_images else None
        rays, ms = ctypes.c_uint64(), ctypes.c_float()
        _check(lib().cvx_batch_render(self._h, cv, len(views), ptrs, ctypes.byref(rays), ctypes.byref(ms)))
        return imgs, rays.value, ms.value

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value and _LIB is not None:
            _LIB.cvx_batch_destroy(self._h)
            self._h = None


class Server:
    """Continuously batched request server over resident scenes."""

    def __init__(self, scenes, framebuffer_bytes=4 << 30, max_groups=1 << 21, traversal=TRAVERSE_SINGLE,
                 use_graph=1, sequential=False, blocks_per_sm=0, refill_mode=REFILL_AFTER_CAMERA, kernel_mode=0,
                 fused_blocks_per_sm=0, wavefront_streams=1, deep_single_launch=0, max_inflight_pixels=0,
                 samples_per_wave=1, sample_buffer_bytes=0):
        self.scenes = list(scenes)
        arr = (ctypes.c_void_p * len(self.scenes))(*[s._h.value for s in self.scenes])
        cfg = _ServerConfig(framebuffer_bytes, max_groups, traversal, use_graph, int(sequential), blocks_per_sm,
                            refill_mode, kernel_mode, fused_blocks_per_sm, wavefront_streams, deep_single_launch,
                            max_inflight_pixels, samples_per_wave, sample_buffer_bytes)
        out = ctypes.c_void_p()
        _check(lib().cvx_server_create(arr, len(self.scenes), ctypes.byref(cfg), ctypes.byref(out)))
        self._h = out
        self._bufs = {}

    def submit(self, scene, width, height, spp, camera, frame_base=0):
        req = _Request(scene, width, height, spp, frame_base, camera._c)
        img = np.empty((height, width), dtype=np.uint32)
        rid = ctypes.c_uint64()
        _check(lib().cvx_server_submit(self._h, ctypes.byref(req), ctypes.c_void_p(img.ctypes.data),
                                       ctypes.byref(rid)))
        self._bufs[rid.value] = img
        return rid.value

    def wait(self, rid, timeout_ms=60000):
        """Returns (status, image or None, result dict); raises CvxError on a timeout."""
        res = _Result()
        _check(lib().cvx_server_wait(self._h, rid, timeout_ms, ctypes.byref(res)))
        img = self._bufs.pop(rid, None)
        info = {"status": res.status, "submit_s": res.submit_s, "start_s": res.start_s, "done_s": res.done_s,
                "rays": res.rays}
        return res.status, (img if res.status == 0 else None), info

    def cancel(self, rid):
        _check(lib().cvx_server_cancel(self._h, rid))

    def set_scene_mode(self, scene, mode):
        """Kernel organisation of one scene's waves: MODE_MEGAKERNEL (single
        launch) or MODE_WAVEFRONT; only while no request is queued or admitted."""
        _check(lib().cvx_server_set_scene_mode(self._h, scene, mode))

    def stats(self):
        now, waves, rays, busy = ctypes.c_double(), ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_double()
        _check(lib().cvx_server_stats(self._h, ctypes.byref(now), ctypes.byref(waves), ctypes.byref(rays),
                                      ctypes.byref(busy)))
        f, w = ctypes.c_double(), ctypes.c_double()
        _check(lib().cvx_server_engine_stats(self._h, ctypes.byref(f), ctypes.byref(w)))
        return {"now_s": now.value, "waves": waves.value, "rays": rays.value, "busy_s": busy.value,
                "fused_busy_s": f.value, "wavefront_busy_s": w.value}

    def close(self):
        if getattr(self, "_h", None) and self._h.value and _LIB is not None:
            _LIB.cvx_server_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()
