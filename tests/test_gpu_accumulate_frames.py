"""cvx_accumulate_frames_f32: the reference's accumulation loop (main.rs: one
accumulate_patch_f32 pass per frame, renderer.rs:339-362) over many frames in
one call. With the single-ray traversal and the per-group RNG order up to 32
frames share a path-refill launch, and a pass adds each pixel's frames in
frame order afterwards; every other form takes a launch per frame. Either way
the accumulator, the last frame's colour buffer and gbuffer, and the ray count
must equal those of one cvx_accumulate_frame_f32 call per frame, bit for bit:
on the deep-tree kernel (the 870k-triangle tube), the shallow one (room, paths
per lane, and a renderer set to one octet per group), the packet, wavefront
and patch-order forms, a moving camera and the debug view, at ragged frame
sizes, and across launch boundaries (33 and 40 frames: 32 + 1 and 32 + 8)."""

import numpy as np
import pytest

from convector_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def room(gpu):
    text, mats = scenes.room_sphere()
    sc = gpu.Scene(gpu.Bvh.from_meshes([gpu.Mesh.parse(text, mats)]))
    scenes.default_camera(sc.camera)
    return sc


@pytest.fixture(scope="module")
def tube(gpu):
    sc = gpu.Scene(gpu.Bvh.build(scenes.random_walk_tube(obj=False)[0]))
    scenes.default_camera(sc.camera)
    return sc


def _one_by_one(gpu, scene, w, h, kw, first, n):
    r = gpu.Renderer(scene, w, h, **kw)
    rays = 0
    gb = None
    for f in range(first, first + n):
        gb = r.accumulate_frame_f32(f, gbuffer=True)
        rays += r.stats()[0]
    return r.read_accumulator(), r.read_frame_f32(), gb, rays


def _in_one_call(gpu, scene, w, h, kw, first, n):
    r = gpu.Renderer(scene, w, h, **kw)
    gb = r.accumulate_frames_f32(first, n, gbuffer=True)
    return r.read_accumulator(), r.read_frame_f32(), gb, r.stats()[0]


def _same(a, b):
    acc_a, col_a, gb_a, rays_a = a
    acc_b, col_b, gb_b, rays_b = b
    assert (acc_a.view(np.uint32) == acc_b.view(np.uint32)).all()
    assert (col_a.view(np.uint32) == col_b.view(np.uint32)).all()
    assert (gb_a == gb_b).all()
    assert rays_a == rays_b


REFILL = dict(rng_order=1, traversal=1, refill_mode=1)


@pytest.mark.parametrize("n", [1, 2, 33])
def test_tube_full_frame(gpu, tube, n):
    w, h = 1280, 736
    _same(_one_by_one(gpu, tube, w, h, REFILL, 42, n), _in_one_call(gpu, tube, w, h, REFILL, 42, n))


@pytest.mark.parametrize("w,h,n", [(200, 120, 3), (136, 72, 40), (1280, 736, 32), (33, 7, 5)])
def test_room_paths_per_lane(gpu, room, w, h, n):
    _same(_one_by_one(gpu, room, w, h, REFILL, 7, n), _in_one_call(gpu, room, w, h, REFILL, 7, n))


@pytest.mark.parametrize("form", ["octet_groups", "packet", "wavefront", "patch_order"])
def test_other_forms(gpu, room, form):
    """One octet per group (shared path-refill launches all the same) and the
    forms that take a launch per frame."""
    kw = {"octet_groups": dict(rng_order=1, traversal=1, refill_mode=2),
          "packet": dict(rng_order=1, traversal=0),
          "wavefront": dict(rng_order=1, traversal=1, mode=1, use_graph=1),
          "patch_order": dict(rng_order=0, traversal=0)}[form]
    _same(_one_by_one(gpu, room, 200, 120, kw, 3, 4), _in_one_call(gpu, room, 200, 120, kw, 3, 4))


def test_moving_camera_and_debug_view(gpu, room):
    """A camera moving over each frame (Renderer::set_time with a time step,
    then update_scene) takes shared launches too; the debug view takes a
    launch per frame. Both equal one call per frame."""
    def moving(r):
        r.set_time(3.5, 0.1)
        r.update_scene()

    def debug(r):
        r.toggle_debug_view(True)

    for prepare in (moving, debug):
        a = gpu.Renderer(room, 200, 120, **REFILL)
        b = gpu.Renderer(room, 200, 120, **REFILL)
        prepare(a)
        prepare(b)
        rays = 0
        for f in range(5, 11):
            a.accumulate_frame_f32(f)
            rays += a.stats()[0]
        b.accumulate_frames_f32(5, 6)
        assert (a.read_accumulator().view(np.uint32) == b.read_accumulator().view(np.uint32)).all()
        assert (a.read_frame_f32().view(np.uint32) == b.read_frame_f32().view(np.uint32)).all()
        assert rays == b.stats()[0]


def test_accumulation_equals_oracle(gpu, orc, room):
    """Five frames in one call against the oracle's restatement of the
    accumulation, then resolved."""
    text, mats = scenes.room_sphere()
    bvh = gpu.Bvh.from_meshes([gpu.Mesh.parse(text, mats)])
    sc = gpu.Scene(bvh)
    scenes.default_camera(sc.camera)
    osc = orc.OracleScene.from_bvh(bvh)
    w, h = 136, 72
    r = gpu.Renderer(sc, w, h, **REFILL)
    r.accumulate_frames_f32(11, 5)
    acc = np.zeros((h, w, 3), np.float32)
    for f in range(11, 16):
        osc.render(sc.camera.as_array(), w, h, f, rng_order=orc.RNG_GROUP, traversal=1, color=False, accum=acc)
    assert (r.read_accumulator().view(np.uint32) == acc.view(np.uint32)).all()
    assert (r.resolve_u8(5) == orc.resolve(acc, 5)).all()


def test_continues_an_accumulation(gpu, room):
    """Calls add to what the accumulator holds, like the one-frame call."""
    w, h = 200, 120
    a = gpu.Renderer(room, w, h, **REFILL)
    for f in range(0, 9):
        a.accumulate_frame_f32(f)
    b = gpu.Renderer(room, w, h, **REFILL)
    b.accumulate_frame_f32(0)
    b.accumulate_frames_f32(1, 5)
    b.accumulate_frames_f32(6, 3)
    assert (a.read_accumulator().view(np.uint32) == b.read_accumulator().view(np.uint32)).all()


def test_bad_arguments(gpu, room):
    r = gpu.Renderer(room, 64, 32, **REFILL)
    with pytest.raises(gpu.CvxError):
        r.accumulate_frames_f32(0, 0)
    with pytest.raises(gpu.CvxError):
        r.accumulate_frames_f32(0xFFFFFFFF, 2)
