"""The reference's patch-sequential random stream (CVX_RNG_PATCH: one
generator per 32x32 patch, consumed block by block and group by group,
renderer.rs:306-362) on the GPU against the oracle's sequential restatement,
bit for bit: frames, gbuffers, linear colour, ray counts and accumulations, at
ragged sizes whose border patches reach past the frame, for both traversals,
and on views whose groups end early (sky seen through the open front, where a
group takes 7 draws) or late (the inside of the room, 31 draws); and a ragged
list of 32-pixel patches through the per-patch call."""

import numpy as np
import pytest

from convector_gb300 import scenes

pytestmark = pytest.mark.gpu

VIEWS = {
    "inside": None,  # the default camera
    "out_of_the_front": ((0.0, 1.2, -1.0), (0.3, 1.4, 3.0)),
    "light_and_walls": ((1.5, 0.6, -1.2), (-0.5, 2.5, -3.0)),
}


@pytest.fixture(scope="module")
def room(gpu, orc):
    text, mats = scenes.room_sphere()
    bvh = gpu.Bvh.from_meshes([gpu.Mesh.parse(text, mats)])
    return gpu.Scene(bvh), orc.OracleScene.from_bvh(bvh)


def _camera(gpu, view):
    cam = gpu.Camera()
    if VIEWS[view] is None:
        return scenes.default_camera(cam)
    eye, target = VIEWS[view]
    return scenes.default_camera(cam, eye=eye, target=target)


@pytest.mark.parametrize("view", sorted(VIEWS))
@pytest.mark.parametrize("traversal", [0, 1])
def test_patch_stream_frame_equals_oracle(room, gpu, orc, view, traversal):
    scene, osc = room
    w, h = 200, 120
    r = gpu.Renderer(scene, w, h, rng_order=gpu.RNG_PATCH, traversal=traversal)
    cam = _camera(gpu, view)
    r.set_camera(cam)
    rgba, gb = r.render_frame_u8(42)
    col = r.read_frame_f32()
    orgba, ogb, ocol, orays = osc.render(cam.as_array(), w, h, 42, rng_order=orc.RNG_PATCH, traversal=traversal)
    assert (rgba == orgba).all() and (gb == ogb).all()
    assert (col.view(np.uint32) == ocol.view(np.uint32)).all()
    assert r.stats()[0] == orays


@pytest.mark.parametrize("traversal", [0, 1])
def test_patch_stream_accumulation_equals_oracle(room, gpu, orc, traversal):
    scene, osc = room
    w, h = 136, 72
    r = gpu.Renderer(scene, w, h, rng_order=gpu.RNG_PATCH, traversal=traversal)
    cam = _camera(gpu, "out_of_the_front")
    r.set_camera(cam)
    acc = np.zeros((h, w, 3), np.float32)
    for f in (3, 4, 5):
        r.accumulate_frame_f32(f)
        osc.render(cam.as_array(), w, h, f, rng_order=orc.RNG_PATCH, traversal=traversal, color=False, accum=acc)
    assert (r.read_accumulator().view(np.uint32) == acc.view(np.uint32)).all()
    assert (r.resolve_u8(3) == orc.resolve(acc, 3)).all()


def test_patch_list_of_32_equals_oracle(room, gpu, orc):
    """A ragged list of 32-pixel patches, some crossing the frame edge."""
    scene, osc = room
    w, h = 150, 90
    r = gpu.Renderer(scene, w, h, rng_order=gpu.RNG_GROUP, traversal=gpu.TRAVERSE_PACKET)
    cam = _camera(gpu, "light_and_walls")
    r.set_camera(cam)
    origins = [(0, 0), (32, 12), (144, 88), (96, 40), (128, 0)]
    sentinel = np.uint32(0xDEADBEEF)
    rgba = np.full((h, w), sentinel, np.uint32)
    gb = np.full((h, w), sentinel, np.uint32)
    r.render_patches_u8(32, origins, 9, rgba, gb)
    orgba = np.full((h, w), sentinel, np.uint32)
    ogb = np.full((h, w), sentinel, np.uint32)
    osc.render_patches(cam.as_array(), w, h, 9, 32, origins, traversal=0, rgba=orgba, gbuf=ogb)
    assert (rgba == orgba).all() and (gb == ogb).all()
    assert (rgba == sentinel).any()
