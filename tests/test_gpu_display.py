"""The debug view and the display post-process on the GPU, against the oracle.

Debug view: Renderer::toggle_debug_view (renderer.rs:150-152, 470-486).
Display: Window::display_buffer (ui.rs:313-364) with gbuffer.glsl, blend.glsl,
median.glsl and id.glsl, restated as CUDA kernels (OpenGL is not available).
"""

import numpy as np
import pytest

from convector_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def room(gpu, orc):
    text, mats = scenes.room_sphere()
    bvh = gpu.Bvh.from_meshes([gpu.Mesh.parse(text, mats)])
    scene = gpu.Scene(bvh)
    scenes.default_camera(scene.camera)
    return scene, orc.OracleScene.from_bvh(bvh)


@pytest.mark.parametrize("rng_order,traversal", [(0, 0), (1, 0), (1, 1)])
def test_debug_view_bitexact(room, gpu, orc, rng_order, traversal):
    scene, osc = room
    r = gpu.Renderer(scene, 160, 96, rng_order=rng_order, traversal=traversal)
    r.toggle_debug_view()
    rgba, gb = r.render_frame_u8(42)
    col = r.read_frame_f32()
    orgba, ogb, ocol, orays = osc.render(scene.camera.as_array(), 160, 96, 42, rng_order=rng_order,
                                         traversal=traversal, debug=True)
    assert (col.view(np.uint32) == ocol.view(np.uint32)).all()
    assert (rgba == orgba).all() and (gb == ogb).all()
    assert r.stats()[0] == orays
    assert col[..., 1].max() > 0.3  # log2 of box counts is visible
    r.toggle_debug_view()
    normal, _ = r.render_frame_u8(42)
    assert not (normal == rgba).all()


def _textures(size=64, seed=3):
    rng = np.random.default_rng(seed)
    t1 = rng.integers(0, 256, (size, size, 3), dtype=np.uint8)
    yy, xx = np.mgrid[0:size, 0:size]
    t2 = np.stack([(xx * 4) % 256, (yy * 4) % 256, ((xx ^ yy) * 8) % 256], -1).astype(np.uint8)
    return t1, t2


def test_display_post_process_bitexact(room, gpu, orc):
    scene, osc = room
    w, h = 160, 96
    t1, t2 = _textures()
    disp = gpu.Display(w, h, t1, t2)
    od = orc.OracleDisplay(w, h, t1, t2)
    r = gpu.Renderer(scene, w, h, rng_order=1, traversal=1)
    for frame in range(10):  # more than the 8-frame ring
        rgba, gb = r.render_frame_u8(42 + frame)
        if frame == 0:
            assert ((gb >> 24) == 1).any()  # the floor carries texture index 1
        for blend, median in ((1, 1), (0, 1), (1, 0)) if frame == 9 else ((1, 1),):
            disp.enable_blend, disp.enable_median = bool(blend), bool(median)
            out = disp.display_buffer(rgba, gb)
            ref = od.frame(rgba, gb, blend=bool(blend), median=bool(median))
            assert (out == ref).all(), (frame, blend, median, np.count_nonzero(out != ref))
