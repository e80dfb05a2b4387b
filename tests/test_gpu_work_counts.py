"""The counting form of the frame kernel (cvx_renderer_count_work), which
gives the frame kernels' algorithmic bytes: its totals of rays, boxes and
triangles tested equal the oracle's single-ray counters (bvh.rs:604-651)
summed over the same frame, and the image it renders is the ordinary frame."""

import numpy as np
import pytest

from convector_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,size", [("room_sphere", (160, 96)), ("displaced_icosphere", (96, 64))])
def test_frame_work_counts_equal_oracle(gpu, orc, name, size):
    kw = {"light": True} if name == "displaced_icosphere" else {}
    text, mats = getattr(scenes, name)(**kw)
    bvh = gpu.Bvh.from_meshes([gpu.Mesh.parse(text, mats)])
    sc = gpu.Scene(bvh)
    scenes.default_camera(sc.camera)
    osc = orc.OracleScene.from_bvh(bvh)
    w, h = size
    r = gpu.Renderer(sc, w, h, rng_order=gpu.RNG_GROUP, traversal=gpu.TRAVERSE_SINGLE)
    work = r.count_work(42)
    rgba_counted = r.read_frame_f32()
    orgba, _, ocol, orays = osc.render(sc.camera.as_array(), w, h, 42, rng_order=orc.RNG_GROUP, traversal=1)
    boxes, tris = osc.last_render_work()
    assert work["rays"] == orays and work["boxes"] == boxes and work["triangles"] == tris
    assert 0 < work["light_shades"] < work["rays"]
    assert (rgba_counted.view(np.uint32) == ocol.view(np.uint32)).all()
    rgba, _ = r.render_frame_u8(42)
    assert (rgba == orgba).all() and r.stats()[0] == orays


def test_count_work_needs_single_ray_group_order(gpu):
    text, mats = scenes.room_sphere()
    sc = gpu.Scene(gpu.Bvh.from_meshes([gpu.Mesh.parse(text, mats)]))
    for kw in (dict(rng_order=gpu.RNG_PATCH, traversal=gpu.TRAVERSE_SINGLE),
               dict(rng_order=gpu.RNG_GROUP, traversal=gpu.TRAVERSE_PACKET)):
        with pytest.raises(gpu.CvxError) as e:
            gpu.Renderer(sc, 64, 32, **kw).count_work(1)
        assert e.value.status == 1
