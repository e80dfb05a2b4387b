"""Properties of the oracle's BVH traversals against brute force over every
triangle (the same triangle test in BVH order, no boxes).

A traversal never reports a hit nearer than brute force does. It agrees with
brute force on nearly every ray; it can miss the nearest hit where the slab
test, computed with the reference's approximate reciprocal (aabb.rs:105-141),
culls a box that holds it. The reference traversal behaves the same way, and
the GPU kernels reproduce it bit for bit, misses included."""

import numpy as np
import pytest

from convector_gb300 import scenes


@pytest.mark.parametrize("scene", ["room_sphere", "spheres_and_boxes", "displaced_icosphere"])
def test_traversals_against_brute_force(cvx, orc, scene):
    if scene == "spheres_and_boxes":
        text, mats = scenes.spheres_and_boxes(3000, seed=5)
    else:
        text, mats = getattr(scenes, scene)()
    osc = orc.OracleScene.from_bvh(cvx.Bvh.from_meshes([cvx.Mesh.parse(text, mats)]))
    o, d = scenes.random_rays(20000, seed=3)
    tb, ib = osc.intersect(o, d, mode=orc.BRUTE_FORCE)
    for mode in (orc.TRAVERSE_PACKET, orc.TRAVERSE_SINGLE):
        t, i = osc.intersect(o, d, mode=mode)
        assert (t >= tb).all()
        differ = (t.view(np.uint32) != tb.view(np.uint32)) | (i != ib)
        assert differ.sum() <= 0.0005 * o.shape[0]
