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


def _scene_and_rays(cvx, orc, scene, n=20000):
    if scene == "spheres_and_boxes":
        text, mats = scenes.spheres_and_boxes(3000, seed=5)
    else:
        text, mats = getattr(scenes, scene)()
    osc = orc.OracleScene.from_bvh(cvx.Bvh.from_meshes([cvx.Mesh.parse(text, mats)]))
    o, d = scenes.random_rays(n, seed=3)
    # and rays along the axes from the scene's corners, which graze box faces
    ax = np.repeat(np.eye(3, dtype=np.float32), 200, axis=0)
    ax *= np.where(np.arange(ax.shape[0]) % 2 == 0, 1.0, -1.0).astype(np.float32)[:, None]
    ao = scenes.random_rays(ax.shape[0], seed=4)[0]
    return osc, np.concatenate([o, ao]), np.concatenate([d, ax])


@pytest.mark.parametrize("scene", ["room_sphere", "spheres_and_boxes", "displaced_icosphere"])
def test_classifier_explains_every_traversal_difference(cvx, orc, scene):
    """The single-ray traversal against the reference's packet traversal, and
    each against brute force: every ray is the same, a tie or grazing."""
    osc, o, d = _scene_and_rays(cvx, orc, scene)
    res = {m: osc.intersect(o, d, mode=m) for m in (orc.TRAVERSE_PACKET, orc.TRAVERSE_SINGLE, orc.BRUTE_FORCE)}
    for a, b in ((orc.TRAVERSE_SINGLE, orc.TRAVERSE_PACKET), (orc.TRAVERSE_PACKET, orc.BRUTE_FORCE),
                 (orc.TRAVERSE_SINGLE, orc.BRUTE_FORCE)):
        cls = osc.classify(o, d, *res[a], *res[b])
        assert (cls != orc.UNCLASSIFIED).all(), (a, b, np.bincount(cls, minlength=4))


def test_classifier_flags_planted_wrong_results(cvx, orc):
    """Wrong results planted in the oracle's own output are not explained."""
    osc, o, d = _scene_and_rays(cvx, orc, "displaced_icosphere", n=4000)
    t, tri = osc.intersect(o, d, mode=orc.TRAVERSE_SINGLE)
    hit = np.nonzero(tri >= 0)[0][:50]
    assert hit.size == 50
    wrong_index = tri.copy()
    wrong_index[hit] = (tri[hit] + 1) % osc.triangles.shape[0]  # same t, another triangle
    missed = tri.copy()
    missed_t = t.copy()
    missed[hit] = -1  # a hit reported as a miss
    missed_t[hit] = 1.0e5
    nudged_t = t.copy()
    nudged_t[hit] = np.nextafter(t[hit], np.float32(np.inf))  # one ulp farther
    for tb, ib in ((t, wrong_index), (missed_t, missed), (nudged_t, tri)):
        cls = osc.classify(o, d, t, tri, tb, ib)
        assert (cls[hit] == orc.UNCLASSIFIED).all()
        rest = np.setdiff1d(np.arange(o.shape[0]), hit)
        assert (cls[rest] == orc.SAME).all()
