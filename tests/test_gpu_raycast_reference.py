"""The ray-cast kernel behind the headline number against the reference's
own traversal, on the full ray-cast workload.

The kernel (k_intersect_refill in select form, with the deferred pass) takes
every traversal decision over its own ray; the reference takes them over an
8-ray packet (bvh.rs:589-657). The two can differ on two kinds of ray only,
and the oracle's classifier decides which (oracle/convector_oracle.cpp
classify_pair):
  * tie: equal t bits, and each index's triangle alone gives that t; the two
    traversals tested them in different orders and the first tested wins
    (triangle.rs:127 rejects t >= dist);
  * grazing: the nearer hit's triangle lies under a box that the
    approximate-reciprocal slab test (aabb.rs:105-141) rejects for the ray at
    the farther distance, while an exact slab test finds the ray inside it.
Every other ray must have the same index and t (the tolerance of the hit
distance is 1e-5 relative; the results are in fact bit-identical).
"""

import numpy as np
import pytest

from convector_gb300 import scenes

pytestmark = pytest.mark.gpu

N_RAYS = 4194304
T_REL_TOL = 1e-5


def test_raycast_kernel_against_reference_packet_traversal(gpu, orc):
    text, mats = scenes.displaced_icosphere()  # 81,920 + 10 triangles, value noise seed 7
    bvh = gpu.Bvh.from_meshes([gpu.Mesh.parse(text, mats)])
    scene = gpu.Scene(bvh)
    osc = orc.OracleScene.from_bvh(bvh)
    o, d = scenes.random_rays(N_RAYS, seed=7)
    t, tri = scene.intersect_nearest(o, d, traversal=gpu.TRAVERSE_SINGLE)
    t_ref, tri_ref = osc.intersect(o, d, mode=orc.TRAVERSE_PACKET)
    cls = osc.classify(o, d, t, tri, t_ref, tri_ref)
    counts = np.bincount(cls, minlength=4)
    print("ray-cast kernel vs reference packet traversal, %d rays: same %d, tie %d, grazing %d, unclassified %d"
          % (N_RAYS, *counts))
    assert counts[orc.UNCLASSIFIED] == 0
    same = cls == orc.SAME
    assert (tri[same] == tri_ref[same]).all()
    rel = np.abs(t[same].astype(np.float64) - t_ref[same]) / np.maximum(np.abs(t_ref[same]), 1e-30)
    assert (rel <= T_REL_TOL).all()
    # differences are rare: 98 grazing rays of 4,194,304 on this workload
    assert counts[orc.SAME] >= N_RAYS - N_RAYS // 10000
    g = cls == orc.GRAZING
    print("grazing rays where the reference's hit is the nearer: %d of %d" % (int((t_ref[g] < t[g]).sum()),
                                                                           int(g.sum())))


def test_packet_query_equals_reference_traversal_on_every_ray(gpu, orc):
    """The packet variant takes the reference's decisions (bvh.rs:589-657:
    an octet is the 8-ray packet): on all 4,194,304 rays of the workload its
    index and t bits equal the oracle's packet traversal, with no exception."""
    text, mats = scenes.displaced_icosphere()
    bvh = gpu.Bvh.from_meshes([gpu.Mesh.parse(text, mats)])
    scene = gpu.Scene(bvh)
    osc = orc.OracleScene.from_bvh(bvh)
    o, d = scenes.random_rays(N_RAYS, seed=7)
    t, tri = scene.intersect_nearest(o, d, traversal=gpu.TRAVERSE_PACKET)
    t_ref, tri_ref = osc.intersect(o, d, mode=orc.TRAVERSE_PACKET)
    assert (tri == tri_ref).all(), np.nonzero(tri != tri_ref)[0][:10]
    assert (t.view(np.uint32) == t_ref.view(np.uint32)).all()
