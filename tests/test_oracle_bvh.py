"""The product's host BVH build against the oracle's independent restatement
of Bvh::build (bvh.rs:488-545, oracle/bvh_oracle.cpp): the same node array,
triangle order (and source index of every BVH-order triangle) and statistics,
bit for bit, on the workloads' scenes and on inputs that reach every branch
of the build: the uniform split for small nodes (bvh.rs:142-145) and as the
crowded-bin fallback (bvh.rs:157-167), equal sort keys (the stable sort of
bvh.rs:178-186), signed zeros in the bounds, and nodes whose barycentres
all coincide. The device build is compared with the same restatement in
tests/test_gpu_bvh_build.py."""

import os

import numpy as np
import pytest

from convector_gb300 import scenes

WHITE = 0x00FFFFFF
REFERENCE = os.environ.get("CONVECTOR_REFERENCE", "")
HAVE_MODELS = bool(REFERENCE) and os.path.isdir(os.path.join(REFERENCE, "models"))


def _tris(v):
    """(n, 3, 3) float32 vertices -> (n, 16) cvx_triangle words."""
    v = np.asarray(v, dtype=np.float32).reshape(-1, 9)
    t = np.zeros((v.shape[0], 16), np.float32)
    t[:, :9] = v
    w = t.view(np.uint32)
    w[:, 15] = WHITE
    return w


def _random_tris(n, seed, spread=4.0, size=0.05):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-spread, spread, (n, 1, 3))
    return _tris(c + rng.normal(0.0, size, (n, 3, 3)))


def _same(cvx, orc, tris):
    a = cvx.Bvh.build(tris)
    b = orc.OracleBvh(tris)
    assert a.nodes.shape == b.nodes.shape
    assert np.array_equal(a.nodes, b.nodes)
    assert np.array_equal(a.triangles, b.triangles)
    assert np.array_equal(a.source_index, b.source_index)
    assert np.float32(a.avg_tris_per_leaf).tobytes() == np.float32(b.avg_tris_per_leaf).tobytes()
    assert np.float32(a.avg_area_ratio).tobytes() == np.float32(b.avg_area_ratio).tobytes()
    assert a.depth == b.depth
    return b


@pytest.mark.parametrize("name", ["room_sphere", "displaced_icosphere"])
def test_workload_scenes(cvx, orc, name):
    tris, _ = getattr(scenes, name)(obj=False)
    _same(cvx, orc, tris)


def test_random_walk_tube(cvx, orc):
    tris, _ = scenes.random_walk_tube(obj=False)
    b = _same(cvx, orc, tris)
    assert b.triangles.shape[0] == 869900 and b.depth == 70


@pytest.mark.parametrize("n,seed", [(500, 3), (3000, 5), (20000, 7)])
def test_spheres_and_boxes(cvx, orc, n, seed):
    tris, _ = scenes.spheres_and_boxes(n, seed, obj=False)
    _same(cvx, orc, tris)


@pytest.mark.parametrize("n", [2, 3, 5, 17, 31, 32, 33, 47, 64, 65, 100, 129, 1000, 4097, 70000])
def test_random_triangles(cvx, orc, n):
    _same(cvx, orc, _random_tris(n, seed=n))


def test_clustered_triangles_take_the_uniform_fallback(cvx, orc):
    wide = _random_tris(300, seed=1, spread=50.0, size=0.5)
    dense = _random_tris(60000, seed=2, spread=0.2, size=0.002)
    _same(cvx, orc, np.concatenate([wide, dense]))


def test_equal_barycentres_keep_node_order(cvx, orc):
    base = _random_tris(40, seed=9)
    copies = np.repeat(_random_tris(1, seed=10), 300, axis=0)
    _same(cvx, orc, np.concatenate([copies[:150], base, copies[150:]]))


def test_coinciding_barycentres_become_a_leaf(cvx, orc):
    """48 copies of one triangle (33..64: the coordinate binning puts them all
    in one bin on every axis, and there is no fallback below 65) beside a
    distant one: the copies end as one leaf, where the reference asserts
    (bvh.rs:302)."""
    copies = np.repeat(_random_tris(1, seed=11), 48, axis=0)
    far = _random_tris(1, seed=12, spread=40.0)
    b = _same(cvx, orc, np.concatenate([copies, far]))
    assert (b.nodes[:, 7] == 48).any()


def test_signed_zero_bounds(cvx, orc):
    rng = np.random.default_rng(4)
    v = rng.uniform(0.1, 1.0, (3000, 3, 3)).astype(np.float32)
    v[:, 0, 0] = np.where(rng.random(3000) < 0.5, np.float32(0.0), np.float32(-0.0))
    v[:, 1, 1] = np.where(rng.random(3000) < 0.5, np.float32(0.0), np.float32(-0.0))
    v[::3, 2, 2] = -0.0
    _same(cvx, orc, _tris(v))


def test_root_that_does_not_split_is_refused(cvx, orc):
    with pytest.raises(ValueError):
        orc.OracleBvh(np.repeat(_random_tris(1, seed=1), 2, axis=0)[:1])


@pytest.mark.skipif(not HAVE_MODELS, reason="CONVECTOR_REFERENCE (the reference checkout) not set")
@pytest.mark.parametrize("name,mats", [
    ("indoor.obj", None),
    ("suzanne.obj", {}),
    ("stanford_bunny.obj", {}),
    ("stanford_dragon.obj", {}),
])
def test_reference_models(cvx, orc, name, mats):
    """The reference's own models, loaded by the restated loader
    (wavefront.rs:83-152), in source order."""
    if mats is None:
        mats = scenes.reference_materials()
    m = cvx.Mesh.load_with_materials(os.path.join(REFERENCE, "models", name), mats)
    a = cvx.Bvh.from_meshes([m])
    src = np.empty_like(a.triangles)
    src[a.source_index] = a.triangles
    _same(cvx, orc, src)
