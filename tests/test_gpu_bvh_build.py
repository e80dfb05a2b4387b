"""Device BVH build against the host build and the oracle's independent
restatement (bvh.rs:488-545): identical node
array, triangle order, source indices and statistics, on the procedural
scenes and on inputs that reach every branch of the build (the uniform split
of bvh.rs:176-201 for small nodes and as the crowded-bin fallback, ties in
the sort key, signed zeros in the bounds, the warp-built subtree sizes)."""

import numpy as np
import pytest

from convector_gb300 import scenes

pytestmark = pytest.mark.gpu

WHITE = 0x00FFFFFF


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


def _same(cvx, tris):
    """Device build == host build == the oracle's independent restatement."""
    from oracle import oracle as orc
    a = cvx.Bvh.build(tris)
    b = cvx.Bvh.build_device(tris)
    c = orc.OracleBvh(tris)
    assert np.array_equal(a.nodes, c.nodes) and np.array_equal(a.source_index, c.source_index)
    assert (a.depth, np.float32(a.avg_area_ratio).tobytes()) == (c.depth, np.float32(c.avg_area_ratio).tobytes())
    assert a.nodes.shape == b.nodes.shape
    assert np.array_equal(a.nodes, b.nodes)
    assert np.array_equal(a.triangles, b.triangles)
    assert np.array_equal(a.source_index, b.source_index)
    assert np.float32(a.avg_tris_per_leaf).tobytes() == np.float32(b.avg_tris_per_leaf).tobytes()
    assert np.float32(a.avg_area_ratio).tobytes() == np.float32(b.avg_area_ratio).tobytes()
    assert a.depth == b.depth
    return b


def test_room_sphere(gpu):
    tris, _ = scenes.room_sphere(obj=False)
    _same(gpu, tris)


def test_displaced_icosphere(gpu):
    tris, _ = scenes.displaced_icosphere(obj=False)
    _same(gpu, tris)


def test_random_walk_tube(gpu):
    tris, _ = scenes.random_walk_tube(obj=False)
    b = _same(gpu, tris)
    assert b.triangles.shape[0] == 869900


@pytest.mark.parametrize("n,seed", [(500, 3), (3000, 5), (20000, 7)])
def test_spheres_and_boxes(gpu, n, seed):
    tris, _ = scenes.spheres_and_boxes(n, seed, obj=False)
    _same(gpu, tris)


@pytest.mark.parametrize("n", [2, 3, 5, 17, 31, 32, 33, 47, 64, 65, 100, 129, 1000, 4097, 70000])
def test_random_triangles(gpu, n):
    _same(gpu, _random_tris(n, seed=n))


def test_clustered_triangles_take_the_uniform_fallback(gpu):
    """A dense cluster inside a wide spread crowds a few coordinate bins, so
    the large nodes near the root take the uniform split."""
    wide = _random_tris(300, seed=1, spread=50.0, size=0.5)
    dense = _random_tris(60000, seed=2, spread=0.2, size=0.002)
    _same(gpu, np.concatenate([wide, dense]))


def test_equal_barycentres_keep_node_order(gpu):
    """Copies of one triangle have equal sort keys: the stable order decides."""
    base = _random_tris(40, seed=9)
    copies = np.repeat(_random_tris(1, seed=10), 300, axis=0)
    _same(gpu, np.concatenate([copies[:150], base, copies[150:]]))


def test_signed_zero_bounds(gpu):
    """Bounds at +0 and -0: a node keeps the bound of its first triangle in
    node order among those at zero."""
    rng = np.random.default_rng(4)
    v = rng.uniform(0.1, 1.0, (3000, 3, 3)).astype(np.float32)
    v[:, 0, 0] = np.where(rng.random(3000) < 0.5, np.float32(0.0), np.float32(-0.0))
    v[:, 1, 1] = np.where(rng.random(3000) < 0.5, np.float32(0.0), np.float32(-0.0))
    v[::3, 2, 2] = -0.0
    _same(gpu, _tris(v))


def test_refuses_nan_and_empty(gpu):
    t = _random_tris(10, seed=1)
    t.view(np.float32)[3, 4] = np.nan
    with pytest.raises(gpu.CvxError) as e:
        gpu.Bvh.build_device(t)
    assert e.value.status == 1
    with pytest.raises(gpu.CvxError):
        gpu.Bvh.build_device(_random_tris(1, seed=1)[:0])
