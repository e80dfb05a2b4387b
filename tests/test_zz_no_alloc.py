"""The no-allocation nearest-hit query (cvx_intersect_nearest_noalloc).

Some callers cannot allocate device memory: a host application that manages
the GPU's memory through its own allocator and does not let plugins call
cudaMalloc, or a real-time loop that cannot afford an allocation's stall. For
them the library stages rays and hits through a static device buffer instead.
These tests call that entry point through the C-ABI and check it against the
allocating cvx_intersect_nearest, bit for bit (the tolerance every other
nearest-hit test here uses), on two calls in a row: the shared buffer keeps
the previous call's contents, and the second call must not see them.
This file is collected last on purpose.
"""

import numpy as np
import pytest

from convector_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene(gpu):
    text, mats = scenes.displaced_icosphere(subdivisions=4)
    return gpu.Scene(gpu.Bvh.from_meshes([gpu.Mesh.parse(text, mats)]))


@pytest.mark.parametrize("traversal", [0, 1])
def test_noalloc_matches_allocating_query_twice(scene, traversal):
    first = scenes.random_rays(100000, seed=21)
    second = scenes.random_rays(4097, seed=22)  # smaller: stale data from the first call would show
    for o, d in (first, second):
        t, tri = scene.intersect_nearest_noalloc(o, d, traversal=traversal)
        rt, rtri = scene.intersect_nearest(o, d, traversal=traversal)
        assert (tri == rtri).all()
        assert (t.view(np.uint32) == rt.view(np.uint32)).all()
        assert (tri >= 0).any()


def test_noalloc_rejects_more_than_its_buffer_holds(scene, gpu):
    o, d = scenes.random_rays(8, seed=1)
    big_o = np.zeros((524289, 3), np.float32)
    big_d = np.tile(d[:1], (524289, 1))
    with pytest.raises(gpu.CvxError) as e:
        scene.intersect_nearest_noalloc(big_o, big_d)
    assert e.value.status == 1 and "524288" in str(e.value)
    t, tri = scene.intersect_nearest_noalloc(o, d)  # still usable afterwards
    rt, rtri = scene.intersect_nearest(o, d)
    assert (tri == rtri).all()


def test_noalloc_leaves_device_memory_unchanged(gpu):
    """A fresh scene's first no-allocation calls change no device memory.

    The allocating query runs first with the same traversal, so the kernels'
    first launches (module loads, local-memory reservation), which any query
    pays once, happen before the measurement; the static buffer was reserved
    when the scene was created. Free device memory is then read before and
    after four no-allocation calls."""
    import torch
    text, mats = scenes.displaced_icosphere(subdivisions=3)
    sc = gpu.Scene(gpu.Bvh.from_meshes([gpu.Mesh.parse(text, mats)]))
    o, d = scenes.random_rays(20000, seed=23)
    for trav in (0, 1):
        sc.intersect_nearest(o, d, traversal=trav)
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for trav in (0, 1):
        for _ in range(2):
            sc.intersect_nearest_noalloc(o, d, traversal=trav)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
