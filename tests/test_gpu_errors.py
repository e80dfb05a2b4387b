"""Error paths of the kernels and of device allocation, run on purpose.

The reference panics where this library returns a status: on a traversal
stack overflow (bvh.rs:594-600) and when memory runs out (main.rs:65-66).
An overflow cannot happen on a scene the library accepted (scene creation
checks the tree's depth against the stack), so these tests lower the stack's
capacity with cvx_set_traversal_stack_limit: a kernel then stops each ray
that would need more entries, sets its status word, and the call that
launched it returns CVX_ERR_DEVICE. Every stack access stays inside the
arrays' full size, so nothing faults and the context stays usable. After the
error the same handle must give the results of a handle that never failed.

Allocation failures are injected on the host (cvx_inject_allocation_failure)
at every allocation of scene, renderer, batch and server creation in turn
(a server with sample slots among them): each must return CVX_ERR_CAPACITY,
hand out no handle and leak no device memory; a renderer whose sample buffers
fail to allocate at its first multi-frame call stays usable.
"""

import contextlib

import numpy as np
import pytest

from convector_gb300 import scenes

pytestmark = pytest.mark.gpu

CVX_ERR_CAPACITY, CVX_ERR_DEVICE = 7, 6


@contextlib.contextmanager
def stack_limit(gpu, entries):
    gpu.set_traversal_stack_limit(entries)
    try:
        yield
    finally:
        gpu.set_traversal_stack_limit(0)


@pytest.fixture(scope="module")
def room(gpu):
    text, mats = scenes.room_sphere()
    sc = gpu.Scene(gpu.Bvh.from_meshes([gpu.Mesh.parse(text, mats)]))
    scenes.default_camera(sc.camera)
    return sc


def test_stack_limit_is_checked(gpu):
    for bad in (1, 129):
        with pytest.raises(gpu.CvxError) as e:
            gpu.set_traversal_stack_limit(bad)
        assert e.value.status == 1
    gpu.set_traversal_stack_limit(0)


@pytest.mark.parametrize("traversal", [0, 1])
def test_query_reports_stack_overflow(room, gpu, traversal):
    o, d = scenes.random_rays(20000, seed=31)
    t_ref, tri_ref = room.intersect_nearest(o, d, traversal=traversal)
    with stack_limit(gpu, 2):
        with pytest.raises(gpu.CvxError) as e:
            room.intersect_nearest(o, d, traversal=traversal)
    assert e.value.status == CVX_ERR_DEVICE and "overflow" in str(e.value)
    t, tri = room.intersect_nearest(o, d, traversal=traversal)
    assert (tri == tri_ref).all() and (t.view(np.uint32) == t_ref.view(np.uint32)).all()


FRAME_FORMS = {
    "octet_groups": dict(rng_order=1, traversal=1, refill_mode=2),
    "paths_per_lane": dict(rng_order=1, traversal=1, refill_mode=1),
    "packet": dict(rng_order=1, traversal=0),
    "patch_order": dict(rng_order=0, traversal=0),
    "wavefront": dict(rng_order=1, traversal=1, mode=1, use_graph=1),
    "wavefront_packet": dict(rng_order=1, traversal=0, mode=1, use_graph=1),
}


@pytest.mark.parametrize("form", sorted(FRAME_FORMS))
def test_frame_reports_stack_overflow(room, gpu, form):
    kw = FRAME_FORMS[form]
    rgba_ref, gb_ref = gpu.Renderer(room, 96, 64, **kw).render_frame_u8(42)
    r = gpu.Renderer(room, 96, 64, **kw)
    r.render_frame_u8(41)  # a wavefront renderer captures its graph here, before the limit
    with stack_limit(gpu, 2):
        with pytest.raises(gpu.CvxError) as e:
            r.render_frame_u8(42)
    assert e.value.status == CVX_ERR_DEVICE
    rgba, gb = r.render_frame_u8(42)
    assert (rgba == rgba_ref).all() and (gb == gb_ref).all()


@pytest.mark.parametrize("kw", [dict(rng_order=1, traversal=1, refill_mode=1), dict(rng_order=1, traversal=0)],
                         ids=["shared_launches", "launch_per_frame"])
def test_multi_frame_accumulation_reports_stack_overflow(room, gpu, kw):
    """cvx_accumulate_frames_f32 returns the kernel's status; after a clear
    the same renderer accumulates what a fresh one does."""
    ref = gpu.Renderer(room, 96, 64, **kw)
    ref.accumulate_frames_f32(3, 5)
    r = gpu.Renderer(room, 96, 64, **kw)
    with stack_limit(gpu, 2):
        with pytest.raises(gpu.CvxError) as e:
            r.accumulate_frames_f32(3, 5)
    assert e.value.status == CVX_ERR_DEVICE
    r.clear_accumulator()
    r.accumulate_frames_f32(3, 5)
    assert (r.read_accumulator().view(np.uint32) == ref.read_accumulator().view(np.uint32)).all()


@pytest.mark.parametrize("mode,refill", [(0, 2), (0, 1), (1, 0)])
def test_batch_reports_stack_overflow(room, gpu, mode, refill):
    """Single-launch waves with one octet per group (k_wave_fused), with paths
    per lane (k_wave_refill), and wavefront waves."""
    views = [gpu.View(0, 64, 32, 2, 10 * k, scenes.default_camera(gpu.Camera(), eye=(0.2 * k, 1.2, 1.6)))
             for k in range(3)]
    batch = gpu.Batch([room], max_groups=1 << 14, max_pixels=1 << 16, mode=mode, refill_mode=refill)
    ref, _, _ = batch.render(views)
    with stack_limit(gpu, 2):
        with pytest.raises(gpu.CvxError) as e:
            batch.render(views)
    assert e.value.status == CVX_ERR_DEVICE
    imgs, _, _ = batch.render(views)
    for a, b in zip(imgs, ref):
        assert (a == b).all()


@pytest.mark.parametrize("kernel_mode,refill,samples_per_wave", [(1, 1, 1), (2, 0, 1), (1, 1, 4)])
def test_server_request_reports_stack_overflow(room, gpu, kernel_mode, refill, samples_per_wave):
    srv = gpu.Server([room], framebuffer_bytes=16 << 20, max_groups=1 << 14, kernel_mode=kernel_mode,
                     refill_mode=refill, samples_per_wave=samples_per_wave)
    cam = scenes.default_camera(gpu.Camera())
    st, ref, _ = srv.wait(srv.submit(0, 64, 48, 2, cam, frame_base=5))
    assert st == 0
    with stack_limit(gpu, 2):
        st, img, info = srv.wait(srv.submit(0, 64, 48, 2, cam, frame_base=5))
    assert st == CVX_ERR_DEVICE and img is None
    st, img, _ = srv.wait(srv.submit(0, 64, 48, 2, cam, frame_base=5))
    assert st == 0 and (img == ref).all()
    srv.close()


def _free_bytes():
    import torch
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def _fail_each_allocation(gpu, create):
    """Runs create() with the k-th device allocation failing, k = 0, 1, ...
    until it succeeds; returns how many allocations failed it."""
    failures = 0
    try:
        for k in range(500):
            gpu.inject_allocation_failure(k)
            try:
                h = create()
            except gpu.CvxError as e:
                assert e.status == CVX_ERR_CAPACITY and "injected" in str(e), str(e)
                failures += 1
                continue
            gpu.inject_allocation_failure(-1)
            del h
            return failures
    finally:
        gpu.inject_allocation_failure(-1)
    raise AssertionError("creation never succeeded")


def test_allocation_failures_at_creation(room, gpu):
    text, mats = scenes.displaced_icosphere(subdivisions=3)
    bvh = gpu.Bvh.from_meshes([gpu.Mesh.parse(text, mats)])
    gpu.Scene(bvh)  # first use of the kernels on this path (module loads) before the baseline
    gpu.Renderer(room, 2048, 2048, rng_order=1, traversal=1).render_frame_u8(1)
    free0 = _free_bytes()
    counts = {
        "scene": _fail_each_allocation(gpu, lambda: gpu.Scene(bvh)),
        # 2048 x 2048: a leaked framebuffer set would be 134 MB
        "renderer": _fail_each_allocation(gpu, lambda: gpu.Renderer(room, 2048, 2048, rng_order=1, traversal=1)),
        "batch": _fail_each_allocation(gpu, lambda: gpu.Batch([room], max_groups=1 << 20, max_pixels=1 << 22)),
        "server": _fail_each_allocation(gpu, lambda: gpu.Server([room], framebuffer_bytes=256 << 20,
                                                                max_groups=1 << 20)),
        "server with sample slots": _fail_each_allocation(
            gpu, lambda: gpu.Server([room], framebuffer_bytes=256 << 20, max_groups=1 << 20,
                                    refill_mode=gpu.REFILL_ALL, samples_per_wave=8)),
    }
    for what, n in counts.items():
        assert n >= 3, (what, n)
    # every partial creation released what it had allocated
    assert abs(_free_bytes() - free0) < (32 << 20), counts
    # the renderer's sample buffers, allocated at its first multi-frame call
    r = gpu.Renderer(room, 256, 128, rng_order=1, traversal=1, refill_mode=1)
    gpu.inject_allocation_failure(0)
    try:
        with pytest.raises(gpu.CvxError) as e:
            r.accumulate_frames_f32(0, 4)
    finally:
        gpu.inject_allocation_failure(-1)
    assert e.value.status == CVX_ERR_CAPACITY
    r.accumulate_frames_f32(0, 4)
    ref = gpu.Renderer(room, 256, 128, rng_order=1, traversal=1, refill_mode=1)
    for f in range(4):
        ref.accumulate_frame_f32(f)
    assert (r.read_accumulator().view(np.uint32) == ref.read_accumulator().view(np.uint32)).all()
    # and the library still works
    o, d = scenes.random_rays(1000, seed=5)
    t, tri = room.intersect_nearest(o, d, traversal=1)
    assert (tri >= 0).any()
