"""GPU parity: the sm_103a kernels, called through the C-ABI, against the
oracle on the same scenes, rays, seeds and BVH.

Both sides compute the reference's x86 arithmetic (approximate reciprocals
from the hardware tables, explicit FMAs only), so the expected agreement is
bit-exact: hit index and t on every ray, and every RGBA, gbuffer and linear
colour value of a frame. The benchmark spec's tolerance for radiance (1e-3
absolute per pixel) is asserted as well, but the test demands equality.
"""

import numpy as np
import pytest

from convector_gb300 import scenes

pytestmark = pytest.mark.gpu

RADIANCE_TOL = 1e-3


@pytest.fixture(scope="module")
def room(gpu, orc):
    text, mats = scenes.room_sphere()
    bvh = gpu.Bvh.from_meshes([gpu.Mesh.parse(text, mats)])
    scene = gpu.Scene(bvh)
    scenes.default_camera(scene.camera)
    return bvh, scene, orc.OracleScene.from_bvh(bvh)


@pytest.fixture(scope="module")
def icosphere(gpu, orc):
    text, mats = scenes.displaced_icosphere()
    bvh = gpu.Bvh.from_meshes([gpu.Mesh.parse(text, mats)])
    assert bvh.triangles.shape[0] == 81930
    return bvh, gpu.Scene(bvh), orc.OracleScene.from_bvh(bvh)


def _edge_rays():
    """Axis-parallel directions, origins on box planes and at the origin."""
    o = np.array([[0, 1, -2], [0, 0, -1], [-2, 1, -2], [0, 2.5, -1], [1.5, 0.5, -3.9], [0, 1.1, -2],
                  [0, 0, 0], [-2, 0, -4]], np.float32)
    d = np.array([[1, 0, 0], [0, 1, 0], [1, 0, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1], [0, 1, -1], [1, 1, 1]],
                 np.float32)
    d = d / np.linalg.norm(d, axis=1, keepdims=True).astype(np.float32)
    return o, d.astype(np.float32)


@pytest.mark.parametrize("traversal", [0, 1])
def test_intersect_bitexact(icosphere, orc, traversal):
    bvh, scene, osc = icosphere
    o, d = scenes.random_rays(1 << 18, seed=7)
    eo, ed = _edge_rays()
    o, d = np.concatenate([eo, o]), np.concatenate([ed, d])
    t, tri = scene.intersect_nearest(o, d, traversal=traversal)
    ot, otri = osc.intersect(o, d, mode=traversal)
    assert (tri == otri).all(), np.nonzero(tri != otri)[0][:10]
    assert (t.view(np.uint32) == ot.view(np.uint32)).all()
    assert (tri >= 0).mean() > 0.5


@pytest.mark.parametrize("traversal", [0, 1])
def test_intersect_origins_on_box_planes_bitexact(icosphere, orc, traversal):
    """Rays starting exactly on node bound planes (zero plane distances, so
    0 * inf and signed-zero slab distances), with unit directions and with
    length-3 ones: hits equal the oracle's bit for bit."""
    bvh, scene, osc = icosphere
    rng = np.random.default_rng(31)
    nodes = bvh.nodes_f32[2:]
    pick = nodes[rng.integers(0, nodes.shape[0], 1 << 15)]
    o = rng.uniform(pick[:, 0:3], pick[:, 3:6]).astype(np.float32)
    axis = rng.integers(0, 3, o.shape[0])
    side = rng.integers(0, 2, o.shape[0])
    o[np.arange(o.shape[0]), axis] = pick[np.arange(o.shape[0]), axis + 3 * side]
    d = rng.normal(size=o.shape).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d[::4] *= np.float32(3.0)  # |d| = 3: reciprocals near 1/3
    d = d.astype(np.float32)
    t, tri = scene.intersect_nearest(o, d, traversal=traversal)
    ot, otri = osc.intersect(o, d, mode=traversal)
    assert (tri == otri).all(), np.nonzero(tri != otri)[0][:10]
    assert (t.view(np.uint32) == ot.view(np.uint32)).all()


def test_intersect_negative_zero_bounds_bitexact(gpu, orc):
    """Leaf bounds at -0 (triangles touching a coordinate plane at a -0
    vertex): the slab test's signed-zero min/max order matches the oracle's."""
    rng = np.random.default_rng(12)
    c = rng.uniform(-1.0, 1.0, (2000, 1, 3))
    v = (c + rng.normal(0.0, 0.04, (2000, 3, 3))).astype(np.float32)
    # Every fifth triangle touches the x = 0 plane from above at a -0 vertex,
    # every seventh the z = 0 plane from below: leaf bounds at -0.
    v[::5, :, 0] = np.abs(v[::5, :, 0])
    v[::5, 0, 0] = np.float32(-0.0)
    v[::7, :, 2] = -np.abs(v[::7, :, 2])
    v[::7, 1, 2] = np.float32(-0.0)
    t16 = np.zeros((2000, 16), np.float32)
    t16[:, :9] = v.reshape(-1, 9)
    w = t16.view(np.uint32)
    w[:, 15] = 0x00FFFFFF
    bvh = gpu.Bvh.build(w)
    scene = gpu.Scene(bvh)
    osc = orc.OracleScene.from_bvh(bvh)
    o, d = scenes.random_rays(1 << 14, seed=3)
    o = (o * np.float32(0.3)).astype(np.float32)
    t, tri = scene.intersect_nearest(o, d, traversal=1)
    ot, otri = osc.intersect(o, d, mode=1)
    assert (tri == otri).all() and (t.view(np.uint32) == ot.view(np.uint32)).all()


@pytest.mark.parametrize("traversal", [0, 1])
def test_intersect_host_access_modes_agree(gpu, icosphere, orc, traversal):
    """The host-buffer query reading the caller's arrays in place (where the
    device shares the host's page tables) and copying them first give the same
    hits, bit for bit, over several chunks with a ragged last one; a sample
    equals the oracle."""
    bvh, scene, osc = icosphere
    n = 3 * (1 << 19) + 123
    o, d = scenes.random_rays(n, seed=17)
    res = {}
    try:
        for mode in (gpu.HOST_ACCESS_COPY, gpu.HOST_ACCESS_AUTO):
            scene.set_host_access(mode)
            res[mode] = scene.intersect_nearest(o, d, traversal=traversal)
    finally:
        scene.set_host_access(gpu.HOST_ACCESS_AUTO)
    (tc, ic), (ta, ia) = res[gpu.HOST_ACCESS_COPY], res[gpu.HOST_ACCESS_AUTO]
    assert (ic == ia).all() and (tc.view(np.uint32) == ta.view(np.uint32)).all()
    pick = np.r_[0:4096, n - 4096:n]
    ot, otri = osc.intersect(o[pick], d[pick], mode=traversal)
    assert (ia[pick] == otri).all() and (ta[pick].view(np.uint32) == ot.view(np.uint32)).all()


def test_intersect_host_access_pinned_buffers(gpu, icosphere):
    """Page-locked host buffers (as an application's staging memory) through
    the C-ABI: in place and copied agree."""
    torch = pytest.importorskip("torch")
    import ctypes
    bvh, scene, osc = icosphere
    n = (1 << 20) + 77
    o, d = scenes.random_rays(n, seed=19)
    cols = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in
            (o[:, 0], o[:, 1], o[:, 2], d[:, 0], d[:, 1], d[:, 2])]
    out = {}
    try:
        for mode in (gpu.HOST_ACCESS_COPY, gpu.HOST_ACCESS_AUTO):
            scene.set_host_access(mode)
            t = torch.empty(n, dtype=torch.float32).pin_memory()
            tri = torch.empty(n, dtype=torch.int32).pin_memory()
            gpu._check(gpu.lib().cvx_intersect_nearest(scene._h, *[ctypes.c_void_p(c.data_ptr()) for c in cols], n,
                                                       1.0e5, 1, ctypes.c_void_p(t.data_ptr()),
                                                       ctypes.c_void_p(tri.data_ptr())))
            out[mode] = (t.numpy().copy(), tri.numpy().copy())
    finally:
        scene.set_host_access(gpu.HOST_ACCESS_AUTO)
    assert (out[0][1] == out[1][1]).all() and (out[0][0].view(np.uint32) == out[1][0].view(np.uint32)).all()
    ref_t, ref_tri = scene.intersect_nearest(o, d, traversal=1)
    assert (out[1][1] == ref_tri).all()


def test_host_access_rejects_bad_mode(gpu, icosphere):
    with pytest.raises(gpu.CvxError):
        icosphere[1].set_host_access(7)


def test_large_leaves_escape_bitexact(gpu, orc):
    """Leaves of 31 or more triangles are stored as escape slots below the node
    pairs. Coincident triangles share one barycentre and end in one leaf (300 and
    40 of them among 2,000 random ones): hits through both traversals, with rays
    aimed into those leaves and axis-parallel rays (the deferred x86-form pass),
    equal the oracle's."""
    rng = np.random.default_rng(21)
    c = rng.uniform(-1.0, 1.0, (2000, 1, 3))
    v = c + rng.normal(0.0, 0.05, (2000, 3, 3))
    big = np.repeat(np.array([[[0.1, 0.2, 0.3], [0.4, 0.2, 0.3], [0.1, 0.6, 0.35]]]), 300, axis=0)
    mid = np.repeat(np.array([[[-0.5, -0.4, 0.2], [-0.2, -0.4, 0.25], [-0.5, -0.1, 0.2]]]), 40, axis=0)
    v = np.concatenate([v[:1000], big, v[1000:], mid]).astype(np.float32)
    t16 = np.zeros((v.shape[0], 16), np.float32)
    t16[:, :9] = v.reshape(-1, 9)
    w = t16.view(np.uint32)
    w[:, 15] = 0x00FFFFFF
    bvh = gpu.Bvh.build(w)
    lens = bvh.nodes.view(np.uint32).reshape(-1, 8)[:, 7]
    assert (lens >= 31).sum() >= 2, "the scene must hold escaped leaves"
    scene = gpu.Scene(bvh)
    osc = orc.OracleScene.from_bvh(bvh)
    n = 1 << 14
    o = rng.uniform(-1.5, 1.5, (n, 3)).astype(np.float32)
    targets = np.where(rng.random((n, 1)) < 0.5, big[0].mean(0), mid[0].mean(0))
    d = np.where(rng.random((n, 1)) < 0.6, targets - o, rng.normal(size=(n, 3)))
    d[:64] = np.eye(3)[rng.integers(0, 3, 64)] * np.sign(rng.normal(size=(64, 1)))  # axis-parallel
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    for traversal in (0, 1):
        t, tri = scene.intersect_nearest(o, d, traversal=traversal)
        ot, otri = osc.intersect(o, d, mode=traversal)
        assert (tri == otri).all(), np.nonzero(tri != otri)[0][:10]
        assert (t.view(np.uint32) == ot.view(np.uint32)).all()
        coincident = np.nonzero(np.abs(bvh.triangles.view(np.float32)[:, :9] - big[0].reshape(9)).max(1) < 1e-6)[0]
        assert np.isin(tri, coincident).any()  # rays reached the escaped leaves


@pytest.mark.parametrize("launch", [8, 10, 12])
def test_intersect_single_launch_shapes_bitexact(icosphere, orc, launch):
    """Every launch shape of the single-ray query (occupancy variants of the
    staged ray supply) returns the oracle's results, ragged tail included."""
    bvh, scene, osc = icosphere
    o, d = scenes.random_rays((1 << 17) + 45, seed=19)
    ot, otri = osc.intersect(o, d, mode=1)
    scene.set_query_launch(launch)
    try:
        t, tri = scene.intersect_nearest(o, d, traversal=1)
    finally:
        scene.set_query_launch(0)
    assert (tri == otri).all(), np.nonzero(tri != otri)[0][:10]
    assert (t.view(np.uint32) == ot.view(np.uint32)).all()


@pytest.mark.parametrize("stack", [0, 4, 12])
def test_intersect_single_stack_depths_bitexact(icosphere, orc, stack):
    """Every shared-memory stack depth of the single-ray query (the query
    autotuner's stack knob) returns the oracle's results."""
    bvh, scene, osc = icosphere
    o, d = scenes.random_rays((1 << 17) + 45, seed=23)
    ot, otri = osc.intersect(o, d, mode=1)
    scene.set_query_stack(stack)
    try:
        t, tri = scene.intersect_nearest(o, d, traversal=1)
    finally:
        scene.set_query_stack(8)
    assert (tri == otri).all(), np.nonzero(tri != otri)[0][:10]
    assert (t.view(np.uint32) == ot.view(np.uint32)).all()


def test_query_autotuner_picks_and_keeps_a_configuration(icosphere, gpu):
    import torch
    from convector_gb300 import autotune
    bvh, scene, osc = icosphere
    o, d = scenes.random_rays(1 << 18, seed=29)
    rays = torch.from_numpy(np.concatenate([o.T, d.T]).copy()).cuda()
    t = torch.empty(o.shape[0], dtype=torch.float32, device="cuda")
    tri = torch.empty(o.shape[0], dtype=torch.int32, device="cuda")
    try:
        best, table = autotune.tune_query(scene, rays, t, tri)
        assert set(table) == {q[0] for q in autotune.QUERY_SHAPES} and best in table
        assert all(ms > 0 for ms in table.values())
        ref_t, ref_tri = scene.intersect_nearest(o, d, traversal=autotune.query_traversal(best))
        scene.intersect_nearest_device(rays, t, tri, traversal=autotune.query_traversal(best))
        torch.cuda.synchronize()
        assert (tri.cpu().numpy() == ref_tri).all()
        with pytest.raises(gpu.CvxError):
            scene.set_query_stack(6)
    finally:
        scene.set_query_launch(0)
        scene.set_query_stack(8)


def test_intersect_deep_tree_bitexact(gpu, orc):
    """A 70-level tree (the 870k-triangle tube) takes the deep-tree launch of
    the single-ray query; results equal the oracle's on rays from the camera
    position into the tube and on random rays in the room."""
    tris, _ = scenes.random_walk_tube(obj=False)
    bvh = gpu.Bvh.build_device(tris)
    assert bvh.depth > 40
    scene = gpu.Scene(bvh)
    osc = orc.OracleScene.from_bvh(bvh)
    o, d = scenes.random_rays(1 << 16, seed=29)
    eye = np.broadcast_to(np.array([0.0, 1.2, 1.6], np.float32), (4096, 3))
    rng = np.random.default_rng(5)
    dc = np.stack([rng.uniform(-0.6, 0.6, 4096), rng.uniform(-0.4, 0.3, 4096), -np.ones(4096)], 1)
    dc = (dc / np.linalg.norm(dc, axis=1, keepdims=True)).astype(np.float32)
    o, d = np.concatenate([eye, o]).astype(np.float32), np.concatenate([dc, d]).astype(np.float32)
    t, tri = scene.intersect_nearest(o, d, traversal=1)
    ot, otri = osc.intersect(o, d, mode=1)
    assert (tri == otri).all(), np.nonzero(tri != otri)[0][:10]
    assert (t.view(np.uint32) == ot.view(np.uint32)).all()
    assert (tri >= 0).mean() > 0.5


@pytest.mark.parametrize("traversal", [0, 1])
def test_intersect_host_pipeline_equals_device_query(icosphere, traversal):
    """The host-buffer query cuts large batches into chunks on several
    streams; its results equal the one-launch device query, ragged end included."""
    import torch
    bvh, scene, _ = icosphere
    n = (1 << 21) + 77
    o, d = scenes.random_rays(n, seed=23)
    t, tri = scene.intersect_nearest(o, d, traversal=traversal)
    rays = torch.from_numpy(np.concatenate([o.T, d.T]).copy()).cuda()
    td = torch.empty(n, dtype=torch.float32, device="cuda")
    trd = torch.empty(n, dtype=torch.int32, device="cuda")
    scene.intersect_nearest_device(rays, td, trd, traversal=traversal)
    torch.cuda.synchronize()
    assert (tri == trd.cpu().numpy()).all()
    assert (t.view(np.uint32) == td.cpu().numpy().view(np.uint32)).all()


@pytest.mark.parametrize("traversal", [0, 1])
def test_intersect_counters_match_reference_debug_counts(icosphere, orc, traversal):
    """Box and triangle counts per packet (bvh.rs:604-651, the debug view) or per ray."""
    import torch
    bvh, scene, osc = icosphere
    o, d = scenes.random_rays(1 << 14, seed=3)
    _, _, na, nt = osc.intersect(o, d, mode=traversal, counters=True)
    rays = torch.from_numpy(np.concatenate([o.T, d.T]).copy()).cuda()
    n = o.shape[0]
    t = torch.empty(n, dtype=torch.float32, device="cuda")
    tri = torch.empty(n, dtype=torch.int32, device="cuda")
    cnt = torch.empty(2 * n, dtype=torch.int32, device="cuda")
    scene.intersect_nearest_device(rays, t, tri, traversal=traversal, counters=cnt)
    torch.cuda.synchronize()
    c = cnt.cpu().numpy().view(np.uint32)
    assert (c[:n] == na).all() and (c[n:] == nt).all()


@pytest.mark.parametrize("n", [0, 1, 7, 13, 4097])
def test_intersect_ragged_sizes(icosphere, orc, n):
    bvh, scene, osc = icosphere
    o, d = scenes.random_rays(max(n, 1), seed=11)
    o, d = o[:n], d[:n]
    t, tri = scene.intersect_nearest(o, d)
    assert t.shape == (n,)
    if n:
        ot, otri = osc.intersect(o, d)
        assert (tri == otri).all() and (t.view(np.uint32) == ot.view(np.uint32)).all()


def test_intersect_far_distance_culls_everything(icosphere):
    bvh, scene, _ = icosphere
    o, d = scenes.random_rays(4096, seed=5)
    t, tri = scene.intersect_nearest(o, d, far=1e-7)
    assert (tri == -1).all() and (t == np.float32(1e-7)).all()


def _render_both(gpu, orc, scene, osc, w, h, frame, rng_order, traversal):
    r = gpu.Renderer(scene, w, h, rng_order=rng_order, traversal=traversal)
    rgba, gb = r.render_frame_u8(frame)
    col = r.read_frame_f32()
    rays, ms = r.stats()
    orgba, ogb, ocol, orays = osc.render(scene.camera.as_array(), w, h, frame, rng_order=rng_order,
                                         traversal=traversal)
    return (rgba, gb, col, rays), (orgba, ogb, ocol, orays)


@pytest.mark.parametrize("traversal", [0, 1])
def test_render_patches_all_equal_frame(room, gpu, traversal):
    """Every 32x32 patch through the patch entry (one call) gives the frame of
    the reference patch order."""
    bvh, scene, osc = room
    w, h = 160, 96
    r = gpu.Renderer(scene, w, h, rng_order=gpu.RNG_PATCH, traversal=traversal)
    rgba, gb = r.render_frame_u8(42)
    origins = [(x, y) for x in range(0, w, 32) for y in range(0, h, 32)]
    prgba, pgb = r.render_patches_u8(32, origins, 42)
    assert (prgba == rgba).all() and (pgb == gb).all()


@pytest.mark.parametrize("patch_width", [16, 64])
def test_render_patches_bitexact_and_local(room, gpu, orc, patch_width):
    """Patches of other widths, some crossing the frame edge, equal the
    oracle's; pixels outside the listed patches keep the caller's values."""
    bvh, scene, osc = room
    w, h = 150, 90
    r = gpu.Renderer(scene, w, h, rng_order=gpu.RNG_GROUP, traversal=gpu.TRAVERSE_PACKET)
    origins = [(0, 0), (patch_width, 4 * 3), (144, 88), (96, 40)]
    sentinel = np.uint32(0xDEADBEEF)
    rgba = np.full((h, w), sentinel, np.uint32)
    gb = np.full((h, w), sentinel, np.uint32)
    r.render_patches_u8(patch_width, origins, 7, rgba, gb)
    orgba = np.full((h, w), sentinel, np.uint32)
    ogb = np.full((h, w), sentinel, np.uint32)
    osc.render_patches(scene.camera.as_array(), w, h, 7, patch_width, origins, traversal=0, rgba=orgba, gbuf=ogb)
    assert (rgba == orgba).all() and (gb == ogb).all()
    assert (rgba == sentinel).any() and (rgba != sentinel).any()


def test_accumulate_patches_equal_frames(room, gpu):
    bvh, scene, osc = room
    w, h = 96, 64
    origins = [(x, y) for x in range(0, w, 32) for y in range(0, h, 32)]
    a = gpu.Renderer(scene, w, h, rng_order=gpu.RNG_PATCH, traversal=gpu.TRAVERSE_PACKET)
    b = gpu.Renderer(scene, w, h, rng_order=gpu.RNG_PATCH, traversal=gpu.TRAVERSE_PACKET)
    for f in (5, 6, 7):
        a.accumulate_frame_f32(f)
        b.accumulate_patches_f32(32, origins, f)
    assert (a.resolve_u8(3) == b.resolve_u8(3)).all()


def test_render_patches_refuses_bad_arguments(room, gpu):
    bvh, scene, osc = room
    r = gpu.Renderer(scene, 64, 64, rng_order=gpu.RNG_PATCH, traversal=gpu.TRAVERSE_PACKET)
    for pw, xy in ((24, [(0, 0)]), (32, [(8, 0)]), (32, [(0, 2)]), (32, [(64, 0)])):
        with pytest.raises(gpu.CvxError) as e:
            r.render_patches_u8(pw, xy, 1)
        assert e.value.status == 1


def test_render_after_update_scene_bitexact(room, gpu, orc):
    """Renderer::set_time + update_scene (renderer.rs:134-147) move the camera
    with a per-frame delta (motion blur); the frame equals the oracle's with
    the same camera."""
    bvh, scene, osc = room
    r = gpu.Renderer(scene, 160, 96, rng_order=gpu.RNG_PATCH, traversal=gpu.TRAVERSE_PACKET)
    r.set_time(7.25, 0.04)
    r.update_scene()
    rgba, gb = r.render_frame_u8(42)
    cam = gpu.Camera().set_interactive(7.25, 0.04)
    orgba, ogb, _, _ = osc.render(cam.as_array(), 160, 96, 42, rng_order=0, traversal=0)
    assert (rgba == orgba).all() and (gb == ogb).all()
    still = gpu.Renderer(scene, 160, 96, rng_order=gpu.RNG_PATCH, traversal=gpu.TRAVERSE_PACKET)
    still.set_camera(gpu.Camera().set_interactive(7.25, 0.0))
    assert not (still.render_frame_u8(42)[0] == rgba).all()  # the delta blurs the frame


@pytest.mark.parametrize("rng_order", [0, 1])
@pytest.mark.parametrize("traversal", [0, 1])
def test_render_small_bitexact(room, gpu, orc, rng_order, traversal):
    bvh, scene, osc = room
    (rgba, gb, col, rays), (orgba, ogb, ocol, orays) = _render_both(gpu, orc, scene, osc, 160, 96, 42, rng_order,
                                                                    traversal)
    assert np.abs(col - ocol).max() <= RADIANCE_TOL
    assert (col.view(np.uint32) == ocol.view(np.uint32)).all()
    assert (rgba == orgba).all() and (gb == ogb).all()
    assert rays == orays


@pytest.mark.parametrize("rng_order", [0, 1])
def test_render_full_frame_bitexact(room, gpu, orc, rng_order):
    """The interactive configuration: 1280x736, 1 spp, 5 bounces, frame 42."""
    bvh, scene, osc = room
    (rgba, gb, col, rays), (orgba, ogb, ocol, orays) = _render_both(gpu, orc, scene, osc, 1280, 736, 42, rng_order,
                                                                    0)
    assert (col.view(np.uint32) == ocol.view(np.uint32)).all()
    assert (rgba == orgba).all() and (gb == ogb).all()
    assert rays == orays and rays > 1280 * 736


@pytest.mark.parametrize("w,h", [(1, 1), (7, 3), (100, 50), (33, 17)])
def test_render_ragged_sizes_pad_and_crop(room, gpu, orc, w, h):
    bvh, scene, osc = room
    for order in (0, 1):
        (rgba, gb, col, rays), (orgba, ogb, ocol, orays) = _render_both(gpu, orc, scene, osc, w, h, 7, order, 0)
        assert (rgba == orgba).all() and (gb == ogb).all() and rays == orays


def _render_refill_forms(gpu, scene, cam, w, h, frame, accumulate=0):
    """The single-launch single-ray frame in its two forms: per-lane path
    refill (REFILL_ALL) and one octet per 8-pixel group (REFILL_NONE)."""
    out = {}
    for refill in (gpu.REFILL_ALL, gpu.REFILL_NONE):
        r = gpu.Renderer(scene, w, h, rng_order=gpu.RNG_GROUP, traversal=gpu.TRAVERSE_SINGLE, refill_mode=refill)
        r.set_camera(cam)
        if accumulate:
            for s in range(accumulate):
                r.accumulate_frame_f32(frame + s)
            out[refill] = (r.read_accumulator(), None, None, r.stats()[0])
        else:
            rgba, gb = r.render_frame_u8(frame)
            out[refill] = (rgba, gb, r.read_frame_f32(), r.stats()[0])
    return out


@pytest.mark.parametrize("eye,target,kind", [
    ((0.0, 1.25, 1.0), (0.0, 1.25, 5.0), "sky"),
    ((1.9, 1.25, 0.5), (3.5, 1.25, -1.5), "wall and sky"),
    ((0.0, 0.8, -2.0), (0.05, 2.5, -2.05), "ceiling light"),
])
def test_refill_frame_emitter_groups_bitexact(room, gpu, orc, eye, target, kind):
    """Per-lane path refill against the oracle where whole 8-pixel groups hit
    an emitter (the sky or the ceiling light) at bounce 0: the reference exits
    such a group before taking its gbuffer values (words 0), while mixed groups
    keep each lane's own word. Every output equals the oracle's and the
    octet-group form's."""
    bvh, scene, osc = room
    cam = scenes.default_camera(gpu.Camera(), eye=eye, target=target)
    w, h = 160, 96
    out = _render_refill_forms(gpu, scene, cam, w, h, 42)
    orgba, ogb, ocol, orays = osc.render(cam.as_array(), w, h, 42, rng_order=1, traversal=1)
    for rgba, gb, col, rays in out.values():
        assert (rgba == orgba).all() and (gb == ogb).all() and rays == orays
        assert (col.view(np.uint32) == ocol.view(np.uint32)).all()
    if kind == "sky":
        assert (ogb == 0).all()
    else:
        assert (ogb == 0).any() and (ogb != 0).any()


def test_refill_full_frame_bitexact(room, gpu, orc):
    """The interactive configuration (1280x736, 1 spp, frame 42) in the
    per-lane path refill form against the oracle's single-ray frame."""
    bvh, scene, osc = room
    out = _render_refill_forms(gpu, scene, scene.camera, 1280, 736, 42)
    orgba, ogb, ocol, orays = osc.render(scene.camera.as_array(), 1280, 736, 42, rng_order=1, traversal=1)
    rgba, gb, col, rays = out[gpu.REFILL_ALL]
    assert (col.view(np.uint32) == ocol.view(np.uint32)).all()
    assert (rgba == orgba).all() and (gb == ogb).all() and rays == orays
    for a, b in zip(out[gpu.REFILL_ALL][:3], out[gpu.REFILL_NONE][:3]):
        assert (a.view(np.uint32) == b.view(np.uint32)).all()


@pytest.mark.parametrize("w,h", [(1, 1), (7, 3), (100, 50), (33, 17)])
def test_refill_ragged_sizes(room, gpu, orc, w, h):
    """Groups partly outside the frame still trace all 8 lanes (ray count and
    the bounce-0 emitter rule see them) but store only pixels inside."""
    bvh, scene, osc = room
    out = _render_refill_forms(gpu, scene, scene.camera, w, h, 7)
    orgba, ogb, ocol, orays = osc.render(scene.camera.as_array(), w, h, 7, rng_order=1, traversal=1)
    for rgba, gb, col, rays in out.values():
        assert (rgba == orgba).all() and (gb == ogb).all() and rays == orays


def test_refill_accumulate_bitexact(room, gpu, orc):
    bvh, scene, osc = room
    w, h, n = 128, 64, 3
    out = _render_refill_forms(gpu, scene, scene.camera, w, h, 42, accumulate=n)
    acc = np.zeros((h, w, 3), np.float32)
    for s in range(n):
        osc.render(scene.camera.as_array(), w, h, 42 + s, rng_order=1, traversal=1, color=False, accum=acc)
    for a, *_ in out.values():
        assert (a.view(np.uint32) == acc.view(np.uint32)).all()


def test_refill_matches_octet_groups_on_larger_scenes(gpu):
    """Path refill against the octet-group form on the 82k-triangle scene
    (claim threshold 16) and on the 70-level tube (threshold 8): the same
    frame bit for bit."""
    tube_tris, _ = scenes.random_walk_tube(obj=False)
    tube = gpu.Scene(gpu.Bvh.build(tube_tris))
    assert tube.bvh.depth > 40
    ico_tris, _ = scenes.displaced_icosphere(obj=False, light=True)
    ico = gpu.Scene(gpu.Bvh.build(ico_tris))
    for sc in (ico, tube):
        cam = scenes.default_camera(gpu.Camera())
        out = _render_refill_forms(gpu, sc, cam, 320, 184, 5)
        for a, b in zip(out[gpu.REFILL_ALL][:3], out[gpu.REFILL_NONE][:3]):
            assert (a.view(np.uint32) == b.view(np.uint32)).all()
        assert out[gpu.REFILL_ALL][3] == out[gpu.REFILL_NONE][3]


def test_accumulate_and_resolve(room, gpu, orc):
    bvh, scene, osc = room
    w, h, n = 128, 64, 4
    r = gpu.Renderer(scene, w, h, rng_order=0)
    acc = np.zeros((h, w, 3), np.float32)
    for s in range(n):
        r.accumulate_frame_f32(42 + s)
        osc.render(scene.camera.as_array(), w, h, 42 + s, rng_order=0, color=False, accum=acc)
    assert (r.read_accumulator().view(np.uint32) == acc.view(np.uint32)).all()
    assert (r.resolve_u8(n) == orc.resolve(acc, n)).all()
    r.clear_accumulator()
    assert (r.read_accumulator() == 0).all()


def test_reference_light_pick_with_eight_lights(gpu, orc):
    """scene.rs:159 picks a light with `bits >> 29`, which needs exactly 8
    direct-sample triangles: a ceiling light split into 8 triangles."""
    text, mats = scenes.room_sphere()
    lines = [ln for ln in text.splitlines()]
    # replace the 2-triangle light by a fan of 8 triangles around its centre
    cut = max(i for i, ln in enumerate(lines) if ln == "usemtl glass")
    nv = sum(1 for ln in lines[:cut] if ln.startswith("v "))
    y = 2.49
    ring = [(-0.5, -2.5), (0.0, -2.5), (0.5, -2.5), (0.5, -2.0), (0.5, -1.5), (0.0, -1.5), (-0.5, -1.5), (-0.5, -2.0)]
    extra = ["usemtl glass", "v 0 %g -2" % y] + ["v %g %g %g" % (x, y, z) for x, z in ring]
    extra += ["f %d %d %d" % (nv + 1, nv + 2 + k, nv + 2 + (k + 1) % 8) for k in range(8)]
    text8 = "\n".join(lines[:cut] + extra) + "\n"
    bvh = gpu.Bvh.from_meshes([gpu.Mesh.parse(text8, mats)])
    assert bvh.direct_sample.shape[0] == 8
    scene = gpu.Scene(bvh, light_pick=0)
    scenes.default_camera(scene.camera)
    osc = orc.OracleScene.from_bvh(bvh, general_pick=False)
    (rgba, gb, col, rays), (orgba, ogb, ocol, orays) = _render_both(gpu, orc, scene, osc, 160, 96, 42, 0, 0)
    assert (col.view(np.uint32) == ocol.view(np.uint32)).all() and rays == orays


def test_device_info(gpu):
    import torch
    ordinal, name = gpu.device_info()
    assert ordinal == torch.cuda.current_device()
    assert isinstance(name, str) and name
