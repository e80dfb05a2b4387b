"""Wavefront form, batching and serving on the GPU.

The wavefront kernels must give the same bits as the oracle (per-group RNG
order); a view rendered in a batch or served in a mix must give the same
image as the same view rendered alone; the server's admission, cancellation
and timeouts are exercised on the host side of its request loop.
"""

import time

import numpy as np
import pytest

from convector_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def two_scenes(gpu, orc):
    out = []
    for text, mats in (scenes.room_sphere(), scenes.spheres_and_boxes(3000, seed=5)):
        bvh = gpu.Bvh.from_meshes([gpu.Mesh.parse(text, mats)])
        sc = gpu.Scene(bvh)
        scenes.default_camera(sc.camera)
        out.append((bvh, sc, orc.OracleScene.from_bvh(bvh)))
    return out


@pytest.mark.parametrize("traversal,refill_mode", [(0, 0), (1, 0), (1, 1), (1, 2)])
@pytest.mark.parametrize("use_graph", [0, 1])
def test_wavefront_frame_bitexact(two_scenes, gpu, orc, traversal, refill_mode, use_graph):
    bvh, scene, osc = two_scenes[0]
    w, h = 200, 120
    r = gpu.Renderer(scene, w, h, rng_order=gpu.RNG_GROUP, traversal=traversal, mode=gpu.MODE_WAVEFRONT,
                     use_graph=use_graph, refill_mode=refill_mode, blocks_per_sm=4 + 4 * refill_mode)
    for frame in (42, 43):
        rgba, gb = r.render_frame_u8(frame)
        col = r.read_frame_f32()
        orgba, ogb, ocol, orays = osc.render(scene.camera.as_array(), w, h, frame, rng_order=1, traversal=traversal)
        assert (col.view(np.uint32) == ocol.view(np.uint32)).all()
        assert (rgba == orgba).all() and (gb == ogb).all()
        assert r.stats()[0] == orays


def test_wavefront_matches_megakernel_full_frame(two_scenes, gpu):
    bvh, scene, osc = two_scenes[0]
    a = gpu.Renderer(scene, 1280, 736, rng_order=gpu.RNG_GROUP, traversal=1)
    b = gpu.Renderer(scene, 1280, 736, rng_order=gpu.RNG_GROUP, traversal=1, mode=gpu.MODE_WAVEFRONT, use_graph=1)
    ra, ga = a.render_frame_u8(42)
    rb, gb = b.render_frame_u8(42)
    assert (ra == rb).all() and (ga == gb).all()
    assert a.stats()[0] == b.stats()[0]


def test_wavefront_rejects_patch_order(two_scenes, gpu):
    bvh, scene, osc = two_scenes[0]
    with pytest.raises(gpu.CvxError):
        gpu.Renderer(scene, 64, 64, rng_order=gpu.RNG_PATCH, mode=gpu.MODE_WAVEFRONT)


def _alone(gpu, scene, view, rays=None):
    r = gpu.Renderer(scene, view.width, view.height, rng_order=gpu.RNG_GROUP, traversal=1)
    r.set_camera(view.camera)
    n = 0
    for s in range(view.spp):
        r.accumulate_frame_f32(view.frame_base + s)
        n += r.stats()[0]
    if rays is not None:
        rays.append(n)
    return r.resolve_u8(view.spp)


@pytest.mark.parametrize("mode,refill", [("fused", 0), ("fused", 1), ("wavefront", 0), ("mixed", 0), ("mixed", 1)])
def test_batch_images_equal_alone(two_scenes, gpu, orc, mode, refill):
    """refill 1 (REFILL_ALL): the single-launch waves take paths per lane
    (k_wave_refill); 0: these shallow scenes keep one octet per group."""
    scs = [s for _, s, _ in two_scenes]
    views = []
    for i, (w, h, spp) in enumerate([(160, 96, 2), (33, 17, 3), (96, 64, 1), (320, 184, 4)]):
        cam = gpu.Camera()
        scenes.default_camera(cam, eye=(0.3 * i, 1.2, 1.6))
        views.append(gpu.View(i % 2, w, h, spp, 100 * i, cam))
    m = {"fused": gpu.MODE_MEGAKERNEL, "wavefront": gpu.MODE_WAVEFRONT, "mixed": gpu.MODE_MEGAKERNEL}[mode]
    batch = gpu.Batch(scs, max_groups=1 << 16, max_pixels=1 << 20, mode=m, refill_mode=refill)
    if mode == "mixed":  # scene 1 through the wavefront kernels, scene 0 fused, in the same waves
        gpu.lib().cvx_batch_set_scene_mode(batch._h, 1, 1)
    imgs, rays, ms = batch.render(views)
    assert rays > 0
    for v, img in zip(views, imgs):
        assert (img == _alone(gpu, scs[v.scene], v)).all()
    # and against the oracle for one view
    v = views[1]
    acc = np.zeros((v.height, v.width, 3), np.float32)
    osc = two_scenes[v.scene][2]
    for s in range(v.spp):
        osc.render(v.camera.as_array(), v.width, v.height, v.frame_base + s, rng_order=1, traversal=1, color=False,
                   accum=acc)
    assert (imgs[1] == orc.resolve(acc, v.spp)).all()


def test_batch_splits_waves_when_queue_is_small(two_scenes, gpu):
    scs = [s for _, s, _ in two_scenes]
    views = [gpu.View(k % 2, 128, 64, 2, 7 * k, scenes.default_camera(gpu.Camera())) for k in range(6)]
    big, _, _ = gpu.Batch(scs, max_groups=1 << 16, max_pixels=1 << 20).render(views)
    small, _, _ = gpu.Batch(scs, max_groups=1100, max_pixels=1 << 20).render(views)
    for a, b in zip(big, small):
        assert (a == b).all()


@pytest.mark.parametrize("kernel_mode,refill", [(1, 0), (1, 1), (2, 0)])
def test_server_mix_equals_alone(two_scenes, gpu, kernel_mode, refill):
    """All requests in single-launch waves (kernel_mode 1; with REFILL_ALL as
    paths per lane, whose ray counts per request are kept per lane and per job)
    or in wavefront waves (2): each image and ray count equals the request
    rendered alone."""
    scs = [s for _, s, _ in two_scenes]
    rng = np.random.default_rng(4)
    reqs = []
    for k in range(12):
        cam = gpu.Camera()
        scenes.default_camera(cam, eye=(rng.uniform(-1, 1), 1.2, 1.6))
        reqs.append((int(k % 2), int(rng.choice([64, 100, 160])), int(rng.choice([32, 50, 96])),
                     int(rng.integers(1, 5)), cam))
    for sequential in (False, True):
        srv = gpu.Server(scs, framebuffer_bytes=64 << 20, max_groups=1 << 14, sequential=sequential,
                         kernel_mode=kernel_mode, refill_mode=refill)
        ids = []
        for i, (sc, w, h, spp, cam) in enumerate(reqs):
            ids.append(srv.submit(sc, w, h, spp, cam, frame_base=10 * i))
            time.sleep(0.002)
        for i, rid in enumerate(ids):
            st, img, info = srv.wait(rid)
            assert st == 0 and info["done_s"] >= info["start_s"] >= info["submit_s"]
            sc, w, h, spp, cam = reqs[i]
            rays = []
            assert (img == _alone(gpu, scs[sc], gpu.View(sc, w, h, spp, 10 * i, cam), rays)).all()
            assert info["rays"] == rays[0]
        assert srv.stats()["waves"] > 0
        srv.close()


@pytest.mark.parametrize("deep_single_launch", [0, 1])
@pytest.mark.parametrize("wavefront_streams", [1, 2])
def test_server_two_engines_concurrent_equal_alone(two_scenes, gpu, wavefront_streams, deep_single_launch):
    """One scene in single-launch waves and one on the deep-scene engines
    (wavefront waves, or with deep_single_launch single-launch waves with paths
    per lane), run concurrently on their streams (the deep ones at higher
    priority) with a reduced single-launch block count: every image equals the
    same request rendered alone, and both engine kinds report device time."""
    scs = [s for _, s, _ in two_scenes]
    srv = gpu.Server(scs, framebuffer_bytes=64 << 20, max_groups=1 << 14, fused_blocks_per_sm=4,
                     blocks_per_sm=10, refill_mode=gpu.REFILL_ALL, wavefront_streams=wavefront_streams,
                     deep_single_launch=deep_single_launch)
    srv.set_scene_mode(0, gpu.MODE_MEGAKERNEL if wavefront_streams == 1 else gpu.MODE_WAVEFRONT)
    srv.set_scene_mode(1, gpu.MODE_WAVEFRONT)
    rng = np.random.default_rng(8)
    reqs, ids = [], []
    for k in range(10):
        cam = gpu.Camera()
        scenes.default_camera(cam, eye=(rng.uniform(-1, 1), 1.2, 1.6))
        reqs.append((k % 2, int(rng.choice([64, 96])), int(rng.choice([40, 64])), int(rng.integers(1, 4)), cam))
    for i, (sc, w, h, spp, cam) in enumerate(reqs):
        ids.append(srv.submit(sc, w, h, spp, cam, frame_base=7 * i))
    for i, rid in enumerate(ids):
        st, img, _ = srv.wait(rid)
        sc, w, h, spp, cam = reqs[i]
        assert st == 0
        assert (img == _alone(gpu, scs[sc], gpu.View(sc, w, h, spp, 7 * i, cam))).all()
    stats = srv.stats()
    assert stats["wavefront_busy_s"] > 0.0
    assert (stats["fused_busy_s"] > 0.0) == (wavefront_streams == 1)
    srv.close()


@pytest.mark.parametrize("samples_per_wave,slot_bytes,cap,two_engines,max_groups", [
    (16, 0, 0, False, 1 << 14),
    (4, 100 * 96 * 12 * 2, 0, False, 1 << 14),  # slots for two extra samples of the largest request per wave
    (16, 0, 64 * 50, False, 1 << 14),           # at most one 64x50 image admitted at a time
    (8, 0, 0, True, 1 << 14),                   # scene 1 on the deep-scene engine (single launch)
    (8, 0, 0, True, 1500),                      # its waves limited to 1500 groups (a 100x96 image: 1344)
])
def test_server_samples_per_wave_equal_alone(two_scenes, gpu, samples_per_wave, slot_bytes, cap, two_engines,
                                             max_groups):
    """Several samples of a request in one wave: the first adds to the
    accumulator in the wave, the others are written to slots and added after
    it in sample order, so every image and ray count equals the request
    rendered alone, with too little slot memory for all samples at once, with
    admission capped by pixels and with a deep-scene engine whose ray-queue
    capacity bounds its waves; and the requests take fewer waves than
    samples."""
    scs = [s for _, s, _ in two_scenes]
    srv = gpu.Server(scs, framebuffer_bytes=64 << 20, max_groups=max_groups, refill_mode=gpu.REFILL_ALL,
                     kernel_mode=1, deep_single_launch=1, samples_per_wave=samples_per_wave,
                     sample_buffer_bytes=slot_bytes, max_inflight_pixels=cap)
    if two_engines:
        srv.set_scene_mode(1, gpu.MODE_WAVEFRONT)
    rng = np.random.default_rng(12)
    reqs, ids = [], []
    for k in range(12):
        cam = gpu.Camera()
        scenes.default_camera(cam, eye=(rng.uniform(-1, 1), 1.2, 1.6))
        reqs.append((k % 2, int(rng.choice([64, 100])), int(rng.choice([50, 96])), int(rng.integers(1, 9)), cam))
    for i, (sc, w, h, spp, cam) in enumerate(reqs):
        ids.append(srv.submit(sc, w, h, spp, cam, frame_base=9 * i))
    for i, rid in enumerate(ids):
        st, img, info = srv.wait(rid)
        sc, w, h, spp, cam = reqs[i]
        assert st == 0
        rays = []
        assert (img == _alone(gpu, scs[sc], gpu.View(sc, w, h, spp, 9 * i, cam), rays)).all(), i
        assert info["rays"] == rays[0]
    assert srv.stats()["waves"] < sum(r[3] for r in reqs)
    srv.close()


def test_server_admission_cancel_timeout(two_scenes, gpu):
    scs = [s for _, s, _ in two_scenes]
    cam = scenes.default_camera(gpu.Camera())
    srv = gpu.Server(scs, framebuffer_bytes=64 * 64 * 16 * 2, max_groups=2048, kernel_mode=2)
    with pytest.raises(gpu.CvxError) as e:  # can never fit the framebuffer budget
        srv.submit(0, 1280, 736, 1, cam)
    assert e.value.status == 7
    long_id = srv.submit(0, 64, 64, 400, cam)
    queued = [srv.submit(1, 64, 64, 1, cam) for _ in range(3)]  # at most two fit at once
    srv.cancel(queued[-1])
    with pytest.raises(gpu.CvxError) as e:
        srv.wait(long_id, timeout_ms=0)
    assert e.value.status == 8
    st, img, info = srv.wait(queued[-1])
    assert st == 9 and img is None
    srv.cancel(long_id)
    st, img, info = srv.wait(long_id)
    assert st == 9
    for rid in queued[:-1]:
        st, img, info = srv.wait(rid)
        assert st == 0 and img.shape == (64, 64)
    with pytest.raises(gpu.CvxError) as e:
        srv.wait(123456)
    assert e.value.status == 10
    srv.close()


def test_size_limits_refused_on_the_host(two_scenes, gpu):
    """Image sides above 16384 pixels and larger patches are refused by the
    renderer, the batch and the server before any device work."""
    scs = [s for _, s, _ in two_scenes]
    cam = scenes.default_camera(gpu.Camera())
    with pytest.raises(gpu.CvxError) as e:
        gpu.Renderer(scs[0], 16385, 16)
    assert e.value.status == 1
    r = gpu.Renderer(scs[0], 64, 32)
    with pytest.raises(gpu.CvxError) as e:
        r.render_patches_u8(16400, [(0, 0)], 1)
    assert e.value.status == 1
    batch = gpu.Batch(scs, max_groups=1 << 14, max_pixels=1 << 20)
    with pytest.raises(gpu.CvxError) as e:
        batch.render([gpu.View(0, 16400, 4, 1, 0, cam)], want_images=False)
    assert e.value.status == 1
    srv = gpu.Server(scs, framebuffer_bytes=64 << 20, max_groups=1 << 14)
    with pytest.raises(gpu.CvxError) as e:
        srv.submit(0, 16, 16400, 1, cam)
    assert e.value.status == 1
    srv.close()
