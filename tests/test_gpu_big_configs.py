"""Image checks at the benchmark workloads' own sizes.

* The large-mesh accumulation (870k-triangle tube, 1280x736, 64 spp, 5
  bounces): the form the autotuner picks for it (single launch, paths per lane,
  per-group RNG order) against the reference's patch-sequential stream on the
  GPU (k_render_patch, bit-exact with the oracle's restatement of the
  reference, test_gpu_parity.py), at matched spp, over the whole frame: per
  pixel, the two means agree within 3 standard errors on all but a small
  fraction of the pixel channels, and the mean image radiance agrees within
  3 sigma (renderer.rs:339-410 accumulates and resolves the samples).
* The 256-scene batch (500..20,000 triangles each, 4 spp): 16 of its views,
  drawn across the three resolutions, equal the same views rendered alone.
* The tube's full frame from the deep-tree path-refill kernel, bit-exact
  against the oracle, and 24 requests of the served benchmark's stream, each
  equal to the request rendered alone, served with one sample per wave, with
  up to 16, and with admission capped by pixels.
"""

import numpy as np
import pytest

from convector_gb300 import scenes

pytestmark = pytest.mark.gpu


class _Moments:
    """Per-pixel running sums of samples and of their squares (float64)."""

    def __init__(self, h, w):
        self.n = 0
        self.s = np.zeros((h, w, 3), np.float64)
        self.q = np.zeros((h, w, 3), np.float64)
        self.frame_means = []

    def add(self, img):
        x = img.astype(np.float64)
        self.n += 1
        self.s += x
        self.q += x * x
        self.frame_means.append(x.mean(axis=(0, 1)))

    def mean(self):
        return self.s / self.n

    def var(self):
        return (self.q - self.s * self.s / self.n) / (self.n - 1)


def test_large_mesh_full_frame_within_3_sigma(gpu):
    tris, _ = scenes.random_walk_tube(obj=False)
    scene = gpu.Scene(gpu.Bvh.build(tris))
    scenes.default_camera(scene.camera)
    w, h, spp = 1280, 736, 64
    ref = gpu.Renderer(scene, w, h, rng_order=gpu.RNG_PATCH, traversal=gpu.TRAVERSE_PACKET)
    fast = gpu.Renderer(scene, w, h, rng_order=gpu.RNG_GROUP, traversal=gpu.TRAVERSE_SINGLE,
                        refill_mode=gpu.REFILL_ALL)
    a, b = _Moments(h, w), _Moments(h, w)
    for s in range(spp):
        ref.render_frame_u8(42 + s, gbuffer=False)
        a.add(ref.read_frame_f32())
        fast.render_frame_u8(4200 + s, gbuffer=False)
        b.add(fast.read_frame_f32())
    se = np.sqrt(a.var() / spp + b.var() / spp)
    ok = np.abs(a.mean() - b.mean()) <= 3.0 * se + 1e-6
    print("tube 1280x736 at %d spp: %.4f of pixel channels within 3 sigma" % (spp, ok.mean()))
    assert ok.mean() >= 0.985
    fa, fb = np.array(a.frame_means), np.array(b.frame_means)  # (spp, 3)
    for c in range(3):
        sigma = np.sqrt(fa[:, c].var(ddof=1) / spp + fb[:, c].var(ddof=1) / spp)
        assert abs(fa[:, c].mean() - fb[:, c].mean()) <= 3.0 * sigma, c


def test_batch_of_256_scenes_equals_views_alone(gpu):
    import bench
    scs, views, _ = bench._c3_views(gpu)
    batch = gpu.Batch(scs, max_groups=1 << 21, max_pixels=sum(v.width * v.height for v in views))
    imgs, rays, _ = batch.render(views)
    assert rays > 0
    rng = np.random.default_rng(17)
    picked = []
    for size in (320, 640, 1280):  # views of every resolution
        idx = [i for i, v in enumerate(views) if v.width == size]
        picked += [int(i) for i in rng.choice(idx, size=min(len(idx), 6 if size < 1280 else 4), replace=False)]
    assert len(picked) == 16
    for i in picked:
        v = views[i]
        r = gpu.Renderer(scs[v.scene], v.width, v.height, rng_order=gpu.RNG_GROUP, traversal=gpu.TRAVERSE_SINGLE)
        r.set_camera(v.camera)
        for s in range(v.spp):
            r.accumulate_frame_f32(v.frame_base + s)
        alone = r.resolve_u8(v.spp)
        assert (imgs[i] == alone).all(), i


def test_large_mesh_full_frame_bitexact_against_oracle(gpu, orc):
    """The deep-tree path-refill kernel (shared stack entries, select-form
    rounds) on the benchmark's own frame: 1280x736 of the 870k-triangle tube,
    frame 42, per-group RNG order, bit-exact RGBA, gbuffer, linear colour and
    ray count against the oracle; then two accumulated samples, bit-exact."""
    tris, _ = scenes.random_walk_tube(obj=False)
    bvh = gpu.Bvh.build(tris)
    scene = gpu.Scene(bvh)
    scenes.default_camera(scene.camera)
    osc = orc.OracleScene.from_bvh(bvh)
    w, h = 1280, 736
    r = gpu.Renderer(scene, w, h, rng_order=gpu.RNG_GROUP, traversal=gpu.TRAVERSE_SINGLE,
                     refill_mode=gpu.REFILL_ALL)
    rgba, gb = r.render_frame_u8(42)
    col = r.read_frame_f32()
    orgba, ogb, ocol, orays = osc.render(scene.camera.as_array(), w, h, 42, rng_order=orc.RNG_GROUP, traversal=1)
    assert (rgba == orgba).all() and (gb == ogb).all()
    assert (col.view(np.uint32) == ocol.view(np.uint32)).all()
    assert r.stats()[0] == orays
    acc = np.zeros((h, w, 3), np.float32)
    for f in (43, 44):
        r.accumulate_frame_f32(f)
        osc.render(scene.camera.as_array(), w, h, f, rng_order=orc.RNG_GROUP, traversal=1, color=False, accum=acc)
    assert (r.read_accumulator().view(np.uint32) == acc.view(np.uint32)).all()


@pytest.fixture(scope="module")
def served_stream(gpu):
    """24 requests of the served workload's own stream and each one's image
    rendered alone (one accumulate_frame_f32 call per sample)."""
    import bench
    scs = []
    for gen in (scenes.room_sphere, lambda obj: scenes.displaced_icosphere(obj=obj, light=True),
                scenes.random_walk_tube):
        scs.append(gpu.Scene(gpu.Bvh.build(gen(obj=False)[0])))
    reqs = bench._served_requests(gpu, scenes, 200.0, 2.0, 4)[:24]
    assert {sc for _, sc, *_ in reqs} == {0, 1, 2}
    alone = []
    for i, (_, sc, w, h, spp, cam) in enumerate(reqs):
        r = gpu.Renderer(scs[sc], w, h, rng_order=gpu.RNG_GROUP, traversal=gpu.TRAVERSE_SINGLE)
        r.set_camera(cam)
        for s in range(spp):
            r.accumulate_frame_f32(16 * i + s)
        alone.append(r.resolve_u8(spp))
    return scs, reqs, alone


@pytest.mark.parametrize("extra", [{}, {"samples_per_wave": 16}, {"samples_per_wave": 16, "max_inflight_pixels": 4 << 20}])
def test_served_benchmark_requests_equal_alone(gpu, served_stream, extra):
    """24 requests of the served workload's own stream (3 resident scenes,
    Poisson arrivals, poses on a radius-3 sphere, 320x184 to 1920x1080, 1 to
    16 spp), served with the benchmark's engine configuration (the tube on a
    single-launch deep engine, paths per lane; one sample per request per
    wave, or up to 16, with admission capped by pixels or not) and all
    submitted at once, so that they share waves: each image equals the request
    rendered alone."""
    scs, reqs, alone = served_stream
    srv = gpu.Server(scs, framebuffer_bytes=4 << 30, max_groups=1 << 21, refill_mode=gpu.REFILL_ALL,
                     deep_single_launch=1, **extra)
    ids = [srv.submit(sc, w, h, spp, cam, frame_base=16 * i) for i, (_, sc, w, h, spp, cam) in enumerate(reqs)]
    for i, rid in enumerate(ids):
        st, img, _ = srv.wait(rid, 600000)
        assert st == 0
        assert (img == alone[i]).all(), i
    srv.close()
