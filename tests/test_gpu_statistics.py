"""Statistical agreement between the fast per-group RNG order and the
reference's patch-sequential stream.

The per-group order draws different random numbers than the reference, so
its frames cannot equal the reference's; its estimator must still converge to
the same image. Mean image radiance over independent seeds must agree within
3 sigma, and per-pixel means of accumulated frames must agree within 3 sigma
of their standard errors on all but a small fraction of pixels. The reference
order runs on the GPU here; its frames are bit-exact with the oracle's
restatement of the reference (test_gpu_parity.py).
"""

import numpy as np
import pytest

from convector_gb300 import scenes

pytestmark = pytest.mark.gpu


def _frames(gpu, scene, w, h, order, traversal, frames, base):
    r = gpu.Renderer(scene, w, h, rng_order=order, traversal=traversal)
    out = np.empty((frames, h, w, 3), np.float32)
    for f in range(frames):
        r.render_frame_u8(base + f, gbuffer=False)
        out[f] = r.read_frame_f32()
    return out


def _room(gpu):
    text, mats = scenes.room_sphere()
    scene = gpu.Scene(gpu.Bvh.from_meshes([gpu.Mesh.parse(text, mats)]))
    scenes.default_camera(scene.camera)
    return scene


def test_mean_radiance_over_seeds_within_3_sigma(gpu):
    scene = _room(gpu)
    w, h, n = 320, 184, 16
    ref = _frames(gpu, scene, w, h, gpu.RNG_PATCH, gpu.TRAVERSE_PACKET, n, 100).mean(axis=(1, 2))  # (n, 3)
    fast = _frames(gpu, scene, w, h, gpu.RNG_GROUP, gpu.TRAVERSE_SINGLE, n, 500).mean(axis=(1, 2))
    for c in range(3):
        diff = abs(ref[:, c].mean() - fast[:, c].mean())
        sigma = np.sqrt(ref[:, c].var(ddof=1) / n + fast[:, c].var(ddof=1) / n)
        assert diff <= 3.0 * sigma, (c, diff, sigma)


def _pixel_agreement(a, b):
    """Fraction of pixel channels whose means agree within 3 standard errors."""
    n = a.shape[0]
    se = np.sqrt(a.var(axis=0, ddof=1) / n + b.var(axis=0, ddof=1) / n)
    diff = np.abs(a.mean(axis=0) - b.mean(axis=0))
    ok = diff <= 3.0 * se + 1e-6
    return ok.mean()


def test_per_pixel_means_within_3_sigma_room(gpu):
    scene = _room(gpu)
    a = _frames(gpu, scene, 96, 64, gpu.RNG_PATCH, gpu.TRAVERSE_PACKET, 64, 1000)
    b = _frames(gpu, scene, 96, 64, gpu.RNG_GROUP, gpu.TRAVERSE_SINGLE, 64, 5000)
    assert _pixel_agreement(a, b) >= 0.985


def test_per_pixel_means_within_3_sigma_large_mesh(gpu):
    """The 64-spp accumulation workload on the ~870k-triangle tube: per-group
    wavefront render against the reference stream at matched spp."""
    tris, _ = scenes.random_walk_tube(obj=False)
    scene = gpu.Scene(gpu.Bvh.build(tris))
    scenes.default_camera(scene.camera)
    w, h, n = 80, 46, 64
    a = _frames(gpu, scene, w, h, gpu.RNG_PATCH, gpu.TRAVERSE_PACKET, n, 2000)
    r = gpu.Renderer(scene, w, h, rng_order=gpu.RNG_GROUP, traversal=gpu.TRAVERSE_SINGLE, mode=gpu.MODE_WAVEFRONT,
                     use_graph=1)
    b = np.empty_like(a)
    for f in range(n):
        r.render_frame_u8(9000 + f, gbuffer=False)
        b[f] = r.read_frame_f32()
    assert _pixel_agreement(a, b) >= 0.985
