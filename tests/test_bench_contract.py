"""bench.py on the CPU. The reference arm (the oracle's restatement of the
reference's AVX packet traversal on the host cores) runs without a GPU: its
JSON line carries the keys the benchmark contract asks for, and under several
ranks only rank 0 does work and prints. The synthetic batch workload has the
shape it is specified with."""

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(env_extra):
    env = dict(os.environ)
    env.update(env_extra)
    p = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "3", "--warmup", "3"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    return [ln for ln in p.stdout.splitlines() if ln.startswith("{")]


def test_reference_arm_json_line(cvx):  # cvx: the library is built
    lines = _run({"RANK": "0", "WORLD_SIZE": "1"})
    assert len(lines) == 1
    r = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in r, key
    assert r["impl"] == "reference" and r["steps"] == 3 and r["warmup"] == 3 and r["n_gpus"] == 1
    assert r["value"] > 0 and r["unit"] == "Mrays/s" and r["higher_is_better"] is True
    assert "workload" in r["config"]
    assert r["config"]["rays_per_step"] == 4194304  # the GPU arm's workload, every step
    cb = r["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == r["value"] and cb["sample"]
    e = r["e2e"]
    assert e["value"] == r["value"] and e["unit"] == r["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_do_nothing(cvx):
    assert _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}) == []


def test_batched_workload_shape(cvx):
    """The 256-scene batch: log-uniform 500..20,000 triangles (mean near
    19,500 / ln 40 = 5,286) and all three resolutions; the spheres-and-boxes
    generator lands within 2 % above each count."""
    import math

    import numpy as np

    import bench
    from convector_gb300 import scenes
    counts, res = bench._c3_plan(np.random.default_rng(3), 256)
    assert counts.min() >= 500 and counts.max() <= 20000
    assert abs(counts.mean() - 19500 / math.log(40)) < 0.1 * 5286
    assert set(res) == {(320, 184), (640, 368), (1280, 736)}
    for n in (500, 1234, 5000, 20000):
        t, _ = scenes.spheres_and_boxes(n, 3, obj=False)
        assert n <= t.shape[0] <= 1.02 * n + 2


def test_served_workload_shape(cvx):
    """The served stream: Poisson arrivals at 200/s over 2 s (415 requests
    with the benchmark's seed), widths log-uniform from 320 to 1920 at the
    320x184 aspect up to a height of 1080, 1..16 spp, all three scenes,
    cameras on the radius-3 sphere around the room centre."""
    import numpy as np

    import bench
    from convector_gb300 import scenes
    reqs = bench._served_requests(cvx, scenes, 200.0, 2.0, 4)
    assert len(reqs) == 415
    at = np.array([r[0] for r in reqs])
    assert (np.diff(at) > 0).all() and 0.0 < at[0] and at[-1] <= 2.0
    assert {r[1] for r in reqs} == {0, 1, 2}
    w = np.array([r[2] for r in reqs])
    h = np.array([r[3] for r in reqs])
    assert w.min() >= 320 and w.max() <= 1920 and h.min() >= 184 and h.max() <= 1080
    # the 320x184 aspect, the height clamped to 1080 (1920 x 184 / 320 is 1104)
    assert (h == np.minimum(1080, np.maximum(184, np.round(w * 184 / 320)))).all()
    # log-uniform: the median width near sqrt(320 * 1920) = 784
    assert 650 < np.median(w) < 950
    spp = np.array([r[4] for r in reqs])
    assert spp.min() == 1 and spp.max() == 16
    center = np.array([0.0, 1.25, -2.0])
    for r in reqs[:20]:
        eye = np.array(r[5].as_array()[:3], dtype=np.float64)
        assert abs(np.linalg.norm(eye - center) - 3.0) < 1e-4
