"""Benchmark of the render hot path on GB300.

Headline workload (one step = one nearest-hit pass of the ray-cast kernel over
one batch): a displaced icosphere of subdivision 6 (81,920 triangles, value
noise seed 7) in a 10-triangle box room, 4,194,304 rays with origins uniform
in the room and directions uniform on the sphere (seed 7), FP32, hit index
and t bit-exact against the oracle. Metric: Mrays/s.

Also reported (extra keys): frame time p50/p99 and Mrays/s of the 1280x736,
1 spp, 5-bounce interactive frame of the room-and-sphere scene.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank runs the same workload on its own GPU
(replicas: rays are independent, there is no collective on the data path);
value = rays of all ranks / max-over-ranks time.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_RAYS = 4194304
# The frame sections time the oracle's CPU frame path beside the GPU (rank 0,
# one GPU); --no-cpu-frames leaves it out.
CPU_BASELINE = True
METRIC = "Mrays/s (nearest-hit rays per second)"
WORKLOAD = "ray-cast isolation: displaced icosphere subdiv 6 (81,920 tris, seed 7) in a 10-tri box room, " \
           "4,194,304 rays uniform in the room / on S^2 (seed 7)"


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


_L2_PEAK = None


def l2_peak():
    """L2 read bandwidth of this GPU (GB/s), measured once by the package's
    L2 probe (libconvector_l2probe.so): an L2-resident buffer read with
    ld.global.cg by a grid filling the GPU, best of 5 launches, at 8, 32 and
    64 MB; the peak is the largest."""
    global _L2_PEAK
    if _L2_PEAK is None:
        import ctypes
        from convector_gb300 import _build
        L = ctypes.CDLL(_build.build_probe())
        L.cvx_probe_l2_read_gbs.restype = ctypes.c_int32
        L.cvx_probe_l2_read_gbs.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32,
                                            ctypes.POINTER(ctypes.c_double)]
        by_size = {}
        for mb, passes in ((8, 400), (32, 100), (64, 50)):
            g = ctypes.c_double()
            rc = L.cvx_probe_l2_read_gbs(mb << 20, passes, 5, ctypes.byref(g))
            if rc != 0:
                raise RuntimeError("L2 probe failed (%d)" % rc)
            by_size["%d MB" % mb] = g.value
        _L2_PEAK = {"gbs": max(by_size.values()), "by_buffer_size": by_size,
                    "how": "ld.global.cg reads of an L2-resident buffer, grid of 8 blocks x 256 threads per SM, "
                           "best of 5 launches (CUDA events)"}
    return _L2_PEAK


def frame_roofline(work, n_lights, pixels, frame_ms, out_bytes_per_px, traffic_key=None):
    """Memory roofline of one frame from its counted work (cvx_renderer_count_work):
    algorithmic bytes = 32 per box tested + 36 per triangle tested (the
    reference's node and vertex records) + 36 per light for every shading step
    that evaluates the light PDFs + the frame's output bytes per pixel."""
    b = 32 * work["boxes"] + 36 * work["triangles"] + 36 * n_lights * work["light_shades"] + \
        out_bytes_per_px * pixels
    achieved = b / (frame_ms * 1e-3) / 1e9
    hbm, hbm_kind = _peaks()
    l2 = l2_peak()["gbs"]
    dram = _traffic(traffic_key) if traffic_key else None
    lts = _traffic(traffic_key + ":lts_bytes") if traffic_key else None
    return {"algorithmic_bytes": b, "bytes_per_ray": b / max(1, work["rays"]), "achieved_gbs": achieved,
            "hbm_peak_gbs": hbm, "hbm_peak_kind": hbm_kind, "hbm_frac": achieved / hbm,
            "l2_peak_gbs": l2, "l2_frac": achieved / l2, "work": work, "traffic": dram, "l2_traffic": lts,
            "l2_frac_measured": None if lts is None else lts / (frame_ms * 1e-3) / 1e9 / l2,
            "boxes_per_ray": work["boxes"] / max(1, work["rays"]),
            "tris_per_ray": work["triangles"] / max(1, work["rays"])}


def cpu_frame_baseline(bvh, camera, w, h, frame, accumulate=False, target_s=10.0, max_frames=10):
    """The reference's frame path on all host cores: the oracle in the
    reference's patch order (one generator per 32x32 patch, main.rs:174-214,
    renderer.rs:306-327), x86 arithmetic, 8-ray packet traversal, patches
    spread over the threads. Frames of the same workload until about
    target_s."""
    from oracle import oracle as orc
    osc = orc.OracleScene.from_bvh(bvh)
    threads = os.cpu_count() or 1
    cam = camera.as_array()
    acc = np.zeros((h, w, 3), np.float32) if accumulate else None
    dt, frames, rays = 0.0, 0, 0
    while frames < max_frames and (dt < target_s or frames == 0):
        t0 = time.perf_counter()
        rays += osc.render(cam, w, h, frame + frames, rng_order=orc.RNG_PATCH, traversal=orc.TRAVERSE_PACKET,
                           nthreads=threads, color=False, accum=acc)[3]
        dt += time.perf_counter() - t0
        frames += 1
    return {"value": 1e3 * dt / frames, "unit": "ms per frame", "mrays_per_s": rays / dt / 1e6,
            "frames": frames, "cores": threads, "kind": "port",
            "sample": "%d frame(s) of %dx%d, %s, patch order, 8-ray packets, %.1f s" % (
                frames, w, h, "accumulated" if accumulate else "1 spp", dt)}


def _traffic(kernel_key):
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f).get(kernel_key)
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
             "clocks_event_reasons.sw_power_cap"

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.2)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() in ("active", "1", "0x1"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def reduce_max(value, dist=None, device=None):
    """Max of a per-rank float over all ranks (replicas: the job takes as long
    as its slowest rank). Works with the nccl (device tensor) and gloo (CPU)
    backends; without an initialised process group returns `value`."""
    if dist is None or not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(rays_per_rank, world, seconds):
    """Whole-job Mrays/s of `world` replicas that each traced rays_per_rank."""
    return world * rays_per_rank / seconds / 1e6


def build_c1():
    import convector_gb300 as cg
    from convector_gb300 import scenes
    text, mats = scenes.displaced_icosphere()
    bvh = cg.Bvh.from_meshes([cg.Mesh.parse(text, mats)])
    o, d = scenes.random_rays(N_RAYS, seed=7)
    return bvh, o, d


def build_c0():
    import convector_gb300 as cg
    from convector_gb300 import scenes
    text, mats = scenes.room_sphere()
    bvh = cg.Bvh.from_meshes([cg.Mesh.parse(text, mats)])
    return bvh


def cpu_sample_rays_per_s(osc, o, d, target_s=10.0):
    """Times the oracle's packet traversal (all host cores) on a bounded sample:
    consecutive 1 Mi-ray slices of the workload until about `target_s`."""
    threads = os.cpu_count() or 1
    chunk = 1 << 20
    osc.intersect(o[:8192], d[:8192], nthreads=threads)
    done, dt, k = 0, 0.0, 0
    while dt < target_s and k < 64:
        lo = (k * chunk) % o.shape[0]
        t0 = time.perf_counter()
        osc.intersect(o[lo:lo + chunk], d[lo:lo + chunk], nthreads=threads)
        dt += time.perf_counter() - t0
        done += min(chunk, o.shape[0] - lo)
        k += 1
    return done / dt, threads, done, dt


def run_reference(args):
    """The reference's CPU path on the host cores: the oracle's C++ restatement
    of the reference AVX packet traversal (the Rust original cannot be built),
    over the same 4,194,304 rays per step as the GPU arm. The scene's BVH is
    built by the oracle's own restatement of Bvh::build (identical to the
    product's build), so this process never loads the product library."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from convector_gb300 import scenes
    from oracle import oracle as orc
    tris, _ = scenes.displaced_icosphere(obj=False)
    obvh = orc.OracleBvh(tris)
    osc = orc.OracleScene(obvh.triangles, obvh.nodes)
    o, d = scenes.random_rays(N_RAYS, seed=7)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        osc.intersect(o, d, nthreads=threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        osc.intersect(o, d, nthreads=threads)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = N_RAYS * args.steps / total / 1e6
    import convector_gb300
    assert convector_gb300._LIB is None, "the reference arm must not load the product library"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "rays_per_step": N_RAYS, "triangles": int(tris.shape[0]),
                   "traversal": "reference 8-ray packets", "bvh": "oracle restatement of Bvh::build"},
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": "all %d rays of the workload per step, %d steps" % (N_RAYS, args.steps)},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_ours(args):
    import torch
    import torch.distributed as dist

    import convector_gb300 as cg

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    cg.lib(build=True)

    bvh, o, d = build_c1()
    scene = cg.Scene(bvh)
    n = o.shape[0]
    rays = torch.from_numpy(np.concatenate([o.T, d.T]).copy()).cuda()
    t_out = torch.empty(n, dtype=torch.float32, device="cuda")
    tri_out = torch.empty(n, dtype=torch.int32, device="cuda")
    cnt = torch.empty(2 * n, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # larger than the 129 MB L2

    # Algorithmic bytes per launch (counters from one untimed pass per variant).
    algo = {}
    for trav in (0, 1):
        scene.intersect_nearest_device(rays, t_out, tri_out, traversal=trav, counters=cnt, stream=stream)
        torch.cuda.synchronize()
        c = cnt.cpu().numpy().view(np.uint32).astype(np.int64)
        na, nt = c[:n], c[n:]
        if trav == 0:  # packet counters repeat on the 8 lanes: node and triangle data once per packet
            b = int((32 * na[::8] + 36 * nt[::8]).sum()) + 32 * n
        else:
            b = int((32 * na + 36 * nt).sum()) + 32 * n
        algo[trav] = {"bytes": b, "boxes_per_ray": float(na.mean()), "tris_per_ray": float(nt.mean())}

    def step(trav):
        scene.intersect_nearest_device(rays, t_out, tri_out, traversal=trav, stream=stream)

    # Pick the traversal variant, launch shape and stack depth on a short
    # untimed trial (the query autotuner).
    from convector_gb300 import autotune
    shapes = None
    if args.launch:  # a fixed configuration (reproducible profiles): no trial
        shapes = [args.launch]
        if not any(q[0] == args.launch for q in autotune.QUERY_SHAPES):
            raise SystemExit("--launch: one of " + ", ".join(q[0] for q in autotune.QUERY_SHAPES))
    best, trial = autotune.tune_query(scene, rays, t_out, tri_out, shapes=shapes)
    trav = autotune.query_traversal(best)
    # Kernels per step: the single-ray query on a scene whose node bounds are
    # finite, ordered and free of -0 runs the select-form kernel and the pass
    # over the rays it deferred (the library's check at scene creation).
    nb = bvh.nodes_f32.reshape(-1, 8)[:, :6]
    select_form = bool(np.isfinite(nb).all() and (nb[:, :3] <= nb[:, 3:]).all()
                       and not ((nb == 0) & np.signbit(nb)).any())
    launches_per_step = 2 if (trav == 1 and select_form) else 1

    for _ in range(args.warmup):
        flush.zero_()
        step(trav)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clocks:
        torch.cuda.synchronize()
        wall0 = time.perf_counter()
        for e0, e1 in evs:
            flush.zero_()  # L2 flush between timed iterations, outside the timed span
            e0.record()
            step(trav)
            e1.record()
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    step_ms = [e0.elapsed_time(e1) for e0, e1 in evs]
    total_ms = reduce_max(sum(step_ms), dist if world > 1 else None, "cuda")
    if world > 1:
        dist.barrier()
    ms_per_step = total_ms / args.steps
    value = replica_value(n * args.steps, world, total_ms * 1e-3)

    # End to end through the C-ABI with page-locked host buffers: every step
    # moves its rays in and its hits out. Where the GPU shares the host's page
    # tables the kernel reads the rays in place over the CPU-GPU link; the
    # same call with the rays copied first is timed beside it.
    pin = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in
           (o[:, 0], o[:, 1], o[:, 2], d[:, 0], d[:, 1], d[:, 2])]
    t_host = torch.empty(n, dtype=torch.float32).pin_memory()
    tri_host = torch.empty(n, dtype=torch.int32).pin_memory()
    L = cg.lib()
    import ctypes
    ptrs = [ctypes.c_void_p(p.data_ptr()) for p in pin]

    def e2e_call():
        st = L.cvx_intersect_nearest(scene._h, *ptrs, n, 1.0e5, trav, ctypes.c_void_p(t_host.data_ptr()),
                                     ctypes.c_void_p(tri_host.data_ptr()))
        if st:
            cg._check(st)

    e2e_steps = max(3, min(args.steps, 20))

    def e2e_run():
        for _ in range(max(1, args.warmup)):
            e2e_call()
        if world > 1:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            e2e_call()
        e2e_s = reduce_max(time.perf_counter() - t0, dist if world > 1 else None, "cuda")
        return replica_value(n * e2e_steps, world, e2e_s)

    scene.set_host_access(cg.HOST_ACCESS_COPY)
    e2e_copy = e2e_run()
    in_place = scene.set_host_access(cg.HOST_ACCESS_AUTO)
    e2e_value = e2e_run()

    render = batched = served = large = bvh_build = None
    if rank == 0 and not args.no_render:
        render = _guard(bench_render, cg)
    if rank == 0 and not args.no_extra:
        large = _guard(bench_large, cg)
        batched = _guard(bench_batched, cg)
        served = _guard(bench_served, cg)
        bvh_build = _guard(bench_bvh_build, cg)

    if rank == 0:
        peak, peak_kind = _peaks()
        bytes_launch = algo[trav]["bytes"]
        achieved = bytes_launch / (ms_per_step * 1e-3) / 1e9
        kname = "k_intersect_packet" if trav == 0 else "k_intersect_refill"
        # The scene is L2-resident: node and triangle fetches are served by
        # L1 and L2, so the kernel is also set against the measured L2 read
        # bandwidth, with its algorithmic bytes and with the L2 bytes ncu
        # counted for one launch (lts__t_bytes.sum, profiles/traffic.json).
        l2 = _guard(l2_peak)
        l2_block = None
        if "gbs" in l2:
            lts = _traffic(kname + ":lts_bytes")
            l2_block = {"peak_gbs": l2["gbs"], "peak_by_buffer_size": l2["by_buffer_size"], "peak_how": l2["how"],
                        "frac_algorithmic": achieved / l2["gbs"], "traffic": lts,
                        "frac_measured": None if lts is None else lts / (ms_per_step * 1e-3) / 1e9 / l2["gbs"]}
        else:
            l2_block = l2
        cpu = None
        if world == 1:
            from oracle import oracle as orc
            osc = orc.OracleScene.from_bvh(bvh)
            rps, cores, sample, dt = cpu_sample_rays_per_s(osc, o, d)
            cpu = {"value": rps / 1e6, "unit": "Mrays/s", "cores": cores, "kind": "port",
                   "sample": "%d rays of the same workload (%.1f s), reference 8-ray packet traversal" % (sample, dt)}
        line = {
            "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "rays_per_step": n, "triangles": int(bvh.triangles.shape[0]),
                       "traversal": "packet8" if trav == 0 else "single", "launch": best, "trial_ms": trial,
                       "l2": "flushed between timed steps (256 MB write)", "parallelism": "replicas"},
            "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": 24 * n, "d2h_bytes_per_step": 8 * n,
                    "host_rays": "read in place by the kernel" if in_place else "copied to the device",
                    "value_rays_copied": e2e_copy},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_kind": peak_kind, "traffic": _traffic(kname),
                         "algorithmic_bytes_per_launch": bytes_launch,
                         "boxes_per_ray": algo[trav]["boxes_per_ray"], "tris_per_ray": algo[trav]["tris_per_ray"],
                         "kernel": kname, "l2": l2_block},
            "cpu_baseline": cpu,
            "clocks": clocks.summary(),
            "gpu_launches": args.steps * launches_per_step,
            "wall_s_timed": wall,
            "step_ms_p50": statistics.median(step_ms),
            "render": render,
            "large_accumulate": large,
            "batched": batched,
            "served": served,
            "bvh_build": bvh_build,
        }
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def _guard(fn, *a):
    try:
        return fn(*a)
    except Exception as e:  # an extra section must not cost the headline line
        return {"error": "%s: %s" % (type(e).__name__, e)}


def _frames(r, frames, first=42, accumulate=False):
    for f in range(3):
        (r.accumulate_frame_f32 if accumulate else r.render_frame_u8)(f)
    ms, rays = [], 0
    for f in range(frames):
        if accumulate:
            r.accumulate_frame_f32(first + f)
        else:
            r.render_frame_u8(first + f, gbuffer=False)
        nr, m = r.stats()
        ms.append(m)
        rays += nr
    # a path is one pixel's sample: camera ray and its bounces
    paths = r.width * r.height * frames
    return {"frame_ms_p50": float(np.percentile(ms, 50)), "frame_ms_p99": float(np.percentile(ms, 99)),
            "mrays_per_s": rays / (sum(ms) * 1e-3) / 1e6, "mpaths_per_s": paths / (sum(ms) * 1e-3) / 1e6,
            "rays_per_frame": rays / frames, "frames": frames}


def bench_render(cg):
    """1280x736, 1 spp, 5 bounces on the room-and-sphere scene: frame p50/p99
    (device time per frame) for every kernel organisation."""
    from convector_gb300 import scenes
    bvh = build_c0()
    scene = cg.Scene(bvh)
    scenes.default_camera(scene.camera)
    out = {}
    # single-launch single-ray: one octet per 8-pixel group (the default for
    # this 19-level tree) and paths per lane with ray refill
    variants = [("megakernel_packet8", cg.RNG_GROUP, 0, cg.MODE_MEGAKERNEL, 0, cg.REFILL_AFTER_CAMERA),
                ("megakernel_single", cg.RNG_GROUP, 1, cg.MODE_MEGAKERNEL, 0, cg.REFILL_NONE),
                ("megakernel_single_path_refill", cg.RNG_GROUP, 1, cg.MODE_MEGAKERNEL, 0, cg.REFILL_ALL),
                ("wavefront_single_graph", cg.RNG_GROUP, 1, cg.MODE_WAVEFRONT, 1, cg.REFILL_AFTER_CAMERA),
                ("wavefront_packet8_graph", cg.RNG_GROUP, 0, cg.MODE_WAVEFRONT, 1, cg.REFILL_AFTER_CAMERA),
                ("patch_exact_packet8", cg.RNG_PATCH, 0, cg.MODE_MEGAKERNEL, 0, cg.REFILL_AFTER_CAMERA)]
    for name, order, trav, mode, graph, refill in variants:
        r = cg.Renderer(scene, 1280, 736, rng_order=order, traversal=trav, mode=mode, use_graph=graph,
                        refill_mode=refill)
        out[name] = _frames(r, 10 if order == cg.RNG_PATCH else 30)
    from convector_gb300 import autotune
    best, table = autotune.tune(scene, 1280, 736, use_cache=False)
    r = cg.Renderer(scene, 1280, 736, **best)
    res = _frames(r, 30)
    res["config"] = best
    res["candidates_ms"] = {k: round(v, 4) for k, v in table.items()}
    out["autotuned"] = res
    # Roofline of the single-ray frame (the work of frame 42, counted on the
    # device; the same for every single-ray kernel form): RGBA and gbuffer out.
    work = cg.Renderer(scene, 1280, 736, rng_order=cg.RNG_GROUP, traversal=cg.TRAVERSE_SINGLE).count_work(42)
    out["roofline"] = frame_roofline(work, scene.direct_sample_num(), 1280 * 736, res["frame_ms_p50"], 8,
                                     "k_render_refill@room")
    out["roofline"]["frame_ms"] = res["frame_ms_p50"]
    if CPU_BASELINE:
        out["cpu_baseline"] = cpu_frame_baseline(bvh, scene.camera, 1280, 736, 42)
    return out


def bench_large(cg):
    """Accumulative 1280x736, 64 spp, 5 bounces on the ~870k-triangle random-walk
    tube (seed 11): wavefront + CUDA graph against the single launch (paths per
    lane with ray refill, the default for this 70-level tree, and one octet per
    group)."""
    from convector_gb300 import scenes
    tris, _ = scenes.random_walk_tube(obj=False)
    bvh = cg.Bvh.build(tris)
    scene = cg.Scene(bvh)
    scenes.default_camera(scene.camera)
    out = {"triangles": int(tris.shape[0]), "bvh_depth": int(bvh.depth)}
    from convector_gb300 import autotune
    best, table = autotune.tune(scene, 1280, 736, use_cache=False, frames=3)
    for name, kw in (("wavefront_single_graph", dict(traversal=1, mode=cg.MODE_WAVEFRONT, use_graph=1)),
                     ("megakernel_single", dict(traversal=1, mode=cg.MODE_MEGAKERNEL)),
                     ("megakernel_single_octets", dict(traversal=1, mode=cg.MODE_MEGAKERNEL,
                                                       refill_mode=cg.REFILL_NONE)),
                     ("autotuned", best)):
        kw = dict(kw)
        kw.setdefault("rng_order", cg.RNG_GROUP)
        r = cg.Renderer(scene, 1280, 736, **kw)
        res = _frames(r, 64, accumulate=True)
        res["spp"] = 64
        if name == "autotuned":
            res["config"] = best
        out[name] = res
    # The 64 samples in one call (cvx_accumulate_frames_f32): in the
    # path-refill form 32 samples share a launch, so the launch's drain is paid
    # once per 32 samples; same accumulator bits as 64 one-sample calls.
    r = cg.Renderer(scene, 1280, 736, **dict(best, rng_order=cg.RNG_GROUP))
    r.accumulate_frames_f32(0, 16)
    ms_calls, rays = [], 0
    for c in range(5):
        r.accumulate_frames_f32(42 + 64 * c, 64)
        nr, m = r.stats()
        ms_calls.append(m)
        rays += nr
    per = float(np.percentile(ms_calls, 50)) / 64.0
    out["in_one_call"] = {"sample_ms_p50": per, "call_ms": [round(m, 3) for m in ms_calls], "spp": 64,
                          "frames_per_launch": 32, "mrays_per_s": rays / (sum(ms_calls) * 1e-3) / 1e6,
                          "mpaths_per_s": 1280 * 736 * 64 * 5 / (sum(ms_calls) * 1e-3) / 1e6, "config": best}
    # Roofline of one accumulated sample (frame 42's work): the accumulator is
    # read and written (24 bytes per pixel).
    work = cg.Renderer(scene, 1280, 736, rng_order=cg.RNG_GROUP, traversal=cg.TRAVERSE_SINGLE).count_work(42)
    ms = out["autotuned"]["frame_ms_p50"]
    out["roofline"] = frame_roofline(work, scene.direct_sample_num(), 1280 * 736, ms, 24, "k_render_refill@tube")
    out["roofline"]["frame_ms"] = ms
    out["in_one_call"]["roofline"] = frame_roofline(work, scene.direct_sample_num(), 1280 * 736, per, 24,
                                                    "k_render_refill@tube-32")
    if CPU_BASELINE:
        out["cpu_baseline"] = cpu_frame_baseline(bvh, scene.camera, 1280, 736, 42, accumulate=True, target_s=5.0,
                                                 max_frames=2)
    return out


def bench_frame_kernel(cg, which):
    """A few frames of one single-ray frame kernel alone (paths per lane, the
    autotuned form for both scenes), for profiling: `room` renders the
    1280x736 interactive frame of the room-and-sphere scene, `tube` samples of
    the 870k-triangle tube accumulated at 1280x736, `tube-multi` two
    accumulate_frames_f32 calls of 32 tube samples (one launch each)."""
    from convector_gb300 import scenes
    if which == "room":
        bvh = build_c0()
    else:
        bvh = cg.Bvh.build(scenes.random_walk_tube(obj=False)[0])
    scene = cg.Scene(bvh)
    scenes.default_camera(scene.camera)
    r = cg.Renderer(scene, 1280, 736, rng_order=cg.RNG_GROUP, traversal=cg.TRAVERSE_SINGLE,
                    refill_mode=cg.REFILL_ALL)
    ms = []
    for f in range(2 if which == "tube-multi" else 4):
        if which == "room":
            r.render_frame_u8(42 + f, gbuffer=False)
        elif which == "tube-multi":
            r.accumulate_frames_f32(42 + 32 * f, 32)
        else:
            r.accumulate_frame_f32(42 + f)
        ms.append(r.stats()[1])
    return {"scene": which, "frame_ms": ms}


def _c3_plan(rng, n):
    """Triangle counts (log-uniform 500..20,000) and resolutions (one of
    320x184, 640x368, 1280x736) of the batch's n scenes."""
    counts = np.exp(rng.uniform(np.log(500), np.log(20000), n)).astype(int)
    sizes = [(320, 184), (640, 368), (1280, 736)]
    res = [sizes[i] for i in rng.integers(0, 3, n)]
    return counts, res


def _c3_views(cg, n=256, seed=3):
    """256 scenes of spheres and boxes, log-uniform 500..20,000 triangles, one
    camera and a resolution from {320x184, 640x368, 1280x736} each, 4 spp."""
    from concurrent.futures import ThreadPoolExecutor
    from convector_gb300 import scenes
    rng = np.random.default_rng(seed)
    counts, res = _c3_plan(rng, n)
    tri_arrays = [scenes.spheres_and_boxes(int(c), seed=seed * 100003 + i, obj=False)[0] for i, c in enumerate(counts)]
    with ThreadPoolExecutor(8) as ex:
        bvhs = list(ex.map(cg.Bvh.build, tri_arrays))
    scs = [cg.Scene(b) for b in bvhs]
    views = []
    for i in range(n):
        cam = scenes.default_camera(cg.Camera(), eye=(rng.uniform(-1, 1), rng.uniform(0.8, 1.6), 1.6))
        views.append(cg.View(i, res[i][0], res[i][1], 4, 1000 * i, cam))
    return scs, views, int(counts.sum())


def bench_batched(cg):
    """256 uneven scenes in shared wavefronts against one scene at a time."""
    scs, views, total_tris = _c3_views(cg)
    batch = cg.Batch(scs, max_groups=1 << 21, max_pixels=sum(v.width * v.height for v in views))
    batch.render(views[:8], want_images=False)  # warm-up (graph capture)
    t0 = time.perf_counter()
    _, rays_b, ms_b = batch.render(views, want_images=False)
    wall_b = time.perf_counter() - t0
    # one at a time: the plain per-scene renderer, 4 accumulated frames + resolve
    rays_p, ms_p = 0, 0.0
    t0 = time.perf_counter()
    for v in views:
        r = cg.Renderer(scs[v.scene], v.width, v.height, rng_order=cg.RNG_GROUP, traversal=cg.TRAVERSE_SINGLE)
        r.set_camera(v.camera)
        for s in range(v.spp):
            r.accumulate_frame_f32(v.frame_base + s)
            nr, m = r.stats()
            rays_p += nr
            ms_p += m
        r.resolve_u8(v.spp)
    wall_p = time.perf_counter() - t0
    return {"scenes": len(scs), "triangles_total": total_tris, "spp": 4, "rays": rays_b,
            "batched_mrays_per_s_device": rays_b / (ms_b * 1e-3) / 1e6, "batched_wall_s": wall_b,
            "batched_mrays_per_s_wall": rays_b / wall_b / 1e6,
            "one_at_a_time_mrays_per_s_device": rays_p / (ms_p * 1e-3) / 1e6, "one_at_a_time_wall_s": wall_p,
            "one_at_a_time_mrays_per_s_wall": rays_p / wall_p / 1e6,
            "speedup_wall": wall_p / wall_b}


def _served_run(cg, scs, reqs, sequential, engine=None, burst=False):
    """The requests through a Server, each submitted at its arrival time
    (burst: all at once, which measures the throughput the server sustains)."""
    engine = engine or {}
    srv = cg.Server(scs, framebuffer_bytes=24 << 30, max_groups=engine.get("max_groups", 1 << 21),
                    traversal=cg.TRAVERSE_SINGLE,
                    sequential=sequential, blocks_per_sm=engine.get("blocks_per_sm", 0),
                    refill_mode=engine.get("refill_mode", cg.REFILL_AFTER_CAMERA),
                    fused_blocks_per_sm=engine.get("fused_blocks_per_sm", 0),
                    wavefront_streams=engine.get("wavefront_streams", 1),
                    deep_single_launch=engine.get("deep_single_launch", 0),
                    max_inflight_pixels=engine.get("max_inflight_pixels", 0),
                    samples_per_wave=engine.get("samples_per_wave", 1))
    # warm-up: one small request per scene
    for k in range(len(scs)):
        srv.wait(srv.submit(k, 64, 64, 1, reqs[0][5]))
    ids = []
    t0 = time.perf_counter()
    for at, sc, w, h, spp, cam in reqs:
        dt = t0 + at - time.perf_counter()
        if dt > 0 and not burst:
            time.sleep(dt)
        ids.append(srv.submit(sc, w, h, spp, cam, frame_base=len(ids) * 16))
    done = [srv.wait(i, 600000) for i in ids]
    failed = sum(1 for st, _, _ in done if st != 0)
    if failed:
        raise RuntimeError("%d of %d served requests failed" % (failed, len(ids)))
    res = [r for _, _, r in done]
    lat = np.array([r["done_s"] - r["submit_s"] for r in res]) * 1e3
    rays = sum(r["rays"] for r in res)
    span = max(r["done_s"] for r in res) - min(r["submit_s"] for r in res)
    st = srv.stats()
    srv.close()
    return {"requests": len(res), "latency_ms_p50": float(np.percentile(lat, 50)),
            "latency_ms_p99": float(np.percentile(lat, 99)), "mrays_per_s": rays / span / 1e6, "span_s": span,
            "waves": st["waves"], "device_busy_s": st["busy_s"], "fused_busy_s": st["fused_busy_s"],
            "wavefront_busy_s": st["wavefront_busy_s"]}


def _plain_renderer_run(cg, scs, bvhs, reqs, modes=None, one_call=False, burst=False):
    """The plain method: the drop-in Renderer API, one request at a time in
    arrival order. Each request gets a Renderer at its resolution, spp
    accumulate_frame_f32 calls (the reference's per-frame loop; one_call: a
    single accumulate_frames_f32 call) and a resolve_u8 read back to the host; the
    scene's kernel form is the server's default rule (wavefront for BVHs
    deeper than 40 or above 200k triangles, else the single-launch form)
    unless `modes` gives one per scene. The time of the requests is broken
    into renderer creation, the sample loop (of which the frames' device
    time is measured by CUDA events) and the resolve with its read-back."""
    if modes is None:
        modes = [cg.MODE_WAVEFRONT if (b.depth > 40 or b.triangles.shape[0] > 200000) else cg.MODE_MEGAKERNEL
                 for b in bvhs]
    parts = {"create_s": 0.0, "samples_s": 0.0, "device_s": 0.0, "resolve_s": 0.0}

    def run(sc, w, h, spp, cam, base, tally):
        t0 = time.perf_counter()
        r = cg.Renderer(scs[sc], w, h, rng_order=cg.RNG_GROUP, traversal=cg.TRAVERSE_SINGLE, mode=modes[sc],
                        use_graph=1 if modes[sc] == cg.MODE_WAVEFRONT else 0)
        r.set_camera(cam)
        t1 = time.perf_counter()
        n, dev = 0, 0.0
        for s in range(1 if one_call else spp):
            if one_call:
                r.accumulate_frames_f32(base, spp)
            else:
                r.accumulate_frame_f32(base + s)
            nr, ms = r.stats()  # rays and device time of the last call
            n += nr
            dev += ms * 1e-3
        t2 = time.perf_counter()
        r.resolve_u8(spp)
        t3 = time.perf_counter()
        if tally:
            parts["create_s"] += t1 - t0
            parts["samples_s"] += t2 - t1
            parts["device_s"] += dev
            parts["resolve_s"] += t3 - t2
        return n

    for k in range(len(scs)):  # warm-up: one small request per scene
        run(k, 64, 64, 1, reqs[0][5], 0, False)
    lat, rays = [], 0
    t0 = time.perf_counter()
    first = last = None
    for i, (at, sc, w, h, spp, cam) in enumerate(reqs):
        dt = t0 + at - time.perf_counter()
        if dt > 0 and not burst:
            time.sleep(dt)
        start = time.perf_counter()
        first = start if first is None else first
        rays += run(sc, w, h, spp, cam, i * 16, True)
        last = time.perf_counter()
        lat.append((last - (t0 if burst else t0 + at)) * 1e3)
    span = last - (t0 if burst else min(t0 + reqs[0][0], first))
    lat = np.array(lat)
    busy = parts["create_s"] + parts["samples_s"] + parts["resolve_s"]
    parts["sample_overhead_s"] = parts["samples_s"] - parts["device_s"]
    parts["idle_s"] = span - busy  # waiting for arrivals
    return {"requests": len(reqs), "latency_ms_p50": float(np.percentile(lat, 50)),
            "latency_ms_p99": float(np.percentile(lat, 99)), "mrays_per_s": rays / span / 1e6, "span_s": span,
            "breakdown": parts}


def _served_requests(cg, scenes, rate, duration, seed):
    """Poisson arrivals at `rate` per second for `duration` seconds over the
    3 scenes: camera on a radius-3 sphere around the room centre, resolution
    log-uniform 320x184..1920x1080, 1..16 spp."""
    rng = np.random.default_rng(seed)
    center = np.array([0.0, 1.25, -2.0])
    reqs, t = [], 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        z = rng.uniform(-1, 1)
        ph = rng.uniform(0, 2 * np.pi)
        eye = center + 3.0 * np.array([np.sqrt(1 - z * z) * np.cos(ph), z, np.sqrt(1 - z * z) * np.sin(ph)])
        cam = scenes.default_camera(cg.Camera(), eye=tuple(eye), target=tuple(center))
        w = int(round(np.exp(rng.uniform(np.log(320), np.log(1920)))))
        h = int(min(1080, max(184, round(w * 184 / 320))))
        reqs.append((t, int(rng.integers(0, 3)), w, h, int(rng.integers(1, 17)), cam))
    return reqs


def bench_served(cg, duration=2.0, rate=200.0, seed=4):
    """Poisson arrivals (200 req/s) over 3 resident scenes (room+sphere,
    displaced icosphere, random-walk tube); camera on a radius-3 sphere around
    the room centre, resolution log-uniform 320x184..1920x1080, 1..16 spp.
    Continuously batched server against the one-request-at-a-time path; the
    same at 100 req/s, which the server sustains (its span stays within the
    arrival window), so that its latency there is service time, not queueing."""
    from convector_gb300 import scenes
    scs, bvhs = [], []
    for gen in (scenes.room_sphere, lambda obj: scenes.displaced_icosphere(obj=obj, light=True),
                scenes.random_walk_tube):
        tris, _ = gen(obj=False)
        bvhs.append(cg.Bvh.build(tris))
        scs.append(cg.Scene(bvhs[-1]))
    reqs = _served_requests(cg, scenes, rate, duration, seed)
    # Served: the deep scene (the tube) on one high-priority engine that runs
    # its waves as single launches with paths per lane, the shallow scenes on the
    # single-launch engine beside it (measured best: 2,082 against 2,023 Mrays/s
    # for two wavefront engines with the autotuner's configuration, p99 1.38
    # against 1.61 s). The tuned wavefront engines and the server's defaults are
    # measured beside it.
    # Up to 16 samples of a request per wave, admission capped at 8M pixels
    # (measured at 200 req/s: 2,158 Mrays/s, p50 369 / p99 791 ms, against
    # 2,140 and 369 / 1,189 ms uncapped, 2,153 and 526 / 1,191 ms with one
    # sample per wave; two deep engines 2,128 and 416 / 838 ms).
    engine = {"refill_mode": cg.REFILL_ALL, "deep_single_launch": 1, "wavefront_streams": 1,
              "samples_per_wave": 16, "max_inflight_pixels": 8 << 20}
    # One sample of each request per wave, no cap (the server before sample slots).
    engine_one = dict(engine, samples_per_wave=1, max_inflight_pixels=0)
    from convector_gb300 import autotune
    wf = [k for k, b in enumerate(bvhs) if b.depth > 40 or b.triangles.shape[0] > 200000]
    wf_engine = {}
    if wf:
        scenes.default_camera(scs[wf[0]].camera)
        best, _ = autotune.tune_wavefront(scs[wf[0]], 1280, 736, frames=3)
        wf_engine = {"blocks_per_sm": best["blocks_per_sm"], "refill_mode": best["refill_mode"],
                     "wavefront_streams": 2}
    served = _served_run(cg, scs, reqs, sequential=False, engine=engine)
    served_one = _served_run(cg, scs, reqs, sequential=False, engine=engine_one)
    served_wf = _served_run(cg, scs, reqs, sequential=False, engine=wf_engine)
    served_default = _served_run(cg, scs, reqs, sequential=False)
    sequential = _served_run(cg, scs, reqs, sequential=True, engine=engine)
    # The plain path is the Renderer's default for every scene: the single
    # launch (paths per lane for the 28- and 70-level trees, one octet per
    # group for the 19-level room). Beside it, the same requests with the deep
    # scene in the wavefront form (the server's default rule for its engines).
    plain = _plain_renderer_run(cg, scs, bvhs, reqs, modes=[cg.MODE_MEGAKERNEL] * len(scs))
    plain_wf = _plain_renderer_run(cg, scs, bvhs, reqs)
    # The same plain path with each request's samples in one
    # accumulate_frames_f32 call (up to 32 samples per launch in the
    # path-refill form).
    plain_one = _plain_renderer_run(cg, scs, bvhs, reqs, modes=[cg.MODE_MEGAKERNEL] * len(scs), one_call=True)
    # Sustained throughput: the same requests all submitted at once.
    burst = {"served": _served_run(cg, scs, reqs, sequential=False, engine=engine, burst=True),
             "plain_renderer": _plain_renderer_run(cg, scs, bvhs, reqs, modes=[cg.MODE_MEGAKERNEL] * len(scs),
                                                   burst=True),
             "plain_renderer_frames_in_one_call": _plain_renderer_run(
                 cg, scs, bvhs, reqs, modes=[cg.MODE_MEGAKERNEL] * len(scs), one_call=True, burst=True)}
    burst["throughput_ratio"] = burst["served"]["mrays_per_s"] / burst["plain_renderer"]["mrays_per_s"]
    burst["throughput_ratio_vs_plain_frames_in_one_call"] = \
        burst["served"]["mrays_per_s"] / burst["plain_renderer_frames_in_one_call"]["mrays_per_s"]
    # Below saturation: half the arrival rate.
    low_rate = rate / 2
    reqs_low = _served_requests(cg, scenes, low_rate, duration, seed + 1)
    served_low = _served_run(cg, scs, reqs_low, sequential=False, engine=engine)
    plain_low = _plain_renderer_run(cg, scs, bvhs, reqs_low, modes=[cg.MODE_MEGAKERNEL] * len(scs))
    plain_one_low = _plain_renderer_run(cg, scs, bvhs, reqs_low, modes=[cg.MODE_MEGAKERNEL] * len(scs),
                                        one_call=True)
    return {"rate_per_s": rate, "duration_s": duration, "served": served, "served_engine": engine,
            "served_one_sample_per_wave": served_one, "all_at_once": burst,
            "served_wavefront_engines": served_wf, "served_wavefront_engine_config": wf_engine,
            "served_default_engine": served_default, "plain_renderer": plain,
            "plain_renderer_wavefront_for_deep": plain_wf,
            "plain_renderer_frames_in_one_call": plain_one,
            "throughput_ratio_vs_plain_frames_in_one_call": served["mrays_per_s"] / plain_one["mrays_per_s"],
            "throughput_ratio_vs_plain_wavefront_for_deep": served["mrays_per_s"] / plain_wf["mrays_per_s"],
            "server_one_at_a_time": sequential,
            "throughput_ratio": served["mrays_per_s"] / plain["mrays_per_s"],
            "throughput_ratio_wavefront_engines": served_wf["mrays_per_s"] / plain["mrays_per_s"],
            "throughput_ratio_default_engine": served_default["mrays_per_s"] / plain["mrays_per_s"],
            "throughput_ratio_vs_server_one_at_a_time": served["mrays_per_s"] / sequential["mrays_per_s"],
            "below_saturation": {"rate_per_s": low_rate, "served": served_low, "plain_renderer": plain_low,
                                 "plain_renderer_frames_in_one_call": plain_one_low,
                                 "latency_p99_ratio_plain_over_served":
                                     plain_low["latency_ms_p99"] / served_low["latency_ms_p99"]}}


def bench_bvh_build(cg):
    """Host build against the device build (same output) for the ray-cast
    scene and the ~870k-triangle tube; best of 3 wall-clock runs."""
    from convector_gb300 import scenes
    out = {}
    for name, gen in (("displaced_icosphere", lambda: scenes.displaced_icosphere(obj=False)[0]),
                      ("random_walk_tube", lambda: scenes.random_walk_tube(obj=False)[0])):
        tris = gen()
        cg.Bvh.build_device(tris[:4096])  # context and table warm-up
        th, td = [], []
        for _ in range(3):
            t0 = time.perf_counter()
            a = cg.Bvh.build(tris)
            th.append(time.perf_counter() - t0)
            t0 = time.perf_counter()
            b = cg.Bvh.build_device(tris)
            td.append(time.perf_counter() - t0)
        same = bool(np.array_equal(a.nodes, b.nodes) and np.array_equal(a.source_index, b.source_index))
        out[name] = {"triangles": int(tris.shape[0]), "host_ms": 1e3 * min(th), "device_ms": 1e3 * min(td),
                     "host_threads": os.cpu_count(), "identical": same}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-render", action="store_true")
    ap.add_argument("--no-cpu-frames", action="store_true",
                    help="leave out the oracle's CPU frame baselines of the render and large sections")
    ap.add_argument("--no-extra", action="store_true", help="skip the large, batched and served sections")
    ap.add_argument("--launch", help="query configuration (packet8/0, single/8, single/8/s0, single/8/s4, "
                                     "single/8/s12, single/10, single/12) instead of the fastest of a short trial")
    ap.add_argument("--section", choices=["render", "large", "batched", "served", "bvh", "frame-room", "frame-tube",
                                          "frame-tube-multi"],
                    help="run one extra section alone and print its JSON (no headline line)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    global CPU_BASELINE
    CPU_BASELINE = not args.no_cpu_frames
    if args.section:
        import convector_gb300 as cg
        cg.lib(build=True)
        fn = {"render": bench_render, "large": bench_large, "batched": bench_batched, "served": bench_served,
              "bvh": bench_bvh_build, "frame-room": lambda c: bench_frame_kernel(c, "room"),
              "frame-tube": lambda c: bench_frame_kernel(c, "tube"),
              "frame-tube-multi": lambda c: bench_frame_kernel(c, "tube-multi")}
        print(json.dumps({args.section: fn[args.section](cg)}))
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
