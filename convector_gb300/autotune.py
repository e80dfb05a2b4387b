"""Autotuner for the render path: times candidate kernel organisations on the
actual scene and frame size and keeps the fastest.

Frames (tune): candidates (all give the same image for a given RNG order and
traversal; the single-ray and packet traversals can differ only on t-ties and
grazing rays): the fused megakernel at several block sizes with one octet per
8-pixel group, the fused megakernel with paths per lane and ray refill, and the
wavefront form with CUDA-graph replay at several persistent grid sizes and
ray-refill modes, each with the single-ray and the 8-ray packet traversal.

Nearest-hit queries (tune_query): the packet traversal and the single-ray
kernel at 8, 10 and 12 resident blocks per SM and, at 8 blocks, with 0, 4, 8
or 12 of each lane's stack entries in shared memory (the stack depth knob: the
rest of the 128-entry stack is local memory, and shared entries take shared
memory from L1, so the best depth depends on the tree).

Results are cached per (GPU model, library build, scene size, BVH depth, frame
size, RNG order) in a JSON file (CONVECTOR_AUTOTUNE_CACHE, default
~/.cache/convector_gb300/autotune.json), so a choice timed on another GPU model
or with other kernels is not reused.
"""

import json
import os

from . import (MODE_MEGAKERNEL, MODE_WAVEFRONT, REFILL_AFTER_CAMERA, REFILL_ALL, REFILL_NONE, RNG_GROUP,
               TRAVERSE_PACKET, TRAVERSE_SINGLE, Renderer, _build, device_info)


def _cache_path():
    return os.environ.get("CONVECTOR_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "convector_gb300", "autotune.json"))


def _build_key():
    """The GPU model and the identity (size, modification time) of the loaded library."""
    st = os.stat(_build.LIB)
    return "gpu=%s lib=%d:%d" % (device_info()[1], st.st_size, int(st.st_mtime))


def candidates(rng_order=RNG_GROUP, allow_packet=True):
    """Render configurations (keyword dicts for Renderer) to try."""
    out = []
    travs = [TRAVERSE_SINGLE, TRAVERSE_PACKET] if allow_packet else [TRAVERSE_SINGLE]
    for trav in travs:
        for block in (64, 128):  # the fused kernels are compiled for at most 128 threads per block
            out.append(dict(rng_order=rng_order, traversal=trav, mode=MODE_MEGAKERNEL, block_size=block,
                            refill_mode=REFILL_NONE))
    if rng_order == RNG_GROUP:  # single launch with paths per lane (its block is fixed at 128)
        out.append(dict(rng_order=rng_order, traversal=TRAVERSE_SINGLE, mode=MODE_MEGAKERNEL, refill_mode=REFILL_ALL))
    if rng_order == RNG_GROUP:
        for bps in (8, 12, 16):
            for refill in (REFILL_AFTER_CAMERA, REFILL_ALL, REFILL_NONE):
                out.append(dict(rng_order=rng_order, traversal=TRAVERSE_SINGLE, mode=MODE_WAVEFRONT, use_graph=1,
                                blocks_per_sm=bps, refill_mode=refill))
            if allow_packet:
                out.append(dict(rng_order=rng_order, traversal=TRAVERSE_PACKET, mode=MODE_WAVEFRONT, use_graph=1,
                                blocks_per_sm=bps))
    return out


def measure(scene, width, height, config, frames=5, warmup=2, first_frame=1000):
    """Median device milliseconds per frame of one configuration."""
    r = Renderer(scene, width, height, **config)
    for f in range(warmup):
        r.render_frame_u8(first_frame + f, gbuffer=False)
    ms = []
    for f in range(frames):
        r.render_frame_u8(first_frame + warmup + f, gbuffer=False)
        ms.append(r.stats()[1])
    ms.sort()
    return ms[len(ms) // 2]


def tune(scene, width, height, rng_order=RNG_GROUP, allow_packet=True, frames=5, use_cache=True):
    """Returns (best config dict, {config key: ms}) for this scene and frame size."""
    b = scene.bvh
    key = None
    if use_cache:
        key = "%s tris=%d nodes=%d depth=%d %dx%d rng=%d packet=%d" % (
            _build_key(), b.triangles.shape[0], b.nodes.shape[0], b.depth, width, height, rng_order,
            int(allow_packet))
    path = _cache_path()
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            with open(path) as f:
                cache = json.load(f)
        except (OSError, ValueError):
            cache = {}
    if use_cache and key in cache:
        return cache[key]["best"], cache[key]["table"]
    table = {}
    best, best_ms = None, None
    for cfg in candidates(rng_order, allow_packet):
        ms = measure(scene, width, height, cfg, frames=frames)
        table[json.dumps(cfg, sort_keys=True)] = ms
        if best_ms is None or ms < best_ms:
            best, best_ms = cfg, ms
    if use_cache:
        cache[key] = {"best": best, "table": table}
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            with open(path, "w") as f:
                json.dump(cache, f, indent=1, sort_keys=True)
        except OSError:
            pass
    return best, table


def tune_wavefront(scene, width, height, frames=5):
    """The fastest single-ray wavefront configuration (blocks per SM, refill
    mode) for this scene: what a batch or server engine running the scene in
    wavefront mode should use. Returns (config dict, {config key: ms})."""
    table = {}
    best, best_ms = None, None
    for cfg in candidates(RNG_GROUP, allow_packet=False):
        if cfg["mode"] != MODE_WAVEFRONT:
            continue
        ms = measure(scene, width, height, cfg, frames=frames)
        table[json.dumps(cfg, sort_keys=True)] = ms
        if best_ms is None or ms < best_ms:
            best, best_ms = cfg, ms
    return best, table


def autotuned_renderer(scene, width, height, rng_order=RNG_GROUP, allow_packet=True):
    best, _ = tune(scene, width, height, rng_order=rng_order, allow_packet=allow_packet)
    return Renderer(scene, width, height, **best)


# (name, traversal, blocks per SM, shared stack entries) of the query candidates
QUERY_SHAPES = [("packet8/0", TRAVERSE_PACKET, 0, 8)] + [
    ("single/%d%s" % (bps, "" if st == 8 else "/s%d" % st), TRAVERSE_SINGLE, bps, st)
    for bps, st in ((8, 8), (8, 0), (8, 4), (8, 12), (10, 8), (12, 8))]


def tune_query(scene, rays_soa, t_out, tri_out, shapes=None, repeats=3):
    """Times the nearest-hit query configurations (QUERY_SHAPES, or the named
    subset `shapes`) on these device rays (a (6, n) float32 CUDA tensor; t_out
    and tri_out its output tensors) on the current CUDA stream, leaves the
    scene set to the fastest and returns (its name, {name: ms per query})."""
    import torch
    stream = torch.cuda.current_stream()
    table = {}
    for name, trav, bps, stack in QUERY_SHAPES:
        if shapes is not None and name not in shapes:
            continue
        scene.set_query_launch(bps)
        scene.set_query_stack(stack)
        for _ in range(2):
            scene.intersect_nearest_device(rays_soa, t_out, tri_out, traversal=trav, stream=stream.cuda_stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(repeats):
            scene.intersect_nearest_device(rays_soa, t_out, tri_out, traversal=trav, stream=stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        table[name] = e0.elapsed_time(e1) / repeats
    if not table:
        raise ValueError("no query configuration named %s" % (shapes,))
    best = min(table, key=table.get)
    _, trav, bps, stack = next(q for q in QUERY_SHAPES if q[0] == best)
    scene.set_query_launch(bps)
    scene.set_query_stack(stack)
    return best, table


def query_traversal(name):
    """The traversal (TRAVERSE_*) of a QUERY_SHAPES name."""
    return next(q[1] for q in QUERY_SHAPES if q[0] == name)
