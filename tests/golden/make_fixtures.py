"""Generates the golden fixtures in this directory. Run on an x86-64 host:

    python tests/golden/make_fixtures.py

x86_approx_vectors.npz: inputs and the hardware's VRCPPS / VRSQRTPS results
    (the instructions behind the reference's recip_fast and rsqrt, simd.rs:
    254-256 and 309-311), recorded by a small C program with AVX intrinsics:
    special values, every exponent, and seeded random bit patterns. These pin
    the table emulation on machines without the instruction.
frame_small.npz: a small room-and-sphere scene (BVH-order triangles and nodes,
    so that the fixture does not depend on the host's libm in the build), a
    camera, and the oracle's frame 42 in both RNG orders: RGBA, gbuffer,
    linear colour and the ray count.
"""

import os
import platform
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

C_SRC = r"""
#include <immintrin.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
int main(int argc, char** argv) {
    FILE* in = fopen(argv[1], "rb"); FILE* out = fopen(argv[2], "wb");
    uint32_t x[8];
    while (fread(x, 4, 8, in) == 8) {
        __m256 v; memcpy(&v, x, 32);
        __m256 r = _mm256_rcp_ps(v), s = _mm256_rsqrt_ps(v);
        fwrite(&r, 4, 8, out); fwrite(&s, 4, 8, out);
    }
    fclose(in); fclose(out); return 0;
}
"""


def x86_vectors():
    if platform.machine() not in ("x86_64", "AMD64"):
        raise SystemExit("the x86 vectors must be recorded on an x86-64 host")
    rng = np.random.default_rng(20161203)
    special = [0, 0x80000000, 1, 0x80000001, 0x007FFFFF, 0x00800000, 0x00800001, 0x7F7FFFFF, 0x7F000000,
               0x7E800000, 0x7E7FFFFF, 0x7E000000, 0x7F800000, 0xFF800000, 0x7FC00000, 0x7F800001, 0xFFC00000,
               0x3F800000, 0xBF800000, 0x3F7FFFFF, 0x40000000, 0xBF000000]
    exps = [(e << 23) | int(m) for e in range(256) for m in rng.integers(0, 1 << 23, 8)]
    exps += [0x80000000 | v for v in exps[::5]]
    rnd = rng.integers(0, 1 << 32, 12288, dtype=np.uint64).tolist()
    xs = np.array(special + exps + rnd, dtype=np.uint32)
    xs = np.concatenate([xs, np.zeros((-len(xs)) % 8, np.uint32)])
    with tempfile.TemporaryDirectory() as td:
        src, exe = os.path.join(td, "v.c"), os.path.join(td, "v")
        open(src, "w").write(C_SRC)
        subprocess.check_call(["gcc", "-O1", "-mavx2", src, "-o", exe])
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        xs.tofile(fin)
        subprocess.check_call([exe, fin, fout])
        res = np.fromfile(fout, dtype=np.uint32).reshape(-1, 2, 8)
    rcp = res[:, 0, :].reshape(-1)
    rsq = res[:, 1, :].reshape(-1)
    np.savez_compressed(os.path.join(HERE, "x86_approx_vectors.npz"), x=xs, rcp=rcp, rsqrt=rsq)
    print("x86_approx_vectors.npz: %d inputs" % xs.shape[0])


def small_scene_text():
    from convector_gb300 import scenes
    w = scenes.ObjWriter()
    scenes._room(w)
    w.material("fauteuil")
    v, f = scenes.uv_sphere((0.0, 0.5, -2.0), 0.5, 16, 8)
    w.faces(f, w.vertices(v))
    scenes._ceiling_light(w)
    return w.text(), scenes.reference_materials()


def frame_small():
    import convector_gb300 as cg
    from convector_gb300 import scenes
    from oracle import oracle as orc
    text, mats = small_scene_text()
    bvh = cg.Bvh.from_meshes([cg.Mesh.parse(text, mats)])
    cam = scenes.default_camera(cg.Camera()).as_array()
    osc = orc.OracleScene(bvh.triangles, bvh.nodes)
    out = {"triangles": bvh.triangles, "nodes": bvh.nodes, "camera": cam, "width": 96, "height": 64, "frame": 42}
    for order in (0, 1):
        rgba, gb, col, rays = osc.render(cam, 96, 64, 42, rng_order=order)
        out["rgba%d" % order], out["gbuffer%d" % order], out["color%d" % order] = rgba, gb, col
        out["rays%d" % order] = np.array([rays], np.uint64)
    np.savez_compressed(os.path.join(HERE, "frame_small.npz"), **out)
    print("frame_small.npz: %d triangles" % bvh.triangles.shape[0])


if __name__ == "__main__":
    x86_vectors()
    frame_small()
