"""Golden fixtures (tests/golden/, made by make_fixtures.py).

CPU: the oracle's rcp / rsqrt emulation against results recorded from the
x86 hardware instructions, and the oracle's small frame against its fixture.
On an x86-64 host the table generator is also rebuilt and re-checked against
the instruction it stands in for. GPU: the kernels against the frame fixture.
"""

import os
import platform
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
CSRC = os.path.join(os.path.dirname(HERE), "convector_gb300", "csrc")


def test_oracle_approx_matches_recorded_x86(orc):
    g = np.load(os.path.join(GOLDEN, "x86_approx_vectors.npz"))
    L = orc.lib()
    xs = g["x"].view(np.float32)
    rcp = np.array([L.orc_rcp(float(x)) for x in xs], np.float32).view(np.uint32)
    rsq = np.array([L.orc_rsqrt(float(x)) for x in xs], np.float32).view(np.uint32)
    # ctypes passes floats through double: NaN payloads survive, signalling NaNs may be quieted
    nan = np.isnan(xs)
    assert (rcp[~nan] == g["rcp"][~nan]).all()
    assert (rsq[~nan] == g["rsqrt"][~nan]).all()
    assert np.isnan(rcp[nan].view(np.float32)).all() and np.isnan(rsq[nan].view(np.float32)).all()


@pytest.mark.skipif(platform.machine() not in ("x86_64", "AMD64"), reason="needs the x86 instructions")
def test_table_generator_against_hardware(tmp_path):
    exe = str(tmp_path / "gen")
    subprocess.check_call(["gcc", "-O2", "-mavx2", os.path.join(CSRC, "gen_x86_approx_tables.c"), "-o", exe])
    out = subprocess.run([exe], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, check=True)
    assert "emulation matches hardware" in out.stderr
    assert out.stdout == open(os.path.join(CSRC, "x86_approx_tables.h")).read()


def test_oracle_small_frame_fixture(orc):
    g = np.load(os.path.join(GOLDEN, "frame_small.npz"))
    osc = orc.OracleScene(g["triangles"], g["nodes"])
    for order in (0, 1):
        rgba, gb, col, rays = osc.render(g["camera"], int(g["width"]), int(g["height"]), int(g["frame"]),
                                         rng_order=order)
        assert (rgba == g["rgba%d" % order]).all() and (gb == g["gbuffer%d" % order]).all()
        assert (col.view(np.uint32) == g["color%d" % order].view(np.uint32)).all()
        assert rays == int(g["rays%d" % order][0])


@pytest.mark.gpu
def test_gpu_small_frame_fixture(gpu):
    traversal = 0
    g = np.load(os.path.join(GOLDEN, "frame_small.npz"))
    bvh_t, bvh_n = g["triangles"], g["nodes"]

    class _Bvh:
        triangles, nodes = np.ascontiguousarray(bvh_t), np.ascontiguousarray(bvh_n)

    scene = gpu.Scene(_Bvh)
    cam = g["camera"]
    scene.camera.set_position(cam[0:3], cam[3:6])
    scene.camera.set_orientation(cam[6:10], cam[10:14])
    for order in (0, 1):
        r = gpu.Renderer(scene, int(g["width"]), int(g["height"]), rng_order=order, traversal=traversal)
        rgba, gb = r.render_frame_u8(int(g["frame"]))
        col = r.read_frame_f32()
        assert (rgba == g["rgba%d" % order]).all() and (gb == g["gbuffer%d" % order]).all()
        assert (col.view(np.uint32) == g["color%d" % order].view(np.uint32)).all()
        assert r.stats()[0] == int(g["rays%d" % order][0])
