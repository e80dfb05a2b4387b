"""Host-side boundary tests (no GPU): C-ABI exports, OBJ loading, BVH build,
camera setters and the procedural scenes."""

import ctypes
import math
import os
import re

import numpy as np
import pytest

from convector_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# The reference checkout (its models/ folder), where one is available: tests
# that read the reference's own files skip without it.
REFERENCE = os.environ.get("CONVECTOR_REFERENCE", "")
HAVE_MODELS = bool(REFERENCE) and os.path.isdir(os.path.join(REFERENCE, "models"))


def test_library_exports_every_declared_symbol(cvx):
    decls = set()
    inc = os.path.join(ROOT, "include")
    for name in os.listdir(inc):
        if name.endswith(".h"):
            text = open(os.path.join(inc, name)).read()
            decls |= set(re.findall(r"\b(cvx_[a-z0-9_]+)\s*\(", text))
    assert len(decls) > 30
    L = ctypes.CDLL(cvx._build.LIB)
    missing = [d for d in sorted(decls) if not hasattr(L, d)]
    assert not missing, missing


def test_obj_fan_triangulation_and_tex_coords(cvx):
    text = "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvt 0 0\nvt 1 0\nvt 1 1\nvt 0 1\nf 1/1 2/2 3/3 4/4\n"
    # a second quad far away, so that the root splits (bvh.rs:509-512)
    text += "v 50 0 0\nv 51 0 0\nv 51 1 0\nv 50 1 0\nf 5 6 7 8\n"
    m = cvx.Mesh.parse(text)
    assert m.num_triangles == 4
    bvh = cvx.Bvh.from_meshes([m])
    tris = bvh.triangles_f32
    assert sorted(bvh.source_index.tolist()) == [0, 1, 2, 3]
    t1 = tris[list(bvh.source_index).index(1)]
    # second fan triangle is (v0, v2, v3) with tex coords (t0, t2, t3) (wavefront.rs:132-139)
    assert t1[0:9].tolist() == [0, 0, 0, 1, 1, 0, 0, 1, 0]
    assert t1[9:15].tolist() == [0, 0, 1, 1, 0, 1]
    assert bvh.triangles[0, 15] == cvx.SMaterial.white()


def test_obj_errors(cvx):
    ok = "v 0 0 0\nv 1 0 0\nv 0 1 0\n"
    with pytest.raises(cvx.CvxError, match="degenerate"):
        cvx.Mesh.parse("v 0 0 0\nv 1 0 0\nv 2 0 0\nf 1 2 3\n")
    with pytest.raises(cvx.CvxError, match="not present"):
        cvx.Mesh.parse(ok + "usemtl nope\nf 1 2 3\n")
    with pytest.raises(cvx.CvxError, match="out of range"):
        cvx.Mesh.parse(ok + "f 1 2 4\n")
    with pytest.raises(cvx.CvxError, match="bad face index"):
        cvx.Mesh.parse(ok + "f 1//1 2 3\n")
    with pytest.raises(cvx.CvxError, match="bad vertex"):
        cvx.Mesh.parse("v 0 x 0\n")
    with pytest.raises(cvx.CvxError) as e:
        cvx.Mesh.load("/nonexistent/file.obj")
    assert e.value.status == 2
    m = cvx.Mesh.parse(ok + "usemtl glass\nf 1 2 3\n", {"glass": cvx.SMaterial.sky()})
    assert m.num_triangles == 1


@pytest.mark.skipif(not HAVE_MODELS, reason="CONVECTOR_REFERENCE (the reference checkout) not set")
@pytest.mark.parametrize("name,mats,count", [
    ("box_walls.obj", {"wall": 0x00ffffff, "glass": 0xC0000000}, 204),
    ("suzanne.obj", {}, 968),
    ("stanford_bunny.obj", {}, 69666),
    ("stanford_dragon.obj", {}, 100000),
])
def test_reference_models_load(cvx, name, mats, count):  # wavefront.rs:155-179
    m = cvx.Mesh.load_with_materials(os.path.join(REFERENCE, "models", name), mats)
    assert m.num_triangles == count


@pytest.mark.skipif(not HAVE_MODELS, reason="CONVECTOR_REFERENCE (the reference checkout) not set")
def test_reference_indoor_scene(cvx):
    """The reference's own interactive scene (main.rs:70-88): 284 triangles,
    8 direct-sample "glass" triangles, which is what the reference's light
    pick `bits >> 29` needs (scene.rs:147-161)."""
    from convector_gb300 import scenes
    m = cvx.Mesh.load_with_materials(os.path.join(REFERENCE, "models", "indoor.obj"), scenes.reference_materials())
    assert m.num_triangles == 284
    bvh = cvx.Bvh.from_meshes([m])
    assert bvh.direct_sample.shape[0] == 8
    _check_bvh(bvh, 284)


def _check_bvh(bvh, n_src):
    nodes, tris = bvh.nodes, bvh.triangles
    f = bvh.nodes_f32
    tf = bvh.triangles_f32
    assert nodes.shape[0] % 2 == 0
    assert sorted(bvh.source_index.tolist()) == list(range(n_src))  # a permutation, no duplicates
    covered = np.zeros(tris.shape[0], np.int64)
    stack = [0, 1]
    seen = 0
    while stack:
        i = stack.pop()
        seen += 1
        lo, hi = f[i, 0:3], f[i, 3:6]
        idx, ln = nodes[i, 6], nodes[i, 7]
        if ln == 0:
            assert idx % 2 == 0 and idx >= 2
            for c in (idx, idx + 1):
                assert (f[c, 0:3] >= lo).all() and (f[c, 3:6] <= hi).all()
                stack.append(c)
            # an internal box encloses its children exactly (Aabb::enclose_aabbs, aabb.rs:185-192)
            assert (np.minimum(f[idx, 0:3], f[idx + 1, 0:3]) == lo).all()
            assert (np.maximum(f[idx, 3:6], f[idx + 1, 3:6]) == hi).all()
        else:
            covered[idx:idx + ln] += 1
            v = tf[idx:idx + ln, 0:9].reshape(-1, 3)
            assert (v >= lo).all() and (v <= hi).all()
            # the node box is the tight box of its triangles (bvh.rs:125-132)
            assert (v.min(0) == lo).all() and (v.max(0) == hi).all()
    assert seen == nodes.shape[0]
    assert (covered == 1).all()


def _area(lo, hi):
    s = (hi - lo).astype(np.float32)
    return np.float32(2.0) * (s[1] * s[2] + s[2] * s[0] + s[0] * s[1])


def test_area_known_answer():  # aabb.rs:194-199: width 4, height 5, depth 6
    assert _area(np.array([1, 2, 3], np.float32), np.array([5, 7, 9], np.float32)) == 40.0 + 60.0 + 48.0


def test_bvh_invariants_room_sphere(cvx):
    from convector_gb300 import scenes
    text, mats = scenes.room_sphere()
    mesh = cvx.Mesh.parse(text, mats)
    assert mesh.num_triangles == 10 + 4960 + 2
    bvh = cvx.Bvh.from_meshes([mesh])
    _check_bvh(bvh, mesh.num_triangles)
    assert bvh.direct_sample.shape[0] == 2
    # smaller-area child first (bvh.rs:343-345)
    f = bvh.nodes_f32
    for i in range(bvh.nodes.shape[0]):
        if bvh.nodes[i, 7] == 0:
            c = bvh.nodes[i, 6]
            assert _area(f[c, 0:3], f[c, 3:6]) <= _area(f[c + 1, 0:3], f[c + 1, 3:6])


def test_bvh_build_is_deterministic(cvx):
    from convector_gb300 import scenes
    text, mats = scenes.spheres_and_boxes(3000, seed=3)
    m = cvx.Mesh.parse(text, mats)
    a, b = cvx.Bvh.from_meshes([m]), cvx.Bvh.from_meshes([m])
    assert (a.nodes == b.nodes).all() and (a.triangles == b.triangles).all()
    _check_bvh(a, m.num_triangles)


def test_bvh_needs_a_root_split(cvx):
    m = cvx.Mesh.parse("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    with pytest.raises(cvx.CvxError, match="root"):
        cvx.Bvh.from_meshes([m])


def test_query_ray_limit_is_checked_first(cvx):
    # Counts above 2^31 would let the 32-bit ray counters of the query kernels
    # wrap; both query forms refuse them before touching the scene or a buffer.
    L = cvx.lib()
    n = 2**31 + 1
    st = L.cvx_intersect_nearest(None, None, None, None, None, None, None, n, 1e5, 1, None, None)
    assert st == 1
    with pytest.raises(cvx.CvxError, match="2\\^31"):
        cvx._check(st)
    st = L.cvx_intersect_nearest_device(None, None, n, 1e5, 1, None, None, None, None)
    assert st == 1
    with pytest.raises(cvx.CvxError, match="2\\^31"):
        cvx._check(st)
    # At the limit the next check (the null scene) answers instead.
    st = L.cvx_intersect_nearest(None, None, None, None, None, None, None, 2**31, 1e5, 1, None, None)
    with pytest.raises(cvx.CvxError, match="null"):
        cvx._check(st)


def test_size_limits_refused_before_work(cvx):
    # Checked on the host before any triangle is read or any device call is made.
    L = cvx.lib()
    tri = np.zeros(16, np.uint32)
    out = ctypes.c_void_p()
    with pytest.raises(cvx.CvxError, match="2\\^27"):
        cvx._check(L.cvx_bvh_build(cvx._ptr(tri), 1 << 27, ctypes.byref(out)))
    tex = np.zeros(3, np.uint8)
    for w, h, tw, th in ((16385, 16, 1, 1), (16, 16385, 1, 1), (16, 16, 16385, 1), (16, 16, 1, 16385)):
        with pytest.raises(cvx.CvxError, match="16384"):
            cvx._check(L.cvx_display_create(w, h, cvx._ptr(tex), cvx._ptr(tex), tw, th, ctypes.byref(out)))
    assert not out.value


def test_wrapper_buffer_checks(cvx):
    # The Python mirror refuses buffers the library would read or write past
    # their end, before any call into it.
    o = np.zeros((10, 3), np.float32)
    n, cols = cvx._host_rays(o, np.ones((10, 3)))
    assert n == 10 and len(cols) == 6 and all(c.dtype == np.float32 and c.shape == (10,) for c in cols)
    for bad in (np.ones((9, 3)), np.ones((10, 2)), np.ones(30)):
        with pytest.raises(ValueError):
            cvx._host_rays(o, bad)
    with pytest.raises(ValueError):
        cvx._host_rays(np.zeros(30), np.zeros(30))
    good = np.zeros((4, 16), np.uint32)
    assert cvx._frame_buffer(good, 4, 16, "rgba") is good
    for bad in (np.zeros((4, 15), np.uint32), np.zeros((4, 16), np.int64), np.zeros((16, 4), np.uint32).T,
                np.zeros(64, np.uint32)):
        with pytest.raises(ValueError):
            cvx._frame_buffer(bad, 4, 16, "rgba")
    torch = pytest.importorskip("torch")
    with pytest.raises(ValueError):  # a host tensor
        cvx._device_tensor(torch.zeros(8), "t_out", 8, True)


def test_icosphere_counts():
    from convector_gb300 import scenes
    v, f = scenes.icosphere(6)
    assert f.shape[0] == 81920
    assert v.shape[0] == 40962


def test_camera_setters(cvx):
    c = cvx.Camera()
    a = c.as_array()
    assert a[6:10].tolist() == [1, 0, 0, 0]
    assert abs(a[14] - 1.0 / math.sin(math.pi / 5)) < 1e-6
    c.set_rotation(1.0, 0.5)
    a = c.as_array()
    assert abs(a[6] - math.cos(0.5)) < 1e-6 and abs(a[8] + math.sin(0.5)) < 1e-6
    assert abs(a[10] - 0.5 * -math.sin(0.5) * 0.5) < 1e-6


def test_look_at_quaternion(orc):
    from convector_gb300 import scenes
    from oracle.oracle import f32
    for eye, target in [((0, 1.2, 1.6), (0, 1, -2)), ((3, 0.5, 0.2), (0, 1, -2)), ((0.1, -2, 0.3), (0, 1, 0))]:
        q = f32(*scenes.look_at_quaternion(eye, target))
        v, out = f32(0, 0, -1), np.zeros(3, np.float32)
        orc.lib().orc_quat_rotate(v.ctypes.data, q.ctypes.data, out.ctypes.data)
        want = np.array(target, float) - np.array(eye, float)
        assert np.allclose(out, want / np.linalg.norm(want), atol=1e-5)


def test_materials_encoding(cvx):  # material.rs:84-136
    M = cvx.SMaterial
    assert M.sky() == 0xC0000000 and M.is_direct_sample(M.sky())
    assert M.white() == 0x00FFFFFF
    assert M.with_glossiness(M.white(), 4) == 0x10FFFFFF
    assert M.with_texture(M.white(), 2) == 0x02FFFFFF
    assert M.diffuse(1.0, 0.1, 0.4) == (0x66 << 16) | (0x19 << 8) | 0xFF


@pytest.mark.parametrize("gen", ["room_sphere", "spheres_and_boxes"])
def test_scene_triangle_arrays_equal_loaded_obj(cvx, gen):
    """The direct triangle arrays are what the OBJ loader gives for the same scene."""
    from convector_gb300 import scenes
    args = (1500, 9) if gen == "spheres_and_boxes" else ()
    text, mats = getattr(scenes, gen)(*args)
    tris, _ = getattr(scenes, gen)(*args, obj=False)
    a = cvx.Bvh.from_meshes([cvx.Mesh.parse(text, mats)])
    b = cvx.Bvh.build(tris)
    assert (a.triangles == b.triangles).all() and (a.nodes == b.nodes).all()


def _parse_with_threads(cvx, monkeypatch, text, mats, threads):
    monkeypatch.setenv("CONVECTOR_OBJ_THREADS", str(threads))
    try:
        m = cvx.Mesh.parse(text, mats)
    except cvx.CvxError as e:
        return ("error", e.status, str(e))
    b = cvx.Bvh.from_meshes([m])
    return ("ok", m.num_triangles, b.triangles.tobytes(), b.nodes.tobytes(), b.source_index.tobytes())


@pytest.mark.parametrize("threads", [2, 3, 7, 16, 61])
def test_parallel_obj_parse_equals_sequential(cvx, monkeypatch, threads):
    """The chunked parser gives the sequential parser's mesh (materials carried
    across chunk boundaries, vertex indices checked against the vertices
    defined before each face) on a mixed scene with quads and tex coords."""
    text, mats = scenes.room_sphere()
    extra = "".join("vt %d 0.5\n" % k for k in range(5)) + "usemtl wall\n" + "f 1/1 2/2 3/3 4/4\n" * 3
    text = text + extra
    seq = _parse_with_threads(cvx, monkeypatch, text, mats, 1)
    assert seq[0] == "ok"
    assert _parse_with_threads(cvx, monkeypatch, text, mats, threads) == seq


@pytest.mark.parametrize("threads", [2, 5, 13])
def test_parallel_obj_parse_reports_the_first_error(cvx, monkeypatch, threads):
    """Whichever chunk holds it, the first error in file order is the one
    reported, with the sequential parser's status, message and line."""
    text, mats = scenes.room_sphere()
    lines = text.splitlines(keepends=True)
    n = len(lines)
    cases = []
    for frac in (0.1, 0.5, 0.9):
        at = int(n * frac)
        # a face before its vertices exist, then a tokenising error later
        cases.append(lines[:at] + ["f 1 2 999999\n"] + lines[at:at + 40] + ["v 0 zz 0\n"] + lines[at + 40:])
        # a tokenising error first, then a degenerate face
        cases.append(lines[:at] + ["usemtl nosuch\n"] + lines[at:] + ["v 9 9 9\nf 1 1 2\n"])
        # degenerate face only
        cases.append(lines[:at] + ["f 1 1 2\n"] + lines[at:])
    for c in cases:
        t = "".join(c)
        seq = _parse_with_threads(cvx, monkeypatch, t, mats, 1)
        assert seq[0] == "error"
        assert _parse_with_threads(cvx, monkeypatch, t, mats, threads) == seq


def test_parallel_obj_parse_edge_inputs(cvx, monkeypatch):
    def count(text, threads):
        monkeypatch.setenv("CONVECTOR_OBJ_THREADS", str(threads))
        return cvx.Mesh.parse(text).num_triangles

    for text, n in [("", 0), ("\n\n", 0), ("v 0 0 0", 0), ("# only a comment\r\n", 0),
                    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3", 1), ("v 0 0 0\r\nv 1 0 0\r\nv 0 1 0\r\nf 1 2 3\r\n", 1)]:
        for threads in (1, 2, 8, 64):
            assert count(text, threads) == n, (text, threads)


@pytest.mark.parametrize("tok", ["1.", ".5", "+1.5", "-0", "1e-50", "2.5e+1", "7E-1", "0.1", "1234567.891",
                                 "0.30000001192092896", "16777217", "1e-40"])
def test_obj_vertex_coordinates_round_like_rust(cvx, tok):
    """Coordinates are parsed as f32::from_str does: correctly rounded, with a
    leading '+', a bare fraction or exponent, and subnormal results."""
    quad = "v 50 0 0\nv 51 0 0\nv 51 1 0\nv 50 1 0\nf 4 5 6 7\n"
    m = cvx.Mesh.parse("v %s 0 0\nv 1 1 0\nv 0 1 1\nf 1 2 3\n" % tok + quad)
    b = cvx.Bvh.from_meshes([m])
    t = b.triangles_f32[list(b.source_index).index(0)]
    assert t[0] == np.float32(float(tok))


@pytest.mark.parametrize("tok,ok", [("1e50", True), ("inf", True), ("-inf", True), ("NaN", True),
                                    ("0x1p3", False), ("1.0f", False), ("--1", False), ("+-1", False),
                                    ("1e", False), (".", False), ("e5", False)])
def test_obj_vertex_coordinate_syntax(cvx, tok, ok):
    text = "v %s 0 0\n" % tok
    if ok:
        assert cvx.Mesh.parse(text).num_triangles == 0
    else:
        with pytest.raises(cvx.CvxError, match="bad vertex coordinate"):
            cvx.Mesh.parse(text)


@pytest.mark.parametrize("time,delta", [(0.0, 0.0), (12.5, 0.016), (-3.0, 0.05), (1000.0, 1.0)])
def test_interactive_camera_path(cvx, time, delta):
    """renderer.rs:140-147 and scene.rs:47-74 in f32, with the sinf/cosf of the
    C library the product is linked against."""
    libm = ctypes.CDLL(None)
    for name in ("sinf", "cosf"):
        getattr(libm, name).restype = ctypes.c_float
        getattr(libm, name).argtypes = [ctypes.c_float]
    f = np.float32
    alpha = f(f(f(time) * f(-0.02)) + f(0.1))
    ad = f(f(delta) * f(-0.02))
    sa, ca = f(libm.sinf(alpha)), f(libm.cosf(alpha))
    c = cvx.Camera().set_interactive(time, delta)
    assert np.array(c._c.position, np.float32).tolist() == [f(f(-3.8) * sa), f(1.6), f(f(3.0) * ca)]
    pd = np.array(c._c.position_delta, np.float32)
    assert pd.tobytes() == np.array([f(f(f(-3.8) * ca) * ad), f(f(0.0) * ad), f(f(f(-3.0) * sa) * ad)],
                                    np.float32).tobytes()
    r = cvx.Camera()
    r.set_rotation(float(alpha), float(ad))
    assert np.array(c._c.orientation, np.float32).tobytes() == np.array(r._c.orientation, np.float32).tobytes()
    assert np.array(c._c.orientation_delta, np.float32).tobytes() == \
        np.array(r._c.orientation_delta, np.float32).tobytes()


def test_device_info_without_a_device(cvx):
    # Nothing falls back to the CPU: without a usable device the call reports CVX_ERR_CUDA.
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(cvx.CvxError) as e:
        cvx.device_info()
    assert e.value.status == 5
