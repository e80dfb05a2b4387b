"""The reference's own unit tests, ported to the oracle (CPU, no GPU).

Each test cites the reference test it ports. The reference's random inputs
come from an unseeded generator (bench.rs:23-223); here they are seeded.
"""

import math

import numpy as np
import pytest

from oracle.oracle import f32


def _biunit(n, seed=0):
    return np.random.default_rng(seed).uniform(-1.0, 1.0, n).astype(np.float32)


def _unit_sphere(n, seed):
    rng = np.random.default_rng(seed)
    phi = rng.uniform(0, 2 * math.pi, n)
    ct = rng.uniform(-1, 1, n)
    st = np.sqrt(1 - ct * ct)
    return np.stack([np.cos(phi) * st, np.sin(phi) * st, ct], 1).astype(np.float32)


def test_recip_precise(orc):  # simd.rs:709-726
    L = orc.lib()
    for x in _biunit(4096, 1):
        if x == 0:
            continue
        approx = np.float32(L.orc_recip_precise(float(x)))
        expected = np.float32(1.0) / x
        assert abs(1.0 - approx / expected) < 1e-6


@pytest.mark.parametrize("fn,ref,tol", [("orc_cos", math.cos, 0.0021), ("orc_sin", math.sin, 0.0082)])
def test_sin_cos(orc, fn, ref, tol):  # simd.rs:728-770
    f = getattr(orc.lib(), fn)
    for x in _biunit(4096, 2):
        y = float(x * np.float32(math.pi))
        assert abs(f(y) - ref(y)) <= tol


def test_acos(orc):  # simd.rs:772-811
    L = orc.lib()
    for x in _biunit(4096, 3):
        assert abs(L.orc_acos_fast(float(x)) - math.acos(float(x))) <= 0.075
        y = float(x * np.float32(0.98))
        assert abs(L.orc_acos(y) - math.acos(y)) <= 0.017


def test_rng_intervals(orc):  # random.rs:197-228
    out = np.empty(4096 * 8, np.float32)
    for kind, lo, hi in [(0, 0.0, 1.0), (1, -1.0, 1.0), (2, -math.pi, math.pi)]:
        orc.lib().orc_rng_samples(2, 5, 7, kind, 4096, out.ctypes.data)
        assert out.min() >= lo and out.max() <= hi


def test_hemisphere_unit_norm(orc):  # random.rs:230-240
    out = np.empty(4096 * 24, np.float32)
    orc.lib().orc_rng_samples(2, 5, 7, 3, 4096, out.ctypes.data)
    v = out.reshape(-1, 3)
    r = np.sqrt((v.astype(np.float64) ** 2).sum(1))
    assert r.min() >= 0.991 and r.max() <= 1.009
    assert v[:, 2].min() >= 0.0


def test_sample_u32_xor_nonzero(orc):  # random.rs:242-259
    out = np.empty(4096 * 8, np.uint32)
    orc.lib().orc_rng_draws(2, 5, 7, 4096, out.ctypes.data)
    x = np.bitwise_xor.reduce(out.reshape(4096, 8), axis=0)
    assert (x != 0).all()


def test_rng_first_draw_known_answer(orc):
    """random.rs:43-90 evaluated with Python integers: the generator the
    oracle (and the GPU) implements is the reference's multiplicative one."""
    M = (1 << 64) - 1
    x, y, i = 2, 5, 7
    seed = (x * 12276630456901467871 + y * 7661526868048087387 + i * 2268244495640532043) & M
    seed = (seed + seed % 9358246936573323101) & M
    primes = [14491630826648200009, 13149596372461506851, 6119410235796056053, 14990141545859273719]
    f = [3 * 1073243692214514217, 5 * 3335100457702756523, 7 * 8789056573444181, 11 * 781436371140792079]
    state = [(seed * p) & M for p in primes]
    expect = []
    for _ in range(3):
        for k in range(4):
            expect += [state[k] & 0xFFFFFFFF, state[k] >> 32]
            state[k] = (state[k] * f[k]) & M
    out = np.empty(24, np.uint32)
    orc.lib().orc_rng_draws(x, y, i, 3, out.ctypes.data)
    assert out.tolist() == expect


def _rot(orc, v, n):
    out, a, b = np.empty(3, np.float32), f32(*v), f32(*n)
    orc.lib().orc_rotate_hemisphere(a.ctypes.data, b.ctypes.data, out.ctypes.data)
    return out


def test_rotate_hemisphere_axes(orc):  # vector3.rs:445-467
    x, y, z = (1, 0, 0), (0, 1, 0), (0, 0, 1)
    cases = [(x, y, x), (y, x, y), (y, y, (0, 0, -1)), (x, x, (0, 0, -1)), (x, z, x), (y, z, y)]
    for v, n, want in cases:
        got = _rot(orc, v, n)
        assert ((got - np.array(want, np.float32)) ** 2).sum() <= 1e-6


def test_rotate_hemisphere_orthogonal_linear(orc):  # vector3.rs:469-490
    ns, xs, ys = _unit_sphere(4096, 4), _unit_sphere(4096, 5), _unit_sphere(4096, 6)
    for n, a, b in zip(ns, xs, ys):
        s = a + b
        m = _rot(orc, s, n)
        assert (float((s.astype(np.float64) ** 2).sum()) - float((m.astype(np.float64) ** 2).sum())) ** 2 <= 1e-5
        lin = _rot(orc, a, n) + _rot(orc, b, n)
        assert ((m - lin) ** 2).sum() <= 1e-6


def test_rotate_hemisphere_extrema(orc):  # vector3.rs:492-510 (exact)
    mz = (0.0, 0.0, -1.0)
    assert _rot(orc, (1, 0, 0), mz).tolist() == [-1.0, 0.0, 0.0]
    assert _rot(orc, (0, 1, 0), mz).tolist() == [0.0, -1.0, 0.0]
    assert _rot(orc, (0, 0, 1), mz).tolist() == [0.0, 0.0, -1.0]


def test_rotate_hemisphere_random_signs(orc):  # vector3.rs:512-540
    out = np.empty(4096 * 24, np.float32)
    orc.lib().orc_rng_samples(1, 2, 3, 3, 4096, out.ctypes.data)
    w = np.array([_rot(orc, v, (1, 0, 0)) for v in out.reshape(-1, 3)[::8]])
    eps = 1e-4
    assert (w[:, 0] + eps >= 0).all()
    assert (w[:, 1] < -eps).any() and (w[:, 1] > eps).any()
    assert (w[:, 2] < -eps).any() and (w[:, 2] > eps).any()


def _qrot(orc, v, q):
    out, a, b = np.empty(3, np.float32), f32(*v), f32(*q)
    orc.lib().orc_quat_rotate(a.ctypes.data, b.ctypes.data, out.ctypes.data)
    return out


def test_quaternion_rotations(orc):  # quaternion.rs:166-221
    h = float(np.float32(0.5) * np.sqrt(np.float32(2.0)))
    for v in _unit_sphere(32 * 8, 7):
        assert ((_qrot(orc, v, (1, 0, 0, 0)) - v) ** 2).sum() <= 1e-14
        assert ((_qrot(orc, v, (h, h, 0, 0)) - np.array([v[0], -v[2], v[1]])) ** 2).sum() <= 1e-12
        assert ((_qrot(orc, v, (h, 0, h, 0)) - np.array([v[2], v[1], -v[0]])) ** 2).sum() <= 1e-12
        assert ((_qrot(orc, v, (h, 0, 0, h)) - np.array([-v[1], v[0], v[2]])) ** 2).sum() <= 1e-12


def test_quaternion_interpolate(orc):  # quaternion.rs:223-234
    h = float(np.float32(0.5) * np.sqrt(np.float32(2.0)))
    q, q0, dq = np.empty(4, np.float32), f32(1, 0, 0, 0), f32(h - 1.0, 0, 0, h)
    orc.lib().orc_quat_interpolate(q0.ctypes.data, dq.ctypes.data, 0.5, q.ctypes.data)
    got = _qrot(orc, (1, 0, 0), q)
    assert ((got - np.array([h, h, 0.0])) ** 2).sum() <= 1e-12


def _normalized(v):  # SVector3::normalized (vector3.rs:104-116)
    v = np.array(v, np.float32)
    return (v * (np.float32(1.0) / np.sqrt((v * v).sum(dtype=np.float32)))).astype(np.float32)


def _any(orc, box, o, d):
    tmin, tmax = np.zeros(1, np.float32), np.zeros(1, np.float32)
    b, oo, dd = f32(*box), f32(*o), f32(*d)
    return orc.lib().orc_aabb_intersect(b.ctypes.data, oo.ctypes.data, dd.ctypes.data, tmin.ctypes.data,
                                        tmax.ctypes.data) == 1


def test_intersect_aabb(orc):  # aabb.rs:201-254
    box = (0.0, 1.0, 2.0, 1.0, 3.0, 5.0)
    cases = [((0, 0, 0), (2, 3, 5), True, False), ((0, 0, 0), (1, 4, 5), True, False),
             ((0, 0, 0), (2, 3, 0), False, False), ((0.2, 1.2, 2.2), (1, 1, 0), True, True),
             ((0.01, 2.0, 3.5), (0, 0, 1), True, True)]
    for o, d, fwd, bwd in cases:
        dn = _normalized(d)
        assert _any(orc, box, o, dn) == fwd
        assert _any(orc, box, o, np.float32(0.0) - dn) == bwd  # Neg for MRay (ray.rs:118-128)


def test_aabb_with_srays(orc):  # bench.rs:141-161, 225-236
    rng = np.random.default_rng(8)
    n, m = 4096, 2048
    dirs = _unit_sphere(n, 9)
    origins = dirs * np.float32(16.0)
    d = np.float32(0.0) - dirs
    up = np.array([0, 0, 1], np.float32)
    for i in range(m, n):
        side = _normalized(np.cross(up, d[i]))
        origins[i] = origins[i] + side * np.float32(16.0)
    perm = rng.permutation(n)
    hits = sum(_any(orc, (-1, -1, -1, 1, 1, 1), origins[i], d[i]) for i in perm)
    assert hits == m


TRI = (0.0, 1.0, 1.0, -1.0, -1.0, 1.0, 1.0, -1.0, 1.0)


def test_intersect_triangle(orc):  # triangle.rs:188-223
    out, tri, o0, o1, d = np.zeros(9, np.float32), f32(*TRI), f32(0, 0, 0), f32(-1, 0, 0), f32(0, 0, 1)
    hit = orc.lib().orc_triangle_intersect(tri.ctypes.data, o0.ctypes.data, d.ctypes.data, 1e5, out.ctypes.data)
    assert hit == 1 and 0.99 < out[0] < 1.01
    assert ((out[1:4] - np.array([0, 0, 1])) ** 2).sum() < 0.01
    hit = orc.lib().orc_triangle_intersect(tri.ctypes.data, o1.ctypes.data, d.ctypes.data, 1e5, out.ctypes.data)
    assert hit == 0 and out[0] == np.float32(1e5)


def test_intersect_triangle_direct(orc):  # triangle.rs:225-259
    out, tri, d = np.zeros(5, np.float32), f32(*TRI), f32(0, 0, 1)
    for o in [(0, 0, 0), (-1, 0, 0)]:
        oo = f32(*o)
        orc.lib().orc_intersect_direct(tri.ctypes.data, oo.ctypes.data, d.ctypes.data, out.ctypes.data)
        assert 0.99 < out[0] < 1.01
        assert 0.99 < (out[2:5].astype(np.float64) ** 2).sum() < 1.01


def test_cvtps_semantics(orc):
    """_mm256_cvtps_epi32: nearest-even, 0x80000000 for NaN and out of range."""
    L = orc.lib()
    assert [L.orc_cvtps(v) for v in (0.5, 1.5, 2.5, -0.5, 254.5, 255.0)] == [0, 2, 2, 0, 254, 255]
    assert L.orc_cvtps(float("nan")) == -2**31 and L.orc_cvtps(3e9) == -2**31


def test_sky_intensity(orc):  # material.rs:205-215
    out, up, down = np.zeros(3, np.float32), f32(0, 0, 1), f32(0, 0, -1)
    orc.lib().orc_sky_intensity(up.ctypes.data, out.ctypes.data)
    assert out.tolist() == [2.5, 2.5, 2.5]
    orc.lib().orc_sky_intensity(down.ctypes.data, out.ctypes.data)
    assert out.tolist() == [0.5, 0.5, 0.5]


@pytest.mark.parametrize("kind,expected", [  # simd.rs:661-686 (mf32_fmadd_ps, fmsub_ps, fnmadd_ps)
    (0, [5.0, 12.0, 7.0, 24.0, 1.0, 5.0, 11.0, 19.0]),
    (1, [-5.0, 0.0, -7.0, 8.0, -1.0, -1.0, 1.0, 5.0]),
    (2, [5.0, 0.0, 7.0, -8.0, 1.0, 1.0, -1.0, -5.0]),
])
def test_fused_multiply_add_forms(orc, kind, expected):
    L = orc.lib()
    a = [0.0, 1.0, 0.0, 2.0, 1.0, 2.0, 3.0, 4.0]
    b = [5.0, 6.0, 7.0, 8.0, 0.0, 1.0, 2.0, 3.0]
    c = [5.0, 6.0, 7.0, 8.0, 1.0, 3.0, 5.0, 7.0]
    assert [L.orc_fma3(kind, x, y, z) for x, y, z in zip(a, b, c)] == expected


def test_any_sign_bit_positive_masked(orc):  # simd.rs:695-707
    L = orc.lib()
    a = f32(-2.0, -1.0, -0.0, 0.0, 1.0, 2.0, 3.0, 4.0)
    on = np.array([0xFFFFFFFF], np.uint32).view(np.float32)[0]

    def mask(*bits):
        return np.array([on if b else 0.0 for b in bits], np.float32)

    cases = [((1, 0, 1, 1, 1, 0, 0, 0), True), ((1, 0, 1, 1, 0, 0, 0, 0), True),
             ((1, 0, 1, 0, 0, 0, 0, 0), False), ((1, 1, 0, 0, 0, 0, 0, 0), False),
             ((1, 0, 0, 1, 0, 0, 0, 0), True)]
    for bits, want in cases:
        m = mask(*bits)
        assert bool(L.orc_any_sign_bit_positive_masked(a.ctypes.data, m.ctypes.data)) == want, bits


def test_abs(orc):  # simd.rs:813-817
    L = orc.lib()
    x = [1.0, -1.0, 0.0, -0.0, 2.0, 3.0, 5.0, -7.0]
    y = [L.orc_abs(v) for v in x]
    assert y == [1.0, 1.0, 0.0, 0.0, 2.0, 3.0, 5.0, 7.0]
    assert all(math.copysign(1.0, v) == 1.0 for v in y)  # -0 loses its sign too
