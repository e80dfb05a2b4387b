// Per-lane shading of the reference's path loop: camera rays (scene.rs:81-99,
// quaternion.rs:62-153), the RNG (random.rs:33-159), continue_path with BRDF
// and direct-light sampling and the one-sample MIS weight (material.rs:
// 205-513, scene.rs:143-202, triangle.rs:152-185) and the pixel packing
// (renderer.rs:239-286). One thread is one lane of a reference packet; the
// operations are the reference's, in its order, with its rounding.
#pragma once
#include "layout.cuh"
#include "traverse.cuh"
#include "x86sem.cuh"

namespace cvx {

// One lane of the reference Rng: lane k reads the low (k even) or high (k odd)
// half of 64-bit state k/2 and then advances it (random.rs:73-102).
struct LaneRng {
    uint64_t s, f;
    uint32_t hi;
    __device__ __forceinline__ void seed(uint32_t x, uint32_t y, uint32_t i, int lane) {
        uint64_t a = (uint64_t)x * 12276630456901467871ull;
        uint64_t b = (uint64_t)y * 7661526868048087387ull;
        uint64_t c = (uint64_t)i * 2268244495640532043ull;
        uint64_t sd = a + b + c;
        sd = sd + sd % 9358246936573323101ull;
        int k = lane >> 1;
        uint64_t p = k == 0 ? 14491630826648200009ull
                   : k == 1 ? 13149596372461506851ull
                   : k == 2 ? 6119410235796056053ull
                            : 14990141545859273719ull;
        f = k == 0 ? 3ull * 1073243692214514217ull
          : k == 1 ? 5ull * 3335100457702756523ull
          : k == 2 ? 7ull * 8789056573444181ull
                   : 11ull * 781436371140792079ull;
        s = sd * p;
        hi = (uint32_t)(lane & 1);
    }
    __device__ __forceinline__ uint32_t next() {
        uint32_t v = hi ? (uint32_t)(s >> 32) : (uint32_t)s;
        s *= f;
        return v;
    }
    // Resumes lane `lane` of a generator from its saved 64-bit state.
    __device__ __forceinline__ void resume(uint64_t state, int lane) {
        int k = lane >> 1;
        f = k == 0 ? 3ull * 1073243692214514217ull
          : k == 1 ? 5ull * 3335100457702756523ull
          : k == 2 ? 7ull * 8789056573444181ull
                   : 11ull * 781436371140792079ull;
        s = state;
        hi = (uint32_t)(lane & 1);
    }
};
__device__ __forceinline__ float unit_from(uint32_t u) { return fmaf((float)(int32_t)u, 0.5f / -2147483648.0f, 0.5f); }
__device__ __forceinline__ float biunit_from(uint32_t u) { return (float)(int32_t)u * (1.0f / -2147483648.0f); }
__device__ __forceinline__ float angle_from(uint32_t u) { return (float)(int32_t)u * (kPi / -2147483648.0f); }

struct Quat {
    float a, b, c, d;
};

__device__ __forceinline__ F3 rotate(F3 v, Quat q) {  // quaternion.rs:110-153
    float pa = q.b * v.x + q.c * v.y + q.d * v.z;
    float pb = q.b * v.x - q.c * v.y + q.d * v.z + (q.a - q.b) * v.x + (q.c - q.d) * (v.y + v.z);
    float pc = q.d * v.x + q.a * v.y - q.b * v.z;
    float pd = q.d * v.x - q.a * v.y - q.b * v.z - (q.c + q.d) * v.x + (q.a + q.b) * (v.y + v.z);
    float rb = (pa + pb) * (q.a + q.b) - (pc - pd) * (q.c + q.d) - pa * q.a - pb * q.b + pc * q.c - pd * q.d;
    float rc = pc * q.a - pd * q.b + pa * q.c + pb * q.d;
    float rd = (pc + pd) * (q.a + q.b) + (pa - pb) * (q.c + q.d) - pc * q.a - pd * q.b - pa * q.c + pb * q.d;
    return f3(rb, rc, rd);
}

__device__ __forceinline__ void camera_ray(const DeviceCamera& c, float x, float y, float t, const ApproxTables& tab,
                                           F3& o, F3& d) {
    o = f3(fmaf(c.pos_delta[0], t, c.pos[0]), fmaf(c.pos_delta[1], t, c.pos[1]), fmaf(c.pos_delta[2], t, c.pos[2]));
    float a = fmaf(c.dq[0], t, c.q[0]), b = fmaf(c.dq[1], t, c.q[1]);
    float cc = fmaf(c.dq[2], t, c.q[2]), dd = fmaf(c.dq[3], t, c.q[3]);
    float nsq = fmaf(a, a, b * b) + fmaf(cc, cc, dd * dd);
    float rn = 1.0f / sqrtf(nsq);
    Quat q{a * rn, b * rn, cc * rn, dd * rn};
    F3 src = normalized(f3(x, y, -c.screen_distance), tab);
    d = rotate(src, q);
}

__device__ __forceinline__ F3 rotate_hemisphere(F3 v, F3 normal, const ApproxTables& tab) {  // vector3.rs:221-251
    bool flip = sneg(normal.z);
    F3 n = flip ? vneg0(normal) : normal;
    float rz = x_rcp(1.0f + n.z, tab);
    float c = n.x * n.y * rz;
    float x = fmsub(v.x, fmaf(n.y, n.y * rz, n.z), fmsub(v.y, c, v.z * n.x));
    float y = fnmadd(v.x, c, fmaf(v.y, fmaf(n.x, n.x * rz, n.z), v.z * n.y));
    float z = fnmadd(v.x, n.x, fnmadd(v.y, n.y, v.z * n.z));
    F3 r = f3(x, y, z);
    return flip ? vneg0(r) : r;
}

__device__ __forceinline__ F3 sky_intensity(F3 d) {  // material.rs:205-215
    float up = d.x * 0.0f + d.y * 0.0f + d.z * 1.0f;
    float k = fmaf(up, 0.5f, 0.5f);
    float r = k, g = k * k, b = k * (k * k);
    return f3(fmaf(r, 2.0f, 0.5f), fmaf(g, 2.0f, 0.5f), fmaf(b, 2.0f, 0.5f));
}

struct Isect {
    F3 pos, normal;
    float dist;
    uint32_t mat;
    float tu, tv;
};

// The hit record the reference builds for the accepted triangle
// (triangle.rs:133-142), or the far intersection (scene.rs:220-228).
__device__ __forceinline__ Isect make_isect(const DeviceScene& s, const Hit& h, F3 o, F3 d,
                                            const ApproxTables& tab) {
    Isect I;
    if (h.tri < 0) {
        I.pos = vfma(d, 1.0e5f, o);
        I.normal = d;
        I.dist = 1.0e5f;
        I.mat = kSkyMaterial;
        I.tu = 0.0f;
        I.tv = 0.0f;
        return I;
    }
    const float4* g = s.geom + 3 * h.tri;
    F3 n = f3(__ldg(&g[0].w), __ldg(&g[1].w), __ldg(&g[2].w));
    const TriShade& sh = s.shade[h.tri];
    float w = (1.0f - h.u) - h.v;
    I.pos = vfma(d, h.t, o);
    I.normal = normalized(n, tab);
    I.dist = h.t;
    I.mat = __ldg(&sh.material);
    I.tu = fmaf(__ldg(&sh.uv[0]), w, fmaf(__ldg(&sh.uv[2]), h.v, __ldg(&sh.uv[4]) * h.u));
    I.tv = fmaf(__ldg(&sh.uv[1]), w, fmaf(__ldg(&sh.uv[3]), h.v, __ldg(&sh.uv[5]) * h.u));
    return I;
}

__device__ __forceinline__ uint32_t light_pick(const DeviceScene& s, uint32_t bits) {
    return s.general_pick ? (uint32_t)(((uint64_t)bits * (uint64_t)s.n_lights) >> 32) : (bits >> 29);
}

// material.rs:281-320
__device__ __forceinline__ float pd_direct_sample(const DeviceScene& s, F3 o, F3 d, const ApproxTables& tab) {
    float pd_total = 0.0f;
    for (uint32_t l = 0; l < s.n_lights; l++) {
        const float4* L = s.lights + 5 * l;
        float4 q0 = __ldg(L), q1 = __ldg(L + 1), q2 = __ldg(L + 2), q3 = __ldg(L + 3), q4 = __ldg(L + 4);
        F3 v0 = f3(q0.x, q0.y, q0.z), e1 = f3(q1.x, q1.y, q1.z), e2 = f3(q2.x, q2.y, q2.z);
        F3 n = f3(q3.x, q3.y, q3.z), normal = f3(q4.x, q4.y, q4.z);
        float area = q0.w;
        F3 fr = sub(v0, o);
        float denom = x_rcp(dot(d, n), tab);
        float t = dot(fr, n) * denom;
        F3 c = cross(d, fr);
        float u = dot(c, e2) * denom;
        float v = dot(c, e1) * denom;
        bool miss = sneg(u) | sneg(v) | sneg(t) | geq(u + v, 1.0f);
        float dsq = t * t;
        float dot_em = fabs_bits(dot(normal, d)) + 0.0001f;
        float pd = dsq * x_rcp(area * dot_em, tab);
        pd_total = miss ? pd_total : pd_total + pd;
    }
    return pd_total * (1.0f / (float)s.n_lights);
}

__device__ __forceinline__ float normal_dist(F3 h, F3 n, int32_t gloss) {  // material.rs:475-513
    float c1 = dot(h, n), c2 = c1 * c1, c4 = c2 * c2, c8 = c4 * c4, c16 = c8 * c8;
    float r = c16 * (8.5f / kPi);
    r = gloss == 4 ? c8 * (4.5f / kPi) : r;
    r = gloss == 3 ? c4 * (2.5f / kPi) : r;
    r = gloss == 2 ? c2 * (1.5f / kPi) : r;
    r = gloss == 1 ? xmax(c1, 0.0f) * (1.0f / kPi) : r;
    r = gloss == 0 ? 0.5f / kPi : r;
    return r;
}

// The ray continue_path samples next (material.rs:228-265 and the one-sample
// pick of 327-411): a BRDF sample or a direct-light sample, chosen by the sixth
// of six draws.
struct NextRay {
    F3 o, d;
    bool direct;
};
__device__ __forceinline__ NextRay sample_next(const DeviceScene& s, const Isect& I, LaneRng& rng,
                                               const ApproxTables& tab) {
    uint32_t dphi = rng.next(), dr = rng.next(), dsel = rng.next(), du = rng.next(), dv = rng.next(),
             drr = rng.next();
    // continue_path_brdf (material.rs:228-242)
    float phi = angle_from(dphi), r_sqr = unit_from(dr), r = sqrtf(r_sqr);
    F3 hv = f3(poly_sin(phi) * r, poly_cos(phi) * r, sqrtf(1.0f - r_sqr));
    F3 dir_b = rotate_hemisphere(hv, I.normal, tab);
    F3 org_b = vfma(dir_b, 1.0e-4f, I.pos);
    // continue_path_direct_sample (material.rs:253-265, scene.rs:143-202)
    const float4* L = s.lights + 5 * light_pick(s, dsel);
    float4 q0 = __ldg(L), q1 = __ldg(L + 1), q2 = __ldg(L + 2);
    float u = unit_from(du), v = unit_from(dv);
    bool fold = sneg((1.0f - u) - v);
    u = fold ? 1.0f - u : u;
    v = fold ? 1.0f - v : v;
    F3 p = f3(fmaf(q2.x, v, fnmadd(q1.x, u, q0.x)), fmaf(q2.y, v, fnmadd(q1.y, u, q0.y)),
              fmaf(q2.z, v, fnmadd(q1.z, u, q0.z)));
    F3 dir_d = normalized(sub(p, I.pos), tab);
    F3 org_d = vfma(dir_d, 1.0e-4f, I.pos);
    // one-sample MIS between the two
    float rr = fmaf(I.normal.z, 0.8f, biunit_from(drr));
    bool pick_direct = sneg(rr);
    return NextRay{pick_direct ? org_d : org_b, pick_direct ? dir_d : dir_b, pick_direct};
}

// The raw Fresnel value of microfacet_fresnel (material.rs:453-469) for the
// incoming direction rd and the sampled direction nd.
__device__ __forceinline__ float fresnel_term(F3 nd, F3 rd, F3& h, const ApproxTables& tab) {
    h = normalized(sub(nd, rd), tab);
    float ct = 1.0f - fabs_bits(dot(h, nd));
    float ct2 = ct * ct, ct3 = ct2 * ct;
    return fabs_bits(ct2 * ct3);
}

// The colour modulation of continue_path (material.rs:327-411, microfacet_brdf
// 415-469) for the sampled next ray n of a lane that continues, from the
// incoming direction rd; returns the raw Fresnel value in `fresnel`.
__device__ __forceinline__ F3 path_modulation(const DeviceScene& s, const Isect& I, const NextRay& n, F3 rd,
                                              bool ignore_fresnel, const ApproxTables& tab, float& fresnel) {
    const bool pick_direct = n.direct;
    const F3 no = n.o, nd = n.d;
    float pd_b = xmax(dot(I.normal, nd), 0.0f) * (1.0f / kPi);
    float pd_d = pd_direct_sample(s, no, nd, tab);
    float wden = pd_b + pd_d + 0.01f;
    float p_brdf = fmaf(I.normal.z, 0.4f, 0.5f);
    float p_direct = fnmadd(I.normal.z, 0.4f, 0.5f);
    float modulation = x_rcp(wden * (pick_direct ? p_direct : p_brdf), tab);
    float cos_theta = xmax(dot(I.normal, nd), 0.0f);
    // microfacet_brdf (material.rs:415-469)
    int32_t mi = (int32_t)I.mat;
    const float k255 = 1.0f / 255.0f;
    F3 col = f3((float)(mi & 0xff) * k255, (float)((mi >> 8) & 0xff) * k255, (float)((mi >> 16) & 0xff) * k255);
    F3 h;
    float ct5 = fresnel_term(nd, rd, h, tab);
    float D = normal_dist(h, I.normal, (mi >> 26) & 7);
    F3 fcol = f3(fmaf(1.0f - col.x, ct5, col.x), fmaf(1.0f - col.y, ct5, col.y), fmaf(1.0f - col.z, ct5, col.z));
    bool has_tex = (((I.mat << 6) | (I.mat << 7)) >> 31) != 0u;
    if (ignore_fresnel && has_tex) fcol = f3(1.0f, 1.0f, 1.0f);
    float k = modulation * cos_theta;
    F3 c = f3((fcol.x * D) * k, (fcol.y * D) * k, (fcol.z * D) * k);
    fresnel = ct5;
    return f3(xmin(c.x, 2.0f), xmin(c.y, 2.0f), xmin(c.z, 2.0f));
}

// material.rs:327-411 for one lane. Advances the ray (unless the lane is or
// becomes inactive) and returns the colour modulation and raw Fresnel value.
__device__ __forceinline__ void continue_path(const DeviceScene& s, F3& ro, F3& rd, bool& active, const Isect& I,
                                              LaneRng& rng, bool ignore_fresnel, const ApproxTables& tab, F3& cm,
                                              float& fresnel) {
    bool inactive = !active | ((I.mat >> 31) != 0u);
    NextRay n = sample_next(s, I, rng, tab);
    F3 c = path_modulation(s, I, n, rd, ignore_fresnel, tab, fresnel);
    if (inactive) {
        cm = f3(1.0f, 1.0f, 1.0f);
        active = false;
    } else {
        cm = c;
        ro = n.o;
        rd = n.d;
    }
}

struct PixelOut {
    F3 color;
    int32_t tex;
    float tu, tv, fresnel;
};

// renderer.rs:413-468 for one lane of an 8-pixel group; the bounce loop exit
// and (PACKET) the traversal are decided over the octet `omask`.
template <bool PACKET>
__device__ __forceinline__ bool render_pixels(const DeviceScene& s, const DeviceCamera& cam, float x, float y,
                                              LaneRng& rng, unsigned omask, const ApproxTables& tab, PixelOut& out,
                                              uint32_t& rays) {
    F3 o, d;
    camera_ray(cam, x, y, unit_from(rng.next()), tab, o, d);
    bool active = true, ok = true;
    F3 color = f3(1.0f, 1.0f, 1.0f);
    uint32_t hit_em = 0u;
    out.tex = 0;
    out.tu = out.tv = out.fresnel = 0.0f;
    for (int i = 0; i < 5; i++) {
        rays += active ? 1u : 0u;
        Hit h{1.0e5f, 0.0f, 0.0f, -1};
        // Packets whose 8 rays all allow it take the select-form slab test,
        // chosen once per bounce outside the traversal loop (room frame in
        // packet traversal 1.32 -> 1.21 ms; the same image).
        if (PACKET && s.slab_sel &&
            oct_all(omask, select_form_ray(f3(x_rcp(d.x, tab), x_rcp(d.y, tab), x_rcp(d.z, tab)))))
            ok &= traverse<true, true>(s, o, d, active, omask, h, tab, nullptr);
        // Likewise a single-ray lane whose reciprocals allow it (room frame in
        // octet groups 0.82 -> 0.74 ms, 256-scene batch 53.4 -> 51.9 ms).
        else if (!PACKET && active && s.slab_sel &&
                 select_form_ray(f3(x_rcp(d.x, tab), x_rcp(d.y, tab), x_rcp(d.z, tab))))
            ok &= traverse<false, true>(s, o, d, active, __activemask(), h, tab, nullptr);
        else if (PACKET || active)
            ok &= traverse<PACKET>(s, o, d, active, PACKET ? omask : __activemask(), h, tab, nullptr);
        Isect I = make_isect(s, h, o, d, tab);
        hit_em = I.mat;
        if (oct_all(omask, (I.mat >> 31) != 0u)) break;
        F3 cm;
        float fr;
        continue_path(s, o, d, active, I, rng, i == 0, tab, cm, fr);
        color = f3(color.x * cm.x, color.y * cm.y, color.z * cm.z);
        if (i == 0) {
            out.tex = ((int32_t)I.mat >> 24) & 3;
            out.tu = I.tu;
            out.tv = I.tv;
            out.fresnel = fr;
        }
    }
    F3 em = sky_intensity(d);
    F3 c = f3(color.x * em.x, color.y * em.y, color.z * em.z);
    out.color = (hit_em >> 31) ? c : f3(0.0f, 0.0f, 0.0f);
    return ok;
}

// renderer.rs:470-486: the debug view of one lane. The time is 0 (no random
// draw); green and blue are log2 of the boxes and triangles the packet (or the
// ray, SINGLE) tested, times 0.1. log2 is taken in double and rounded to
// float, which equals a correctly rounded f32 log2.
template <bool PACKET>
__device__ __forceinline__ bool render_pixels_debug(const DeviceScene& s, const DeviceCamera& cam, float x, float y,
                                                    unsigned omask, const ApproxTables& tab, PixelOut& out,
                                                    uint32_t& rays) {
    F3 o, d;
    camera_ray(cam, x, y, 0.0f, tab, o, d);
    Hit h{1.0e5f, 0.0f, 0.0f, -1};
    Counters c{0u, 0u};
    bool ok = traverse<PACKET>(s, o, d, true, omask, h, tab, &c);
    rays += 1u;
    float g = (float)log2((double)c.aabb) * 0.1f, b = (float)log2((double)c.tri) * 0.1f;
    out.color = f3(0.0f, g, b);
    out.tex = 0;
    out.tu = out.tv = out.fresnel = 0.0f;
    return ok;
}

__device__ __forceinline__ uint32_t pack_color(F3 c) {  // renderer.rs:239-256
    float r = xmin(1.0f, c.x * 2.0f) * 255.0f, g = xmin(1.0f, c.y * 2.0f) * 255.0f,
          b = xmin(1.0f, c.z * 2.0f) * 255.0f;
    return ((uint32_t)x_cvtps(r) | ((uint32_t)x_cvtps(g) << 8)) | ((uint32_t)x_cvtps(b) << 16);
}
__device__ __forceinline__ uint32_t pack_gbuffer(const PixelOut& p) {  // renderer.rs:260-286
    uint32_t r = (uint32_t)x_cvtps(p.tu * 255.0f) & 0xffu;
    uint32_t g = ((uint32_t)x_cvtps(p.tv * 255.0f) & 0xffu) << 8;
    uint32_t b = (uint32_t)x_cvtps(p.fresnel * 255.0f) << 16;
    uint32_t a = (uint32_t)p.tex << 24;
    return (r | g) | (b | a);
}

}  // namespace cvx
