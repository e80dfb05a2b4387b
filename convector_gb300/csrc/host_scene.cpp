// Host side of the boundary: OBJ loading (wavefront.rs), the BVH build
// (bvh.rs) and the camera setters (scene.rs), restated in C++. The BVH build
// is the reference's algorithm step for step, so the device sees the same
// node order and triangle order as the reference's traversal. Compiled with
// -ffp-contract=off so that every float operation rounds where the Rust
// original rounds.
#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <future>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <string_view>
#include <thread>
#include <vector>

#include "internal.h"

namespace cvx {

static thread_local std::string g_last_error;
static thread_local int32_t g_last_status = CVX_OK;

int32_t set_error(int32_t status, const std::string& msg) {
    g_last_status = status;
    g_last_error = msg;
    return status;
}

// ---------------------------------------------------------------------------
// Scalar vector helpers (SVector3, vector3.rs:39-143)

struct S3 {
    float x, y, z;
};
static inline S3 s3(const float* p) { return S3{p[0], p[1], p[2]}; }
static inline S3 operator-(S3 a, S3 b) { return S3{a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline S3 operator+(S3 a, S3 b) { return S3{a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline S3 operator*(S3 a, float k) { return S3{a.x * k, a.y * k, a.z * k}; }
// SVector3::cross is cross_fma with `mul_add(b, -c)` (vector3.rs:63-70).
static inline S3 scross(S3 a, S3 b) {
    return S3{std::fma(a.y, b.z, -(a.z * b.y)), std::fma(a.z, b.x, -(a.x * b.z)), std::fma(a.x, b.y, -(a.y * b.x))};
}
// SVector3::dot is dot_fma (vector3.rs:86-98).
static inline float sdot(S3 a, S3 b) { return std::fma(a.x, b.x, std::fma(a.y, b.y, a.z * b.z)); }
// f32::min / f32::max (IEEE minNum / maxNum). On equal operands (+0 / -0) the
// x86 lowering of llvm.minnum / maxnum returns the first operand.
static inline float fmin_rs(float a, float b) { return a != a ? b : (b < a ? b : a); }
static inline float fmax_rs(float a, float b) { return a != a ? b : (b > a ? b : a); }
static inline S3 smin(S3 a, S3 b) { return S3{fmin_rs(a.x, b.x), fmin_rs(a.y, b.y), fmin_rs(a.z, b.z)}; }
static inline S3 smax(S3 a, S3 b) { return S3{fmax_rs(a.x, b.x), fmax_rs(a.y, b.y), fmax_rs(a.z, b.z)}; }
static inline float coord(S3 v, int axis) { return axis == 0 ? v.x : axis == 1 ? v.y : v.z; }

// ---------------------------------------------------------------------------
// OBJ loading (wavefront.rs:83-152)

// Tokens are views into the OBJ text; nothing is allocated per token.
using Tok = std::string_view;

// Rust's f32::from_str: decimal or exponent notation, inf / nan, correctly
// rounded; strtof also takes hexadecimal floats, which are refused here.
static bool parse_f32(Tok tok, float* out) {
    if (tok.empty() || tok.size() >= 128) return false;
    // Plain decimal tokens in range: std::from_chars, correctly rounded like
    // strtof and several times faster. Everything else goes through strtof.
    if (tok[0] != '+') {
        float v;
        auto r = std::from_chars(tok.data(), tok.data() + tok.size(), v, std::chars_format::general);
        bool plain = true;
        for (char c : tok) plain = plain && ((c >= '0' && c <= '9') || c == '.' || c == '-' || c == 'e' || c == 'E');
        if (plain && r.ec == std::errc() && r.ptr == tok.data() + tok.size()) {
            *out = v;
            return true;
        }
    }
    if (tok.find("0x") != Tok::npos || tok.find("0X") != Tok::npos) return false;
    char buf[128];
    std::memcpy(buf, tok.data(), tok.size());
    buf[tok.size()] = 0;
    char* end = nullptr;
    float v = std::strtof(buf, &end);
    if (end != buf + tok.size()) return false;
    *out = v;
    return true;
}

static bool parse_u32(Tok tok, uint32_t* out) {
    size_t i = 0;
    if (i < tok.size() && tok[i] == '+') i++;
    if (i == tok.size()) return false;
    uint64_t v = 0;
    for (; i < tok.size(); i++) {
        if (tok[i] < '0' || tok[i] > '9') return false;
        v = v * 10 + (uint64_t)(tok[i] - '0');
        if (v > 0xffffffffull) return false;
    }
    *out = (uint32_t)v;
    return true;
}

// wavefront.rs:49-55: "v" or "v/t" (further parts parsed and ignored).
static bool parse_vertex_index(Tok tok, uint32_t* v, int64_t* t) {
    uint32_t vi = 0, ti = 0;
    size_t start = 0, part = 0;
    for (;; part++) {
        size_t p = tok.find('/', start);
        Tok s = tok.substr(start, p == Tok::npos ? Tok::npos : p - start);
        uint32_t x;
        if (!parse_u32(s, &x) || x == 0) return false;
        if (part == 0) vi = x;
        if (part == 1) ti = x;
        if (p == Tok::npos) break;
        start = p + 1;
    }
    *v = vi - 1;
    *t = part >= 1 ? (int64_t)ti - 1 : -1;
    return true;
}

// ASCII white space: space and \t \n \v \f \r.
static inline bool is_ws(char c) { return c == ' ' || (c >= '\t' && c <= '\r'); }

// Splits [pos, end) at ASCII white space.
static void tokenize(const char* text, size_t pos, size_t end, std::vector<Tok>& toks) {
    toks.clear();
    for (size_t i = pos; i < end;) {
        while (i < end && is_ws(text[i])) i++;
        size_t j = i;
        while (j < end && !is_ws(text[j])) j++;
        if (j > i) toks.emplace_back(text + i, j - i);
        i = j;
    }
}

static int32_t parse_obj_sequential(const char* text, size_t len, const char* const* names,
                                    const uint32_t* materials, uint32_t n_materials, cvx_mesh** out) {
    std::unique_ptr<cvx_mesh> mesh(new cvx_mesh());
    uint32_t material = 0x00ffffffu;  // SMaterial::white() (material.rs:93-95)
    size_t pos = 0;
    uint32_t line_nr = 0;
    std::vector<Tok> toks;
    std::vector<uint32_t> vi;
    std::vector<int64_t> ti;
    while (pos < len) {
        size_t eol = pos;
        while (eol < len && text[eol] != '\n') eol++;
        size_t end = eol;
        if (end > pos && text[end - 1] == '\r') end--;
        line_nr++;
        tokenize(text, pos, end, toks);
        pos = eol + 1;
        if (toks.empty()) continue;
        Tok kw = toks[0];
        // the location suffix of an error message, made only on error
        auto where = [line_nr] { return " (line " + std::to_string(line_nr) + ")"; };
        if (kw == "v") {
            float c[3];
            if (toks.size() < 4) return set_error(CVX_ERR_PARSE, std::string("missing vertex coordinate") + where());
            for (int k = 0; k < 3; k++)
                if (!parse_f32(toks[1 + k], &c[k]))
                    return set_error(CVX_ERR_PARSE, std::string("bad vertex coordinate") + where());
            mesh->vertices.insert(mesh->vertices.end(), c, c + 3);
        } else if (kw == "vt") {
            float c[2];
            if (toks.size() < 3) return set_error(CVX_ERR_PARSE, std::string("missing texture coordinate") + where());
            for (int k = 0; k < 2; k++)
                if (!parse_f32(toks[1 + k], &c[k]))
                    return set_error(CVX_ERR_PARSE, std::string("bad texture coordinate") + where());
            mesh->tex_coords.insert(mesh->tex_coords.end(), c, c + 2);
        } else if (kw == "usemtl") {
            if (toks.size() < 2) return set_error(CVX_ERR_PARSE, std::string("missing material name") + where());
            bool found = false;
            for (uint32_t k = 0; k < n_materials; k++)
                if (toks[1] == names[k]) {
                    material = materials[k];
                    found = true;
                }
            if (!found)
                return set_error(CVX_ERR_PARSE, "material '" + std::string(toks[1]) + "' not present in material dictionary" + where());
        } else if (kw == "f") {
            if (toks.size() < 4) return set_error(CVX_ERR_PARSE, std::string("missing triangle index") + where());
            vi.resize(toks.size() - 1);
            ti.resize(toks.size() - 1);
            for (size_t k = 1; k < toks.size(); k++)
                if (!parse_vertex_index(toks[k], &vi[k - 1], &ti[k - 1]))
                    return set_error(CVX_ERR_PARSE, "bad face index '" + std::string(toks[k]) + "'" + where());
            size_t nv = mesh->vertices.size() / 3;
            // Fan triangulation of convex n-gons (wavefront.rs:132-139).
            for (size_t k = 2; k < vi.size(); k++) {
                uint32_t a = vi[0], b = vi[k - 1], c = vi[k];
                if (a >= nv || b >= nv || c >= nv)
                    return set_error(CVX_ERR_PARSE, std::string("vertex index out of range") + where());
                // wavefront.rs:30-46
                S3 v0 = s3(&mesh->vertices[3 * a]), v1 = s3(&mesh->vertices[3 * b]), v2 = s3(&mesh->vertices[3 * c]);
                S3 e1 = v0 - v2, e2 = v1 - v0;
                S3 cr = scross(e1, e2);
                if (sdot(cr, cr) == 0.0f)
                    return set_error(CVX_ERR_DEGENERATE, std::string("encountered degenerate triangle") + where());
                MeshTri t;
                t.v[0] = a;
                t.v[1] = b;
                t.v[2] = c;
                bool has_t = ti[0] >= 0 && ti[k - 1] >= 0 && ti[k] >= 0;
                t.t[0] = has_t ? ti[0] : -1;
                t.t[1] = has_t ? ti[k - 1] : -1;
                t.t[2] = has_t ? ti[k] : -1;
                t.material = material;
                mesh->triangles.push_back(t);
            }
        }
    }
    *out = mesh.release();
    return CVX_OK;
}

// Parallel form of the same parser for large inputs. The text is cut into
// chunks at line starts; every chunk is tokenised concurrently into vertices,
// texture coordinates and an ordered list of records (material switches and
// faces, with the vertex and texture counts seen before them in the chunk).
// Prefix sums give every record its file-global counts and active material,
// then faces are checked (index range, degeneracy) and fan-triangulated
// concurrently. The result, and the first error in file order, equal the
// sequential parser's.
struct ChunkFace {
    uint32_t line;             // line number within the chunk (1-based)
    uint32_t v_before, t_before;  // vertices / texture coords earlier in the chunk
    int32_t mat_record;        // index of the last material switch in the chunk, -1: none
    uint32_t first, count;     // the face's corners in Chunk::vi / Chunk::ti
};
struct Chunk {
    size_t begin, end;
    uint32_t lines = 0;
    std::vector<float> v, vt;
    std::vector<uint32_t> mats;  // material values of the chunk's switches, in order
    std::vector<ChunkFace> faces;
    std::vector<uint32_t> vi;
    std::vector<int64_t> ti;
    int32_t err = CVX_OK;
    uint32_t err_line = 0;
    std::string err_msg;
};

static void parse_chunk(const char* text, Chunk& c, const char* const* names, const uint32_t* materials,
                        uint32_t n_materials) {
    std::vector<Tok> toks;
    size_t pos = c.begin;
    while (pos < c.end) {
        size_t eol = pos;
        while (eol < c.end && text[eol] != '\n') eol++;
        size_t end = eol;
        if (end > pos && text[end - 1] == '\r') end--;
        c.lines++;
        tokenize(text, pos, end, toks);
        pos = eol + 1;
        if (toks.empty()) continue;
        auto fail = [&](int32_t st, const std::string& m) {
            c.err = st;
            c.err_line = c.lines;
            c.err_msg = m;
        };
        Tok kw = toks[0];
        if (kw == "v") {
            float f[3];
            if (toks.size() < 4) return fail(CVX_ERR_PARSE, "missing vertex coordinate");
            for (int k = 0; k < 3; k++)
                if (!parse_f32(toks[1 + k], &f[k])) return fail(CVX_ERR_PARSE, "bad vertex coordinate");
            c.v.insert(c.v.end(), f, f + 3);
        } else if (kw == "vt") {
            float f[2];
            if (toks.size() < 3) return fail(CVX_ERR_PARSE, "missing texture coordinate");
            for (int k = 0; k < 2; k++)
                if (!parse_f32(toks[1 + k], &f[k])) return fail(CVX_ERR_PARSE, "bad texture coordinate");
            c.vt.insert(c.vt.end(), f, f + 2);
        } else if (kw == "usemtl") {
            if (toks.size() < 2) return fail(CVX_ERR_PARSE, "missing material name");
            bool found = false;
            uint32_t m = 0;
            for (uint32_t k = 0; k < n_materials; k++)
                if (toks[1] == names[k]) {
                    m = materials[k];
                    found = true;
                }
            if (!found) return fail(CVX_ERR_PARSE, "material '" + std::string(toks[1]) + "' not present in material dictionary");
            c.mats.push_back(m);
        } else if (kw == "f") {
            if (toks.size() < 4) return fail(CVX_ERR_PARSE, "missing triangle index");
            ChunkFace f;
            f.line = c.lines;
            f.v_before = (uint32_t)(c.v.size() / 3);
            f.t_before = (uint32_t)(c.vt.size() / 2);
            f.mat_record = (int32_t)c.mats.size() - 1;
            f.first = (uint32_t)c.vi.size();
            f.count = (uint32_t)(toks.size() - 1);
            for (size_t k = 1; k < toks.size(); k++) {
                uint32_t v;
                int64_t t;
                if (!parse_vertex_index(toks[k], &v, &t)) return fail(CVX_ERR_PARSE, "bad face index '" + std::string(toks[k]) + "'");
                c.vi.push_back(v);
                c.ti.push_back(t);
            }
            c.faces.push_back(f);
        }
    }
}

static int32_t parse_obj(const char* text, size_t len, const char* const* names, const uint32_t* materials,
                         uint32_t n_materials, cvx_mesh** out) {
    // CONVECTOR_OBJ_THREADS=n fixes the number of chunks (1: the sequential
    // parser) whatever the input size; by default inputs under 1 MiB are
    // parsed sequentially and larger ones on every hardware thread.
    unsigned hw = std::thread::hardware_concurrency();
    size_t nchunks = std::min<size_t>(hw ? hw : 1, 64);
    bool forced = false;
    if (const char* env = std::getenv("CONVECTOR_OBJ_THREADS")) {
        long n = std::strtol(env, nullptr, 10);
        if (n >= 1) {
            nchunks = (size_t)std::min<long>(n, 256);
            forced = true;
        }
    }
    if ((!forced && len < (1u << 20)) || nchunks < 2 || len == 0)
        return parse_obj_sequential(text, len, names, materials, n_materials, out);
    // Cut at line starts.
    std::vector<Chunk> ch(nchunks);
    size_t at = 0;
    for (size_t k = 0; k < nchunks; k++) {
        ch[k].begin = at;
        size_t e = k + 1 == nchunks ? len : std::max(at, len * (k + 1) / nchunks);
        while (e > 0 && e < len && text[e - 1] != '\n') e++;
        ch[k].end = e;
        at = e;
    }
    {
        std::vector<std::thread> pool;
        for (auto& c : ch) pool.emplace_back([&, cp = &c] { parse_chunk(text, *cp, names, materials, n_materials); });
        for (auto& t : pool) t.join();
    }
    // Global counts before each chunk; the first tokenising error in file order.
    std::vector<uint32_t> line0(nchunks), v0(nchunks), t0(nchunks), mat0(nchunks);
    uint32_t lines = 0, nv = 0, nt = 0, mat = 0x00ffffffu;  // SMaterial::white()
    for (size_t k = 0; k < nchunks; k++) {
        line0[k] = lines;
        v0[k] = nv;
        t0[k] = nt;
        mat0[k] = mat;
        if (ch[k].err) {
            char where[64];
            std::snprintf(where, sizeof where, " (line %u)", lines + ch[k].err_line);
            // a face error earlier in the file must win over this one
            ch[k].err_line += lines;
            ch[k].err_msg += where;
        }
        lines += ch[k].lines;
        nv += (uint32_t)(ch[k].v.size() / 3);
        nt += (uint32_t)(ch[k].vt.size() / 2);
        if (!ch[k].mats.empty()) mat = ch[k].mats.back();
    }
    std::unique_ptr<cvx_mesh> mesh(new cvx_mesh());
    mesh->vertices.reserve((size_t)nv * 3);
    mesh->tex_coords.reserve((size_t)nt * 2);
    for (auto& c : ch) {
        mesh->vertices.insert(mesh->vertices.end(), c.v.begin(), c.v.end());
        mesh->tex_coords.insert(mesh->tex_coords.end(), c.vt.begin(), c.vt.end());
    }
    // Faces: range and degeneracy checks and fan triangulation, per chunk.
    std::vector<std::vector<MeshTri>> tris(nchunks);
    std::vector<uint32_t> face_err_line(nchunks, 0);
    std::vector<int32_t> face_err(nchunks, CVX_OK);
    std::vector<std::string> face_msg(nchunks);
    {
        std::vector<std::thread> pool;
        for (size_t k = 0; k < nchunks; k++)
            pool.emplace_back([&, k] {
                for (const ChunkFace& f : ch[k].faces) {
                    const uint32_t* vi = &ch[k].vi[f.first];
                    const int64_t* ti = &ch[k].ti[f.first];
                    uint32_t visible = v0[k] + f.v_before;  // vertices defined before this line
                    uint32_t material = f.mat_record >= 0 ? ch[k].mats[f.mat_record] : mat0[k];
                    auto where = [&] { return " (line " + std::to_string(line0[k] + f.line) + ")"; };
                    for (size_t j = 2; j < f.count; j++) {
                        uint32_t a = vi[0], b = vi[j - 1], c = vi[j];
                        if (a >= visible || b >= visible || c >= visible) {
                            face_err[k] = CVX_ERR_PARSE;
                            face_err_line[k] = line0[k] + f.line;
                            face_msg[k] = std::string("vertex index out of range") + where();
                            return;
                        }
                        S3 va = s3(&mesh->vertices[3 * (size_t)a]), vb = s3(&mesh->vertices[3 * (size_t)b]),
                           vc = s3(&mesh->vertices[3 * (size_t)c]);
                        S3 cr = scross(va - vc, vb - va);
                        if (sdot(cr, cr) == 0.0f) {
                            face_err[k] = CVX_ERR_DEGENERATE;
                            face_err_line[k] = line0[k] + f.line;
                            face_msg[k] = std::string("encountered degenerate triangle") + where();
                            return;
                        }
                        MeshTri t;
                        t.v[0] = a;
                        t.v[1] = b;
                        t.v[2] = c;
                        bool has_t = ti[0] >= 0 && ti[j - 1] >= 0 && ti[j] >= 0;
                        t.t[0] = has_t ? ti[0] : -1;
                        t.t[1] = has_t ? ti[j - 1] : -1;
                        t.t[2] = has_t ? ti[j] : -1;
                        t.material = material;
                        tris[k].push_back(t);
                    }
                }
            });
        for (auto& t : pool) t.join();
    }
    // The first error in file order: a chunk's tokenising error stops that
    // chunk, so its face errors can only come from lines before it.
    for (size_t k = 0; k < nchunks; k++) {
        bool fe = face_err[k] != CVX_OK, te = ch[k].err != CVX_OK;
        if (fe && (!te || face_err_line[k] < ch[k].err_line)) return set_error(face_err[k], face_msg[k]);
        if (te) return set_error(ch[k].err, ch[k].err_msg);
    }
    size_t total = 0;
    for (auto& t : tris) total += t.size();
    mesh->triangles.reserve(total);
    for (auto& t : tris) mesh->triangles.insert(mesh->triangles.end(), t.begin(), t.end());
    *out = mesh.release();
    return CVX_OK;
}

// ---------------------------------------------------------------------------
// BVH build (bvh.rs:44-545)

struct Aabb {
    S3 lo, hi;
};
static inline Aabb enclose(const Aabb& a, const Aabb& b) { return Aabb{smin(a.lo, b.lo), smax(a.hi, b.hi)}; }
// aabb.rs:97-103
static inline float area(const Aabb& a) {
    S3 s = a.hi - a.lo;
    float x = s.y * s.z, y = s.z * s.x, z = s.x * s.y;
    return 2.0f * (x + y + z);
}

struct TriRef {  // bvh.rs:44-50
    Aabb aabb;
    S3 bc;
    uint32_t index;
};

struct Interim {  // bvh.rs:52-62
    Aabb outer, inner;
    std::vector<Interim> children;
    std::vector<TriRef> tris;
};

static Interim from_refs(std::vector<TriRef>&& refs) {  // bvh.rs:125-132
    Interim n;
    n.outer = refs[0].aabb;
    n.inner = Aabb{refs[0].bc, refs[0].bc};
    for (size_t i = 1; i < refs.size(); i++) {
        n.outer = enclose(n.outer, refs[i].aabb);
        n.inner.lo = smin(n.inner.lo, refs[i].bc);
        n.inner.hi = smax(n.inner.hi, refs[i].bc);
    }
    n.tris = std::move(refs);
    return n;
}

struct Bin {  // bvh.rs:64-121
    std::vector<const TriRef*> tris;
    Aabb aabb;
    void push(const TriRef* t) {
        aabb = tris.empty() ? t->aabb : enclose(aabb, t->aabb);
        tris.push_back(t);
    }
    void clear() { tris.clear(); }
};

// TreeSurfaceAreaHeuristic (bvh.rs:452-474) with the constants of bvh.rs:500-504:
//   aabb_term = 1 + ac_ap * (2p - n p^m) / (p - 2p^2),  m = log2(n)
//   tri_term  = n p^(m-1) * ac_ap
// The factors that depend on n alone (tsah_x, tsah_t) are shared with the
// device build, which reads them from a table made here, so that both builds
// round every operation alike.
static const float kTsahP = 0.8f;
static inline float tsah_x(float n) { return 2.0f * kTsahP - n * std::pow(kTsahP, std::log2(n)); }
static inline float tsah_t(float n) { return n * std::pow(kTsahP, std::log2(n) - 1.0f); }
static inline float tsah_y() { return kTsahP - 2.0f * kTsahP * kTsahP; }
static inline float tsah_aabb_cost(const Aabb& parent, const Aabb& box, size_t num_tris) {
    const float aabb_cost = 40.0f, tri_cost = 120.0f;
    float ac_ap = area(box) / area(parent);
    float n = (float)num_tris;
    float aabb_term = 1.0f + ac_ap * tsah_x(n) / tsah_y();
    float tri_term = tsah_t(n) * ac_ap;
    return aabb_term * aabb_cost + tri_term * tri_cost;
}
static inline float tsah_tris_cost(size_t n) { return (float)n * 120.0f; }

static void bin_uniform(const Interim& node, std::vector<Bin>& bins, int axis) {  // bvh.rs:176-201
    std::vector<const TriRef*> ptrs;
    ptrs.reserve(node.tris.size());
    for (const TriRef& t : node.tris) ptrs.push_back(&t);
    std::stable_sort(ptrs.begin(), ptrs.end(),
                     [axis](const TriRef* a, const TriRef* b) { return coord(a->bc, axis) < coord(b->bc, axis); });
    size_t per = (ptrs.size() + bins.size() - 1) / bins.size();
    if (per == 0) per = 1;
    size_t b = 0;
    for (size_t i = 0; i < ptrs.size(); i += per, b++)
        for (size_t k = i; k < std::min(i + per, ptrs.size()); k++) bins[b].push(ptrs[k]);
}

static void bin_tris(const Interim& node, std::vector<Bin>& bins, int axis) {  // bvh.rs:142-171
    size_t n = node.tris.size();
    if (n <= bins.size() / 2) return bin_uniform(node, bins, axis);
    float mn = coord(node.inner.lo, axis);
    float size = coord(node.inner.hi, axis) - mn;
    for (const TriRef& t : node.tris) {
        float f = std::floor((float)bins.size() * (coord(t.bc, axis) - mn) / size);
        // `as usize`: NaN and negative values saturate to 0.
        size_t idx = (f != f || f <= 0.0f) ? 0 : (f >= 1.8446744e19f ? SIZE_MAX : (size_t)f);
        if (idx >= bins.size()) idx = bins.size() - 1;
        bins[idx].push(&t);
        if (bins[idx].tris.size() > n / 8 && n > bins.size()) {
            for (Bin& b : bins) b.clear();
            return bin_uniform(node, bins, axis);
        }
    }
}

static bool enclose_bins(const std::vector<Bin>& bins, size_t from, size_t to, Aabb* out, size_t* count) {
    bool any = false;
    size_t c = 0;
    for (size_t i = from; i < to; i++) {
        if (bins[i].tris.empty()) continue;
        *out = any ? enclose(*out, bins[i].aabb) : bins[i].aabb;
        any = true;
        c += bins[i].tris.size();
    }
    *count = c;
    return any;
}

// bvh.rs:218-261
static float cheapest_split(const Interim& node, const std::vector<Bin>& bins, size_t* at) {
    size_t first = 0, last = 0;
    for (size_t i = 0; i < bins.size(); i++)
        if (!bins[i].tris.empty()) {
            first = i + 1;
            break;
        }
    for (size_t i = bins.size(); i-- > 0;)
        if (!bins[i].tris.empty()) {
            last = i + 1;
            break;
        }
    float best = 0.0f;
    bool is_first = true;
    for (size_t i = first; i < last; i++) {
        Aabb la, ra;
        size_t lc, rc;
        enclose_bins(bins, 0, i, &la, &lc);
        enclose_bins(bins, i, bins.size(), &ra, &rc);
        float cost = tsah_aabb_cost(node.outer, la, lc) + tsah_aabb_cost(node.outer, ra, rc);
        if (cost < best || is_first) {
            best = cost;
            *at = i;
            is_first = false;
        }
    }
    return best;
}

// bvh.rs:265-322
static void split(Interim& node) {
    if (node.tris.size() <= 1) return;
    std::vector<Bin> bins(64);
    std::vector<TriRef> best_l, best_r;
    float best_cost = 0.0f;
    bool is_first = true;
    for (int axis = 0; axis < 3; axis++) {
        bin_tris(node, bins, axis);
        size_t nonempty = 0;
        for (const Bin& b : bins) nonempty += !b.tris.empty();
        if (nonempty > 1) {
            size_t at = 0;
            float cost = cheapest_split(node, bins, &at);
            if (cost < best_cost || is_first) {
                best_l.clear();
                best_r.clear();
                for (size_t i = 0; i < bins.size(); i++)
                    for (const TriRef* t : bins[i].tris) (i < at ? best_l : best_r).push_back(*t);
                best_cost = cost;
                is_first = false;
            }
        }
        for (Bin& b : bins) b.clear();
    }
    if (is_first) return;  // the reference asserts here; all barycentres coincide
    if (tsah_tris_cost(node.tris.size()) < best_cost) return;
    node.children.push_back(from_refs(std::move(best_l)));
    node.children.push_back(from_refs(std::move(best_r)));
    node.tris.clear();
    node.tris.shrink_to_fit();
}

// bvh.rs:325-356. Subtrees are built concurrently, as with rayon::join; the
// result does not depend on the schedule.
static void split_recursive(Interim& node, int par_depth) {
    split(node);
    if (node.children.empty()) return;
    if (area(node.children[0].outer) > area(node.children[1].outer)) std::swap(node.children[0], node.children[1]);
    size_t n = node.children[0].tris.size() + node.children[1].tris.size();
    if (par_depth > 0 && n > 20000) {
        auto fut = std::async(std::launch::async, [&]() { split_recursive(node.children[0], par_depth - 1); });
        split_recursive(node.children[1], par_depth - 1);
        fut.get();
    } else {
        split_recursive(node.children[0], 0);
        split_recursive(node.children[1], 0);
    }
}

static void count(const Interim& n, size_t* nodes, size_t* leaves, size_t* tris) {
    (*nodes)++;
    if (n.children.empty()) (*leaves)++;
    *tris += n.tris.size();
    for (const Interim& c : n.children) count(c, nodes, leaves, tris);
}
static float summed_area_ratio(const Interim& n) {  // bvh.rs:380-385
    float child_contrib = 0.0f;
    for (const Interim& c : n.children) child_contrib += summed_area_ratio(c);
    float self_area = area(n.outer);
    float child_sum = 0.0f;
    for (const Interim& c : n.children) child_sum += area(c.outer) / self_area;
    return child_sum + child_contrib;
}

// bvh.rs:389-428
static void crystallize(const Interim& n, const std::vector<cvx_triangle>& src, cvx_bvh& out, size_t into,
                        uint32_t depth) {
    cvx_bvh_node& nd = out.nodes[into];
    nd.origin[0] = n.outer.lo.x;
    nd.origin[1] = n.outer.lo.y;
    nd.origin[2] = n.outer.lo.z;
    nd.far_[0] = n.outer.hi.x;
    nd.far_[1] = n.outer.hi.y;
    nd.far_[2] = n.outer.hi.z;
    out.depth = std::max(out.depth, depth);
    if (n.tris.empty()) {
        size_t child = out.nodes.size();
        out.nodes.push_back(cvx_bvh_node{});
        out.nodes.push_back(cvx_bvh_node{});
        crystallize(n.children[0], src, out, child, depth + 1);
        crystallize(n.children[1], src, out, child + 1, depth + 1);
        out.nodes[into].index = (uint32_t)child;
        out.nodes[into].len = 0;
    } else {
        out.nodes[into].index = (uint32_t)out.triangles.size();
        out.nodes[into].len = (uint32_t)n.tris.size();
        for (const TriRef& t : n.tris) {
            out.triangles.push_back(src[t.index]);
            out.source_index.push_back(t.index);
        }
    }
}

void tsah_tables(uint32_t n, std::vector<float>& x, std::vector<float>& t, float* y) {
    // Grown on demand and kept: the factors depend on the count alone.
    static std::mutex mu;
    static std::vector<float> cx{0.0f}, ct{0.0f};
    {
        std::lock_guard<std::mutex> lk(mu);
        for (uint32_t k = (uint32_t)cx.size(); k <= n; k++) {
            cx.push_back(tsah_x((float)k));
            ct.push_back(tsah_t((float)k));
        }
        x.assign(cx.begin(), cx.begin() + (size_t)n + 1);
        t.assign(ct.begin(), ct.begin() + (size_t)n + 1);
    }
    *y = tsah_y();
}

// crystallize (bvh.rs:389-428) and the statistics of bvh.rs:536-545 over an
// interim tree built elsewhere (the device build): node 0 is the root, a
// leaf's triangles are order[beg .. beg + cnt) in leaf order, and every child
// has a larger id than its parent. The recursion of crystallize becomes two
// linear passes: bottom-up (decreasing ids) subtree sizes and the summed area
// ratio, then top-down (increasing ids) each node's place in the depth-first
// order. A node's first child goes to 2 + 2 * (internal nodes before it in
// depth-first order), a leaf's triangles follow those of the leaves before it.
static float interim_area(const InterimNode& n) {
    Aabb a{S3{n.lo[0], n.lo[1], n.lo[2]}, S3{n.hi[0], n.hi[1], n.hi[2]}};
    return area(a);
}

int32_t bvh_from_interim(const std::vector<InterimNode>& t, const std::vector<uint32_t>& order,
                         const cvx_triangle* src, uint32_t n, cvx_bvh** out) {
    const size_t N = t.size();
    if (N == 0 || !t[0].c0)
        return set_error(CVX_ERR_INVALID,
                         "the BVH root did not split: the reference needs at least two root nodes (bvh.rs:509-512)");
    for (size_t v = 0; v < N; v++)
        if (t[v].c0 && (t[v].c0 <= v || t[v].c1 <= v || t[v].c0 >= N || t[v].c1 >= N))
            return set_error(CVX_ERR_DEVICE, "device BVH build: malformed interim tree");
    // Bottom-up: internal nodes and triangles per subtree; summed area ratio
    // with the operation order of bvh.rs:380-385.
    std::vector<uint32_t> sint(N), stri(N);
    std::vector<float> sar(N);
    for (size_t v = N; v-- > 0;) {
        const InterimNode& x = t[v];
        if (!x.c0) {
            sint[v] = 0;
            stri[v] = x.cnt;
            sar[v] = 0.0f;
            continue;
        }
        sint[v] = 1 + sint[x.c0] + sint[x.c1];
        stri[v] = stri[x.c0] + stri[x.c1];
        float child_contrib = 0.0f;
        child_contrib += sar[x.c0];
        child_contrib += sar[x.c1];
        float self_area = interim_area(x);
        float child_sum = 0.0f;
        child_sum += interim_area(t[x.c0]) / self_area;
        child_sum += interim_area(t[x.c1]) / self_area;
        sar[v] = child_sum + child_contrib;
    }
    if (stri[0] != n) return set_error(CVX_ERR_DEVICE, "device BVH build lost triangles");
    // Top-down: crystal index, internal nodes before in depth-first order,
    // first triangle, depth.
    std::vector<uint32_t> cidx(N), ipre(N), toff(N), dep(N);
    const InterimNode& root = t[0];
    cidx[root.c0] = 0;
    cidx[root.c1] = 1;
    ipre[root.c0] = 0;
    ipre[root.c1] = sint[root.c0];
    toff[root.c0] = 0;
    toff[root.c1] = stri[root.c0];
    dep[root.c0] = dep[root.c1] = 1;
    for (size_t v = 1; v < N; v++) {
        const InterimNode& x = t[v];
        if (!x.c0) continue;
        uint32_t child = 2 + 2 * ipre[v];
        cidx[x.c0] = child;
        cidx[x.c1] = child + 1;
        ipre[x.c0] = ipre[v] + 1;
        ipre[x.c1] = ipre[v] + 1 + sint[x.c0];
        toff[x.c0] = toff[v];
        toff[x.c1] = toff[v] + stri[x.c0];
        dep[x.c0] = dep[x.c1] = dep[v] + 1;
    }
    std::unique_ptr<cvx_bvh> bvh(new cvx_bvh());
    const size_t M = 2 + 2 * (size_t)(sint[0] - 1);
    if (M != N - 1) return set_error(CVX_ERR_DEVICE, "device BVH build: unreachable interim nodes");
    bvh->nodes.assign(M, cvx_bvh_node{});
    bvh->triangles.resize(n);
    bvh->source_index.resize(n);
    size_t leaves = 0;
    uint32_t depth = 0;
    std::vector<uint32_t> leaf_ids;
    leaf_ids.reserve(N / 2 + 1);
    for (size_t v = 1; v < N; v++) {
        const InterimNode& x = t[v];
        cvx_bvh_node& nd = bvh->nodes[cidx[v]];
        for (int k = 0; k < 3; k++) {
            nd.origin[k] = x.lo[k];
            nd.far_[k] = x.hi[k];
        }
        nd.index = x.c0 ? 2 + 2 * ipre[v] : toff[v];
        nd.len = x.c0 ? 0u : x.cnt;
        depth = std::max(depth, dep[v]);
        if (!x.c0) {
            leaves++;
            leaf_ids.push_back((uint32_t)v);
        }
    }
    // Triangles in leaf order, gathered on all host threads.
    unsigned hw = std::thread::hardware_concurrency();
    size_t nth = std::max<size_t>(1, std::min<size_t>(hw ? hw : 1, (leaf_ids.size() + 4095) / 4096));
    std::vector<std::thread> pool;
    for (size_t k = 0; k < nth; k++)
        pool.emplace_back([&, k] {
            for (size_t i = k; i < leaf_ids.size(); i += nth) {
                const InterimNode& x = t[leaf_ids[i]];
                uint32_t o = toff[leaf_ids[i]];
                for (uint32_t j = 0; j < x.cnt; j++) {
                    uint32_t tri = order[x.beg + j];
                    bvh->triangles[o + j] = src[tri];
                    bvh->source_index[o + j] = tri;
                }
            }
        });
    for (auto& th : pool) th.join();
    bvh->depth = depth;
    size_t num_nodes = M + 1;  // the interim nodes: crystallized ones and the root
    bvh->avg_area_ratio = sar[0] / (float)num_nodes;
    bvh->avg_tris_per_leaf = (float)n / (float)leaves;
    *out = bvh.release();
    return CVX_OK;
}

static int32_t build(const cvx_triangle* tris, uint32_t n, cvx_bvh** out) {
    if (n == 0) return set_error(CVX_ERR_INVALID, "cannot build a BVH of zero triangles");
    // Node and triangle indices are 32-bit, and a scene holds fewer than 2^27
    // triangles (cvx_scene_create).
    if (n >= (1u << 27)) return set_error(CVX_ERR_INVALID, "a BVH holds fewer than 2^27 triangles");
    std::vector<cvx_triangle> src(tris, tris + n);
    std::vector<TriRef> refs(n);
    const float third = 1.0f / 3.0f;  // 3.0f32.recip()
    for (uint32_t i = 0; i < n; i++) {
        S3 v0 = s3(tris[i].v0), v1 = s3(tris[i].v1), v2 = s3(tris[i].v2);
        refs[i].aabb = Aabb{smin(smin(v0, v1), v2), smax(smax(v0, v1), v2)};
        refs[i].bc = (v0 + v1 + v2) * third;
        refs[i].index = i;
    }
    Interim root = from_refs(std::move(refs));
    split_recursive(root, 4);
    if (root.children.size() != 2)
        return set_error(CVX_ERR_INVALID,
                         "the BVH root did not split: the reference needs at least two root nodes (bvh.rs:509-512)");
    std::unique_ptr<cvx_bvh> bvh(new cvx_bvh());
    size_t num_nodes = 0, num_leaves = 0, num_tris = 0;
    count(root, &num_nodes, &num_leaves, &num_tris);
    bvh->nodes.reserve(num_nodes);
    bvh->triangles.reserve(num_tris);
    bvh->nodes.push_back(cvx_bvh_node{});
    bvh->nodes.push_back(cvx_bvh_node{});
    crystallize(root.children[0], src, *bvh, 0, 1);
    crystallize(root.children[1], src, *bvh, 1, 1);
    bvh->avg_area_ratio = summed_area_ratio(root) / (float)num_nodes;
    bvh->avg_tris_per_leaf = (float)num_tris / (float)num_leaves;
    *out = bvh.release();
    return CVX_OK;
}

}  // namespace cvx

using namespace cvx;

extern "C" {

int32_t cvx_last_error(char* buf, size_t len) {
    if (buf && len) {
        std::strncpy(buf, g_last_error.c_str(), len - 1);
        buf[len - 1] = '\0';
    }
    return g_last_status;
}

int32_t cvx_mesh_parse_obj(const char* text, size_t len, const char* const* names, const uint32_t* materials,
                           uint32_t n_materials, cvx_mesh** out) {
    if (!out || (!text && len)) return set_error(CVX_ERR_INVALID, "null argument");
    return parse_obj(text, len, names, materials, n_materials, out);
}

int32_t cvx_mesh_load_obj(const char* path, const char* const* names, const uint32_t* materials,
                          uint32_t n_materials, cvx_mesh** out) {
    if (!path || !out) return set_error(CVX_ERR_INVALID, "null argument");
    std::ifstream f(path, std::ios::binary);
    if (!f) return set_error(CVX_ERR_IO, std::string("failed to open file ") + path);
    std::stringstream ss;
    ss << f.rdbuf();
    std::string s = ss.str();
    return parse_obj(s.data(), s.size(), names, materials, n_materials, out);
}

uint32_t cvx_mesh_num_triangles(const cvx_mesh* m) { return m ? (uint32_t)m->triangles.size() : 0u; }
void cvx_mesh_destroy(cvx_mesh* m) { delete m; }

int32_t cvx_bvh_from_meshes(const cvx_mesh* const* meshes, uint32_t n_meshes, cvx_bvh** out) {
    if (!out || (!meshes && n_meshes)) return set_error(CVX_ERR_INVALID, "null argument");
    std::vector<cvx_triangle> tris;
    for (uint32_t m = 0; m < n_meshes; m++) {
        const cvx_mesh& mesh = *meshes[m];
        size_t ntc = mesh.tex_coords.size() / 2;
        for (const MeshTri& t : mesh.triangles) {
            cvx_triangle tr;
            std::memset(&tr, 0, sizeof tr);
            std::memcpy(tr.v0, &mesh.vertices[3 * t.v[0]], 12);
            std::memcpy(tr.v1, &mesh.vertices[3 * t.v[1]], 12);
            std::memcpy(tr.v2, &mesh.vertices[3 * t.v[2]], 12);
            if (t.t[0] >= 0) {
                for (int k = 0; k < 3; k++)
                    if ((size_t)t.t[k] >= ntc) return set_error(CVX_ERR_PARSE, "texture coordinate index out of range");
                std::memcpy(tr.uv0, &mesh.tex_coords[2 * t.t[0]], 8);
                std::memcpy(tr.uv1, &mesh.tex_coords[2 * t.t[1]], 8);
                std::memcpy(tr.uv2, &mesh.tex_coords[2 * t.t[2]], 8);
            }
            tr.material = t.material;
            tris.push_back(tr);
        }
    }
    return build(tris.data(), (uint32_t)tris.size(), out);
}

int32_t cvx_bvh_build(const cvx_triangle* triangles, uint32_t n, cvx_bvh** out) {
    if (!out || (!triangles && n)) return set_error(CVX_ERR_INVALID, "null argument");
    return build(triangles, n, out);
}

uint32_t cvx_bvh_num_nodes(const cvx_bvh* b) { return b ? (uint32_t)b->nodes.size() : 0u; }
uint32_t cvx_bvh_num_triangles(const cvx_bvh* b) { return b ? (uint32_t)b->triangles.size() : 0u; }
void cvx_bvh_copy_nodes(const cvx_bvh* b, cvx_bvh_node* out) {
    std::memcpy(out, b->nodes.data(), b->nodes.size() * sizeof(cvx_bvh_node));
}
void cvx_bvh_copy_triangles(const cvx_bvh* b, cvx_triangle* out) {
    std::memcpy(out, b->triangles.data(), b->triangles.size() * sizeof(cvx_triangle));
}
void cvx_bvh_copy_source_index(const cvx_bvh* b, uint32_t* out) {
    std::memcpy(out, b->source_index.data(), b->source_index.size() * sizeof(uint32_t));
}
void cvx_bvh_stats(const cvx_bvh* b, float* avg_tris_per_leaf, float* avg_area_ratio, uint32_t* depth) {
    if (avg_tris_per_leaf) *avg_tris_per_leaf = b->avg_tris_per_leaf;
    if (avg_area_ratio) *avg_area_ratio = b->avg_area_ratio;
    if (depth) *depth = b->depth;
}
void cvx_bvh_destroy(cvx_bvh* b) { delete b; }

// scene.rs:34-42
void cvx_camera_default(cvx_camera* c) {
    std::memset(c, 0, sizeof *c);
    c->orientation[0] = 1.0f;
    c->screen_distance = 1.0f / std::sin(3.14159265358979323846f / 5.0f);
}
// scene.rs:66-74
void cvx_camera_set_rotation(cvx_camera* c, float radians, float delta) {
    float x = std::cos(radians * 0.5f), y = std::sin(radians * 0.5f);
    c->orientation[0] = x;
    c->orientation[1] = 0.0f;
    c->orientation[2] = -y;
    c->orientation[3] = 0.0f;
    float x_delta = 0.5f * -std::sin(radians * 0.5f) * delta;
    float y_delta = 0.5f * std::cos(radians * 0.5f) * delta;
    c->orientation_delta[0] = x_delta;
    c->orientation_delta[1] = 0.0f;
    c->orientation_delta[2] = -y_delta;
    c->orientation_delta[3] = 0.0f;
}
// scene.rs:61-63
void cvx_camera_set_fov(cvx_camera* c, float fov) { c->screen_distance = 1.0f / std::sin(fov / 2.0f); }

// Renderer::update_scene (renderer.rs:140-147): the interactive camera path
// around the scene at `time` seconds, moving by `time_delta` over one frame.
void cvx_camera_set_interactive(cvx_camera* c, float time, float time_delta) {
    float alpha = time * -0.02f + 0.1f;
    float alpha_delta = time_delta * -0.02f;
    float sa = std::sin(alpha), ca = std::cos(alpha);
    // scene.rs:47-50 (set_position) with SVector3 * f32 (vector3.rs)
    c->position[0] = -3.8f * sa;
    c->position[1] = 1.6f;
    c->position[2] = 3.0f * ca;
    c->position_delta[0] = (-3.8f * ca) * alpha_delta;
    c->position_delta[1] = 0.0f * alpha_delta;
    c->position_delta[2] = (-3.0f * sa) * alpha_delta;
    cvx_camera_set_rotation(c, alpha, alpha_delta);
}

}  // extern "C"
