// The device half of the C-ABI (include/convector_gpu.h): scene upload,
// nearest-hit queries and frame rendering.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "device_guard.cuh"
#include "engine.h"
#include "internal.h"
#include "kernels.h"
#include "x86_approx_tables.h"

using namespace cvx;

namespace {

const uint32_t kRcp32[2048] = CVX_RCP_TABLE_INIT;
const uint32_t kRsqrt32[2048] = CVX_RSQRT_TABLE_INIT;

std::mutex g_init_mu;
std::vector<bool> g_tables_ready;

int32_t cuda_fail(cudaError_t e, const char* what) {
    return set_error(CVX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call, what)                                \
    do {                                              \
        cudaError_t e_ = (call);                      \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

// Uploads the approximation tables once per device.
int32_t ensure_device(int* dev_out) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) return set_error(CVX_ERR_CUDA, "no CUDA device available");
    int dev = 0;
    CK(cudaGetDevice(&dev), "cudaGetDevice");
    std::lock_guard<std::mutex> lk(g_init_mu);
    if ((int)g_tables_ready.size() < n) g_tables_ready.resize(n, false);
    if (!g_tables_ready[dev]) {
        uint16_t r[2048], s[2048];
        for (int i = 0; i < 2048; i++) {
            r[i] = (uint16_t)(kRcp32[i] >> 11);
            s[i] = (uint16_t)(kRsqrt32[i] >> 11);
        }
        CK(upload_tables(r, s), "upload approximation tables");
        CK(upload_tables_wave(r, s), "upload approximation tables");
        g_tables_ready[dev] = true;
    }
    *dev_out = dev;
    return CVX_OK;
}

// Device allocations that succeed before an injected failure (-1: none
// pending). Process-wide: the allocation helpers of every thread count down.
std::atomic<int64_t> g_alloc_countdown{-1};

template <class T>
int32_t dalloc(T** p, size_t count, const char* what) {
    *p = nullptr;
    if (count == 0) count = 1;
    if (injected_allocation_failure())
        return set_error(CVX_ERR_CAPACITY, std::string("cudaMalloc ") + what + ": out of memory (injected)");
    cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(e == cudaErrorMemoryAllocation ? CVX_ERR_CAPACITY : CVX_ERR_CUDA,
                         std::string("cudaMalloc ") + what + ": " + cudaGetErrorString(e));
    }
    return CVX_OK;
}

// Host memory the driver can copy without staging (allocated or registered
// page-locked through CUDA).
bool page_locked(const void* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

}  // namespace

bool cvx::injected_allocation_failure() {
    int64_t v = g_alloc_countdown.load();
    while (v >= 0)
        if (g_alloc_countdown.compare_exchange_weak(v, v - 1)) return v == 0;
    return false;
}

struct cvx_scene {
    int device = 0;
    float4* d_nodes = nullptr;  // escape slots (node_offset float4), then the node pairs
    size_t node_offset = 0;
    float4* d_geom = nullptr;
    TriShade* d_shade = nullptr;
    float4* d_lights = nullptr;
    uint32_t* d_err = nullptr;
    uint32_t n_nodes = 0, n_tris = 0, n_lights = 0, depth = 0;
    uint32_t general_pick = 1;
    uint32_t blocks_per_sm = 0;  // launch shape of the nearest-hit query (0: default)
    uint32_t query_stack = 8;    // stack entries per lane in shared memory (cvx_scene_set_query_stack)
    // The device reads host memory through the host's page tables (address
    // translation over a coherent CPU-GPU link): the host-buffer query may
    // read the caller's ray arrays in place. host_access: CVX_HOST_ACCESS_*.
    bool host_page_tables = false;
    bool slab_sel = false;  // DeviceScene::slab_sel
    uint32_t host_access = CVX_HOST_ACCESS_AUTO;
    bool reads_host_in_place() const { return host_page_tables && host_access == CVX_HOST_ACCESS_AUTO; }
    // scratch for the host-buffer query
    float* d_rays = nullptr;
    float* d_t = nullptr;
    int32_t* d_tri = nullptr;
    size_t scratch_n = 0;
    cudaStream_t stream = nullptr;
    // the host-buffer query's copy/compute pipeline: streams and per-chunk
    // (status, ray counter) words
    cudaStream_t qstreams[3] = {nullptr, nullptr, nullptr};
    uint32_t* d_qerr = nullptr;
    uint32_t* h_qerr = nullptr;  // page-locked copy of d_qerr

    DeviceScene view() const {
        DeviceScene s;
        s.nodes = d_nodes + node_offset;
        s.geom = d_geom;
        s.shade = d_shade;
        s.lights = d_lights;
        s.n_nodes = n_nodes;
        s.n_tris = n_tris;
        s.n_lights = n_lights;
        s.general_pick = general_pick;
        s.depth = depth;
        s.slab_sel = slab_sel ? 1u : 0u;
        return s;
    }
    ~cvx_scene() {
        cudaFree(d_nodes);
        cudaFree(d_geom);
        cudaFree(d_shade);
        cudaFree(d_lights);
        cudaFree(d_err);
        cudaFree(d_rays);
        cudaFree(d_t);
        cudaFree(d_tri);
        cudaFree(d_qerr);
        if (h_qerr) cudaFreeHost(h_qerr);
        for (cudaStream_t q : qstreams)
            if (q) cudaStreamDestroy(q);
        if (stream) cudaStreamDestroy(stream);
    }
};

DeviceScene cvx::scene_view(const cvx_scene* s) { return s->view(); }
cudaStream_t cvx::scene_stream(const cvx_scene* s) { return s->stream; }
uint32_t cvx::scene_depth(const cvx_scene* s) { return s->depth; }
uint32_t cvx::scene_num_lights(const cvx_scene* s) { return s->n_lights; }
int cvx::scene_device(const cvx_scene* s) { return s->device; }
uint32_t cvx::scene_query_blocks_per_sm(const cvx_scene* s) { return s->blocks_per_sm; }
uint32_t cvx::scene_query_stack(const cvx_scene* s) { return s->query_stack; }

struct cvx_renderer {
    std::unique_ptr<WaveEngine> engine;  // wavefront mode
    cvx_scene* scene = nullptr;
    int device = 0;  // the scene's
    uint32_t w = 0, h = 0;
    cvx_render_config cfg{};
    DeviceCamera cam{};
    uint32_t* d_rgba = nullptr;
    uint32_t* d_gbuf = nullptr;
    float* d_color = nullptr;
    float* d_accum = nullptr;
    unsigned long long* d_rays = nullptr;
    uint32_t* d_err = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    uint64_t last_rays = 0;
    float time = 0.0f, time_delta = 0.0f;  // Renderer::set_time (renderer.rs:134-137)
    float last_ms = 0.0f;
    bool debug = false;
    uint32_t* d_patches = nullptr;  // patch origins of the patch entry points
    uint32_t patch_cap = 0;
    uint32_t* d_group_em = nullptr;  // per 8-pixel group: lanes that hit an emitter at bounce 0
    unsigned long long* d_work = nullptr;  // cvx_renderer_count_work's counters (allocated at first use)
    float* d_samples = nullptr;  // cvx_accumulate_frames_f32's sample colours (allocated at first use)
    size_t samples_cap = 0;      // floats
    ~cvx_renderer() {
        cudaFree(d_samples);
        cudaFree(d_work);
        cudaFree(d_group_em);
        cudaFree(d_patches);
        cudaFree(d_rgba);
        cudaFree(d_gbuf);
        cudaFree(d_color);
        cudaFree(d_accum);
        cudaFree(d_rays);
        cudaFree(d_err);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (stream) cudaStreamDestroy(stream);
    }
};

// Checks the tree and returns its depth (roots at depth 1).
static int32_t validate_tree(const cvx_bvh_node* nodes, uint32_t n_nodes, uint32_t n_tris, uint32_t* depth_out) {
    if (n_nodes < 2 || (n_nodes & 1u)) return set_error(CVX_ERR_INVALID, "node count must be even and at least 2");
    std::vector<std::pair<uint32_t, uint32_t>> stack{{0u, 1u}, {1u, 1u}};
    uint32_t depth = 0;
    size_t visited = 0;
    while (!stack.empty()) {
        auto [i, dep] = stack.back();
        stack.pop_back();
        if (++visited > n_nodes) return set_error(CVX_ERR_INVALID, "BVH nodes form a cycle");
        depth = dep > depth ? dep : depth;
        const cvx_bvh_node& nd = nodes[i];
        if (nd.len == 0) {
            if ((nd.index & 1u) || nd.index + 1 >= n_nodes || nd.index < 2)
                return set_error(CVX_ERR_INVALID, "internal node child index out of range");
            stack.push_back({nd.index, dep + 1});
            stack.push_back({nd.index + 1, dep + 1});
        } else if ((uint64_t)nd.index + nd.len > n_tris) {
            return set_error(CVX_ERR_INVALID, "leaf triangle range out of range");
        }
    }
    *depth_out = depth;
    return CVX_OK;
}

extern "C" {

int32_t cvx_device_info(int32_t* ordinal, char* name, size_t name_len) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return set_error(CVX_ERR_CUDA, "no CUDA device available");
    }
    int dev = 0;
    CK(cudaGetDevice(&dev), "cudaGetDevice");
    cudaDeviceProp prop{};
    CK(cudaGetDeviceProperties(&prop, dev), "cudaGetDeviceProperties");
    if (ordinal) *ordinal = dev;
    if (name && name_len) {
        std::strncpy(name, prop.name, name_len - 1);
        name[name_len - 1] = '\0';
    }
    return CVX_OK;
}

int32_t cvx_set_traversal_stack_limit(uint32_t entries) {
    if (entries == 0) entries = (uint32_t)kStackDepth;
    if (entries < 2 || entries > (uint32_t)kStackDepth)
        return set_error(CVX_ERR_INVALID, "the traversal stack limit must be 2.." + std::to_string(kStackDepth));
    int dev = 0;
    int32_t st = ensure_device(&dev);
    if (st) return st;
    CK(set_stack_limit((int)entries), "set the traversal stack limit");
    CK(set_stack_limit_wave((int)entries), "set the traversal stack limit");
    return CVX_OK;
}

int32_t cvx_inject_allocation_failure(int32_t after) {
    g_alloc_countdown.store(after < 0 ? -1 : (int64_t)after);
    return CVX_OK;
}

int32_t cvx_scene_create(const cvx_triangle* tris, uint32_t n_tris, const cvx_bvh_node* nodes, uint32_t n_nodes,
                         cvx_scene** out) {
    if (!tris || !nodes || !out || n_tris == 0) return set_error(CVX_ERR_INVALID, "null argument or empty scene");
    if (n_tris >= (1u << 27) || n_nodes >= (1u << 27))
        return set_error(CVX_ERR_INVALID, "scenes are limited to 2^27 triangles and 2^27 nodes");
    uint32_t depth = 0;
    int32_t st = validate_tree(nodes, n_nodes, n_tris, &depth);
    if (st) return st;
    if (depth + 2 > (uint32_t)kStackDepth)
        return set_error(CVX_ERR_INVALID, "BVH deeper than the device traversal stack (" +
                                              std::to_string(depth) + " levels)");
    std::vector<uint32_t> ds;
    for (uint32_t i = 0; i < n_tris; i++) {
        if (((tris[i].material >> 26) & 7u) > 5u)
            return set_error(CVX_ERR_INVALID, "glossiness index above 5 (material.rs:497-512 has six entries)");
        if ((tris[i].material >> 30) & 1u) ds.push_back(i);  // scene.rs:117-122
    }
    int dev = 0;
    st = ensure_device(&dev);
    if (st) return st;
    std::unique_ptr<cvx_scene> s(new cvx_scene());
    s->device = dev;
    int host_tables = 0;
    if (cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess) {
        cudaGetLastError();
        host_tables = 0;
    }
    s->host_page_tables = host_tables == 1;
    s->n_nodes = n_nodes;
    s->n_tris = n_tris;
    s->n_lights = (uint32_t)ds.size();
    s->depth = depth;
    CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    // The no-allocation query's static buffer is reserved here, where
    // allocating is expected, not at that query's first call.
    if ((st = noalloc_setup_device())) return st;
    if ((st = dalloc(&s->d_geom, (size_t)n_tris * 3, "triangles"))) return st;
    if ((st = dalloc(&s->d_shade, n_tris, "shading data"))) return st;
    if ((st = dalloc(&s->d_lights, (size_t)s->n_lights * 5, "lights"))) return st;
    if ((st = dalloc(&s->d_err, 2, "status"))) return st;  // [0] status, [1] ray counter
    // The select-form slab test (box_test_sel) needs every bound finite and
    // ordered, and none -0.
    s->slab_sel = true;
    for (uint32_t i = 0; i < n_nodes && s->slab_sel; i++)
        for (int c = 0; c < 3; c++) {
            const float lo = nodes[i].origin[c], hi = nodes[i].far_[c];
            if (!std::isfinite(lo) || !std::isfinite(hi) || !(lo <= hi) || (lo == 0.0f && std::signbit(lo)) ||
                (hi == 0.0f && std::signbit(hi)))
                s->slab_sel = false;
        }
    // Node pairs: q0 = lo0 hi0.x | q1 = hi0.yz lo1.xy | q2 = lo1.z hi1 | q3 = index/len x2
    // q3 holds the two children's stack references, the form the traversal
    // pushes (traverse.cuh): (index << 5) | len for internal nodes (len 0, index =
    // first child) and leaves of up to 30 triangles; (slot << 5) | 31 for larger
    // leaves, whose (index, len) is escape slot `slot`, the float4 at
    // nodes[-1 - slot] below the pairs (the region is padded to 8 float4, so the
    // pairs keep their 128-byte alignment).
    std::vector<uint2> esc;
    auto child_ref = [&esc](const cvx_bvh_node& nd) -> uint32_t {
        if (nd.len < 31u) return (nd.index << 5) | nd.len;
        esc.push_back(make_uint2(nd.index, nd.len));
        return ((uint32_t)(esc.size() - 1) << 5) | 31u;
    };
    std::vector<float4> pairs((size_t)n_nodes / 2 * 4);
    for (uint32_t p = 0; p < n_nodes / 2; p++) {
        const cvx_bvh_node& a = nodes[2 * p];
        const cvx_bvh_node& b = nodes[2 * p + 1];
        float4* q = &pairs[4 * (size_t)p];
        q[0] = make_float4(a.origin[0], a.origin[1], a.origin[2], a.far_[0]);
        q[1] = make_float4(a.far_[1], a.far_[2], b.origin[0], b.origin[1]);
        q[2] = make_float4(b.origin[2], b.far_[0], b.far_[1], b.far_[2]);
        uint32_t w[4] = {child_ref(a), child_ref(b), 0u, 0u};
        std::memcpy(&q[3], w, 16);
    }
    s->node_offset = (esc.size() + 7) / 8 * 8;
    std::vector<float4> node_buf(s->node_offset + pairs.size());
    for (size_t k = 0; k < esc.size(); k++) {
        uint32_t e[4] = {esc[k].x, esc[k].y, 0u, 0u};
        std::memcpy(&node_buf[s->node_offset - 1 - k], e, 16);
    }
    std::copy(pairs.begin(), pairs.end(), node_buf.begin() + (std::ptrdiff_t)s->node_offset);
    if ((st = dalloc(&s->d_nodes, node_buf.size(), "nodes"))) return st;
    CK(cudaMemcpyAsync(s->d_nodes, node_buf.data(), node_buf.size() * sizeof(float4), cudaMemcpyHostToDevice,
                       s->stream),
       "upload nodes");
    cvx_triangle* d_src = nullptr;
    uint32_t* d_ds = nullptr;
    if ((st = dalloc(&d_src, n_tris, "staging"))) return st;
    if ((st = dalloc(&d_ds, ds.size(), "staging"))) {
        cudaFree(d_src);
        return st;
    }
    cudaError_t e = cudaMemcpyAsync(d_src, tris, (size_t)n_tris * sizeof(cvx_triangle), cudaMemcpyHostToDevice,
                                    s->stream);
    if (e == cudaSuccess && !ds.empty())
        e = cudaMemcpyAsync(d_ds, ds.data(), ds.size() * 4, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = launch_prep_geom(d_src, n_tris, s->d_geom, s->d_shade, s->stream);
    if (e == cudaSuccess && !ds.empty()) e = launch_prep_lights(d_src, d_ds, s->n_lights, s->d_lights, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(d_src);
    cudaFree(d_ds);
    if (e != cudaSuccess) return cuda_fail(e, "scene upload");
    *out = s.release();
    return CVX_OK;
}

int32_t cvx_scene_from_bvh(const cvx_bvh* bvh, cvx_scene** out) {
    if (!bvh) return set_error(CVX_ERR_INVALID, "null bvh");
    return cvx_scene_create(bvh->triangles.data(), (uint32_t)bvh->triangles.size(), bvh->nodes.data(),
                            (uint32_t)bvh->nodes.size(), out);
}

uint32_t cvx_scene_num_direct_samples(const cvx_scene* s) { return s ? s->n_lights : 0u; }

int32_t cvx_scene_set_light_pick(cvx_scene* s, uint32_t light_pick) {
    if (!s) return set_error(CVX_ERR_INVALID, "null scene");
    if (light_pick == 0 && s->n_lights != 8)
        return set_error(CVX_ERR_INVALID, "the reference light pick (bits >> 29) needs exactly 8 direct-sample triangles");
    s->general_pick = light_pick ? 1u : 0u;
    return CVX_OK;
}

int32_t cvx_scene_set_host_access(cvx_scene* s, uint32_t mode, uint32_t* in_place) {
    if (!s || mode > CVX_HOST_ACCESS_COPY) return set_error(CVX_ERR_INVALID, "bad host access mode");
    s->host_access = mode;
    if (in_place) *in_place = s->reads_host_in_place() ? 1u : 0u;
    return CVX_OK;
}

int32_t cvx_scene_set_query_stack(cvx_scene* s, uint32_t shared_entries) {
    if (!s || (shared_entries != 0 && shared_entries != 4 && shared_entries != 8 && shared_entries != 12))
        return set_error(CVX_ERR_INVALID, "shared stack entries must be 0, 4, 8 or 12");
    s->query_stack = shared_entries;
    return CVX_OK;
}

int32_t cvx_scene_set_query_launch(cvx_scene* s, uint32_t blocks_per_sm) {
    if (!s || blocks_per_sm > 32) return set_error(CVX_ERR_INVALID, "bad launch shape");
    s->blocks_per_sm = blocks_per_sm;
    return CVX_OK;
}

void cvx_scene_destroy(cvx_scene* s) {
    if (!s) return;
    DeviceGuard g(s->device);
    delete s;
}

int32_t cvx_intersect_nearest_device(cvx_scene* s, const float* rays, uint32_t n, float far_dist, uint32_t traversal,
                                     float* t_out, int32_t* tri_out, uint32_t* counters, void* stream) {
    if (n > CVX_MAX_QUERY_RAYS) return set_error(CVX_ERR_INVALID, "a query takes at most 2^31 rays per call");
    if (!s || (!rays && n) || (!t_out && n) || (!tri_out && n)) return set_error(CVX_ERR_INVALID, "null argument");
    if (traversal > 1) return set_error(CVX_ERR_INVALID, "unknown traversal variant");
    if (n == 0) return CVX_OK;
    CVX_ON_DEVICE(s->device);
    cudaStream_t st = (cudaStream_t)stream;
    CK(launch_intersect(s->view(), soa_cols(rays, n), n, far_dist, traversal == CVX_TRAVERSE_PACKET, t_out, tri_out,
                        counters, s->d_err, 0, s->blocks_per_sm, st, s->query_stack),
       "intersect launch");
    return CVX_OK;
}

int32_t cvx_intersect_nearest(cvx_scene* s, const float* ox, const float* oy, const float* oz, const float* dx,
                              const float* dy, const float* dz, uint32_t n, float far_dist, uint32_t traversal,
                              float* t_out, int32_t* tri_out) {
    if (n > CVX_MAX_QUERY_RAYS) return set_error(CVX_ERR_INVALID, "a query takes at most 2^31 rays per call");
    if (!s) return set_error(CVX_ERR_INVALID, "null scene");
    if (n == 0) return CVX_OK;
    if (!ox || !oy || !oz || !dx || !dy || !dz || !t_out || !tri_out) return set_error(CVX_ERR_INVALID, "null buffer");
    if (traversal > 1) return set_error(CVX_ERR_INVALID, "unknown traversal variant");
    CVX_ON_DEVICE(s->device);
    int32_t st = 0;
    // In place: the kernel reads the caller's six arrays over the CPU-GPU
    // link as it consumes them (a warp stages each batch of 32 rays one batch
    // ahead), so the transfer overlaps traversal and no ray copy is made.
    const bool in_place = s->reads_host_in_place();
    if (s->scratch_n < n || (!in_place && !s->d_rays)) {
        cudaFree(s->d_rays);
        cudaFree(s->d_t);
        cudaFree(s->d_tri);
        s->d_rays = nullptr;
        s->d_t = nullptr;
        s->d_tri = nullptr;
        s->scratch_n = 0;
        if (!in_place && (st = dalloc(&s->d_rays, (size_t)n * 6, "ray buffer"))) return st;
        if ((st = dalloc(&s->d_t, n, "hit buffer"))) return st;
        if ((st = dalloc(&s->d_tri, n, "hit buffer"))) return st;
        s->scratch_n = n;
    }
    // Chunked pipeline: the rays are cut into chunks that go round-robin to
    // three streams, so the copies of one chunk overlap the traversal of
    // another (a chunk's kernel starts on the SMs the previous one leaves).
    // Chunk counts, measured on 4M rays: 4 when rays are copied from page-locked
    // memory (against 1, 2 and 8); 2 when they are read in place (only the hits
    // remain to overlap); 1 when any buffer is pageable, as the driver stages
    // each pageable copy through its own buffers and every extra chunk adds
    // one such round trip.
    constexpr uint32_t kMaxChunks = 4, kMinChunk = 1u << 19;
    if (!s->d_qerr && (st = dalloc(&s->d_qerr, 2 * kMaxChunks, "status"))) return st;
    if (!s->h_qerr) {
        CK(cudaHostAlloc((void**)&s->h_qerr, 8 * kMaxChunks, cudaHostAllocDefault), "cudaHostAlloc status");
    }
    for (cudaStream_t& q : s->qstreams)
        if (!q) CK(cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking), "cudaStreamCreate");
    StreamSync sync(s->qstreams[0], s->qstreams[1], s->qstreams[2]);
    const float* src[6] = {ox, oy, oz, dx, dy, dz};
    bool locked = page_locked(t_out) && page_locked(tri_out);
    for (int k = 0; k < 6 && locked && !in_place; k++) locked = page_locked(src[k]);
    uint32_t max_chunks = !locked ? 1u : (in_place ? 2u : kMaxChunks);
    uint32_t chunks = n / kMinChunk;
    chunks = chunks < 1 ? 1 : (chunks > max_chunks ? max_chunks : chunks);
    uint32_t per = (n + chunks - 1) / chunks;
    per = (per + 31u) & ~31u;
    uint32_t c = 0;
    for (uint32_t off = 0; off < n; off += per, c++) {
        uint32_t len = n - off < per ? n - off : per;
        cudaStream_t q = s->qstreams[c % 3];
        RayCols cols;
        if (in_place) {
            for (int k = 0; k < 6; k++) cols.c[k] = src[k] + off;
        } else {
            float* rays = s->d_rays + (size_t)6 * off;
            for (int k = 0; k < 6; k++)
                CK(cudaMemcpyAsync(rays + (size_t)k * len, src[k] + off, (size_t)len * 4, cudaMemcpyHostToDevice,
                                   q),
                   "copy rays");
            cols = soa_cols(rays, len);
        }
        CK(cudaMemsetAsync(s->d_qerr + 2 * c, 0, 8, q), "reset status");
        CK(launch_intersect(s->view(), cols, len, far_dist, traversal == CVX_TRAVERSE_PACKET, s->d_t + off,
                            s->d_tri + off, nullptr, s->d_qerr + 2 * c, 0, s->blocks_per_sm, q, s->query_stack),
           "intersect launch");
        CK(cudaMemcpyAsync(t_out + off, s->d_t + off, (size_t)len * 4, cudaMemcpyDeviceToHost, q), "copy distances");
        CK(cudaMemcpyAsync(tri_out + off, s->d_tri + off, (size_t)len * 4, cudaMemcpyDeviceToHost, q),
           "copy indices");
        CK(cudaMemcpyAsync(s->h_qerr + 2 * c, s->d_qerr + 2 * c, 8, cudaMemcpyDeviceToHost, q), "copy status");
    }
    for (cudaStream_t q : s->qstreams) CK(cudaStreamSynchronize(q), "intersect");
    for (uint32_t k = 0; k < c; k++)
        if (s->h_qerr[2 * k]) return set_error(CVX_ERR_DEVICE, "traversal stack overflow reported by the kernel");
    return CVX_OK;
}

int32_t cvx_renderer_create(cvx_scene* scene, uint32_t w, uint32_t h, const cvx_render_config* cfg,
                            cvx_renderer** out) {
    if (!scene || !out) return set_error(CVX_ERR_INVALID, "null argument");
    CVX_ON_DEVICE(scene->device);
    if (w == 0 || h == 0 || w > kMaxImageSide || h > kMaxImageSide)
        return set_error(CVX_ERR_INVALID, "frame size out of range");
    if (scene->n_lights == 0)
        return set_error(CVX_ERR_INVALID, "rendering needs at least one direct-sample triangle (scene.rs:143-161)");
    cvx_render_config c{};
    if (cfg) c = *cfg;
    if (c.rng_order > 1 || c.traversal > 1 || c.mode > 1 || (c.block_size % 32) || c.block_size > 128 ||
        c.refill_mode > 2 || c.blocks_per_sm > 64)
        return set_error(CVX_ERR_INVALID, "bad render configuration");
    if (c.mode == CVX_MODE_WAVEFRONT && c.rng_order != CVX_RNG_GROUP)
        return set_error(CVX_ERR_INVALID,
                         "the wavefront form needs the per-group RNG order (the patch order is one serial chain "
                         "per patch)");
    std::unique_ptr<cvx_renderer> r(new cvx_renderer());
    r->scene = scene;
    r->device = scene->device;
    r->w = w;
    r->h = h;
    r->cfg = c;
    cvx_camera cam;
    cvx_camera_default(&cam);
    std::memcpy(&r->cam, &cam, sizeof cam);
    size_t npx = (size_t)w * h;
    int32_t st = 0;
    if ((st = dalloc(&r->d_rgba, npx, "colour buffer"))) return st;
    if ((st = dalloc(&r->d_gbuf, npx, "gbuffer"))) return st;
    if ((st = dalloc(&r->d_color, npx * 3, "frame buffer"))) return st;
    if ((st = dalloc(&r->d_accum, npx * 3, "accumulator"))) return st;
    if ((st = dalloc(&r->d_rays, 1, "counters"))) return st;
    if ((st = dalloc(&r->d_err, 2, "status"))) return st;  // [0] status, [1] group counter
    if ((st = dalloc(&r->d_group_em, ((size_t)(w + 15) / 16) * ((h + 3) / 4) * 8, "group counters"))) return st;
    CK(cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    CK(cudaEventCreate(&r->e0), "cudaEventCreate");
    CK(cudaEventCreate(&r->e1), "cudaEventCreate");
    CK(cudaMemsetAsync(r->d_accum, 0, npx * 12, r->stream), "clear accumulator");
    CK(cudaStreamSynchronize(r->stream), "renderer init");
    if (c.mode == CVX_MODE_WAVEFRONT) {
        r->engine.reset(new WaveEngine());
        if ((st = r->engine->init(groups_of(w, h), 1, c.traversal == CVX_TRAVERSE_PACKET, c.use_graph != 0,
                                  c.blocks_per_sm, c.refill_mode)))
            return st;
        cvx_scene* sc[1] = {scene};
        if ((st = r->engine->set_scenes(sc, 1))) return st;
    }
    *out = r.release();
    return CVX_OK;
}

void cvx_renderer_destroy(cvx_renderer* r) {
    if (!r) return;
    DeviceGuard g(r->device);
    delete r;
}

int32_t cvx_renderer_set_time(cvx_renderer* r, float time, float time_delta) {
    if (!r) return set_error(CVX_ERR_INVALID, "null renderer");
    r->time = time;
    r->time_delta = time_delta;
    return CVX_OK;
}

int32_t cvx_renderer_update_scene(cvx_renderer* r) {
    if (!r) return set_error(CVX_ERR_INVALID, "null renderer");
    cvx_camera cam;
    std::memcpy(&cam, &r->cam, sizeof cam);
    cvx_camera_set_interactive(&cam, r->time, r->time_delta);
    std::memcpy(&r->cam, &cam, sizeof cam);
    return CVX_OK;
}

int32_t cvx_renderer_set_camera(cvx_renderer* r, const cvx_camera* cam) {
    if (!r || !cam) return set_error(CVX_ERR_INVALID, "null argument");
    static_assert(sizeof(DeviceCamera) == sizeof(cvx_camera), "camera layout");
    std::memcpy(&r->cam, cam, sizeof *cam);
    return CVX_OK;
}

static int32_t run_frame_wavefront(cvx_renderer* r, uint32_t frame, bool accumulate, uint32_t* rgba,
                                   uint32_t* gbuf) {
    size_t npx = (size_t)r->w * r->h;
    Job j{};
    j.cam = r->cam;
    j.scene = 0;
    j.w = r->w;
    j.h = r->h;
    j.frame = frame;
    j.out_offset = 0;
    WaveOutputs out{};
    out.rgba = accumulate ? nullptr : r->d_rgba;
    out.gbuf = r->d_gbuf;
    out.color = r->d_color;
    out.accum = accumulate ? r->d_accum : nullptr;
    uint64_t rays = 0;
    float ms = 0.0f;
    StreamSync sync(r->stream);
    int32_t st = r->engine->run(std::vector<Job>{j}, out, r->stream, &rays, nullptr, &ms);
    if (st) return st;
    r->last_rays = rays;
    r->last_ms = ms;
    if (rgba) CK(cudaMemcpyAsync(rgba, r->d_rgba, npx * 4, cudaMemcpyDeviceToHost, r->stream), "copy colour");
    if (gbuf) CK(cudaMemcpyAsync(gbuf, r->d_gbuf, npx * 4, cudaMemcpyDeviceToHost, r->stream), "copy gbuffer");
    CK(cudaStreamSynchronize(r->stream), "render");
    return CVX_OK;
}

static int32_t run_frame(cvx_renderer* r, uint32_t frame, bool accumulate, uint32_t* rgba, uint32_t* gbuf) {
    if (r->engine && !r->debug) return run_frame_wavefront(r, frame, accumulate, rgba, gbuf);
    size_t npx = (size_t)r->w * r->h;
    unsigned long long rays = 0;
    uint32_t err = 0;
    StreamSync sync(r->stream);
    CK(cudaMemsetAsync(r->d_rays, 0, 8, r->stream), "reset counters");
    CK(cudaMemsetAsync(r->d_err, 0, 8, r->stream), "reset status");
    CK(cudaEventRecord(r->e0, r->stream), "event");
    CK(launch_render(r->scene->view(), r->cam, r->w, r->h, frame, r->cfg.traversal == CVX_TRAVERSE_PACKET,
                     r->cfg.rng_order == CVX_RNG_PATCH, accumulate ? nullptr : r->d_rgba, r->d_gbuf, r->d_color,
                     accumulate ? r->d_accum : nullptr, r->d_rays, r->d_err, r->cfg.block_size, r->debug,
                     r->stream, 32, nullptr, 0,
                     path_refill_frames(r->cfg.refill_mode, r->scene->depth) ? r->d_group_em : nullptr),
       "render launch");
    CK(cudaEventRecord(r->e1, r->stream), "event");
    if (rgba) CK(cudaMemcpyAsync(rgba, r->d_rgba, npx * 4, cudaMemcpyDeviceToHost, r->stream), "copy colour");
    if (gbuf) CK(cudaMemcpyAsync(gbuf, r->d_gbuf, npx * 4, cudaMemcpyDeviceToHost, r->stream), "copy gbuffer");
    CK(cudaMemcpyAsync(&rays, r->d_rays, 8, cudaMemcpyDeviceToHost, r->stream), "copy counters");
    CK(cudaMemcpyAsync(&err, r->d_err, 4, cudaMemcpyDeviceToHost, r->stream), "copy status");
    CK(cudaStreamSynchronize(r->stream), "render");
    cudaEventElapsedTime(&r->last_ms, r->e0, r->e1);
    r->last_rays = rays;
    if (err) return set_error(CVX_ERR_DEVICE, "traversal stack overflow reported by the kernel");
    return CVX_OK;
}

int32_t cvx_renderer_count_work(cvx_renderer* r, uint32_t frame, uint64_t* out) {
    if (!r || !out) return set_error(CVX_ERR_INVALID, "null argument");
    CVX_ON_DEVICE(r->device);
    if (r->cfg.traversal != CVX_TRAVERSE_SINGLE || r->cfg.rng_order != CVX_RNG_GROUP || r->debug)
        return set_error(CVX_ERR_INVALID,
                         "work counts are defined for single-ray frames in the per-group RNG order");
    int32_t st = 0;
    if (!r->d_work && (st = dalloc(&r->d_work, 3, "work counters"))) return st;
    unsigned long long rays = 0, work[3] = {0, 0, 0};
    uint32_t err = 0;
    StreamSync sync(r->stream);
    CK(cudaMemsetAsync(r->d_rays, 0, 8, r->stream), "reset counters");
    CK(cudaMemsetAsync(r->d_err, 0, 8, r->stream), "reset status");
    CK(cudaMemsetAsync(r->d_work, 0, 24, r->stream), "reset counters");
    CK(launch_render(r->scene->view(), r->cam, r->w, r->h, frame, false, false, r->d_rgba, r->d_gbuf, r->d_color,
                     nullptr, r->d_rays, r->d_err, r->cfg.block_size, false, r->stream, 32, nullptr, 0,
                     r->d_group_em, r->d_work),
       "render launch");
    CK(cudaMemcpyAsync(&rays, r->d_rays, 8, cudaMemcpyDeviceToHost, r->stream), "copy counters");
    CK(cudaMemcpyAsync(work, r->d_work, 24, cudaMemcpyDeviceToHost, r->stream), "copy counters");
    CK(cudaMemcpyAsync(&err, r->d_err, 4, cudaMemcpyDeviceToHost, r->stream), "copy status");
    CK(cudaStreamSynchronize(r->stream), "render");
    if (err) return set_error(CVX_ERR_DEVICE, "traversal stack overflow reported by the kernel");
    out[0] = rays;
    out[1] = work[0];
    out[2] = work[1];
    out[3] = work[2];
    return CVX_OK;
}

int32_t cvx_renderer_set_debug_view(cvx_renderer* r, uint32_t enable) {
    if (!r) return set_error(CVX_ERR_INVALID, "null renderer");
    r->debug = enable != 0;
    return CVX_OK;
}

// The listed patches with the reference's per-patch generator, in one launch
// (one octet per patch); only the patches' pixels are copied to the caller's
// full-frame buffers.
static int32_t run_patches(cvx_renderer* r, uint32_t pw, const uint32_t* xy, uint32_t n, uint32_t frame,
                           bool accumulate, uint32_t* rgba, uint32_t* gbuf) {
    if (!r) return set_error(CVX_ERR_INVALID, "null renderer");
    CVX_ON_DEVICE(r->device);
    if (pw == 0 || (pw & 15u) || pw > kMaxImageSide)
        return set_error(CVX_ERR_INVALID, "patch width must be a positive multiple of 16, at most " +
                                              std::to_string(kMaxImageSide));
    if (n && !xy) return set_error(CVX_ERR_INVALID, "null patch list");
    for (uint32_t i = 0; i < n; i++) {
        uint32_t x = xy[2 * i], y = xy[2 * i + 1];
        if ((x & 15u) || (y & 3u) || x >= r->w || y >= r->h)
            return set_error(CVX_ERR_INVALID, "patch origin " + std::to_string(x) + "," + std::to_string(y) +
                                                  " must lie in the frame at a multiple of 16 (x) and 4 (y)");
    }
    if (n == 0) return CVX_OK;
    int32_t st = 0;
    unsigned long long rays = 0;
    uint32_t err = 0;
    StreamSync sync(r->stream);
    if (n > r->patch_cap) {
        cudaFree(r->d_patches);
        r->d_patches = nullptr;
        r->patch_cap = 0;
        if ((st = dalloc(&r->d_patches, (size_t)2 * n, "patch list"))) return st;
        r->patch_cap = n;
    }
    CK(cudaMemcpyAsync(r->d_patches, xy, (size_t)8 * n, cudaMemcpyHostToDevice, r->stream), "copy patch list");
    CK(cudaMemsetAsync(r->d_rays, 0, 8, r->stream), "reset counters");
    CK(cudaMemsetAsync(r->d_err, 0, 8, r->stream), "reset status");
    CK(cudaEventRecord(r->e0, r->stream), "event");
    CK(launch_render(r->scene->view(), r->cam, r->w, r->h, frame, r->cfg.traversal == CVX_TRAVERSE_PACKET, true,
                     accumulate ? nullptr : r->d_rgba, r->d_gbuf, r->d_color, accumulate ? r->d_accum : nullptr,
                     r->d_rays, r->d_err, r->cfg.block_size, r->debug, r->stream, pw, r->d_patches, n),
       "render launch");
    CK(cudaEventRecord(r->e1, r->stream), "event");
    size_t pitch = (size_t)r->w * 4;
    for (uint32_t i = 0; i < n; i++) {
        uint32_t x = xy[2 * i], y = xy[2 * i + 1];
        size_t cols = std::min<size_t>(pw, r->w - x), rows = std::min<size_t>(pw, r->h - y);
        size_t off = (size_t)y * r->w + x;
        if (rgba && !accumulate)
            CK(cudaMemcpy2DAsync(rgba + off, pitch, r->d_rgba + off, pitch, cols * 4, rows, cudaMemcpyDeviceToHost,
                                 r->stream),
               "copy colour");
        if (gbuf)
            CK(cudaMemcpy2DAsync(gbuf + off, pitch, r->d_gbuf + off, pitch, cols * 4, rows, cudaMemcpyDeviceToHost,
                                 r->stream),
               "copy gbuffer");
    }
    CK(cudaMemcpyAsync(&rays, r->d_rays, 8, cudaMemcpyDeviceToHost, r->stream), "copy counters");
    CK(cudaMemcpyAsync(&err, r->d_err, 4, cudaMemcpyDeviceToHost, r->stream), "copy status");
    CK(cudaStreamSynchronize(r->stream), "render");
    cudaEventElapsedTime(&r->last_ms, r->e0, r->e1);
    r->last_rays = rays;
    if (err) return set_error(CVX_ERR_DEVICE, "traversal stack overflow reported by the kernel");
    return CVX_OK;
}

int32_t cvx_render_patches_u8(cvx_renderer* r, uint32_t patch_width, const uint32_t* origins, uint32_t n_patches,
                              uint32_t frame, uint32_t* rgba, uint32_t* gbuffer) {
    return run_patches(r, patch_width, origins, n_patches, frame, false, rgba, gbuffer);
}

int32_t cvx_accumulate_patches_f32(cvx_renderer* r, uint32_t patch_width, const uint32_t* origins,
                                   uint32_t n_patches, uint32_t frame, uint32_t* gbuffer) {
    return run_patches(r, patch_width, origins, n_patches, frame, true, nullptr, gbuffer);
}

int32_t cvx_render_frame_u8(cvx_renderer* r, uint32_t frame, uint32_t* rgba, uint32_t* gbuffer) {
    if (!r) return set_error(CVX_ERR_INVALID, "null renderer");
    CVX_ON_DEVICE(r->device);
    return run_frame(r, frame, false, rgba, gbuffer);
}

int32_t cvx_accumulate_frame_f32(cvx_renderer* r, uint32_t frame, uint32_t* gbuffer) {
    if (!r) return set_error(CVX_ERR_INVALID, "null renderer");
    CVX_ON_DEVICE(r->device);
    return run_frame(r, frame, true, nullptr, gbuffer);
}

// Frames per launch of cvx_accumulate_frames_f32. The paths of up to
// kMaxLaunchFrames frames share one path-refill launch, so the launch's drain
// (lanes running out of paths while the last ones finish: 1.1 of 2.9 ms of a
// one-frame launch on the 870k-triangle tube) is paid once per launch instead
// of once per frame. Measured per 1280x736 tube sample at 1, 2, 4, 8, 16
// frames per launch: 2.94, 2.61, 2.40, 2.30, 2.25 ms (room: 0.709, 0.650,
// 0.614, 0.596, 0.588 ms), about 2.20 + 0.82 / frames. The colour buffers of
// all frames of a launch but the last take at most kSampleBufferBytes.
constexpr uint32_t kMaxLaunchFrames = 32;
constexpr size_t kSampleBufferBytes = (size_t)512 << 20;

int32_t cvx_accumulate_frames_f32(cvx_renderer* r, uint32_t first_frame, uint32_t n_frames, uint32_t* gbuffer) {
    if (!r) return set_error(CVX_ERR_INVALID, "null renderer");
    if (n_frames == 0) return set_error(CVX_ERR_INVALID, "number of frames must be positive");
    if (first_frame + (n_frames - 1u) < first_frame) return set_error(CVX_ERR_INVALID, "frame numbers overflow");
    CVX_ON_DEVICE(r->device);
    const size_t npx = (size_t)r->w * r->h;
    const uint64_t paths = (uint64_t)((r->w + 15u) / 16u) * ((r->h + 3u) / 4u) * 64u;  // per frame
    uint32_t per_launch = std::min(n_frames, kMaxLaunchFrames);
    per_launch = (uint32_t)std::min<uint64_t>(per_launch, kSampleBufferBytes / (npx * 12u) + 1u);
    per_launch = (uint32_t)std::min<uint64_t>(per_launch, (1ull << 31) / paths);  // 32-bit path numbers
    // Shared launches use the path-refill kernel whatever the refill mode: its
    // frames have the bits of the octet-group kernel's, and with the drain
    // shared it is the faster form on every scene measured (room 0.588 against
    // 0.744 ms per 1280x736 sample for one octet per group).
    const bool shared_launch = !r->engine && !r->debug && r->cfg.traversal == CVX_TRAVERSE_SINGLE &&
                               r->cfg.rng_order == CVX_RNG_GROUP && per_launch > 1;
    if (!shared_launch) {  // one launch per frame
        uint64_t rays = 0;
        float ms = 0.0f;
        for (uint32_t i = 0; i < n_frames; i++) {
            int32_t st = run_frame(r, first_frame + i, true, nullptr, i + 1u == n_frames ? gbuffer : nullptr);
            if (st) return st;
            rays += r->last_rays;
            ms += r->last_ms;
        }
        r->last_rays = rays;
        r->last_ms = ms;
        return CVX_OK;
    }
    int32_t st = 0;
    const size_t need = (size_t)(per_launch - 1u) * npx * 3u;
    if (r->samples_cap < need) {
        cudaFree(r->d_samples);
        r->d_samples = nullptr;
        r->samples_cap = 0;
        if ((st = dalloc(&r->d_samples, need, "sample colour buffers"))) return st;
        r->samples_cap = need;
    }
    unsigned long long rays = 0;
    uint32_t err = 0;
    StreamSync sync(r->stream);
    CK(cudaMemsetAsync(r->d_rays, 0, 8, r->stream), "reset counters");
    CK(cudaMemsetAsync(r->d_err, 0, 8, r->stream), "reset status");
    CK(cudaEventRecord(r->e0, r->stream), "event");
    for (uint32_t done = 0; done < n_frames;) {
        const uint32_t n = std::min(per_launch, n_frames - done);
        if (done) CK(cudaMemsetAsync(r->d_err + 1, 0, 4, r->stream), "reset path counter");
        CK(launch_render(r->scene->view(), r->cam, r->w, r->h, first_frame + done, false, false, nullptr, r->d_gbuf,
                         r->d_color, r->d_accum, r->d_rays, r->d_err, r->cfg.block_size, false, r->stream, 32,
                         nullptr, 0, r->d_group_em, nullptr, n, r->d_samples),
           "render launch");
        done += n;
    }
    CK(cudaEventRecord(r->e1, r->stream), "event");
    if (gbuffer) CK(cudaMemcpyAsync(gbuffer, r->d_gbuf, npx * 4, cudaMemcpyDeviceToHost, r->stream), "copy gbuffer");
    CK(cudaMemcpyAsync(&rays, r->d_rays, 8, cudaMemcpyDeviceToHost, r->stream), "copy counters");
    CK(cudaMemcpyAsync(&err, r->d_err, 4, cudaMemcpyDeviceToHost, r->stream), "copy status");
    CK(cudaStreamSynchronize(r->stream), "render");
    cudaEventElapsedTime(&r->last_ms, r->e0, r->e1);
    r->last_rays = rays;
    if (err) return set_error(CVX_ERR_DEVICE, "traversal stack overflow reported by the kernel");
    return CVX_OK;
}

int32_t cvx_resolve_u8(cvx_renderer* r, uint32_t n, uint32_t* rgba) {
    if (!r || !rgba) return set_error(CVX_ERR_INVALID, "null argument");
    if (n == 0) return set_error(CVX_ERR_INVALID, "number of samples must be positive");
    CVX_ON_DEVICE(r->device);
    size_t npx = (size_t)r->w * r->h;
    StreamSync sync(r->stream);
    CK(launch_resolve(r->d_accum, (uint32_t)npx, 1.0f / (float)n, r->d_rgba, r->stream), "resolve launch");
    CK(cudaMemcpyAsync(rgba, r->d_rgba, npx * 4, cudaMemcpyDeviceToHost, r->stream), "copy colour");
    CK(cudaStreamSynchronize(r->stream), "resolve");
    return CVX_OK;
}

int32_t cvx_read_accumulator(cvx_renderer* r, float* out) {
    if (!r || !out) return set_error(CVX_ERR_INVALID, "null argument");
    CVX_ON_DEVICE(r->device);
    CK(cudaMemcpy(out, r->d_accum, (size_t)r->w * r->h * 12, cudaMemcpyDeviceToHost), "copy accumulator");
    return CVX_OK;
}

int32_t cvx_clear_accumulator(cvx_renderer* r) {
    if (!r) return set_error(CVX_ERR_INVALID, "null renderer");
    CVX_ON_DEVICE(r->device);
    CK(cudaMemsetAsync(r->d_accum, 0, (size_t)r->w * r->h * 12, r->stream), "clear accumulator");
    CK(cudaStreamSynchronize(r->stream), "clear accumulator");
    return CVX_OK;
}

int32_t cvx_read_frame_f32(cvx_renderer* r, float* out) {
    if (!r || !out) return set_error(CVX_ERR_INVALID, "null argument");
    CVX_ON_DEVICE(r->device);
    CK(cudaMemcpy(out, r->d_color, (size_t)r->w * r->h * 12, cudaMemcpyDeviceToHost), "copy frame");
    return CVX_OK;
}

int32_t cvx_renderer_stats(cvx_renderer* r, uint64_t* rays, float* ms) {
    if (!r) return set_error(CVX_ERR_INVALID, "null renderer");
    if (rays) *rays = r->last_rays;
    if (ms) *ms = r->last_ms;
    return CVX_OK;
}

}  // extern "C"
