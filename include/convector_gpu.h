/*
 * convector_gpu.h -- C-ABI of the GB300 render hot path of ruuda/convector.
 *
 * The reference exposes its hot path as Rust methods, not an FFI; each entry
 * point below names the reference interface it stands in for (paths relative
 * to the reference's src/). The reference panics on bad input; here every call
 * returns a status (0 = CVX_OK) and cvx_last_error() gives the message of the
 * calling thread's last failure.
 *
 * Ownership and threading: the caller owns every host buffer it passes;
 * handles own their device memory. A handle must be used by one thread at a
 * time; distinct handles may be used concurrently. Calls that take host
 * buffers are synchronous. Nothing here falls back to the CPU: without a
 * usable CUDA device the GPU entry points return CVX_ERR_CUDA.
 *
 * Devices: a scene or display belongs to the device current in the calling
 * thread when it is created; a renderer, batch or server to its scenes' device
 * (the scenes of one batch or server must share it). Every call on a handle
 * runs on the handle's device, whatever device is current in the calling
 * thread, and leaves the thread's current device as it found it. Device
 * pointers and streams passed in must belong to that device.
 */
#ifndef CONVECTOR_GPU_H
#define CONVECTOR_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    CVX_OK = 0,
    CVX_ERR_INVALID = 1,    /* bad argument or unsupported size */
    CVX_ERR_IO = 2,         /* file could not be read */
    CVX_ERR_PARSE = 3,      /* malformed OBJ text */
    CVX_ERR_DEGENERATE = 4, /* collinear triangle (wavefront.rs:30-46) */
    CVX_ERR_CUDA = 5,       /* CUDA runtime failure or no device */
    CVX_ERR_DEVICE = 6,     /* a kernel reported an error (e.g. stack overflow) */
    CVX_ERR_CAPACITY = 7,   /* admission refused: not enough device memory */
    CVX_ERR_TIMEOUT = 8,    /* a request did not finish in time */
    CVX_ERR_CANCELLED = 9,  /* a request was cancelled */
    CVX_ERR_NOT_FOUND = 10  /* unknown request or scene id */
};

/* Reference `Triangle` (triangle.rs:24-32), 64 bytes. `material` is the
 * reference's 32-bit SMaterial encoding (material.rs:10-31). */
typedef struct cvx_triangle {
    float v0[3], v1[3], v2[3];
    float uv0[2], uv1[2], uv2[2];
    uint32_t material;
} cvx_triangle;

/* Reference `BvhNode` (bvh.rs:21-30), 32 bytes: len == 0 marks an internal
 * node whose children are nodes index and index + 1; a leaf covers triangles
 * index .. index + len. Nodes 0 and 1 are the two roots. */
typedef struct cvx_bvh_node {
    float origin[3];
    float far_[3];
    uint32_t index;
    uint32_t len;
} cvx_bvh_node;

/* Reference `Camera` (scene.rs:20-30). */
typedef struct cvx_camera {
    float position[3];
    float position_delta[3];
    float orientation[4];       /* quaternion a, b, c, d */
    float orientation_delta[4];
    float screen_distance;
} cvx_camera;

typedef struct cvx_mesh cvx_mesh;
typedef struct cvx_bvh cvx_bvh;
typedef struct cvx_scene cvx_scene;
typedef struct cvx_renderer cvx_renderer;

/* Copies the calling thread's last error message; returns its status. */
int32_t cvx_last_error(char* buf, size_t len);

/* ---- host: scene loading and BVH build -------------------------------- */

/* Mesh::load_with_materials (wavefront.rs:83-152). `names[i]` maps to the
 * SMaterial bits `materials[i]`; an unknown `usemtl` name is an error. */
int32_t cvx_mesh_load_obj(const char* path, const char* const* names, const uint32_t* materials,
                          uint32_t n_materials, cvx_mesh** out);
/* The same parser over OBJ text in memory. */
int32_t cvx_mesh_parse_obj(const char* text, size_t len, const char* const* names, const uint32_t* materials,
                           uint32_t n_materials, cvx_mesh** out);
uint32_t cvx_mesh_num_triangles(const cvx_mesh* mesh);
void cvx_mesh_destroy(cvx_mesh* mesh);

/* Bvh::from_meshes (bvh.rs:547-568) and Bvh::build (bvh.rs:488-545): the
 * reference's binned tree-SAH build, node order and triangle order. Fewer
 * than 2^27 triangles (CVX_ERR_INVALID beyond). */
int32_t cvx_bvh_from_meshes(const cvx_mesh* const* meshes, uint32_t n_meshes, cvx_bvh** out);
int32_t cvx_bvh_build(const cvx_triangle* triangles, uint32_t n, cvx_bvh** out);
/* Bvh::build (bvh.rs:488-545) run on the device: the same nodes, triangle
 * order, source indices and statistics as cvx_bvh_build, for scene admission
 * in serving. Refuses NaN or infinite vertex coordinates (CVX_ERR_INVALID)
 * and more than 2^26 triangles (CVX_ERR_CAPACITY). */
int32_t cvx_bvh_build_device(const cvx_triangle* triangles, uint32_t n, cvx_bvh** out);
uint32_t cvx_bvh_num_nodes(const cvx_bvh* bvh);
uint32_t cvx_bvh_num_triangles(const cvx_bvh* bvh);
/* Copies nodes / triangles (BVH order) / source index of each BVH-order
 * triangle into caller buffers sized by the counts above. */
void cvx_bvh_copy_nodes(const cvx_bvh* bvh, cvx_bvh_node* out);
void cvx_bvh_copy_triangles(const cvx_bvh* bvh, cvx_triangle* out);
void cvx_bvh_copy_source_index(const cvx_bvh* bvh, uint32_t* out);
/* Bvh::print_stats (bvh.rs:570-583) figures, plus the tree depth. */
void cvx_bvh_stats(const cvx_bvh* bvh, float* avg_tris_per_leaf, float* avg_area_ratio, uint32_t* depth);
void cvx_bvh_destroy(cvx_bvh* bvh);

/* Camera::new / set_rotation / set_fov (scene.rs:34-74), computed on the host. */
void cvx_camera_default(cvx_camera* cam);
void cvx_camera_set_rotation(cvx_camera* cam, float radians, float delta);
void cvx_camera_set_fov(cvx_camera* cam, float fov);
/* The camera step of Renderer::update_scene (renderer.rs:140-147): position
 * and rotation on the interactive path at `time`, with the deltas of a frame
 * lasting `time_delta` (motion blur over the frame). */
void cvx_camera_set_interactive(cvx_camera* cam, float time, float time_delta);

/* ---- diagnostics: error paths ------------------------------------------
 * No counterpart in the reference, which panics where these calls make the
 * library return a status (bvh.rs:594-600 on a stack overflow, main.rs:65-66
 * on allocation). They exist so that tests can run the error paths. */

/* Lowers the number of entries a traversal stack may hold (2 .. 128; 0
 * restores the default of 128) on the calling thread's current device, for
 * kernels launched after the call returns; call it while no kernel of this
 * library runs there. A ray that would need more entries stops, the kernel
 * sets its status word and the call that launched it returns CVX_ERR_DEVICE;
 * every access stays inside the stacks' full size. */
int32_t cvx_set_traversal_stack_limit(uint32_t entries);
/* Makes the library's device allocations fail as if the device were out of
 * memory (CVX_ERR_CAPACITY): the next `after` allocations succeed and the one
 * after them fails, once; a negative value cancels a pending failure.
 * Process-wide, on every device. */
int32_t cvx_inject_allocation_failure(int32_t after);

/* ---- device: scenes ------------------------------------------------------ */

/* The device that handles created now by the calling thread would belong to:
 * its ordinal and its name (NUL-terminated, truncated to name_len). No
 * counterpart in the reference; the autotuner keys its cache on it. */
int32_t cvx_device_info(int32_t* ordinal, char* name, size_t name_len);

/* Scene::from_meshes (scene.rs:114-129) given a built BVH: uploads nodes and
 * triangles in BVH order and the direct-sample list (triangles with material
 * bit 30). Rejects trees deeper than the device traversal stack and
 * glossiness indices above 5 (material.rs:497-512 has six entries). */
int32_t cvx_scene_create(const cvx_triangle* triangles_bvh_order, uint32_t n_triangles, const cvx_bvh_node* nodes,
                         uint32_t n_nodes, cvx_scene** out);
int32_t cvx_scene_from_bvh(const cvx_bvh* bvh, cvx_scene** out);
uint32_t cvx_scene_num_direct_samples(const cvx_scene* scene);
/* light_pick 0: `bits >> 29` as scene.rs:159 (requires exactly 8 direct-sample
 * triangles); 1 (default): `(bits * n) >> 32`, identical to it when n == 8. */
int32_t cvx_scene_set_light_pick(cvx_scene* scene, uint32_t light_pick);
/* Launch shape of this scene's nearest-hit queries: resident 128-thread
 * blocks per SM (0: default 8; the single-ray kernel is built for 8, 10 and
 * 12, trading registers for occupancy). Results do not depend on it. */
int32_t cvx_scene_set_query_launch(cvx_scene* scene, uint32_t blocks_per_sm);
/* Stack depth of this scene's single-ray nearest-hit queries at the default
 * launch shape: how many of each lane's traversal stack entries are kept in
 * shared memory (0, 4, 8 or 12; default 8), the deeper ones in local memory.
 * Shared entries never miss a cache, but take shared memory from L1; the
 * best depth depends on the tree (convector_gb300.autotune.tune_query times
 * them). Results do not depend on it. No counterpart in the reference, whose
 * stack is a Vec (bvh.rs:594-600). */
int32_t cvx_scene_set_query_stack(cvx_scene* scene, uint32_t shared_entries);
/* How cvx_intersect_nearest brings the caller's host ray arrays to the device.
 * AUTO (default): where the device translates addresses through the host's
 * page tables (a coherent CPU-GPU link, as on Grace systems; pinned or pageable
 * memory alike), the query kernel reads the six arrays in place while it
 * traverses, and no copy of the rays is made; elsewhere, and always under
 * COPY, each chunk of rays is copied to device memory first. Hits are copied
 * back either way, and the results are the same. `in_place` (optional)
 * receives 1 when this scene's calls will read in place. No counterpart in
 * the reference, whose query reads its own memory (bvh.rs:659-662). */
enum { CVX_HOST_ACCESS_AUTO = 0, CVX_HOST_ACCESS_COPY = 1 };
int32_t cvx_scene_set_host_access(cvx_scene* scene, uint32_t mode, uint32_t* in_place);
void cvx_scene_destroy(cvx_scene* scene);

/* Traversal variants (flags of cvx_intersect_nearest, traversal of cvx_render_config). */
enum { CVX_TRAVERSE_PACKET = 0, CVX_TRAVERSE_SINGLE = 1 };

/* Bvh::intersect_nearest (bvh.rs:659-662) over n rays in SoA form, packed
 * 8 per reference packet in input order; the hit record starts at
 * `far_dist` (MIntersection::with_max_distance, ray.rs:95-103). Outputs the
 * hit distance and the BVH-order triangle index (-1 for no hit). Host
 * buffers, read in place or copied in (cvx_scene_set_host_access); hits are
 * copied out inside the call. Both query forms take at most
 * CVX_MAX_QUERY_RAYS rays per call (CVX_ERR_INVALID beyond: split the rays
 * over several calls). */
#define CVX_MAX_QUERY_RAYS 2147483648u
int32_t cvx_intersect_nearest(cvx_scene* scene, const float* ox, const float* oy, const float* oz,
                              const float* dx, const float* dy, const float* dz, uint32_t n, float far_dist,
                              uint32_t traversal, float* t_out, int32_t* tri_out);
/* Device-pointer form: `rays` holds 6 arrays of n floats (ox oy oz dx dy dz);
 * `stream` is a cudaStream_t (NULL: the default stream). Asynchronous.
 * `counters`, when not NULL, receives 2 * n u32: per ray the boxes and the
 * triangles its packet (or the ray, single mode) tested (bvh.rs:604-651). */
int32_t cvx_intersect_nearest_device(cvx_scene* scene, const float* rays, uint32_t n, float far_dist,
                                     uint32_t traversal, float* t_out, int32_t* tri_out, uint32_t* counters,
                                     void* stream);

/* The query of cvx_intersect_nearest for callers that must not allocate device
 * memory: a host application that owns the GPU's memory budget through its
 * own allocator and forbids plugins to call cudaMalloc, or a real-time loop in
 * which an allocation (which can synchronise the device and take an
 * unpredictable time) would break the frame budget. The scene must already
 * exist; this call allocates nothing and loads nothing. Rays and hits are
 * staged through one static device buffer of 16 MiB + 256 B, reserved on a
 * device (and its address looked up) when the first scene is created there,
 * and held until the process exits: at most 524,288 rays per call
 * (CVX_ERR_INVALID beyond). Every call shares that buffer: calls that overlap
 * on the GPU (from several threads or scenes at once) race on it and must be
 * serialised by the caller. No counterpart in the reference. */
int32_t cvx_intersect_nearest_noalloc(cvx_scene* scene, const float* ox, const float* oy, const float* oz,
                                      const float* dx, const float* dy, const float* dz, uint32_t n,
                                      float far_dist, uint32_t traversal, float* t_out, int32_t* tri_out);

/* ---- device: renderer ---------------------------------------------------- */

/* RNG order: CVX_RNG_PATCH reproduces the reference's stream exactly (one
 * generator per 32x32 patch, renderer.rs:306-327; one octet per patch on the
 * GPU); CVX_RNG_GROUP seeds each 8-pixel group from its own pixel
 * coordinates so that every group renders in parallel. */
enum { CVX_RNG_PATCH = 0, CVX_RNG_GROUP = 1 };
/* Kernel organisation: one fused kernel per frame, or the wavefront form
 * (ray generation, traversal, shading and accumulation kernels over SoA ray
 * queues with compaction), optionally replayed as a CUDA graph. */
enum { CVX_MODE_MEGAKERNEL = 0, CVX_MODE_WAVEFRONT = 1, CVX_MODE_AUTO = 2 };

/* Ray refill in the single-ray traversal: persistent lanes take the next ray
 * when theirs finishes, rather than one octet working through an 8-pixel group.
 * Wavefront form: which bounces fetch rays with refill (the camera rays of a
 * group are coherent and share warps well by octets).
 * Single-launch form, per-group RNG order: CVX_REFILL_NONE renders one 8-pixel
 * group per octet through all its bounces; CVX_REFILL_ALL gives each lane one
 * path at a time, refilled ray by ray (a lane whose ray is finished shades it
 * together with the others of its warp that are, then traces the next);
 * CVX_REFILL_AFTER_CAMERA (default) takes the second for scenes of 25 levels
 * and more (for a wave of a batch or server: when at least half of its groups
 * belong to such scenes), the first below. The image is the same either way. */
enum { CVX_REFILL_AFTER_CAMERA = 0, CVX_REFILL_ALL = 1, CVX_REFILL_NONE = 2 };

typedef struct cvx_render_config {
    uint32_t rng_order;     /* CVX_RNG_* */
    uint32_t traversal;     /* CVX_TRAVERSE_* */
    uint32_t mode;          /* CVX_MODE_* */
    uint32_t block_size;    /* megakernel, octet groups: threads per block, 32, 64, 96 or 128 (0: 128) */
    uint32_t use_graph;     /* wavefront: capture the bounce loop in a CUDA graph */
    uint32_t blocks_per_sm; /* wavefront: persistent blocks per SM (0: 12) */
    uint32_t refill_mode;   /* CVX_REFILL_* */
} cvx_render_config;

/* Renderer::new (renderer.rs:121-130). Widths and heights from 1 to
 * CVX_MAX_IMAGE_SIDE are accepted (CVX_ERR_INVALID beyond; the same bound
 * holds for batch views and server requests); sizes off the reference tiling
 * are padded and cropped. */
#define CVX_MAX_IMAGE_SIDE 16384u
int32_t cvx_renderer_create(cvx_scene* scene, uint32_t width, uint32_t height, const cvx_render_config* config,
                            cvx_renderer** out);
void cvx_renderer_destroy(cvx_renderer* r);
/* The scene's camera (scene.rs:103 `pub camera`). */
int32_t cvx_renderer_set_camera(cvx_renderer* r, const cvx_camera* cam);
/* Renderer::set_time (renderer.rs:134-137): the time of the next frame and
 * the frame's duration. */
int32_t cvx_renderer_set_time(cvx_renderer* r, float time, float time_delta);
/* Renderer::update_scene (renderer.rs:140-147): moves this renderer's camera
 * to the interactive path position of the time set above. */
int32_t cvx_renderer_update_scene(cvx_renderer* r);
/* Renderer::toggle_debug_view (renderer.rs:150-152): frames show log2 of the
 * boxes (green) and triangles (blue) tested per packet, times 0.1
 * (renderer.rs:470-486). The debug view always runs the fused kernel. */
int32_t cvx_renderer_set_debug_view(cvx_renderer* r, uint32_t enable);
/* Renderer::render_patch_u8 (renderer.rs:306-327) over every patch of the
 * frame: RGBA8 colour and gbuffer words, row-major, row 0 at the bottom
 * (renderer.rs:210-235 stores rows bottom-up). Either output may be NULL. */
int32_t cvx_render_frame_u8(cvx_renderer* r, uint32_t frame_number, uint32_t* rgba, uint32_t* gbuffer);
/* Renderer::accumulate_patch_f32 (renderer.rs:339-362) over the frame: adds
 * this frame's colour to the device accumulator; gbuffer may be NULL. */
int32_t cvx_accumulate_frame_f32(cvx_renderer* r, uint32_t frame_number, uint32_t* gbuffer);
/* The accumulation loop of main.rs (one accumulate_patch_f32 pass per frame,
 * renderer.rs:339-362) over frames first_frame .. first_frame + n_frames - 1
 * in one call: the accumulator, the frame buffer (cvx_read_frame_f32) and the
 * gbuffer (may be NULL) end with the same bits as after n_frames calls of
 * cvx_accumulate_frame_f32 in frame order, and cvx_renderer_stats reports
 * their total rays and time. A single-launch renderer with the single-ray
 * traversal and the per-group RNG order renders up to 32 frames per launch
 * with the per-lane path refill (whatever its refill_mode: the frames' bits
 * are the same), each pixel's frames being added in frame order afterwards;
 * this takes up to 512 MiB of device memory for their colours, allocated at
 * the first call. Other forms take one launch per frame. */
int32_t cvx_accumulate_frames_f32(cvx_renderer* r, uint32_t first_frame, uint32_t n_frames, uint32_t* gbuffer);
/* Renderer::render_patch_u8 (renderer.rs:306-327) for a list of patches in
 * one call: origins holds n_patches (x, y) pairs, each patch patch_width
 * pixels square (a multiple of 16, at most CVX_MAX_IMAGE_SIDE; pixels of a
 * patch beyond the frame are not stored) with its own generator seeded (x, y,
 * frame_number), as in the reference whatever the renderer's rng_order.
 * x must be a multiple of 16 and y of 4, inside the frame. Only the patches'
 * pixels of the full-frame rgba / gbuffer buffers (either may be NULL) are
 * written; the rest of the caller's buffers is left as it is. */
int32_t cvx_render_patches_u8(cvx_renderer* r, uint32_t patch_width, const uint32_t* origins, uint32_t n_patches,
                              uint32_t frame_number, uint32_t* rgba, uint32_t* gbuffer);
/* Renderer::accumulate_patch_f32 (renderer.rs:339-362) for a list of
 * patches: adds their colour to the device accumulator (read it with
 * cvx_resolve_u8) and writes their gbuffer pixels (may be NULL). */
int32_t cvx_accumulate_patches_f32(cvx_renderer* r, uint32_t patch_width, const uint32_t* origins,
                                   uint32_t n_patches, uint32_t frame_number, uint32_t* gbuffer);
/* Renderer::buffer_f32_into_render_buffer (renderer.rs:378-410). */
int32_t cvx_resolve_u8(cvx_renderer* r, uint32_t num_samples, uint32_t* rgba);
/* Reads (row-major, 3 floats per pixel) or zeroes the accumulator
 * (Renderer::new_buffer_f32, renderer.rs:366-374). */
int32_t cvx_read_accumulator(cvx_renderer* r, float* out);
int32_t cvx_clear_accumulator(cvx_renderer* r);
/* Per-pixel linear colour of the last rendered frame (3 floats per pixel),
 * before quantisation. */
int32_t cvx_read_frame_f32(cvx_renderer* r, float* out);
/* Rays traced by the last frame (camera plus bounce rays, active lanes only)
 * and its device time. */
int32_t cvx_renderer_stats(cvx_renderer* r, uint64_t* rays, float* ms);
/* The work of one frame, for the memory roofline of the frame kernels:
 * renders frame_number as cvx_render_frame_u8 does (the image stays on the
 * device) with the per-lane path refill kernel in a counting form, and writes
 * out[0] the rays traced (camera and bounce rays), out[1] the boxes and
 * out[2] the triangles they tested (two boxes per internal node visited, the
 * reference's counters of bvh.rs:604-651), out[3] the shading steps that
 * evaluated every light's PDF (material.rs:281-320). A ray's counts do not
 * depend on which kernel traces it, so they hold for every single-ray form
 * of the frame. Single-ray traversal and per-group RNG order only
 * (CVX_ERR_INVALID otherwise). No counterpart in the reference. */
int32_t cvx_renderer_count_work(cvx_renderer* r, uint32_t frame_number, uint64_t* out);

/* ---- device: batched rendering -----------------------------------------
 * Many images of many resident scenes in shared wavefronts: sample s of
 * every view goes into wave s, so each view accumulates its samples in order
 * and its image equals the one cvx_accumulate_frame_f32 + cvx_resolve_u8
 * give for it alone. No reference counterpart: the reference renders one
 * frame of one scene (main.rs:124-217). */
typedef struct cvx_view {
    uint32_t scene;       /* index into the scenes given to cvx_batch_create */
    uint32_t width, height;
    uint32_t spp;         /* samples, frames frame_base .. frame_base + spp - 1 */
    uint32_t frame_base;
    cvx_camera camera;
} cvx_view;

typedef struct cvx_batch cvx_batch;
/* max_groups bounds the 8-pixel groups of one wave (ray-queue capacity);
 * max_pixels bounds the pixels of all views of one call. config->mode picks
 * the kernel organisation of every scene: CVX_MODE_MEGAKERNEL (fused),
 * CVX_MODE_WAVEFRONT, or CVX_MODE_AUTO (wavefront for BVHs deeper than 40
 * levels or above 200k triangles, fused otherwise). A wave's fused and
 * wavefront jobs run concurrently on two streams. */
int32_t cvx_batch_create(cvx_scene* const* scenes, uint32_t n_scenes, uint32_t max_groups, uint64_t max_pixels,
                         const cvx_render_config* config, cvx_batch** out);
/* Renders every view; rgba[i] (host, width*height words, may be NULL)
 * receives view i. rays and ms (may be NULL) receive the totals. */
int32_t cvx_batch_render(cvx_batch* b, const cvx_view* views, uint32_t n_views, uint32_t* const* rgba,
                         uint64_t* rays, float* ms);
/* Overrides one scene's kernel organisation (0 fused, 1 wavefront). */
int32_t cvx_batch_set_scene_mode(cvx_batch* b, uint32_t scene, uint32_t mode);
void cvx_batch_destroy(cvx_batch* b);

/* ---- device: request server ----------------------------------------------
 * A request loop on its own host thread over resident scenes: submitted
 * requests wait in FIFO order and are admitted while their framebuffer and
 * ray-queue memory fit the budget; every wave renders the next sample (or,
 * with samples_per_wave, the next samples) of every admitted request, so
 * requests that arrive while others are on the GPU join the next wave
 * (continuous batching). No reference counterpart. */
typedef struct cvx_server_config {
    uint64_t framebuffer_bytes; /* device memory for admitted requests' images */
    uint32_t max_groups;        /* ray-queue capacity of one wave, in 8-pixel groups */
    uint32_t traversal;         /* CVX_TRAVERSE_* */
    uint32_t use_graph;
    uint32_t sequential;        /* 1: one request at a time (the plain path, for comparison) */
    uint32_t blocks_per_sm;     /* persistent blocks per SM (0: 12) */
    uint32_t refill_mode;       /* CVX_REFILL_* */
    uint32_t kernel_mode;       /* 0: per scene as CVX_MODE_AUTO; 1: all fused; 2: all wavefront */
    uint32_t fused_blocks_per_sm; /* blocks per SM of the single-launch waves (0: 16) */
    uint32_t wavefront_streams; /* wavefront engines, each on its own stream (0, 1: one; at most
                                   4): requests are spread over them and their waves, running
                                   out of phase, fill each other's bounce tails */
    uint32_t deep_single_launch; /* 1: the engines of the deep scenes (those in wavefront mode)
                                    run their waves as single launches instead of the wavefront
                                    kernels, keeping their streams and priority */
    uint64_t max_inflight_pixels; /* 0: admit while framebuffer memory lasts; else admitted
                                     requests hold at most this many pixels (the oldest queued
                                     request is admitted whenever none is), so that in overload
                                     requests finish in arrival order instead of all together */
    uint32_t samples_per_wave;    /* 0, 1: a wave takes the next sample of each admitted request;
                                     n > 1: up to n of its next samples, on the single-launch
                                     engines that take paths per lane (CVX_REFILL_ALL, single-ray
                                     traversal; the others take one). The samples are added to the
                                     request's accumulator in sample order, so its image is the
                                     same either way */
    uint64_t sample_buffer_bytes; /* device memory for those samples' colours (0: as much as
                                     framebuffer_bytes), shared among the engines */
} cvx_server_config;

typedef struct cvx_request {
    uint32_t scene, width, height, spp, frame_base;
    cvx_camera camera;
} cvx_request;

typedef struct cvx_request_result {
    int32_t status;          /* CVX_OK, or the request's error */
    double submit_s, start_s, done_s; /* server clock, seconds */
    uint64_t rays;
} cvx_request_result;

typedef struct cvx_server cvx_server;
int32_t cvx_server_create(cvx_scene* const* scenes, uint32_t n_scenes, const cvx_server_config* config,
                          cvx_server** out);
/* Queues a request; rgba (host, width*height words, may be NULL) must stay
 * valid until cvx_server_wait has returned the request's result (or the
 * server is destroyed): a cancelled request whose image was already being
 * copied out still writes it. CVX_ERR_CAPACITY if it can never be admitted. */
int32_t cvx_server_submit(cvx_server* s, const cvx_request* req, uint32_t* rgba, uint64_t* id);
/* Waits up to timeout_ms (0: just polls) for a request; CVX_ERR_TIMEOUT if
 * it is not done yet. The result is returned once and then forgotten. */
int32_t cvx_server_wait(cvx_server* s, uint64_t id, uint32_t timeout_ms, cvx_request_result* result);
/* Cancels a queued or running request: its result status becomes
 * CVX_ERR_CANCELLED, unless its last sample had already finished (then the
 * request completes normally). Returns at once; wait for the result before
 * releasing the request's image buffer. */
int32_t cvx_server_cancel(cvx_server* s, uint64_t id);
/* Overrides one scene's kernel organisation (0 fused, 1 wavefront); only
 * while the server has no queued or admitted request. */
int32_t cvx_server_set_scene_mode(cvx_server* s, uint32_t scene, uint32_t mode);
/* The server clock (seconds), waves run, rays traced and device busy time. */
int32_t cvx_server_stats(cvx_server* s, double* now_s, uint64_t* waves, uint64_t* rays, double* busy_s);
/* Device time spent so far by each of the server's two engines (single-launch
 * waves and wavefront waves; they run concurrently, so the sum can exceed
 * the busy time above). No counterpart in the reference. */
int32_t cvx_server_engine_stats(cvx_server* s, double* fused_busy_s, double* wavefront_busy_s);
void cvx_server_destroy(cvx_server* s);

/* ---- device: display post-process ----------------------------------------
 * Window::display_buffer (ui.rs:313-364) and the shaders it runs
 * (src/gpu/gbuffer.glsl, blend.glsl, median.glsl, id.glsl), restated as CUDA
 * kernels over device buffers instead of OpenGL textures: the gbuffer
 * composite of the material textures into a ring of 8 frames, the mean of the
 * ring (or the newest frame), the 5-tap median in CIE XYZ (or the identity),
 * and the sRGB encode of the window's framebuffer. Textures are RGB8 sRGB,
 * tex_w x tex_h, for texture indices 1 and 2. Every side is at most
 * CVX_MAX_IMAGE_SIDE. */
typedef struct cvx_display cvx_display;
int32_t cvx_display_create(uint32_t width, uint32_t height, const uint8_t* texture1_rgb, const uint8_t* texture2_rgb,
                           uint32_t tex_w, uint32_t tex_h, cvx_display** out);
/* One displayed frame from a rendered frame and its gbuffer (host buffers);
 * out_srgb receives sRGB RGBA8, row-major, row 0 at the bottom. */
int32_t cvx_display_frame(cvx_display* d, const uint32_t* rgba, const uint32_t* gbuffer, uint32_t enable_blend,
                          uint32_t enable_median, uint32_t* out_srgb);
void cvx_display_destroy(cvx_display* d);

#ifdef __cplusplus
}
#endif
#endif
