/*
 * crt_gb300.h -- C ABI of the GB300 (sm_103a) path-tracing library.
 *
 * Drop-in replacement for CudaRT's GPU render path.  The reference binds its
 * renderer through the abstract C++ class `Renderer`
 * (src/include/renderer.h:78-100) and its GPU implementation
 * `ParallelRenderer` (src/renderer/parallel_renderer.cu); this header exposes
 * the same operations as plain C functions over opaque handles so that any
 * host (the C++ shim in cudart_gb300/shim/, ctypes, cgo, JNI) can call them.
 *
 * Conventions
 *  - Every function returns a crt_status; CRT_OK is 0.  On failure the
 *    message is available from crt_last_error() (thread-local).  Nothing in
 *    the library calls exit() (the reference's CUDA_CHECK_RETURN does,
 *    src/include/cuda_error_check.h:9-21).
 *  - Handles own all device memory they allocate and free it on *_destroy.
 *  - Pointers named d_* are device pointers; all others are host pointers.
 *  - Triangle indices are the caller's face order (the order of
 *    crt_scene_desc.positions), independent of the BVH layout.
 *  - There is no CPU fallback: without a usable sm_103a GPU the create
 *    calls fail with CRT_ERR_CUDA.
 */
#ifndef CRT_GB300_H
#define CRT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CRT_API_VERSION 1

#if defined(__GNUC__)
#define CRT_EXPORT __attribute__((visibility("default")))
#else
#define CRT_EXPORT
#endif

typedef enum {
    CRT_OK = 0,
    CRT_ERR_INVALID = 1,      /* bad argument or scene description */
    CRT_ERR_CUDA = 2,         /* CUDA runtime error (message has details) */
    CRT_ERR_NOMEM = 3,        /* host or device allocation failed */
    CRT_ERR_UNSUPPORTED = 4,  /* option not supported by this library */
    CRT_ERR_WATCHDOG = 5,     /* a device traversal exceeded its step or stack limit */
    CRT_ERR_LIMIT = 6         /* a size exceeds a documented maximum */
} crt_status;

/* refl_t (src/include/material.h:8-15). */
typedef enum {
    CRT_BSDF_DIFFUSE = 0,
    CRT_BSDF_SPECULAR = 1,
    CRT_BSDF_DIFFSPEC = 2,
    CRT_BSDF_MICROFACET = 3,
    CRT_BSDF_REFRACTIVE = 4,
    CRT_BSDF_EMISSIVE = 5
} crt_bsdf;

#define CRT_NO_TEXTURE (-1)

/* One material with the values of its MTL entry; replaces the reference's
 * Material (src/include/material.h:17-55) as produced by materialFromMtl
 * (src/geometry/scene.cpp:175-190).  `ka` is the MTL Ka: the library applies
 * the reference's emission scaling Ka * 3 * (total light area)
 * (scene.cpp:19,163,177). */
typedef struct {
    int32_t bsdf;        /* crt_bsdf */
    int32_t texture;     /* index into the scene's textures or CRT_NO_TEXTURE */
    float kd[3];
    float ka[3];
    float ks[3];
    float ns;
    float ni;            /* index of refraction for CRT_BSDF_REFRACTIVE */
    float diffuse;       /* diffuse probability for CRT_BSDF_DIFFSPEC */
} crt_material;

/* Camera (src/include/camera.h:9-22), already derived from the JSON file. */
typedef struct {
    float eye[3];
    float dir[3];
    float up[3];
    float right[3];
    float fov;           /* tan(vertical fov / 2) */
    float aspect;
    float aperture;      /* focalLength / fStop; 0 for a pinhole */
    float focus;         /* |viewDirection| */
    int32_t xpixels;
    int32_t ypixels;
} crt_camera;

/* Scene description: everything Scene::loadTriangles, constructLightList and
 * TextureStore produce (scene.cpp:74-165, texture_store.cpp:18-71). */
typedef struct {
    uint32_t num_triangles;
    const float* positions;        /* [n][3 vertices][xyz] */
    const float* normals;          /* [n][3 vertices][xyz] shading normals */
    const float* uvs;              /* [n][3 vertices][uv]; may be NULL (all 0) */
    const uint32_t* material_ids;  /* [n] */
    uint32_t num_materials;
    const crt_material* materials;
    uint32_t num_lights;           /* 0: every triangle whose material is
                                      CRT_BSDF_EMISSIVE, in face order */
    const uint32_t* light_indices; /* [num_lights] face indices in pick order */
    uint32_t num_textures;
    const uint32_t* texture_dims;  /* [num_textures][width, height] */
    const float* texels;           /* [sum(w*h)][rgb] linear floats, as
                                      stbi_loadf returns them (or NULL with
                                      texels_rgba8) */
    uint32_t node_format;          /* crt_node_format renders use by default; both
                                      encodings are uploaded */
    uint32_t bvh_width;            /* children per node: 4 or 8 (0 = 8) */
    uint32_t flags;                /* crt_scene_flags */
    uint32_t builder;              /* crt_bvh_builder */
    const uint8_t* texels_rgba8;   /* instead of texels: [sum(w*h)][rgba] bytes,
                                      converted on the device as stbi_loadf
                                      converts 8-bit data (alpha dropped) */
} crt_scene_desc;

/* Inputs as the reference's Scene holds them after construction, so a
 * Renderer shim can pass its arrays unchanged: */
typedef enum {
    CRT_SCENE_EDGES = 1u,      /* positions are v1, e1, e2 per face (Triangle::_v1,
                                  _e1, _e2) instead of three vertices */
    CRT_SCENE_KA_SCALED = 2u   /* material ka already includes the emission
                                  scaling Ka * 3 * lights area (scene.cpp:163,177) */
} crt_scene_flags;

/* Where the BVH is built.  Both produce the same node and triangle layouts,
 * so every query gives the same result; the trees differ, and with them the
 * nodes a ray visits. */
typedef enum {
    CRT_BVH_HOST = 0u,   /* binned SAH (32 bins; exact sweep below 33 triangles),
                            host threads: the best trees */
    CRT_BVH_GPU = 1u     /* PLOC clustering (Meister and Bittner 2018) over
                            63-bit Morton order on the device, then the same
                            collapse and encoding: a few milliseconds for
                            millions of triangles */
} crt_bvh_builder;

/* BVH node encoding on the device (same tree either way). */
typedef enum {
    CRT_NODES_Q8 = 0,    /* 80-byte nodes, child planes quantised to 8 bits
                            relative to the node and rounded outward */
    CRT_NODES_F32 = 1    /* 208-byte nodes with FP32 child planes: more bytes
                            per visit, half the ALU work per child test */
} crt_node_format;

typedef struct crt_scene_s* crt_scene;
typedef struct crt_render_s* crt_render;

/* Build-time statistics of a scene's BVH and buffers. */
typedef struct {
    uint32_t num_triangles;
    uint32_t num_nodes;        /* 8-wide nodes (80 bytes each) */
    uint32_t max_depth;        /* levels from the root to the deepest leaf */
    uint32_t num_lights;
    uint32_t num_materials;
    uint32_t num_textures;
    uint64_t node_bytes;
    uint64_t triangle_bytes;   /* intersection records (48 bytes each) */
    uint64_t shading_bytes;    /* normals/uv/material records */
    uint64_t texture_bytes;
    float lights_area;
    float build_ms;
    uint32_t bvh_width;        /* children per node of the current BVH: 4 or 8 */
} crt_scene_info;

/* ---- version / errors ------------------------------------------------ */
CRT_EXPORT int crt_api_version(void);
CRT_EXPORT const char* crt_last_error(void);

/* ---- camera -------------------------------------------------------------
 * CameraJsonLoader::getCamera (src/context/json_loader.cpp:26-48): fov from
 * `fieldOfView` degrees, aperture = focalLength / fStop, focus = |viewDirection|. */
CRT_EXPORT int crt_camera_from_json(float fov_deg, float focal_length, float fstop, const float eye[3],
                         const float view_dir[3], const float up[3], uint32_t width,
                         uint32_t height, crt_camera* out);

/* ---- scene --------------------------------------------------------------
 * Replaces Scene::constructBvh + constructLightList (scene.cpp:140-165) and
 * the uploads in the ParallelRenderer constructor
 * (parallel_renderer.cu:37-126): builds an 8-wide BVH with quantised child
 * bounds on the host and uploads it with the triangle, shading, material,
 * light and texture buffers to the current device. */
CRT_EXPORT int crt_scene_create(const crt_scene_desc* desc, crt_scene* out);
CRT_EXPORT int crt_scene_destroy(crt_scene scene);
CRT_EXPORT int crt_scene_get_info(crt_scene scene, crt_scene_info* out);
/* Host copies of the BVH as uploaded: nodes [num_nodes][80 bytes],
 * triangle records [num_triangles][48 bytes] (v1.xyz + face index bits,
 * e1.xyz + 0, e2.xyz + 0).  Either pointer may be NULL. */
CRT_EXPORT int crt_scene_export_bvh(crt_scene scene, void* nodes, void* triangles);
/* Replaces the material table (n = the scene's material count; ka is taken
 * as crt_scene_create took it, scaled or not per CRT_SCENE_KA_SCALED).  The light list and the total light
 * area stay those of crt_scene_create.  Waits for the device to go idle
 * first, so passes already queued finish with the old table.
 * No reference counterpart (the optimisation loop of the adjoint). */
CRT_EXPORT int crt_scene_set_materials(crt_scene scene, const crt_material* materials, uint32_t n);
/* Failure detection.  Every traversal counts the nodes it visits; past the
 * limit (default 2^20, 0 restores it) the ray ends as a miss and the scene's
 * device error word records it, so that the next crt_render_resolve /
 * _accum / _synchronize returns CRT_ERR_WATCHDOG (as it does for a traversal
 * stack overflow) instead of a GPU hang.  The error word stays set until
 * crt_scene_clear_errors.  Both wait for the device to go idle first; the
 * limit applies to passes started afterwards.  No reference counterpart
 * (the reference's traversal has no bound, renderer.cu:283-330). */
CRT_EXPORT int crt_scene_set_visit_limit(crt_scene scene, uint32_t max_visits);
CRT_EXPORT int crt_scene_clear_errors(crt_scene scene);
/* Reads the scene's sticky device error word into *bits (CRT_SCENE_ERR_*;
 * 0 when every traversal so far finished within its limits) after the work
 * queued on `stream` (NULL = default stream) before this call: one 4-byte
 * copy and a wait for that stream, nothing allocated.  The word is shared by
 * every render of the scene, so a bit may come from any of them since the
 * last crt_scene_clear_errors.  Callers of crt_render_tile_noalloc, which
 * returns before its kernels run and never reads the word, use this to learn
 * whether a tile had rays cut short. */
#define CRT_SCENE_ERR_WATCHDOG 1u   /* a traversal passed the node-visit limit */
#define CRT_SCENE_ERR_STACK 2u      /* a traversal stack overflowed */
CRT_EXPORT int crt_scene_errors(crt_scene scene, void* stream, uint32_t* bits);
/* Rebuilds the scene's BVH with 4 or 8 children per node from its own
 * triangle records (the geometry is unchanged, so every query answers the
 * same) and uploads it in place of the current one; the autotuner's BVH
 * width axis.  Waits for the device to go idle before the old nodes are
 * freed; render handles of the scene pick up the new BVH at their next pass.
 * No reference counterpart: the reference's BVH is binary. */
CRT_EXPORT int crt_scene_set_bvh_width(crt_scene scene, uint32_t bvh_width);
/* The same BVH build on the host alone, without a device (inspection and
 * build statistics): call once with nodes/triangles NULL to learn
 * num_nodes, then again with buffers of num_nodes*80 and n*48 bytes.
 * bvh_width: children per node, 4 or 8 (0 = 8).
 * Replaces constructBVH (src/geometry/bvh.cpp:65-77). */
CRT_EXPORT int crt_bvh_build_host(const float* positions, uint32_t num_triangles, uint32_t bvh_width,
                                  uint32_t* num_nodes, uint32_t* max_depth, void* nodes, void* triangles);

/* ---- ray queries ---------------------------------------------------------
 * Closest hit of a batch of rays; replaces intersectBVH
 * (src/renderer/renderer.cu:283-330) with Triangle::intersect
 * (src/geometry/geometry.cu:38-65).  d_rays: [n][8] floats
 * (o.x o.y o.z tmin d.x d.y d.z tmax).  A hit is the smallest t with
 * tmin < t < tmax; equal t goes to the lowest face index.  d_index gets the
 * face index or -1, d_t the distance (FLT_MAX on a miss), d_uv (optional)
 * the barycentrics.  Asynchronous on `stream` (NULL = default stream). */
CRT_EXPORT int crt_trace_closest(crt_scene scene, const float* d_rays, uint32_t n, int32_t* d_index,
                      float* d_t, float* d_uv, void* stream);
/* Node visits and triangle tests of each ray of crt_trace_closest
 * (instrumented traversal for the memory roofline). */
CRT_EXPORT int crt_trace_counts(crt_scene scene, const float* d_rays, uint32_t n, uint32_t* d_nodes,
                     uint32_t* d_tris, void* stream);

/* Measurement aid with no counterpart in the reference: the ceiling of the
 * traversal's access pattern.  n_threads (a multiple of 256) threads each
 * fetch loads_per_thread records of record_bytes (a multiple of 16) from
 * pseudo-random record indices of d_buf (bytes long, 16-byte aligned),
 * through L2 only, or through L1 as node fetches go with CRT_GATHER_L1.
 * d_sink gets one word per thread (keeps the loads live).  Bytes fetched =
 * n_threads * loads_per_thread * record_bytes; time it with events on
 * `stream`.  A working set below the L2 size gives the L2 gather ceiling. */
#define CRT_GATHER_L1 1u
CRT_EXPORT int crt_measure_gather(const void* d_buf, uint64_t bytes, uint32_t record_bytes,
                                  uint32_t n_threads, uint32_t loads_per_thread, uint32_t flags,
                                  uint32_t* d_sink, void* stream);

/* ---- progressive render -------------------------------------------------
 * Replaces ParallelRenderer (src/include/renderer.h:102-126). */
typedef enum {
    CRT_MODE_MEGAKERNEL = 0,   /* one kernel per pass runs whole paths */
    CRT_MODE_WAVEFRONT = 1     /* generate / extend / shade / shadow queues */
} crt_mode;

/* Traversal scheduling of the wavefront's persistent kernels.  The default
 * (0): a warp takes 32 rays and finishes them all before taking more, and a
 * node visit tests all triangles of the leaves it hits. */
enum {
    CRT_FLAG_LANE_REFILL = 1u,  /* a lane whose ray finished takes the next one
                                   at once (warp-local pool of queue entries) */
    CRT_FLAG_SPLIT_LEAF = 2u,   /* one triangle test per traversal step, so lanes
                                   in leaves and lanes in inner nodes interleave */
    CRT_FLAG_OCTANT_QUEUES = 4u, /* shade files surviving paths by the octant of
                                   their next direction (8 queue regions, each in
                                   path order), so a warp of the extend kernel
                                   mostly holds rays of one octant: the same child
                                   order at every node.  8x the queue memory; not
                                   used by crt_render_tile_noalloc */
    CRT_FLAG_SERIAL_SHADOW = 8u, /* trace each bounce's shadow rays before the next
                                   bounce's extension rays.  By default the two
                                   (independent) traversals are branches of the
                                   wave graph and fill each other's tails */
    CRT_FLAG_NO_WINDOW_SORT = 16u /* by default the shade kernel groups each
                                   block's 1024 consecutive queue entries before
                                   appending them: surviving paths by direction
                                   (7 x 7 cells of the octahedral map), shadow
                                   requests by light face, so that a traversal
                                   warp takes rays from one image region heading
                                   one way.  This flag appends in warp order
                                   instead.  The sort is also off with
                                   CRT_FLAG_OCTANT_QUEUES and in
                                   crt_render_tile_noalloc */
};

typedef struct {
    uint32_t max_depth;        /* bounces per path; the reference hard-codes 6
                                  (renderer.cu:25,33) */
    uint64_t seed;             /* Philox key */
    uint32_t view_id;          /* Philox counter word: separates views */
    uint32_t mode;             /* crt_mode */
    uint32_t block_size;       /* wavefront traversal kernels: threads per block,
                                  64, 128 or 256 (0 = 128) */
    uint32_t wave_paths;       /* wavefront: paths in flight per wave set; 0 = about
                                  16 samples of every pixel of the handle's views,
                                  a power of two in [2^16, 2^25] (32M at 1080p:
                                  ~4.7 GB of path state per set) */
    uint32_t flags;            /* CRT_FLAG_* */
    uint32_t wave_sets;        /* wavefront: waves in flight at once, each with its
                                  own buffers and stream, 0..8 (0 = default 4) */
    uint32_t stack_depth;      /* wavefront traversal kernels: stack entries per
                                  thread kept in shared memory, 4..32 (0 = 8);
                                  deeper entries go to local memory */
    int32_t node_format;       /* crt_node_format, or -1 for the scene's format */
    uint32_t queue_chunk;      /* wavefront traversal kernels: queue entries a warp
                                  claims per fetch, 32, 64, 128 or 256 (0 = 32);
                                  unused with CRT_FLAG_LANE_REFILL */
    uint32_t top_nodes;        /* wavefront traversal kernels: the first top_nodes
                                  BVH nodes (breadth-first: the top levels) are
                                  copied to shared memory at kernel start, 0..128
                                  (0 = none; 9 = two levels, the default of
                                  crt_render_options_default; 73 = three) */
    uint32_t refill_busy;      /* with CRT_FLAG_LANE_REFILL: idle lanes of a warp
                                  take new rays together once at most this many
                                  lanes are still busy, 1..31 (0 = 31: as soon as
                                  one lane is idle) */
} crt_render_options;

CRT_EXPORT void crt_render_options_default(crt_render_options* opts);

/* Constructor `ParallelRenderer(scene, w, h, spp)` (parallel_renderer.cu:37-77);
 * the accumulator starts at zero (the reference leaves it uninitialised). */
CRT_EXPORT int crt_render_create(crt_scene scene, const crt_camera* camera, uint32_t width,
                      uint32_t height, const crt_render_options* opts, crt_render* out);
CRT_EXPORT int crt_render_destroy(crt_render r);
/* Render n_spp more samples per pixel: n_spp calls of
 * renderOneSamplePerPixel (parallel_renderer.cu:288-301).  Asynchronous. */
CRT_EXPORT int crt_render_pass(crt_render r, uint32_t n_spp);
CRT_EXPORT int crt_render_samples_rendered(crt_render r, uint32_t* out);
CRT_EXPORT int crt_render_synchronize(crt_render r);
/* copyImageBytes (parallel_renderer.cu:303-310): RGBA8 of the average with
 * float3ToUchar4 (renderer.h:149-156) then gammaCorrectPixel
 * (renderer.cu:495-504); host_rgba holds width*height*4 bytes. */
CRT_EXPORT int crt_render_resolve(crt_render r, uint8_t* host_rgba);
/* renderKernel's own device image (parallel_renderer.cu:338-341): RGBA8 of
 * the average through float3ToUchar4 only (the gamma table is applied on
 * the host by copyImageBytes), written to the caller's device buffer of
 * width*height*4 bytes on the handle's stream.  Asynchronous. */
CRT_EXPORT int crt_render_resolve_device(crt_render r, void* d_rgba);
/* crt_render_resolve without the wait: the resolve kernel and the copy into
 * host_rgba (pinned memory, width*height*4 bytes) are queued on the handle's
 * stream behind the passes already queued, so a caller can queue the next
 * pass right away and overlap it with the copy; the bytes are valid after
 * crt_render_synchronize.  Uses a device staging buffer owned by the handle.
 * No reference counterpart. */
CRT_EXPORT int crt_render_resolve_async(crt_render r, uint8_t* host_rgba);
/* Progressive resume: replaces the accumulator of view `view` with
 * host_rgb ([width*height][3] FP32 sums, as crt_render_view_accum returns
 * them) holding `samples` samples that started at sample index
 * `first_sample`; the next pass continues at first_sample + samples.  With
 * the sums and the two counters saved, a render resumes bit for bit where it
 * stopped.  No reference counterpart. */
CRT_EXPORT int crt_render_load_accum(crt_render r, uint32_t view, const float* host_rgb, uint32_t samples,
                                     uint32_t first_sample);
/* FP32 per-pixel radiance sums [width*height][3] (host copy). */
CRT_EXPORT int crt_render_accum(crt_render r, float* host_rgb);
/* Device pointer of the accumulator, valid until destroy. */
CRT_EXPORT int crt_render_accum_device(crt_render r, float** d_rgb);
CRT_EXPORT int crt_render_reset(crt_render r);
/* As crt_render_reset, but the next pass renders from sample index
 * first_sample on (every view): a fresh, independent estimate per call, as
 * an optimisation loop wants.  No reference counterpart. */
CRT_EXPORT int crt_render_restart(crt_render r, uint32_t first_sample);
CRT_EXPORT int crt_render_set_camera(crt_render r, const crt_camera* camera);
/* Use the caller's CUDA stream (cudaStream_t) instead of the handle's own. */
CRT_EXPORT int crt_render_set_stream(crt_render r, void* stream);
/* Per-stage timing of a wavefront pass, for the memory roofline. */
typedef struct {
    double ms[6];              /* generate, extend, shade, shadow, accumulate, bookkeeping */
    uint64_t launches[6];
    uint64_t extension_rays, extension_nodes, extension_tris;
    uint64_t shadow_rays, shadow_nodes, shadow_tris;
    double extend_ms_by_bounce[16];      /* bounces >= 15 add to the last entry */
    uint64_t extend_rays_by_bounce[16];
    double shadow_ms_by_bounce[16];
    uint64_t shadow_rays_by_bounce[16];
    uint64_t extension_top_nodes, shadow_top_nodes;   /* visits (in *_nodes) to the nodes
                                                         staged in shared memory (top_nodes) */
} crt_stage_profile;

/* Renders n_spp more samples per pixel (like crt_render_pass, same result)
 * with the wavefront stages launched one by one instead of through the
 * graph, each timed with CUDA events on the handle's stream; every
 * extension and shadow traversal is re-run untimed in counting mode to
 * report node visits and triangle tests.  Wavefront handles only. */
CRT_EXPORT int crt_render_profile_pass(crt_render r, uint32_t n_spp, crt_stage_profile* out);

/* ---- batched views ------------------------------------------------------
 * No reference counterpart (the reference renders one camera per process).
 * A batch is a render handle over many camera views of one scene, each with
 * its own resolution, samples per pixel and Philox view word.  With
 * CRT_MODE_WAVEFRONT, crt_batch_render runs every view's samples as one
 * stream of waves: a wave packs whole sample layers or pixel ranges of
 * several views, so small views share the GPU instead of each launching
 * alone, and each wave replays the same captured CUDA graph.  With
 * CRT_MODE_MEGAKERNEL the views render one after another (one launch
 * sequence per view).  Either way view v's image equals, bit for bit, a
 * single render of that view with view_id = views[v].view_id.
 * crt_render_pass on a batch adds n_spp to every view; the single-view
 * functions (crt_render_resolve, _accum, _samples_rendered, _set_camera) act
 * on view 0, and crt_render_accum_device returns the accumulator of all
 * views, view v at pixel offset crt_render_view_info(...).pixel_offset. */
#define CRT_MAX_VIEWS 8192u
typedef struct {
    crt_camera camera;
    uint32_t width, height;
    uint32_t spp;              /* samples per pixel one crt_batch_render adds */
    uint32_t view_id;          /* Philox counter word of this view */
} crt_view;

CRT_EXPORT int crt_batch_create(crt_scene scene, const crt_view* views, uint32_t num_views,
                                const crt_render_options* opts, crt_render* out);
/* Renders views[v].spp more samples per pixel of every view.  Asynchronous. */
CRT_EXPORT int crt_batch_render(crt_render r);
/* Size, spp and view word of a view (camera left zeroed), its samples so far
 * and the offset of its first pixel in the accumulator; outputs may be NULL. */
CRT_EXPORT int crt_render_view_info(crt_render r, uint32_t view, crt_view* desc, uint32_t* samples_rendered,
                                    uint32_t* pixel_offset);
CRT_EXPORT int crt_render_view_resolve(crt_render r, uint32_t view, uint8_t* host_rgba);
CRT_EXPORT int crt_render_view_accum(crt_render r, uint32_t view, float* host_rgb);

/* ---- adjoint (differentiable rendering) -----------------------------------
 * No reference counterpart (the reference computes no derivatives).
 * Gradient of  Phi = sum over pixels p, channels c of adjoint[p][c] * S[p][c],
 * S being the radiance sum that samples [spp0, spp0 + n_spp) add to each
 * pixel (the samples crt_render_pass renders there), with respect to every
 * material's kd (diffuse albedo; diffuse vertices of untextured materials)
 * and ka (emission as given in crt_material).  For an image loss L(I) with
 * I = accum / spp, pass adjoint = dL/dI / spp.
 * Path-replay backpropagation: each path is traced twice from the same
 * Philox counters, first for its radiance, then again turning every vertex
 * into gradient terms, so nothing per vertex is stored.  By default Russian
 * roulette's survival probability counts as a constant: the gradient is
 * unbiased for the expected image (roulette is unbiased whatever the
 * probability).  CRT_ADJOINT_EXACT_ROULETTE also differentiates the
 * division by max(throughput) after each surviving roulette: the exact
 * derivative of every sample with its decisions held, what central finite
 * differences with common random numbers measure (max_depth <= 16; keeps a
 * 16-entry material history per path).  Gradients are summed per warp and
 * block before global atomics.  Always the wavefront form.
 * d_adjoint: device float4 per pixel of every view (the layout of
 * crt_render_accum_device; .w ignored).  d_grad_kd, d_grad_ka: device float
 * [num_materials][3], ADDED to.  At most 1024 materials.  Asynchronous on the
 * handle's stream; the accumulator and sample counts do not change. */
enum { CRT_ADJOINT_EXACT_ROULETTE = 1u };
CRT_EXPORT int crt_render_adjoint(crt_render r, uint32_t spp0, uint32_t n_spp, const float* d_adjoint,
                                  float* d_grad_kd, float* d_grad_ka, uint32_t flags);

/* ---- allocation-free tile render ----------------------------------------
 * No counterpart in the reference: an addition for callers that cannot
 * allocate device memory while rendering, such as a host application that
 * owns every device allocation through its own pool (a plugin inside a DCC
 * tool or engine), or a latency-critical loop that must not pay for
 * cudaMalloc / cudaFree and the device synchronisation they cause.
 *
 * Renders samples [spp0, spp0 + nspp) of the pixels [pixel0, pixel0 +
 * pixel_count) of a width x height image with the wavefront kernels and
 * adds each pixel's per-sample radiance, in sample order, to d_accum[pixel]
 * (the caller's device buffer of width*height x 4 floats: rgb + unused,
 * 16-byte aligned; same layout as crt_render_accum_device).  Sums are
 * bit-identical to crt_render_pass when calls cover each pixel's samples in
 * increasing order.  Asynchronous on `stream` (NULL = legacy default).
 *
 * The call allocates nothing: paths in flight, queues and counters live in
 * a fixed scratch array compiled into the library (about 8.5 MiB of device
 * memory on every GPU that loads it, held until the process exits).  Hence
 * pixel_count * nspp may not exceed CRT_NOALLOC_MAX_PATHS; larger requests
 * fail with CRT_ERR_LIMIT, so render big images as several tiles.  The
 * first call on a device looks up the scratch array's device address; make
 * that first call before any stream capture.  All calls share the one
 * scratch array, so calls that can overlap on the GPU (different streams,
 * or different threads without ordering) race: serialise them.
 * The call only queues kernels on `stream`: a traversal cut short by the
 * scene's visit limit or a stack overflow sets the scene's error word, which
 * this function does not read; check it with crt_scene_errors.  A CUDA error
 * already pending on the calling thread from earlier work is reported
 * (CRT_ERR_CUDA, not cleared) and nothing is launched.  The cached device
 * address of the scratch belongs to the device's primary context: after
 * cudaDeviceReset on that device, do not call this function again in the
 * process.  CRT_FLAG_OCTANT_QUEUES is ignored here (the scratch holds
 * single-region queues); like every launch option it does not change the
 * sums. */
#define CRT_NOALLOC_MAX_PATHS 65536u
CRT_EXPORT int crt_render_tile_noalloc(crt_scene scene, const crt_camera* camera, uint32_t width,
                                       uint32_t height, const crt_render_options* opts,
                                       uint32_t pixel0, uint32_t pixel_count, uint32_t spp0,
                                       uint32_t nspp, float* d_accum, void* stream);

/* Extension and shadow rays traced by the passes since the last reset. */
CRT_EXPORT int crt_render_ray_counts(crt_render r, uint64_t* extension_rays, uint64_t* shadow_rays);

/* ---- autotuner ------------------------------------------------------
 * No reference counterpart: the reference's launch shape is fixed at
 * compile time (16x16 blocks, renderer.cu:543-551).  crt_autotune times
 * short wavefront renders of the given scene, camera and image size and
 * searches, by coordinate descent, the options that change speed but not
 * the image: node_format, block_size, stack_depth, queue_chunk, wave_sets,
 * wave_paths, CRT_FLAG_LANE_REFILL, top_nodes and (tune_bvh_width) the BVH
 * width.
 * The device must be otherwise idle for the timings to mean anything.  With
 * tune_bvh_width the scene's BVH is rebuilt (crt_scene_set_bvh_width) and
 * the faster width is left in place. */
typedef struct {
    uint32_t trial_spp;        /* samples per pixel of each timed render (0 = 8) */
    uint32_t repeats;          /* timed renders per candidate, fastest kept (0 = 3) */
    uint32_t rounds;           /* coordinate-descent sweeps at most (0 = 2) */
    uint32_t tune_bvh_width;   /* nonzero: also try the other BVH width */
    uint64_t max_wave_bytes;   /* skip candidates whose path state exceeds this
                                  (0 = 32 GiB) */
} crt_tune_params;

typedef struct {
    crt_render_options options;  /* fastest options (mode = wavefront, defaults spelled out) */
    uint32_t bvh_width;          /* BVH width left in the scene */
    uint32_t candidates;         /* distinct candidates timed */
    float ms_per_spp;            /* fastest: milliseconds per sample per pixel */
    float start_ms_per_spp;      /* the starting options, for comparison */
    float tune_ms;               /* wall time spent tuning */
} crt_tune_result;

CRT_EXPORT void crt_tune_params_default(crt_tune_params* params);
CRT_EXPORT int crt_autotune(crt_scene scene, const crt_camera* camera, uint32_t width, uint32_t height,
                            const crt_render_options* start, const crt_tune_params* params,
                            crt_tune_result* out);

/* ---- scene files ----------------------------------------------------------
 * The reference's input files read without its loaders, into the arrays
 * crt_scene_desc takes (host memory owned by the handle):
 *  - Wavefront OBJ with its `mtllib` libraries: objl::Loader::LoadFile /
 *    LoadMaterials (src/include/obj_load.h:441-720, :1015-1186) as
 *    Scene::loadObj + loadTriangles assemble them (src/geometry/scene.cpp:
 *    40-46, 74-138): one record per face in file order; faces without
 *    normals get (p0 - p1) x (p2 - p1) at every vertex; `usemtl` names map
 *    to meshes by position as LoadFile maps them;
 *  - the material table of populateMaterialsMap + materialFromMtl
 *    (scene.cpp:175-203), including the reference's merging of materials
 *    (unless CRT_LOAD_EXACT_MATERIALS); ka is the MTL Ka, scaled by
 *    crt_scene_create as the reference scales it;
 *  - PNG textures named by `map_Kd` (Scene::loadTextures, scene.cpp:55-71;
 *    TextureStore::load, texture_store.cpp:18-35): linear texels
 *    (float)pow(b / 255, 2.2) as stbi_loadf returns them.
 * Departures, each for files the reference misreads or rejects: polygons
 * are fanned into triangles; grey images give grey texels; runs of blanks
 * separate tokens; a missing library, texture or malformed number is an
 * error (CRT_ERR_INVALID with file:line in crt_last_error()).  The light
 * list is left to crt_scene_create (emissive faces in face order). */
typedef struct crt_scene_files_s* crt_scene_files;

typedef enum {
    CRT_LOAD_EXACT_MATERIALS = 1u   /* one table entry per MTL material in use
                                       instead of the reference's merged table */
} crt_load_flags;

typedef struct {
    uint32_t num_triangles;
    uint32_t num_meshes;         /* meshes as LoadFile splits them (o, g, usemtl) */
    uint32_t num_materials;      /* entries of the material table */
    uint32_t num_mtl_materials;  /* materials read from the libraries */
    uint32_t num_textures;
    uint32_t num_positions;      /* v records */
    uint32_t num_texcoords;      /* vt records */
    uint32_t num_normals;        /* vn records */
    uint32_t num_polygons;       /* faces of more than 3 vertices (fanned) */
    uint64_t file_bytes;         /* OBJ + MTL + PNG bytes read */
    float parse_ms;              /* OBJ + MTL */
    float texture_ms;            /* PNG decode */
} crt_scene_files_info;

/* texture_dir is prefixed to each map_Kd name (a '/' is added if missing). */
CRT_EXPORT int crt_scene_files_load(const char* obj_path, const char* texture_dir, uint32_t flags,
                                    crt_scene_files* out);
/* Fills desc with pointers into the handle (valid until it is destroyed);
 * node_format, bvh_width, flags and builder are zero. */
CRT_EXPORT int crt_scene_files_desc(crt_scene_files files, crt_scene_desc* desc);
CRT_EXPORT int crt_scene_files_get_info(crt_scene_files files, crt_scene_files_info* out);
CRT_EXPORT int crt_scene_files_mesh(crt_scene_files files, uint32_t mesh, const char** name,
                                    uint32_t* first_triangle, uint32_t* num_triangles);
CRT_EXPORT int crt_scene_files_destroy(crt_scene_files files);
/* CameraJsonLoader (src/context/json_loader.cpp:15-48): keys fieldOfView,
 * focalLength, fStop, eye, viewDirection, upDirection. */
CRT_EXPORT int crt_camera_load_json(const char* path, uint32_t width, uint32_t height, crt_camera* out);
/* One PNG as stbi_loadf + TextureStore::load read it: dims = {width,
 * height}; with texels != NULL (capacity in texels) writes [w*h][rgb]. */
CRT_EXPORT int crt_texture_load_png(const char* path, uint32_t dims[2], float* texels, uint64_t capacity);
/* RGBA8 image to a PNG file (Launcher::saveToImage, src/context/
 * launcher.cpp:13-21). */
CRT_EXPORT int crt_image_write_png(const char* path, uint32_t width, uint32_t height, const uint8_t* rgba);

#ifdef __cplusplus
}
#endif
#endif
