/*
 * crt_oracle.h -- CPU restatement of CudaRT's path-tracing hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the
 * GB300 kernels in cudart_gb300/csrc.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load it; the product never calls it.
 *
 * Every function restates the reference's CPU code path (the `--cpu`
 * SequentialRenderer, which runs the shared `samplePixel` estimator on the
 * host) and cites the reference file:line it follows.  Arithmetic is FP32
 * in the reference's operation order; the library must be compiled with
 * -ffp-contract=off so that no multiply-add is fused (the reference's host
 * pass on x86-64 never fuses).  FP64 appears only in the per-pixel
 * statistics accumulators of orc_render().
 *
 * Deliberate, documented departures from the as-shipped reference:
 *  - RNG: libc rand() (renderer.cu:76) is replaced by a counter-based
 *    Philox4x32-10 stream keyed by (seed, view, pixel, sample), so results
 *    are deterministic and thread-safe.  A draw is (x >> 8) * 2^-24, which
 *    is exactly what `rand()/(float)RAND_MAX` yields when rand() returns
 *    (x >> 8) << 7; the pinning harness interposes rand() that way.
 *  - BVH build (bvh.cpp:114-307) initialises the centroid and bucket bounds
 *    that the reference leaves uninitialised (bvh.cpp:133,205,231), and the
 *    traversal stack holds 1024 entries instead of 16 (renderer.cu:289).
 *  - Closest-hit ties (equal t) go to the lowest original triangle index;
 *    the reference's tie winner depends on traversal order
 *    (renderer.cu:271).
 *  - Texel reads outside the padded texture array return 0 instead of
 *    reading out of bounds (renderer.cu:108-111, texture_store.cpp:68).
 */
#ifndef CRT_ORACLE_H
#define CRT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { float x, y, z; } orc_f3;
typedef struct { float x, y; } orc_f2;

/* refl_t (material.h:8-15) */
enum { ORC_DIFFUSE = 0, ORC_SPECULAR = 1, ORC_DIFFSPEC = 2, ORC_MICROFACET = 3,
       ORC_REFRACTIVE = 4, ORC_EMISSIVE = 5 };

/* Triangle (geometry.h:30-51): v1, e1 = v2 - v1, e2 = v3 - v1, vertex
 * normals, vertex uvs, area = |e1 x e2| / 2 (scene.cpp:114-130). */
typedef struct {
    orc_f3 v1, e1, e2, n1, n2, n3;
    orc_f2 uv1, uv2, uv3;
    float area;
    uint32_t material;
} orc_triangle;

/* One row of the material tables (parallel_renderer.cu:252-279):
 * kd, ka (already multiplied by 3 * lightsSurfaceArea, scene.cpp:163,177),
 * ks, (ns, ni, diffuseCoefficient), (bsdf, texKdIdx). */
typedef struct {
    orc_f3 kd, ka, ks;
    float ns, ni, diffuse;
    int32_t bsdf, tex;
} orc_material;

/* Camera (camera.h:9-22). */
typedef struct {
    orc_f3 eye, dir, up, right;
    float fov, aspect, aperture, focus;
    int32_t xpixels, ypixels;
} orc_camera;

/* LinearBVHNode (bvh.h:18-27): leaf if ntris > 0; then `offset` is the
 * first triangle position, else it is the second child's node index. */
typedef struct {
    orc_f3 bmin, bmax;
    int32_t offset;
    int16_t ntris, axis;
} orc_bvh_node;

typedef struct {
    uint32_t n_tris;
    const orc_triangle* tris;      /* original (caller) order */
    uint32_t n_mats;
    const orc_material* mats;
    uint32_t n_lights;
    const uint32_t* lights;        /* original triangle indices, pick order */
    float lights_area;             /* sum of light areas in pick order */
    uint32_t n_tex;
    const uint32_t* tex_dims;      /* [n_tex][2] width, height */
    const uint32_t* tex_offsets;   /* [n_tex] first texel of each texture */
    const orc_f3* tex_data;        /* flattened texels + zero padding */
    uint32_t tex_total;            /* texels in tex_data incl. padding */
    /* binary BVH built by orc_bvh_build */
    uint32_t n_nodes;
    const orc_bvh_node* nodes;
    const uint32_t* tri_perm;      /* BVH position -> original index */
} orc_scene;

/* ---- RNG ---------------------------------------------------------------- */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

typedef struct {
    uint32_t key[2];
    uint32_t ctr[4];
    uint32_t buf[4];
    uint32_t n;            /* draws consumed */
} orc_sampler;

void orc_sampler_init(orc_sampler* s, uint64_t seed, uint32_t view,
                      uint32_t pixel, uint32_t sample);
float orc_next_float(orc_sampler* s);

/* ---- scene preparation -------------------------------------------------- */
/* Fill one triangle from three vertices (scene.cpp:111-130). */
void orc_make_triangle(orc_triangle* t, const float v[9], const float n[9],
                       const float uv[6], uint32_t material);
/* orc_make_triangle over arrays: pos/nor [n][9], uv [n][6]. */
void orc_prepare_tris(const float* pos, const float* nor, const float* uv,
                      const uint32_t* mat, uint32_t n, orc_triangle* out);
/* Sum of light areas in list order (scene.cpp:167-173). */
float orc_lights_area(const orc_triangle* tris, const uint32_t* lights, uint32_t n);
/* Material row from MTL values (scene.cpp:175-190) and the area scaling
 * of ka (scene.cpp:163). */
void orc_make_material(orc_material* m, int32_t bsdf, int32_t tex, const float kd[3],
                       const float ka_mtl[3], const float ks[3], float ns,
                       float ni, float diffuse, float lights_area);
/* Camera from the camera-JSON fields (json_loader.cpp:26-48). */
void orc_make_camera(orc_camera* c, float fov_deg, float focal_length, float fstop,
                     const float eye[3], const float view_dir[3], const float up[3],
                     uint32_t width, uint32_t height);

/* Binary SAH BVH (bvh.cpp:65-323).  Writes at most 2*n_tris-1 nodes and a
 * permutation of n_tris entries; returns the node count. */
uint32_t orc_bvh_build(const orc_triangle* tris, uint32_t n_tris,
                       orc_bvh_node* nodes_out, uint32_t* perm_out);

/* ---- intersection ------------------------------------------------------- */
/* Moller-Trumbore, Triangle::intersect (geometry.cu:38-65): returns t or
 * FLT_MAX. */
float orc_tri_intersect(const orc_triangle* t, orc_f3 o, orc_f3 d, float* u, float* v);

/* Closest hit over all triangles in index order (lowest index wins ties).
 * rays: [n][8] = ox oy oz tmin dx dy dz tmax.  idx = -1 on miss. */
void orc_closest_hit_brute(const orc_scene* s, const float* rays, uint32_t n,
                           int32_t* idx, float* t, float* uv);
/* Same result through the scene's binary BVH (renderer.cu:283-330). */
void orc_closest_hit_bvh(const orc_scene* s, const float* rays, uint32_t n,
                         int32_t* idx, float* t, float* uv, int threads);
/* Node visits and triangle tests per ray through the binary BVH. */
void orc_traversal_counts(const orc_scene* s, const float* rays, uint32_t n,
                          uint32_t* nodes_visited, uint32_t* tris_tested);

/* ---- estimator ---------------------------------------------------------- */
/* samplePixel (renderer.cu:119-262) for one (x, y, sample). */
orc_f3 orc_sample_pixel(const orc_scene* s, const orc_camera* cam, int x, int y,
                        orc_sampler* smp, uint32_t max_depth);

/* Render samples [spp0, spp0+spp) of every pixel.  acc (optional, [W*H*3])
 * accumulates FP32 sums in sample order exactly like the reference's
 * accumulator (sequential_renderer.cu:106-107); mean/m2 (optional, FP64,
 * [W*H*3]) receive Welford statistics of the per-sample radiance.
 * pixels (optional) restricts the render to a list of pixel indices; then
 * acc/mean/m2 are indexed by list position. */
void orc_render(const orc_scene* s, const orc_camera* cam, uint64_t seed, uint32_t view,
                uint32_t spp0, uint32_t spp, uint32_t max_depth,
                const uint32_t* pixels, uint32_t n_pixels,
                float* acc, double* mean, double* m2, int threads);

/* FP64 reference gradient of  sum_p,c adjoint[p][c] * S[p][c]  (S = the
 * radiance sum of samples [spp0, spp0+spp) of pixel p) with respect to each
 * material's kd (untextured diffuse vertices) and ka (emission as given,
 * stored as ka * 3 * lights_area): each path is traced, then replayed from
 * the same sampler with every event turned into derivative terms, summed in
 * FP64.  exact_roulette = 0: Russian roulette's survival probability is held
 * constant (unbiased for the gradient of the expected image); 1: its
 * renormalisation mask / max(mask) is differentiated too, the exact
 * derivative of each sample with its decisions fixed (what central
 * differences with common random numbers measure; kd history of at most 64
 * vertices).  adjoint [W*H][3]; grad_kd / grad_ka [n_mats][3] are added to. */
void orc_adjoint(const orc_scene* s, const orc_camera* cam, uint64_t seed, uint32_t view,
                 uint32_t spp0, uint32_t spp, uint32_t max_depth, const float* adjoint,
                 uint32_t n_mats, double* grad_kd, double* grad_ka, int exact_roulette, int threads);

/* ---- output formatting -------------------------------------------------- */
/* float3ToUchar4 (renderer.h:149-156) of acc / spp, then gammaCorrectPixel
 * (renderer.cu:495-504) on the host (parallel_renderer.cu:303-310). */
void orc_resolve(const float* acc, uint32_t n_pixels, uint32_t spp, uint8_t* rgba);
uint8_t orc_gamma_u8(uint8_t v);

#ifdef __cplusplus
}
#endif
#endif
