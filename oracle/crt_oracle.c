/*
 * crt_oracle.c -- CPU restatement of CudaRT's path-tracing hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the parity checker; see crt_oracle.h).
 * Build with: -O2 -ffp-contract=off -fno-fast-math (-fopenmp optional).
 * Reference citations are paths inside the CudaRT source tree.
 */
#include "crt_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846   /* the value <math.h> gives under _GNU_SOURCE */
#endif

#define ORC_EPS 0.00001f     /* EPSILON   geometry.h:9 */
#define ORC_EPS2 0.000005f   /* EPSILON_2 geometry.h:10 */
#define ORC_NO_TEXTURE (-1)  /* material.h:6 */
#define ORC_STACK 1024       /* renderer.cu:289 holds 16, which overflows on deep trees */

/* ---- float3 helpers, linalg.h:15-40 (same operation order) ---------------- */
static inline orc_f3 f3(float x, float y, float z) { orc_f3 r = {x, y, z}; return r; }
static inline orc_f3 add3(orc_f3 a, orc_f3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline orc_f3 sub3(orc_f3 a, orc_f3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline orc_f3 mul3(orc_f3 a, orc_f3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline orc_f3 muls(orc_f3 a, float b) { return f3(a.x * b, a.y * b, a.z * b); }
static inline orc_f3 divs(orc_f3 a, float b) { return f3(a.x / b, a.y / b, a.z / b); }
static inline float dot3(orc_f3 a, orc_f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline orc_f3 cross3(orc_f3 a, orc_f3 b) {
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline orc_f3 normalize3(orc_f3 v) {
    float n = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
    return f3(v.x / n, v.y / n, v.z / n);
}
static inline float maxc3(orc_f3 v) { float m = v.x > v.y ? v.x : v.y; return m > v.z ? m : v.z; }
static inline orc_f3 min2(orc_f3 a, orc_f3 b) {   /* bvh.cpp:348-353 */
    return f3(a.x < b.x ? a.x : b.x, a.y < b.y ? a.y : b.y, a.z < b.z ? a.z : b.z);
}
static inline orc_f3 max2(orc_f3 a, orc_f3 b) {   /* bvh.cpp:355-360 */
    return f3(a.x > b.x ? a.x : b.x, a.y > b.y ? a.y : b.y, a.z > b.z ? a.z : b.z);
}
static inline float comp3(orc_f3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

/* ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) -------------------- */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

void orc_sampler_init(orc_sampler* s, uint64_t seed, uint32_t view, uint32_t pixel,
                      uint32_t sample) {
    s->key[0] = (uint32_t)seed;
    s->key[1] = (uint32_t)(seed >> 32);
    s->ctr[0] = 0;
    s->ctr[1] = sample;
    s->ctr[2] = pixel;
    s->ctr[3] = view;
    s->n = 0;
}

/* Sampler::getNextFloat (renderer.cu:72-78): one uniform draw in [0, 1). */
float orc_next_float(orc_sampler* s) {
    if ((s->n & 3u) == 0) {
        s->ctr[0] = s->n >> 2;
        orc_philox4x32_10(s->ctr, s->key, s->buf);
    }
    uint32_t x = s->buf[s->n & 3u];
    s->n++;
    return (float)(x >> 8) * 0x1p-24f;
}

/* ---- scene preparation ------------------------------------------------- */
void orc_make_triangle(orc_triangle* t, const float v[9], const float n[9],
                       const float uv[6], uint32_t material) {
    orc_f3 a = f3(v[0], v[1], v[2]), b = f3(v[3], v[4], v[5]), c = f3(v[6], v[7], v[8]);
    t->v1 = a;
    t->n1 = f3(n[0], n[1], n[2]);
    t->n2 = f3(n[3], n[4], n[5]);
    t->n3 = f3(n[6], n[7], n[8]);
    t->uv1.x = uv[0]; t->uv1.y = uv[1];
    t->uv2.x = uv[2]; t->uv2.y = uv[3];
    t->uv3.x = uv[4]; t->uv3.y = uv[5];
    t->e1 = sub3(b, a);                       /* scene.cpp:124 */
    t->e2 = sub3(c, a);                       /* scene.cpp:125 */
    t->material = material;
    orc_f3 cr = cross3(t->e1, t->e2);         /* scene.cpp:130 */
    t->area = sqrtf(cr.x * cr.x + cr.y * cr.y + cr.z * cr.z) / 2.0f;
}

float orc_lights_area(const orc_triangle* tris, const uint32_t* lights, uint32_t n) {
    float sa = 0;                             /* scene.cpp:167-173 */
    for (uint32_t i = 0; i < n; ++i) sa += tris[lights[i]].area;
    return sa;
}

void orc_make_material(orc_material* m, int32_t bsdf, int32_t tex, const float kd[3],
                       const float ka_mtl[3], const float ks[3], float ns, float ni,
                       float diffuse, float lights_area) {
    orc_f3 ka = muls(f3(ka_mtl[0], ka_mtl[1], ka_mtl[2]), 3.0f);  /* scene.cpp:177 */
    m->ka = muls(ka, lights_area);                                  /* scene.cpp:163 */
    m->kd = f3(kd[0], kd[1], kd[2]);
    m->ks = f3(ks[0], ks[1], ks[2]);
    m->ns = ns;
    m->ni = ni;
    m->diffuse = diffuse;
    m->bsdf = bsdf;
    m->tex = tex;
}

void orc_make_camera(orc_camera* c, float fov_deg, float focal_length, float fstop,
                     const float eye[3], const float view_dir[3], const float up[3],
                     uint32_t width, uint32_t height) {
    /* json_loader.cpp:26-48 */
    c->xpixels = (int32_t)width;
    c->ypixels = (int32_t)height;
    c->fov = tanf((float)((double)(fov_deg * 0.5f) * M_PI / 180.0));
    c->eye = f3(eye[0], eye[1], eye[2]);
    orc_f3 d = f3(view_dir[0], view_dir[1], view_dir[2]);
    c->focus = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
    c->dir = normalize3(d);
    c->up = normalize3(f3(up[0], up[1], up[2]));
    c->right = normalize3(cross3(c->dir, c->up));
    c->aperture = focal_length / fstop;
    c->aspect = (float)width / (float)height;
}

/* ---- binary BVH build, bvh.cpp:65-323 ------------------------------------- */
typedef struct { uint32_t tri; orc_f3 bmin, bmax, center; } orc_tbox;  /* bvh.cpp:18-30 */

typedef struct {
    orc_tbox* info;
    const orc_triangle* tris;
    orc_bvh_node* nodes;
    uint32_t* perm;
    uint32_t n_nodes;
    uint32_t n_ordered;
} orc_build;

static float bvh_volume(orc_f3 lo, orc_f3 hi) {  /* surfaceArea(), bvh.cpp:334-337 */
    orc_f3 d = sub3(hi, lo);
    return d.x * d.y * d.z;
}

static int bvh_max_extent(orc_f3 lo, orc_f3 hi) {  /* bvh.cpp:339-346 */
    orc_f3 d = sub3(hi, lo);
    if (d.x > d.y && d.x > d.z) return 0;
    if (d.y > d.z) return 1;
    return 2;
}

static float bvh_offset(orc_f3 lo, orc_f3 hi, orc_f3 p, int dim) {  /* bvh.cpp:326-332 */
    orc_f3 r = sub3(p, lo);
    if (hi.x > lo.x) r.x /= (hi.x - lo.x);
    if (hi.y > lo.y) r.y /= (hi.y - lo.y);
    if (hi.z > lo.z) r.z /= (hi.z - lo.z);
    return comp3(r, dim);
}

static int bvh_bucket(orc_f3 cmin, orc_f3 cmax, orc_f3 c, int dim) {
    int b = (int)(8 * bvh_offset(cmin, cmax, c, dim));
    if (b == 8) b = 7;
    return b;
}

static void tbox_swap(orc_tbox* a, orc_tbox* b) { orc_tbox t = *a; *a = *b; *b = t; }

/* In-place quickselect: element `k` ends in sorted position by centre[dim]
 * (std::nth_element, bvh.cpp:189-199). */
static void bvh_nth_element(orc_tbox* a, uint32_t lo, uint32_t hi, uint32_t k, int dim) {
    while (hi - lo > 1) {
        uint32_t mid = lo + (hi - lo) / 2;
        float pv = comp3(a[mid].center, dim);
        tbox_swap(&a[mid], &a[hi - 1]);
        uint32_t st = lo;
        for (uint32_t i = lo; i < hi - 1; ++i)
            if (comp3(a[i].center, dim) < pv) tbox_swap(&a[i], &a[st++]);
        tbox_swap(&a[st], &a[hi - 1]);
        if (st == k) return;
        if (k < st) hi = st; else lo = st + 1;
    }
}

static uint32_t bvh_push_leaf(orc_build* b, uint32_t start, uint32_t end) {
    uint32_t first = b->n_ordered;
    for (uint32_t i = start; i < end; ++i) b->perm[b->n_ordered++] = b->info[i].tri;
    return first;
}

/* recursiveBuild (bvh.cpp:114-307) fused with flattenBVHTree (:309-323):
 * nodes are written depth first, first child (upper partition) at i+1. */
static uint32_t bvh_recurse(orc_build* b, uint32_t start, uint32_t end) {
    uint32_t my = b->n_nodes++;
    orc_bvh_node* node = &b->nodes[my];
    orc_f3 wmin = f3(FLT_MAX, FLT_MAX, FLT_MAX), wmax = f3(-FLT_MAX, -FLT_MAX, -FLT_MAX);
    for (uint32_t i = start; i < end; ++i) {
        wmin = min2(wmin, b->info[i].bmin);
        wmax = max2(wmax, b->info[i].bmax);
    }
    node->bmin = wmin;
    node->bmax = wmax;
    node->axis = 0;   /* interior axis stays 0: flattenBVHTree never sets it */
    uint32_t n = end - start;
    if (n <= 3) {
        node->offset = (int32_t)bvh_push_leaf(b, start, end);
        node->ntris = (int16_t)n;
        return my;
    }
    orc_f3 cmin = f3(FLT_MAX, FLT_MAX, FLT_MAX), cmax = f3(-FLT_MAX, -FLT_MAX, -FLT_MAX);
    for (uint32_t i = start; i < end; ++i) {
        cmin = min2(cmin, b->info[i].center);
        cmax = max2(cmax, b->info[i].center);
    }
    int dim = bvh_max_extent(cmin, cmax);
    uint32_t mid = (start + end) / 2;
    if (comp3(cmax, dim) == comp3(cmin, dim)) {
        node->offset = (int32_t)bvh_push_leaf(b, start, end);
        node->ntris = (int16_t)n;
        return my;
    }
    if (n <= 4) {
        bvh_nth_element(b->info, start, end, mid, dim);
    } else {
        int count[8] = {0};
        orc_f3 lo[8], hi[8];
        for (int k = 0; k < 8; ++k) { lo[k] = f3(FLT_MAX, FLT_MAX, FLT_MAX); hi[k] = f3(-FLT_MAX, -FLT_MAX, -FLT_MAX); }
        for (uint32_t i = start; i < end; ++i) {
            int bk = bvh_bucket(cmin, cmax, b->info[i].center, dim);
            count[bk]++;
            lo[bk] = min2(lo[bk], b->info[i].bmin);
            hi[bk] = max2(hi[bk], b->info[i].bmax);
        }
        float cost[7];
        for (int i = 0; i < 7; ++i) {
            orc_f3 b0lo = f3(FLT_MAX, FLT_MAX, FLT_MAX), b0hi = f3(-FLT_MAX, -FLT_MAX, -FLT_MAX);
            orc_f3 b1lo = b0lo, b1hi = b0hi;
            int c0 = 0, c1 = 0;
            for (int j = 0; j <= i; ++j) { b0lo = min2(b0lo, lo[j]); b0hi = max2(b0hi, hi[j]); c0 += count[j]; }
            for (int j = i + 1; j < 8; ++j) { b1lo = min2(b1lo, lo[j]); b1hi = max2(b1hi, hi[j]); c1 += count[j]; }
            cost[i] = 1.f + (c0 * bvh_volume(b0lo, b0hi) + c1 * bvh_volume(b1lo, b1hi)) /
                            bvh_volume(wmin, wmax);
        }
        int best = 0;                                   /* std::min_element */
        for (int i = 1; i < 7; ++i) if (cost[i] < cost[best]) best = i;
        /* std::partition by bucket <= best (bvh.cpp:254-271) */
        uint32_t st = start;
        for (uint32_t i = start; i < end; ++i)
            if (bvh_bucket(cmin, cmax, b->info[i].center, dim) <= best) tbox_swap(&b->info[i], &b->info[st++]);
        mid = st;
        if (mid == start || mid == end) {
            mid = (start + end) / 2;
            bvh_nth_element(b->info, start, end, mid, dim);
        }
    }
    node->ntris = 0;
    /* children[0] = upper partition [mid, end), children[1] = [start, mid)
     * (bvh.cpp:302-304); DFS flatten puts children[0] at my + 1. */
    bvh_recurse(b, mid, end);
    uint32_t second = bvh_recurse(b, start, mid);
    b->nodes[my].offset = (int32_t)second;
    return my;
}

uint32_t orc_bvh_build(const orc_triangle* tris, uint32_t n_tris, orc_bvh_node* nodes_out,
                       uint32_t* perm_out) {
    if (n_tris == 0) return 0;
    orc_build b;
    b.info = (orc_tbox*)malloc(sizeof(orc_tbox) * n_tris);
    b.tris = tris;
    b.nodes = nodes_out;
    b.perm = perm_out;
    b.n_nodes = 0;
    b.n_ordered = 0;
    for (uint32_t i = 0; i < n_tris; ++i) {   /* createTriangleBboxes, bvh.cpp:79-96 */
        const orc_triangle* t = &tris[i];
        orc_f3 v2 = add3(t->v1, t->e1), v3 = add3(t->v1, t->e2);
        orc_f3 lo = min2(t->v1, min2(v2, v3)), hi = max2(t->v1, max2(v2, v3));
        b.info[i].tri = i;
        b.info[i].bmin = lo;
        b.info[i].bmax = hi;
        b.info[i].center = muls(add3(lo, hi), 0.5f);
    }
    bvh_recurse(&b, 0, n_tris);
    free(b.info);
    return b.n_nodes;
}

/* ---- intersection ------------------------------------------------------- */
float orc_tri_intersect(const orc_triangle* tr, orc_f3 o, orc_f3 d, float* ou, float* ov) {
    /* Triangle::intersect, geometry.cu:38-65 */
    orc_f3 P = cross3(d, tr->e2);
    float det = dot3(tr->e1, P);
    if (fabsf(det) < ORC_EPS) return FLT_MAX;
    float inv_det = 1.f / det;
    orc_f3 T = sub3(o, tr->v1);
    float u = dot3(T, P) * inv_det;
    if (u < 0.f || u > 1.f) return FLT_MAX;
    orc_f3 Q = cross3(T, tr->e1);
    float v = dot3(d, Q) * inv_det;
    if (v < 0.f || u + v > 1.f) return FLT_MAX;
    float t = dot3(tr->e2, Q) * inv_det;
    if (t > ORC_EPS) { *ou = u; *ov = v; return t; }
    return FLT_MAX;
}

/* rayIntersectsBox, renderer.cu:333-373: slab test against the infinite line. */
static int orc_ray_box(orc_f3 o, orc_f3 d, orc_f3 lo, orc_f3 hi) {
    float t0 = -FLT_MAX, t1 = FLT_MAX;
    for (int k = 0; k < 3; ++k) {
        float inv = 1.f / comp3(d, k);
        float tn = (comp3(lo, k) - comp3(o, k)) * inv;
        float tf = (comp3(hi, k) - comp3(o, k)) * inv;
        if (tn > tf) { float tmp = tn; tn = tf; tf = tmp; }
        t0 = tn > t0 ? tn : t0;
        t1 = tf < t1 ? tf : t1;
        if (t0 > t1) return 0;
    }
    return 1;
}

typedef struct { orc_f3 o, d; float tmin, tmax; int32_t idx; float u, v; } orc_ray;

/* intersectTriangles (renderer.cu:264-280) with the lowest-index tie rule. */
static inline void orc_test_tri(const orc_scene* s, uint32_t orig, orc_ray* r) {
    float u, v;
    float t = orc_tri_intersect(&s->tris[orig], r->o, r->d, &u, &v);
    if (t == FLT_MAX || !(t > r->tmin)) return;
    if (t < r->tmax || (t == r->tmax && r->idx >= 0 && (int32_t)orig < r->idx)) {
        r->tmax = t; r->idx = (int32_t)orig; r->u = u; r->v = v;
    }
}

/* intersectBVH, renderer.cu:283-330 (stack of 64). */
static int orc_trace(const orc_scene* s, orc_ray* r, uint32_t* nv, uint32_t* nt) {
    if (s->n_nodes == 0) {
        for (uint32_t i = 0; i < s->n_tris; ++i) orc_test_tri(s, i, r);
        if (nt) *nt += s->n_tris;
        return r->idx >= 0;
    }
    orc_f3 inv = f3(1 / r->d.x, 1 / r->d.y, 1 / r->d.z);
    int neg[3] = {inv.x < 0, inv.y < 0, inv.z < 0};
    int stack[ORC_STACK];
    int top = 0, cur = 0;
    for (;;) {
        const orc_bvh_node* n = &s->nodes[cur];
        if (nv) (*nv)++;
        if (orc_ray_box(r->o, r->d, n->bmin, n->bmax)) {
            if (n->ntris > 0) {
                for (int i = 0; i < n->ntris; ++i) orc_test_tri(s, s->tri_perm[n->offset + i], r);
                if (nt) *nt += (uint32_t)n->ntris;
                if (top == 0) break;
                cur = stack[--top];
            } else {
                if (top >= ORC_STACK) abort();   /* stack overflow is a build bug */
                if (neg[n->axis]) { stack[top++] = cur + 1; cur = n->offset; }
                else { stack[top++] = n->offset; cur = cur + 1; }
            }
        } else {
            if (top == 0) break;
            cur = stack[--top];
        }
    }
    return r->idx >= 0;
}

static void ray_from(const float* p, orc_ray* r) {
    r->o = f3(p[0], p[1], p[2]);
    r->tmin = p[3];
    r->d = f3(p[4], p[5], p[6]);
    r->tmax = p[7];
    r->idx = -1;
    r->u = r->v = 0.f;
}

void orc_closest_hit_brute(const orc_scene* s, const float* rays, uint32_t n, int32_t* idx,
                           float* t, float* uv) {
    for (uint32_t k = 0; k < n; ++k) {
        orc_ray r;
        ray_from(rays + 8 * k, &r);
        for (uint32_t i = 0; i < s->n_tris; ++i) orc_test_tri(s, i, &r);
        idx[k] = r.idx;
        t[k] = r.idx >= 0 ? r.tmax : FLT_MAX;
        if (uv) { uv[2 * k] = r.u; uv[2 * k + 1] = r.v; }
    }
}

void orc_closest_hit_bvh(const orc_scene* s, const float* rays, uint32_t n, int32_t* idx,
                         float* t, float* uv, int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 256)
#endif
    for (int64_t k = 0; k < (int64_t)n; ++k) {
        orc_ray r;
        ray_from(rays + 8 * k, &r);
        orc_trace(s, &r, NULL, NULL);
        idx[k] = r.idx;
        t[k] = r.idx >= 0 ? r.tmax : FLT_MAX;
        if (uv) { uv[2 * k] = r.u; uv[2 * k + 1] = r.v; }
    }
    (void)threads;
}

void orc_traversal_counts(const orc_scene* s, const float* rays, uint32_t n,
                          uint32_t* nodes_visited, uint32_t* tris_tested) {
    for (uint32_t k = 0; k < n; ++k) {
        orc_ray r;
        ray_from(rays + 8 * k, &r);
        uint32_t nv = 0, nt = 0;
        orc_trace(s, &r, &nv, &nt);
        nodes_visited[k] = nv;
        tris_tested[k] = nt;
    }
}

/* ---- estimator ---------------------------------------------------------- */
static const float orc_skybox[3] = {0.0f, 0.025f, 0.05f};   /* renderer.cu:66-68 */

static orc_f3 tri_normal(const orc_triangle* t, float u, float v) {
    /* Triangle::getNormal, geometry.cu:67-71 */
    float w = 1.f - u - v;
    return normalize3(add3(add3(muls(t->n1, w), muls(t->n2, u)), muls(t->n3, v)));
}

/* sampleTexture host branch, renderer.cu:92-115. */
static orc_f3 sample_texture(const orc_scene* s, int tex, float u, float v) {
    uint32_t W = s->tex_dims[2 * tex], H = s->tex_dims[2 * tex + 1];
    const orc_f3* p = s->tex_data + s->tex_offsets[tex];
    uint32_t avail = s->tex_total - s->tex_offsets[tex];
    float pu = u * (float)W;
    float pv = v * (float)H;
    uint32_t i = (uint32_t)truncf(pu);
    uint32_t j = (uint32_t)truncf(pv);
    float fu = floorf(pu), fv = floorf(pv), cu = ceilf(pu), cv = ceilf(pv);
    uint32_t ia = j * W + i + 1, ib = j * W + i, ic = (j + 1) * W + i + 1, id = (j + 1) * W + i;
    orc_f3 z = f3(0, 0, 0);
    orc_f3 ta = ia < avail ? p[ia] : z, tb = ib < avail ? p[ib] : z;
    orc_f3 tc = ic < avail ? p[ic] : z, td = id < avail ? p[id] : z;
    orc_f3 a1 = muls(ta, pu - fu);
    orc_f3 a2 = muls(tb, cu - pu);
    orc_f3 b1 = muls(tc, pu - fu);
    orc_f3 b2 = muls(td, cu - pu);
    orc_f3 c1 = muls(add3(a1, a2), cv - pv);
    orc_f3 c2 = muls(add3(b1, b2), pv - fv);
    return add3(c1, c2);
}

/* tentFilter + Camera::computeCameraRay, camera.cu:13-57. */
static void camera_ray(const orc_camera* c, int i, int j, orc_sampler* smp, orc_ray* r) {
    float r1 = 2.f * orc_next_float(smp);
    float r2 = 2.f * orc_next_float(smp);
    float dx = r1 < 1.f ? sqrtf(r1) - 1.f : 1.f - sqrtf(2.f - r1);
    float dy = r2 < 1 ? sqrtf(r2) - 1.f : 1.f - sqrtf(2.f - r2);
    float ni = (float)((double)(((float)i + dx) / (float)c->xpixels) - 0.5);
    float nj = 0.5f - (((float)j + dy) / (float)c->ypixels);
    orc_f3 dir = c->dir, origin = c->eye;
    dir = add3(dir, muls(muls(muls(c->right, c->fov), c->aspect), ni));
    dir = add3(dir, muls(muls(c->up, c->fov), nj));
    if (c->aperture > 0.0f) {
        float q1 = (float)((double)orc_next_float(smp) - 0.5f * 2 * M_PI);
        float q2 = orc_next_float(smp) - 0.5f;
        float rj = cosf(q1) * q2 * c->aperture;
        float uj = sinf(q1) * q2 * c->aperture;
        origin = add3(origin, add3(muls(c->right, rj), muls(c->up, uj)));
        orc_f3 focal = add3(c->eye, muls(dir, c->focus));
        dir = sub3(focal, origin);
    }
    r->o = origin;
    r->d = normalize3(dir);
    r->tmin = ORC_EPS;
    r->tmax = FLT_MAX;
    r->idx = -1;
}

static inline void reset_ray(orc_ray* r, orc_f3 o, orc_f3 d) {
    r->o = o; r->d = d; r->tmin = ORC_EPS; r->tmax = FLT_MAX; r->idx = -1; r->u = r->v = 0.f;
}

/* Gradient context of the adjoint replay (orc_adjoint): w is the pixel's
 * adjoint weight, total the radiance of the path's first trace; the
 * gradient terms are formed and summed in FP64. */
typedef struct {
    double w[3];
    orc_f3 total;
    double ka_scale;            /* d(stored emission)/d(material ka) = 3 * lights area */
    double* gkd;                /* [n_mats][3] */
    double* gka;
    /* exact roulette: materials of the kd factors in the throughput so far,
     * and the previous surviving roulette's channel and history length */
    int exact;
    uint32_t hist[64];
    int n_hist, prev_c, prev_n;
} orc_grad;

static orc_f3 sample_path(const orc_scene* s, const orc_camera* cam, int x, int y,
                          orc_sampler* smp, uint32_t max_depth, orc_grad* g);

orc_f3 orc_sample_pixel(const orc_scene* s, const orc_camera* cam, int x, int y,
                        orc_sampler* smp, uint32_t max_depth) {
    return sample_path(s, cam, x, y, smp, max_depth, NULL);
}

/* samplePixel with optional gradient hooks: with g, each event of the path
 * adds its derivative terms (path-replay backpropagation; Russian roulette's
 * survival probability held constant):
 *  - emission term mask * ka / lights_area:  d/d ka_m = mask * 3 SA / SA;
 *  - diffuse vertex of untextured material m: every later term carries one
 *    factor kd_m, so d/d kd_m += (total - radiance so far) / kd_m;
 *  - visible light sample: d/d ka_light = mask * weight * 3 SA. */
static orc_f3 sample_path(const orc_scene* s, const orc_camera* cam, int x, int y,
                          orc_sampler* smp, uint32_t max_depth, orc_grad* g) {
    orc_ray ray;
    camera_ray(cam, x, y, smp, &ray);
    orc_f3 color = f3(0.f, 0.f, 0.f);
    orc_f3 mask = f3(1.f, 1.f, 1.f);
    orc_f3 in_dir = f3(0.f, 0.f, 0.f);   /* SurfaceInteraction() value-initialised */
    int prev = ORC_DIFFUSE;
    float one_over_sa = 1.f / s->lights_area;
    for (uint32_t bounce = 0; bounce < max_depth; ++bounce) {
        if (!orc_trace(s, &ray, NULL, NULL)) {
            color = add3(color, mul3(mask, f3(orc_skybox[0], orc_skybox[1], orc_skybox[2])));
            break;
        }
        uint32_t hit = (uint32_t)ray.idx;
        const orc_triangle* tri = &s->tris[hit];
        const orc_material* m = &s->mats[tri->material];
        if (bounce == 0 || prev == ORC_SPECULAR || prev == ORC_REFRACTIVE) {
            color = add3(color, muls(mul3(mask, m->ka), one_over_sa));
            if (g) {
                const double mk[3] = {mask.x, mask.y, mask.z};
                for (int c = 0; c < 3; ++c)
                    g->gka[3 * tri->material + c] += g->w[c] * mk[c] * g->ka_scale * (double)one_over_sa;
            }
        }
        orc_f3 normal = tri_normal(tri, ray.u, ray.v);
        orc_f3 position = add3(add3(ray.o, muls(ray.d, ray.tmax)), muls(normal, ORC_EPS2));
        orc_f3 out_dir = normalize3(ray.d);
        int bsdf = m->bsdf;
        if (bsdf == ORC_DIFFSPEC) {                          /* renderer.cu:171-181 */
            float p = m->diffuse;
            if (orc_next_float(smp) < p) { bsdf = ORC_DIFFUSE; mask = muls(mask, 1.0f / p); }
            else { bsdf = ORC_SPECULAR; mask = muls(mask, 1.0f / (1.0f - p)); }
        }
        if (bsdf == ORC_REFRACTIVE) {                        /* renderer.cu:183-205, 464-493 */
            float cosi = dot3(out_dir, normal);
            float etai = 1, etat = m->ni;
            orc_f3 n = normal;
            if (cosi < 0.0f) cosi = -cosi;
            else { float tmp = etai; etai = etat; etat = tmp; n = muls(normal, -1.0f); }
            float eta = etai / etat;
            float k = 1 - eta * eta * (1 - cosi * cosi);
            float pr, pt;
            orc_f3 tdir = f3(0, 0, 0);
            if (k < 0) { pr = 1.0f; pt = 0.0f; }
            else {
                tdir = add3(muls(out_dir, eta), muls(n, eta * cosi - sqrtf(k)));
                float R0 = (etai - etat) * (etai - etat) / (etat + etai) * (etat + etai);
                float c = 1.f - dot3(tdir, normal);
                float Re = R0 + (1.f - R0) * c * c * c * c * c;
                pr = Re; pt = 1.f - Re;
            }
            if (pr == 1.0f) bsdf = ORC_SPECULAR;
            else {
                float P = 0.25f + .5f * pr;
                float RP = pr / P;
                float TP = pt / (1.f - P);
                if (orc_next_float(smp) > 0.25f) {
                    in_dir = tdir;
                    mask = muls(mul3(mask, m->ks), TP);
                } else {
                    mask = muls(mask, RP);
                    bsdf = ORC_SPECULAR;
                }
            }
        }
        if (bsdf == ORC_DIFFUSE) {                           /* renderer.cu:207-236, 375-402 */
            float r1 = (float)(2 * M_PI * (double)orc_next_float(smp));
            float r2 = orc_next_float(smp);
            float r2sq = sqrtf(r2);
            orc_f3 w = normal;
            orc_f3 u = normalize3(cross3(fabsf(w.x) > 0.1f ? f3(0.f, 1.f, 0.f) : f3(1.f, 0.f, 0.f), w));
            orc_f3 v = cross3(w, u);
            in_dir = normalize3(add3(add3(muls(muls(u, cosf(r1)), r2sq), muls(muls(v, sinf(r1)), r2sq)),
                                     muls(w, sqrtf(1.f - r2))));
            float cosw = dot3(in_dir, normal);
            orc_f3 kd = m->kd;
            if (m->tex != ORC_NO_TEXTURE) {
                float tu = ray.u, tv = ray.v;
                float tw = 1.f - tu - tv;
                float uvx = tri->uv1.x * tw + tri->uv2.x * tu + tri->uv3.x * tv;
                float uvy = tri->uv1.y * tw + tri->uv2.y * tu + tri->uv3.y * tv;
                kd = sample_texture(s, m->tex, uvx, uvy);
            } else if (g) {
                const double rest[3] = {(double)g->total.x - color.x, (double)g->total.y - color.y,
                                        (double)g->total.z - color.z};
                const double k[3] = {kd.x, kd.y, kd.z};
                for (int c = 0; c < 3; ++c)
                    if (k[c] != 0.0) g->gkd[3 * tri->material + c] += g->w[c] * rest[c] / k[c];
                if (g->exact && g->n_hist < 64) g->hist[g->n_hist++] = tri->material;
            }
            mask = divs(mul3(mask, muls(kd, cosw)), 0.5f);
            /* light pick, renderer.cu:218-221 */
            float rn = orc_next_float(smp) * ((float)s->n_lights - .00001f);
            uint32_t li = (uint32_t)truncf(rn);
            if (li >= s->n_lights) li = s->n_lights - 1;
            uint32_t light = s->lights[li];
            const orc_triangle* lt = &s->tris[light];
            orc_f3 lcolor = s->mats[lt->material].ka;
            orc_f3 direct = f3(0.0f, 0.0f, 0.0f);
            if (hit != light) {                              /* estimateDirectLighting, :414-445 */
                orc_f3 ro = add3(position, muls(normal, ORC_EPS));
                float pu = orc_next_float(smp), pv = orc_next_float(smp);
                if (pu + pv >= 1.0f) { pu = 1.0f - pu; pv = 1.0f - pv; }
                orc_f3 pt = add3(add3(lt->v1, muls(lt->e1, pu)), muls(lt->e2, pv));
                orc_ray sr;
                reset_ray(&sr, ro, normalize3(sub3(pt, position)));
                if (orc_trace(s, &sr, NULL, NULL) && (uint32_t)sr.idx == light) {
                    float sa = lt->area;
                    float d2 = sr.tmax * sr.tmax;
                    float cost = fabsf(dot3(tri_normal(lt, sr.u, sr.v), muls(sr.d, -1.0f)));
                    float wgt = sa / (d2 * s->lights_area) * cost;
                    direct = add3(direct, muls(lcolor, wgt));
                    if (g) {
                        const double mk[3] = {mask.x, mask.y, mask.z};
                        for (int c = 0; c < 3; ++c)
                            g->gka[3 * lt->material + c] += g->w[c] * mk[c] * (double)wgt * g->ka_scale;
                    }
                }
            }
            color = add3(color, mul3(mask, direct));
        }
        if (bsdf == ORC_SPECULAR) {                          /* renderer.cu:238-243, 404-412 */
            in_dir = sub3(out_dir, muls(muls(normal, dot3(out_dir, normal)), 2.f));
            mask = divs(mul3(mask, m->ks), 1.0f);
        }
        prev = bsdf;
        reset_ray(&ray, add3(position, muls(in_dir, ORC_EPS)), in_dir);
        if (bounce >= 3) {                                   /* renderer.cu:252-259 */
            float p = maxc3(mask);
            if (orc_next_float(smp) > p) break;
            if (g && g->exact) {
                /* After this roulette the throughput is mask / mask[c], c the
                 * channel max_component picks: every term from here on gets
                 * -1/kd[c] per kd factor so far, in channel c, replacing the
                 * previous roulette's correction (only the latest counts). */
                const int c01 = mask.x > mask.y ? 0 : 1;
                const float v01 = mask.x > mask.y ? mask.x : mask.y;
                const int cs = v01 > mask.z ? c01 : 2;
                const double sdot = g->w[0] * ((double)g->total.x - color.x) +
                                    g->w[1] * ((double)g->total.y - color.y) +
                                    g->w[2] * ((double)g->total.z - color.z);
                for (int i = 0; i < g->n_hist; ++i) {
                    const orc_f3 k = s->mats[g->hist[i]].kd;
                    const double kc = cs == 0 ? k.x : cs == 1 ? k.y : k.z;
                    if (kc != 0.0) g->gkd[3 * g->hist[i] + cs] -= sdot / kc;
                }
                for (int i = 0; i < g->prev_n; ++i) {
                    const orc_f3 k = s->mats[g->hist[i]].kd;
                    const double kc = g->prev_c == 0 ? k.x : g->prev_c == 1 ? k.y : k.z;
                    if (kc != 0.0) g->gkd[3 * g->hist[i] + g->prev_c] += sdot / kc;
                }
                g->prev_c = cs;
                g->prev_n = g->n_hist;
            }
            mask = divs(mask, p);
        }
    }
    return color;
}

void orc_render(const orc_scene* s, const orc_camera* cam, uint64_t seed, uint32_t view,
                uint32_t spp0, uint32_t spp, uint32_t max_depth, const uint32_t* pixels,
                uint32_t n_pixels, float* acc, double* mean, double* m2, int threads) {
    uint32_t W = (uint32_t)cam->xpixels, H = (uint32_t)cam->ypixels;
    int64_t total = pixels ? (int64_t)n_pixels : (int64_t)W * H;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int64_t k = 0; k < total; ++k) {
        uint32_t pix = pixels ? pixels[k] : (uint32_t)k;
        int x = (int)(pix % W), y = (int)(pix / W);
        float a[3] = {0, 0, 0};
        if (acc) { a[0] = acc[3 * k]; a[1] = acc[3 * k + 1]; a[2] = acc[3 * k + 2]; }
        double mu[3] = {0, 0, 0}, q[3] = {0, 0, 0};
        for (uint32_t si = 0; si < spp; ++si) {
            orc_sampler smp;
            orc_sampler_init(&smp, seed, view, pix, spp0 + si);
            orc_f3 c = orc_sample_pixel(s, cam, x, y, &smp, max_depth);
            a[0] = a[0] + c.x; a[1] = a[1] + c.y; a[2] = a[2] + c.z;
            double cv[3] = {c.x, c.y, c.z};
            for (int ch = 0; ch < 3; ++ch) {
                double dlt = cv[ch] - mu[ch];
                mu[ch] += dlt / (double)(si + 1);
                q[ch] += dlt * (cv[ch] - mu[ch]);
            }
        }
        if (acc) { acc[3 * k] = a[0]; acc[3 * k + 1] = a[1]; acc[3 * k + 2] = a[2]; }
        if (mean) for (int ch = 0; ch < 3; ++ch) mean[3 * k + ch] = mu[ch];
        if (m2) for (int ch = 0; ch < 3; ++ch) m2[3 * k + ch] = q[ch];
    }
    (void)H;
    (void)threads;
}

void orc_adjoint(const orc_scene* s, const orc_camera* cam, uint64_t seed, uint32_t view,
                 uint32_t spp0, uint32_t spp, uint32_t max_depth, const float* adjoint,
                 uint32_t n_mats, double* grad_kd, double* grad_ka, int exact_roulette, int threads) {
    uint32_t W = (uint32_t)cam->xpixels, H = (uint32_t)cam->ypixels;
    int64_t total = (int64_t)W * H;
    const double ka_scale = 3.0 * (double)s->lights_area;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel
#endif
    {
        double* gkd = (double*)calloc(3 * (size_t)n_mats, sizeof(double));
        double* gka = (double*)calloc(3 * (size_t)n_mats, sizeof(double));
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
        for (int64_t k = 0; k < total; ++k) {
            const float* a = adjoint + 3 * k;
            if (a[0] == 0.f && a[1] == 0.f && a[2] == 0.f) continue;
            int x = (int)((uint32_t)k % W), y = (int)((uint32_t)k / W);
            for (uint32_t si = 0; si < spp; ++si) {
                orc_sampler smp;
                orc_sampler_init(&smp, seed, view, (uint32_t)k, spp0 + si);
                orc_grad g;
                g.w[0] = a[0]; g.w[1] = a[1]; g.w[2] = a[2];
                g.ka_scale = ka_scale;
                g.gkd = gkd;
                g.gka = gka;
                g.exact = exact_roulette;
                g.n_hist = 0;
                g.prev_c = 0;
                g.prev_n = 0;
                g.total = sample_path(s, cam, x, y, &smp, max_depth, NULL);
                orc_sampler_init(&smp, seed, view, (uint32_t)k, spp0 + si);   /* replay */
                sample_path(s, cam, x, y, &smp, max_depth, &g);
            }
        }
#ifdef _OPENMP
#pragma omp critical
#endif
        for (uint32_t i = 0; i < 3 * n_mats; ++i) {
            grad_kd[i] += gkd[i];
            grad_ka[i] += gka[i];
        }
        free(gkd);
        free(gka);
    }
    (void)H;
    (void)threads;
}

/* ---- output formatting -------------------------------------------------- */
uint8_t orc_gamma_u8(uint8_t v) {
    /* gammaCorrectPixel, renderer.cu:495-504: pow(float, float) resolves to
     * the float overload in C++ (powf). */
    float inv_gamma = 1.f / 2.2f;
    float fp = powf((float)v * 1.f / 255.f, inv_gamma);
    return (uint8_t)(fp * 255.f);
}

void orc_resolve(const float* acc, uint32_t n_pixels, uint32_t spp, uint8_t* rgba) {
    for (uint32_t i = 0; i < n_pixels; ++i) {
        for (int ch = 0; ch < 3; ++ch) {
            float v = acc[3 * i + ch] / (float)spp;               /* renderer.h:149-156 */
            uint8_t q = (uint8_t)((v > 1.0f ? 1.0f : v) * (255.f));
            rgba[4 * i + ch] = orc_gamma_u8(q);
        }
        rgba[4 * i + 3] = 255u;
    }
}

void orc_prepare_tris(const float* pos, const float* nor, const float* uv, const uint32_t* mat,
                      uint32_t n, orc_triangle* out) {
    for (uint32_t i = 0; i < n; ++i)
        orc_make_triangle(&out[i], pos + 9 * (size_t)i, nor + 9 * (size_t)i, uv + 6 * (size_t)i, mat[i]);
}
