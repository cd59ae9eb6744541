/*
 * ref_harness.cpp -- pins the oracle to the reference itself.
 *
 * TEST INFRASTRUCTURE ONLY.  Linked (by oracle/Makefile, target `ref`) with
 * CudaRT's own renderer.cu, geometry.cu, camera.cu, scene.cpp, bvh.cpp,
 * texture_store.cpp and json_loader.cpp, compiled unmodified from the
 * reference tree.  It loads a scene through the reference's Scene class
 * (scene.h:13-75), then exposes the reference's closest-hit traversal
 * (intersectBVH, renderer.cu:283-330), its per-sample estimator
 * (samplePixel, renderer.cu:119-262) and its gamma step
 * (gammaCorrectPixel, renderer.cu:495-504) through a C ABI.
 *
 * libc rand() is interposed (the library links with -Bsymbolic) by a
 * thread-local Philox4x32-10 stream keyed per (seed, view, pixel, sample),
 * returning (x >> 8) << 7 so that `rand()/(float)RAND_MAX` equals the
 * oracle's draw (x >> 8) * 2^-24 bit for bit.
 *
 * The reference keeps scene-build state in file-static globals
 * (bvh.cpp:60-61, scene.cpp:24-25), so one process loads one scene.
 */
#include "renderer.h"
#include "scene.h"

#include <cfloat>
#include <chrono>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <vector>

typedef void* dataPtr_t;
__host__ __device__ bool intersectBVH(dataPtr_t p_bvhData, Triangle* p_triangles,
                                      SurfaceInteraction& interaction, Ray& ray);
__host__ __device__ bool rayIntersectsBox(Ray& ray, const float3& min, const float3& max);

/* Host-only harness: the device compilation pass sees an empty file body. */
#ifndef __CUDA_ARCH__

/* The traversal stack and bounce count the linked renderer.cu was compiled
 * with: 16 and 6 as shipped (renderer.cu:289, 25/33); the Makefile's
 * ref-deep target builds a copy with both raised and passes them here. */
#ifndef CRT_REF_STACK
#define CRT_REF_STACK 16
#endif
#ifndef CRT_REF_DEPTH
#define CRT_REF_DEPTH 6
#endif

namespace {

struct PhiloxStream {
    uint32_t key[2];
    uint32_t ctr[4];
    uint32_t buf[4];
    uint32_t n;
};

thread_local PhiloxStream g_rng = {{0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}, 0};

void philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        c0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        c1 = (uint32_t)p1;
        c2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c3 = (uint32_t)p0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

void rng_key(uint64_t seed, uint32_t view, uint32_t pixel, uint32_t sample) {
    g_rng.key[0] = (uint32_t)seed;
    g_rng.key[1] = (uint32_t)(seed >> 32);
    g_rng.ctr[0] = 0;
    g_rng.ctr[1] = sample;
    g_rng.ctr[2] = pixel;
    g_rng.ctr[3] = view;
    g_rng.n = 0;
}

Scene* g_scene = nullptr;
std::vector<uint32_t> g_perm;          // BVH position -> original face index
std::vector<uint32_t> g_inv;           // original face index -> BVH position
std::vector<float3> g_mat_floats;      // createMaterialsData layout
std::vector<int2> g_mat_ints;
SceneData g_scene_data;
int g_width = 0, g_height = 0;

int bvh_depth(const LinearBVHNode* nodes, int i) {
    if (nodes[i].numTriangles > 0) return 1;
    int a = bvh_depth(nodes, i + 1), b = bvh_depth(nodes, nodes[i].secondChildOffset);
    return 1 + (a > b ? a : b);
}

/* Deepest traversal stack intersectBVH would use for this ray: the same
 * visit order (renderer.cu:290-328), which depends only on the box tests
 * because the reference never culls by distance. */
int stack_need(const LinearBVHNode* nodes, Ray ray) {
    float3 inv = make_float3(1 / ray.dir.x, 1 / ray.dir.y, 1 / ray.dir.z);
    int neg[3] = {inv.x < 0, inv.y < 0, inv.z < 0};
    std::vector<int> stack;
    int cur = 0, need = 0;
    for (;;) {
        const LinearBVHNode& n = nodes[cur];
        if (rayIntersectsBox(ray, n.min, n.max) && n.numTriangles == 0) {
            if (neg[n.axis]) { stack.push_back(cur + 1); cur = n.secondChildOffset; }
            else { stack.push_back(n.secondChildOffset); cur = cur + 1; }
            need = need > (int)stack.size() ? need : (int)stack.size();
        } else {
            if (stack.empty()) break;
            cur = stack.back();
            stack.pop_back();
        }
    }
    return need;
}

}  // namespace

extern "C" int rand(void) noexcept {
    PhiloxStream& s = g_rng;
    if ((s.n & 3u) == 0) {
        s.ctr[0] = s.n >> 2;
        philox(s.ctr, s.key, s.buf);
    }
    uint32_t x = s.buf[s.n & 3u];
    s.n++;
    return (int)((x >> 8) << 7);
}

extern "C" {

/* Load obj + camera json + textures through the reference (main.cpp:133-139). */
__attribute__((visibility("default"))) int ref_load(const char* obj, const char* cam,
                                                    const char* tex_dir, int width,
                                                    int height) {
    try {
        g_scene = new Scene();
        g_scene->loadObj(obj);
        g_scene->loadCamera(cam, (pixels_t)width, (pixels_t)height);
        g_scene->loadTextures(tex_dir);
        g_scene->loadTriangles();
        g_scene->constructBvh();
        uint32_t n = (uint32_t)g_scene->getNumTriangles();
        g_perm.resize(n);
        g_inv.resize(n);
        for (uint32_t i = 0; i < n; ++i) {
            g_perm[i] = g_scene->getTriPtr()[i]._triId;
            g_inv[g_perm[i]] = i;
        }
        g_scene->constructLightList();
        uint32_t nm = g_scene->getNumMaterials();
        Material* m = g_scene->getMaterialsPtr();
        g_mat_floats.assign(MAX_MATERIALS * MATERIALS_FLOAT_COMPONENTS, make_float3(0, 0, 0));
        g_mat_ints.assign(MAX_MATERIALS, make_int2(0, 0));
        for (uint32_t i = 0; i < nm; ++i) {  // sequential_renderer.cu:48-64
            g_mat_floats[4 * i + 0] = m[i].kd;
            g_mat_floats[4 * i + 1] = m[i].ka;
            g_mat_floats[4 * i + 2] = m[i].ks;
            g_mat_floats[4 * i + 3] = make_float3(m[i].ns, m[i].ni, m[i].diffuseCoefficient);
            g_mat_ints[i] = make_int2((int32_t)m[i].bsdf, (int32_t)m[i].texKdIdx);
        }
        std::memset(&g_scene_data, 0, sizeof(g_scene_data));  // sequential_renderer.cu:73-89
        g_scene_data.p_triangles = g_scene->getTriPtr();
        g_scene_data.p_bvh = g_scene->getBvhPtr();
        g_scene_data.p_textureData = g_scene->getTexturePtr();
        g_scene_data.p_textureDimensions = g_scene->getTextureDimensionsPtr();
        g_scene_data.p_textureOffsets = g_scene->getTextureOffsetsPtr();
        g_scene_data.numBVHNodes = g_scene->getNumBvhNodes();
        g_scene_data.numTextures = g_scene->getNumTextures();
        g_width = width;
        g_height = height;
        return (int)n;
    } catch (const std::exception&) {
        return -1;
    }
}

/* counts: n_tris, n_nodes, n_materials, n_lights, n_textures, bvh_depth,
 * total_texels (without padding), padding texels. */
__attribute__((visibility("default"))) void ref_counts(uint32_t out[8]) {
    Scene* s = g_scene;
    out[0] = (uint32_t)s->getNumTriangles();
    out[1] = s->getNumBvhNodes();
    out[2] = s->getNumMaterials();
    out[3] = (uint32_t)s->getNumLights();
    out[4] = s->getNumTextures();
    out[5] = out[1] ? (uint32_t)bvh_depth(s->getBvhPtr(), 0) : 0;
    out[6] = out[4] ? s->getTotalTexturePixels() : 0;
    out[7] = out[4] ? s->getTextureDimensionsPtr()[2 * (out[4] - 1)] : 0;
}

/* Triangles in original face order: v1 e1 e2 n1 n2 n3 (18) uv1 uv2 uv3 (6)
 * area (1) -> 25 floats, plus the material id. */
__attribute__((visibility("default"))) void ref_export_tris(float* out, uint32_t* mat) {
    Triangle* t = g_scene->getTriPtr();
    for (size_t o = 0; o < g_perm.size(); ++o) {
        const Triangle& x = t[g_inv[o]];
        float* p = out + 25 * o;
        const float3* v[6] = {&x._v1, &x._e1, &x._e2, &x._n1, &x._n2, &x._n3};
        for (int k = 0; k < 6; ++k) { p[3 * k] = v[k]->x; p[3 * k + 1] = v[k]->y; p[3 * k + 2] = v[k]->z; }
        p[18] = x._uv1.x; p[19] = x._uv1.y; p[20] = x._uv2.x; p[21] = x._uv2.y;
        p[22] = x._uv3.x; p[23] = x._uv3.y; p[24] = x._surfaceArea;
        mat[o] = x._materialId;
    }
}

/* Material rows: kd ka ks (ns ni diffuse) -> 12 floats; (bsdf, tex). */
__attribute__((visibility("default"))) void ref_export_materials(float* out, int32_t* ints) {
    uint32_t nm = g_scene->getNumMaterials();
    for (uint32_t i = 0; i < nm; ++i) {
        for (int k = 0; k < 4; ++k) {
            float3 f = g_mat_floats[4 * i + k];
            out[12 * i + 3 * k] = f.x; out[12 * i + 3 * k + 1] = f.y; out[12 * i + 3 * k + 2] = f.z;
        }
        ints[2 * i] = g_mat_ints[i].x;
        ints[2 * i + 1] = g_mat_ints[i].y;
    }
}

/* Light list in the reference's pick order, as original face indices. */
__attribute__((visibility("default"))) float ref_export_lights(uint32_t* orig) {
    uint32_t n = (uint32_t)g_scene->getNumLights();
    uint32_t* li = g_scene->getLightsIndicesPtr();
    for (uint32_t i = 0; i < n; ++i) orig[i] = g_perm[li[i]];
    return g_scene->getLightsSurfaceArea();
}

/* Camera: eye dir up right (12) fov aspect aperture focus (4) x y pixels. */
__attribute__((visibility("default"))) void ref_export_camera(float* out, int32_t* px) {
    Camera* c = g_scene->getCameraPtr();
    const float3* v[4] = {&c->eye, &c->dir, &c->up, &c->right};
    for (int k = 0; k < 4; ++k) { out[3 * k] = v[k]->x; out[3 * k + 1] = v[k]->y; out[3 * k + 2] = v[k]->z; }
    out[12] = c->fov; out[13] = c->aspect; out[14] = c->apertureWidth; out[15] = c->focusDistance;
    px[0] = c->xpixels; px[1] = c->ypixels;
}

/* Texture dims [n][2], offsets [n], texels incl. padding [total][3]. */
__attribute__((visibility("default"))) void ref_export_textures(uint32_t* dims, uint32_t* offs,
                                                                float* texels) {
    uint32_t c[8];
    ref_counts(c);
    for (uint32_t i = 0; i < c[4]; ++i) {
        dims[2 * i] = g_scene->getTextureDimensionsPtr()[2 * i];
        dims[2 * i + 1] = g_scene->getTextureDimensionsPtr()[2 * i + 1];
        offs[i] = g_scene->getTextureOffsetsPtr()[i];
    }
    float3* p = g_scene->getTexturePtr();
    for (uint32_t i = 0; i < c[6] + c[7]; ++i) {
        texels[3 * i] = p[i].x; texels[3 * i + 1] = p[i].y; texels[3 * i + 2] = p[i].z;
    }
}

/* Traversal stack entries and maximum bounces of the linked estimator. */
__attribute__((visibility("default"))) void ref_limits(uint32_t out[2]) {
    out[0] = CRT_REF_STACK;
    out[1] = CRT_REF_DEPTH;
}

/* Closest hit through the reference's own traversal.  rays [n][8] =
 * o.xyz tmin d.xyz tmax; idx is the original face index, -1 on a miss, or
 * -2 when the ray's traversal would overflow the linked build's stack
 * (16 entries as shipped, renderer.cu:289) and was therefore not run. */
__attribute__((visibility("default"))) void ref_closest_hit(const float* rays, uint32_t n,
                                                            int32_t* idx, float* t, float* uv) {
    for (uint32_t k = 0; k < n; ++k) {
        const float* r = rays + 8 * k;
        Ray ray(make_float3(r[0], r[1], r[2]), make_float3(r[4], r[5], r[6]));
        ray.tMin = r[3];
        ray.tMax = r[7];
        if (stack_need(g_scene->getBvhPtr(), ray) > CRT_REF_STACK) {
            idx[k] = -2;
            t[k] = FLT_MAX;
            uv[2 * k] = uv[2 * k + 1] = 0.f;
            continue;
        }
        SurfaceInteraction si;
        std::memset(&si, 0, sizeof(si));
        bool hit = intersectBVH((dataPtr_t)g_scene->getBvhPtr(), g_scene->getTriPtr(), si, ray);
        idx[k] = hit ? (int32_t)g_perm[si.hitTriIdx] : -1;
        t[k] = hit ? ray.tMax : FLT_MAX;
        uv[2 * k] = hit ? si.u : 0.f;
        uv[2 * k + 1] = hit ? si.v : 0.f;
    }
}

/* One call of the reference samplePixel with the keyed stream; returns the
 * number of random draws it consumed. */
__attribute__((visibility("default"))) uint32_t ref_sample_pixel(int x, int y, uint64_t seed,
                                                                 uint32_t view, uint32_t sample,
                                                                 float* rgb) {
    rng_key(seed, view, (uint32_t)(y * g_width + x), sample);
    Sampler sampler;
    float3 c = samplePixel(x, y, *g_scene->getCameraPtr(), &g_scene_data,
                           g_scene->getLightsIndicesPtr(), (uint)g_scene->getNumLights(),
                           g_scene->getLightsSurfaceArea(), &sampler, g_mat_floats.data(),
                           g_mat_ints.data());
    rgb[0] = c.x; rgb[1] = c.y; rgb[2] = c.z;
    return g_rng.n;
}

/* Per-pixel FP32 accumulation (sequential_renderer.cu:106-107) and FP64
 * Welford statistics over samples [spp0, spp0+spp) of listed pixels. */
__attribute__((visibility("default"))) void ref_render(const uint32_t* pixels, uint32_t n,
                                                       uint64_t seed, uint32_t view,
                                                       uint32_t spp0, uint32_t spp, float* acc,
                                                       double* mean, double* m2) {
    float lsa = g_scene->getLightsSurfaceArea();
    Camera cam = *g_scene->getCameraPtr();
    uint numLights = (uint)g_scene->getNumLights();
    uint* lights = g_scene->getLightsIndicesPtr();
#pragma omp parallel for schedule(dynamic, 8)
    for (int64_t k = 0; k < (int64_t)n; ++k) {
        uint32_t pix = pixels[k];
        int x = (int)(pix % (uint32_t)g_width), y = (int)(pix / (uint32_t)g_width);
        float3 a = make_float3(0, 0, 0);
        double mu[3] = {0, 0, 0}, q[3] = {0, 0, 0};
        for (uint32_t s = 0; s < spp; ++s) {
            rng_key(seed, view, pix, spp0 + s);
            Sampler sampler;
            float3 c = samplePixel(x, y, cam, &g_scene_data, lights, numLights, lsa, &sampler,
                                   g_mat_floats.data(), g_mat_ints.data());
            a = a + c;
            double cv[3] = {c.x, c.y, c.z};
            for (int ch = 0; ch < 3; ++ch) {
                double d = cv[ch] - mu[ch];
                mu[ch] += d / (double)(s + 1);
                q[ch] += d * (cv[ch] - mu[ch]);
            }
        }
        acc[3 * k] = a.x; acc[3 * k + 1] = a.y; acc[3 * k + 2] = a.z;
        for (int ch = 0; ch < 3; ++ch) { mean[3 * k + ch] = mu[ch]; m2[3 * k + ch] = q[ch]; }
    }
}

/* Wall time of the reference's file loading alone (main.cpp:133-137 up to
 * loadTriangles: OBJ + MTL, camera JSON, textures, triangle assembly), in
 * milliseconds; -1 on an exception.  Leaves the scene half built: call it
 * in a process of its own. */
__attribute__((visibility("default"))) double ref_time_load(const char* obj, const char* cam,
                                                            const char* tex_dir, int width,
                                                            int height) {
    try {
        auto t0 = std::chrono::steady_clock::now();
        Scene* s = new Scene();
        s->loadObj(obj);
        s->loadCamera(cam, (pixels_t)width, (pixels_t)height);
        s->loadTextures(tex_dir);
        s->loadTriangles();
        auto t1 = std::chrono::steady_clock::now();
        return std::chrono::duration<double, std::milli>(t1 - t0).count();
    } catch (const std::exception&) {
        return -1.0;
    }
}

/* gammaCorrectPixel for every byte value (red channel path). */
__attribute__((visibility("default"))) void ref_gamma_table(uint8_t* out256) {
    for (int v = 0; v < 256; ++v) {
        uchar4 p = make_uchar4((unsigned char)v, 0, 0, 255);
        gammaCorrectPixel(p);
        out256[v] = p.x;
    }
}

/* float3ToUchar4 (renderer.h:149-156) of acc / spp. */
__attribute__((visibility("default"))) void ref_quantise(const float* acc, uint32_t n, uint32_t spp,
                                                         uint8_t* rgba) {
    for (uint32_t i = 0; i < n; ++i) {
        float3 v = make_float3(acc[3 * i], acc[3 * i + 1], acc[3 * i + 2]) / (float)spp;
        uchar4 q = float3ToUchar4(v);
        rgba[4 * i] = q.x; rgba[4 * i + 1] = q.y; rgba[4 * i + 2] = q.z; rgba[4 * i + 3] = q.w;
    }
}

}  // extern "C"

#endif  // __CUDA_ARCH__
