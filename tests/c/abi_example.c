/* A plain C host of the library: builds the Cornell box from a few quads,
 * renders it with the plain kernel and the wavefront form, and prints both
 * images' byte sums and whether the FP32 accumulators are identical.  The
 * GPU tests compile it with gcc against include/crt_gb300.h. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "crt_gb300.h"

#define CHECK(call)                                                        \
    do {                                                                   \
        int st_ = (call);                                                  \
        if (st_ != CRT_OK) {                                               \
            fprintf(stderr, "%s failed: %d %s\n", #call, st_, crt_last_error()); \
            return 1;                                                      \
        }                                                                  \
    } while (0)

/* two triangles per quad: corners a, b, c, d counter-clockwise */
static int quad(float* pos, float* nor, unsigned* mid, int f, const float q[4][3], unsigned m) {
    const int tri[2][3] = {{0, 1, 2}, {0, 2, 3}};
    float e1[3], e2[3], n[3];
    for (int k = 0; k < 3; ++k) { e1[k] = q[1][k] - q[0][k]; e2[k] = q[2][k] - q[0][k]; }
    n[0] = e1[1] * e2[2] - e1[2] * e2[1];
    n[1] = e1[2] * e2[0] - e1[0] * e2[2];
    n[2] = e1[0] * e2[1] - e1[1] * e2[0];
    float l = 0.f;
    for (int k = 0; k < 3; ++k) l += n[k] * n[k];
    for (int k = 0; k < 3; ++k) n[k] /= (l > 0.f ? __builtin_sqrtf(l) : 1.f);
    for (int t = 0; t < 2; ++t, ++f) {
        for (int v = 0; v < 3; ++v)
            for (int k = 0; k < 3; ++k) {
                pos[9 * f + 3 * v + k] = q[tri[t][v]][k];
                nor[9 * f + 3 * v + k] = n[k];
            }
        mid[f] = m;
    }
    return f;
}

int main(void) {
    const float walls[6][4][3] = {
        {{-1, -1, -1}, {1, -1, -1}, {1, -1, 1}, {-1, -1, 1}},     /* floor   (inward normal +y) */
        {{-1, 1, -1}, {-1, 1, 1}, {1, 1, 1}, {1, 1, -1}},         /* ceiling */
        {{-1, -1, -1}, {-1, 1, -1}, {1, 1, -1}, {1, -1, -1}},     /* back */
        {{-1, -1, -1}, {-1, -1, 1}, {-1, 1, 1}, {-1, 1, -1}},     /* left */
        {{1, -1, -1}, {1, 1, -1}, {1, 1, 1}, {1, -1, 1}},         /* right */
        {{-.25f, .99f, -.25f}, {-.25f, .99f, .25f}, {.25f, .99f, .25f}, {.25f, .99f, -.25f}}, /* light */
    };
    const unsigned wall_mat[6] = {0, 0, 0, 1, 2, 3};
    float pos[12 * 9], nor[12 * 9];
    unsigned mid[12];
    int f = 0;
    for (int w = 0; w < 6; ++w) f = quad(pos, nor, mid, f, walls[w], wall_mat[w]);
    crt_material mats[4];
    memset(mats, 0, sizeof(mats));
    const float kd[3][3] = {{.725f, .71f, .68f}, {.63f, .065f, .05f}, {.14f, .45f, .09f}};
    for (int m = 0; m < 3; ++m) {
        mats[m].bsdf = CRT_BSDF_DIFFUSE;
        mats[m].texture = CRT_NO_TEXTURE;
        memcpy(mats[m].kd, kd[m], sizeof(kd[m]));
        mats[m].ni = 1.f;
        mats[m].diffuse = 1.f;
    }
    mats[3].bsdf = CRT_BSDF_EMISSIVE;
    mats[3].texture = CRT_NO_TEXTURE;
    mats[3].ka[0] = 17.f / 3.f;
    mats[3].ka[1] = 12.f / 3.f;
    mats[3].ka[2] = 4.f / 3.f;

    crt_scene_desc d;
    memset(&d, 0, sizeof(d));
    d.num_triangles = (uint32_t)f;
    d.positions = pos;
    d.normals = nor;
    d.material_ids = mid;
    d.num_materials = 4;
    d.materials = mats;
    crt_scene scene;
    CHECK(crt_scene_create(&d, &scene));

    const float eye[3] = {0.f, 0.f, 3.9f}, dir[3] = {0.f, 0.f, -1.f}, up[3] = {0.f, 1.f, 0.f};
    const uint32_t W = 64, H = 48, SPP = 8;
    crt_camera cam;
    CHECK(crt_camera_from_json(40.f, 0.f, 1.f, eye, dir, up, W, H, &cam));

    unsigned long sums[2] = {0, 0};
    float* acc[2];
    for (int mode = 0; mode < 2; ++mode) {
        crt_render_options o;
        crt_render_options_default(&o);
        o.mode = mode ? CRT_MODE_WAVEFRONT : CRT_MODE_MEGAKERNEL;
        o.max_depth = 5;
        crt_render r;
        CHECK(crt_render_create(scene, &cam, W, H, &o, &r));
        CHECK(crt_render_pass(r, SPP));
        uint8_t* img = (uint8_t*)malloc((size_t)W * H * 4);
        acc[mode] = (float*)malloc((size_t)W * H * 12);
        CHECK(crt_render_resolve(r, img));
        CHECK(crt_render_accum(r, acc[mode]));
        for (size_t i = 0; i < (size_t)W * H * 4; ++i) sums[mode] += img[i];
        free(img);
        CHECK(crt_render_destroy(r));
    }
    const int same = memcmp(acc[0], acc[1], (size_t)W * H * 12) == 0;
    printf("megakernel %lu wavefront %lu identical %d\n", sums[0], sums[1], same);
    free(acc[0]);
    free(acc[1]);
    CHECK(crt_scene_destroy(scene));
    return same ? 0 : 2;
}
