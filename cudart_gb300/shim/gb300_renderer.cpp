// gb300_renderer.cpp -- see gb300_renderer.h.  Errors from the library are
// thrown as std::runtime_error with crt_last_error()'s message; the reference
// itself prints and exits (cuda_error_check.h:9-21), which the shim leaves to
// its caller.
#include "gb300_renderer.h"

#include <cuda_runtime.h>

#include <stdexcept>
#include <string>
#include <vector>

namespace {

void check(int status, const char* what) {
    if (status != CRT_OK) throw std::runtime_error(std::string(what) + ": " + crt_last_error());
}

void put3(float* dst, const float3& v) {
    dst[0] = v.x;
    dst[1] = v.y;
    dst[2] = v.z;
}

}  // namespace

Gb300Renderer::Gb300Renderer(Scene* scene, pixels_t w, pixels_t h, uint spp, bool progressive_)
    : Renderer(scene, w, h, spp), progressive(progressive_) {
    const uint n = (uint)scene->getNumTriangles();
    const Triangle* tris = scene->getTriPtr();
    // per-face arrays in the Scene's (BVH) order, with the exact v1/e1/e2 the
    // reference intersects against
    std::vector<float> pos(9ull * n), nor(9ull * n), uv(6ull * n);
    std::vector<uint32_t> mat(n);
    for (uint i = 0; i < n; ++i) {
        const Triangle& t = tris[i];
        put3(&pos[9ull * i], t._v1);
        put3(&pos[9ull * i + 3], t._e1);
        put3(&pos[9ull * i + 6], t._e2);
        put3(&nor[9ull * i], t._n1);
        put3(&nor[9ull * i + 3], t._n2);
        put3(&nor[9ull * i + 6], t._n3);
        const float2 u[3] = {t._uv1, t._uv2, t._uv3};
        for (int k = 0; k < 3; ++k) {
            uv[6ull * i + 2 * k] = u[k].x;
            uv[6ull * i + 2 * k + 1] = u[k].y;
        }
        mat[i] = t._materialId;
    }
    // the deduplicated material table; ka already holds Ka * 3 * lights area
    const uint nm = scene->getNumMaterials();
    const Material* ms = scene->getMaterialsPtr();
    std::vector<crt_material> mats(nm);
    for (uint m = 0; m < nm; ++m) {
        crt_material& c = mats[m];
        c.bsdf = (int32_t)ms[m].bsdf;
        c.texture = ms[m].texKdIdx;
        put3(c.kd, ms[m].kd);
        put3(c.ka, ms[m].ka);
        put3(c.ks, ms[m].ks);
        c.ns = ms[m].ns;
        c.ni = ms[m].ni;
        c.diffuse = ms[m].diffuseCoefficient;
    }
    const uint nt = scene->getNumTextures();
    std::vector<uint32_t> dims(2ull * nt);
    for (uint t = 0; t < 2 * nt; ++t) dims[t] = scene->getTextureDimensionsPtr()[t];
    crt_scene_desc d = {};
    d.num_triangles = n;
    d.positions = pos.data();
    d.normals = nor.data();
    d.uvs = uv.data();
    d.material_ids = mat.data();
    d.num_materials = nm;
    d.materials = mats.data();
    d.num_lights = (uint32_t)scene->getNumLights();
    d.light_indices = scene->getLightsIndicesPtr();
    d.num_textures = nt;
    d.texture_dims = nt ? dims.data() : nullptr;
    d.texels = nt ? reinterpret_cast<const float*>(scene->getTexturePtr()) : nullptr;
    d.flags = CRT_SCENE_EDGES | CRT_SCENE_KA_SCALED;
    check(crt_scene_create(&d, &scene_handle), "crt_scene_create");

    const Camera& cam = *scene->getCameraPtr();
    crt_camera c = {};
    put3(c.eye, cam.eye);
    put3(c.dir, cam.dir);
    put3(c.up, cam.up);
    put3(c.right, cam.right);
    c.fov = cam.fov;
    c.aspect = cam.aspect;
    c.aperture = cam.apertureWidth;
    c.focus = cam.focusDistance;
    c.xpixels = cam.xpixels;
    c.ypixels = cam.ypixels;
    crt_render_options o;
    crt_render_options_default(&o);   // 6 bounces, seed 1234: the reference's values
    o.mode = CRT_MODE_WAVEFRONT;
    o.node_format = CRT_NODES_F32;    // the faster encoding on the 1080p and mixed scenes
    check(crt_render_create(scene_handle, &c, w, h, &o, &render_handle), "crt_render_create");
    // h_imgPtr comes from the Renderer constructor (renderer.cu:80-85)
    if (cudaMalloc(&d_img, sizeof(uchar4) * (size_t)w * h) != cudaSuccess)
        throw std::runtime_error("cudaMalloc of the RGBA8 image failed");
}

Gb300Renderer::~Gb300Renderer() {
    crt_render_destroy(render_handle);
    crt_scene_destroy(scene_handle);
    cudaFree(d_img);
}

void Gb300Renderer::flush() {
    if (!pending) return;
    check(crt_render_pass(render_handle, pending), "crt_render_pass");
    pending = 0;
}

void Gb300Renderer::renderOneSamplePerPixel(uchar4* p_img) {
    ++pending;
    samplesRendered = samplesRendered + 1;
    if (progressive) {
        flush();
        check(crt_render_resolve_device(render_handle, p_img), "crt_render_resolve_device");
    }
}

void Gb300Renderer::copyImageBytes(uchar4*) {
    flush();
    // quantise-then-gamma exactly like copyImageBytes + gammaCorrectPixel
    check(crt_render_resolve(render_handle, reinterpret_cast<uint8_t*>(h_imgPtr)), "crt_render_resolve");
}
