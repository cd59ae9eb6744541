// scene.cu -- scene construction, upload and the library's error handling.
//
// Replaces the reference's scene preparation (src/geometry/scene.cpp:74-165)
// and the ParallelRenderer uploads (src/renderer/parallel_renderer.cu:37-279):
// triangles become 48-byte intersection records in BVH leaf order plus
// per-face shading records, materials a small float4 table, and the BVH an
// 8-wide quantised tree (bvh8.cpp) instead of two 1-D textures.
#include "crt_internal.h"

#include <chrono>
#include <cmath>
#include <cstring>

namespace crt {

// stbi_loadf's 8-bit to float table (defined with the PNG reader).
const float* stb_texel_table();

namespace {
thread_local std::string g_last_error;
}

int set_error(int status, const std::string& msg) {
    g_last_error = msg;
    return status;
}

int cuda_error(cudaError_t e, const char* what) {
    return set_error(CRT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

namespace {

template <typename T>
int upload(DevBuf& b, const std::vector<T>& v) {
    size_t bytes = v.size() * sizeof(T);
    cudaError_t e = b.alloc(bytes ? bytes : 16);
    if (e != cudaSuccess) return cuda_error(e, "cudaMalloc");
    if (bytes) {
        e = cudaMemcpy(b.p, v.data(), bytes, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_error(e, "cudaMemcpy");
    }
    return CRT_OK;
}

// Uploads a built BVH (both node encodings while child indices fit 24 bits)
// and points the device view and the statistics at it.  The buffers it
// replaces are freed on return: callers make sure no work still reads them.
static int install_bvh(crt_scene s, Bvh8& b, uint32_t width) {
    DevBuf nodes, fnodes, tris;
    int st = CRT_OK;
    if (b.fnodes_ok && (st = upload(fnodes, b.fnodes))) return st;
    if ((st = upload(nodes, b.nodes)) || (st = upload(tris, b.tris))) return st;
    s->nodes.swap(nodes);
    s->fnodes.swap(fnodes);
    s->tris.swap(tris);
    s->bvh = std::move(b);
    s->dev.nodes = s->nodes.as<float4>();
    s->dev.fnodes = s->bvh.fnodes_ok ? s->fnodes.as<float4>() : nullptr;
    s->dev.tris = s->tris.as<float4>();
    crt_scene_info& I = s->info;
    I.num_nodes = (uint32_t)s->bvh.nodes.size();
    I.max_depth = s->bvh.max_depth;
    I.node_bytes = s->default_f32 ? s->bvh.fnodes.size() * sizeof(Bvh8FloatNode)
                                  : s->bvh.nodes.size() * sizeof(Bvh8Node);
    I.triangle_bytes = s->bvh.tris.size() * sizeof(TriRecord);
    I.bvh_width = width;
    ++s->generation;
    return CRT_OK;
}

// The GPU build leaves the BVH on the device only; export and rebuilds copy
// it back on demand.
static int ensure_host_bvh(crt_scene s) {
    if (s->host_bvh) return CRT_OK;
    Bvh8& b = s->bvh;
    b.nodes.resize(s->info.num_nodes);
    b.tris.resize(s->info.num_triangles);
    b.fnodes.resize(b.fnodes_ok ? s->info.num_nodes : 0);
    CRT_CUDA(cudaMemcpy(b.nodes.data(), s->nodes.p, b.nodes.size() * sizeof(Bvh8Node), cudaMemcpyDeviceToHost));
    CRT_CUDA(cudaMemcpy(b.tris.data(), s->tris.p, b.tris.size() * sizeof(TriRecord), cudaMemcpyDeviceToHost));
    if (b.fnodes_ok)
        CRT_CUDA(cudaMemcpy(b.fnodes.data(), s->fnodes.p, b.fnodes.size() * sizeof(Bvh8FloatNode),
                            cudaMemcpyDeviceToHost));
    s->host_bvh = true;
    return CRT_OK;
}

// Builds the BVH of device arrays v1/e1/e2 ([n][3]) on the GPU and installs it.
static int build_on_device(crt_scene s, const float* dv1, const float* de1, const float* de2, uint32_t n,
                           uint32_t width) {
    DevBuf nodes, fnodes, tris;
    uint32_t nn = 0, depth = 0;
    bool fok = false;
    if (int st = build_bvh_gpu(dv1, de1, de2, n, (uint32_t)kMaxLevels, (int)width, nodes, fnodes, tris, &nn, &depth,
                               &fok, nullptr))
        return st;
    if (s->default_f32 && !fok)
        return set_error(CRT_ERR_LIMIT, "FP32 nodes hold 24-bit child indices; scene has more than 2^24 nodes");
    CRT_CUDA(cudaDeviceSynchronize());
    s->nodes.swap(nodes);
    s->fnodes.swap(fnodes);
    s->tris.swap(tris);
    s->bvh = Bvh8{};
    s->bvh.fnodes_ok = fok;
    s->bvh.max_depth = depth;
    s->host_bvh = false;
    s->dev.nodes = s->nodes.as<float4>();
    s->dev.fnodes = fok ? s->fnodes.as<float4>() : nullptr;
    s->dev.tris = s->tris.as<float4>();
    crt_scene_info& I = s->info;
    I.num_nodes = nn;
    I.max_depth = depth;
    I.node_bytes = (size_t)nn * (s->default_f32 ? sizeof(Bvh8FloatNode) : sizeof(Bvh8Node));
    I.triangle_bytes = (size_t)n * sizeof(TriRecord);
    I.bvh_width = width;
    ++s->generation;
    return CRT_OK;
}

// Builds the BVH of host arrays v1/e1/e2 ([n][3]) with the scene's builder and installs it.
static int build_and_install(crt_scene s, const std::vector<float>& v1, const std::vector<float>& e1,
                             const std::vector<float>& e2, uint32_t n, uint32_t width) {
    if (s->builder == CRT_BVH_GPU) {
        DevBuf dv1, de1, de2;
        int st = CRT_OK;
        if ((st = upload(dv1, v1)) || (st = upload(de1, e1)) || (st = upload(de2, e2))) return st;
        return build_on_device(s, dv1.as<float>(), de1.as<float>(), de2.as<float>(), n, width);
    }
    Bvh8 bvh;
    const char* msg = nullptr;
    if (!build_bvh8(v1.data(), e1.data(), e2.data(), n, (uint32_t)kMaxLevels, bvh, &msg, (int)width))
        return set_error(CRT_ERR_LIMIT, msg ? msg : "BVH build failed");
    if (s->default_f32 && !bvh.fnodes_ok)
        return set_error(CRT_ERR_LIMIT, "FP32 nodes hold 24-bit child indices; scene has more than 2^24 nodes");
    s->host_bvh = true;
    return install_bvh(s, bvh, width);
}

inline float4 f4(float x, float y, float z, float w) { return make_float4(x, y, z, w); }
inline float bits(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
inline float bits(int32_t i) { float f; std::memcpy(&f, &i, 4); return f; }

// Per-face records on the device, in the operation order of
// Scene::loadTriangles (scene.cpp:111-130): v1, e1 = v2 - v1, e2 = v3 - v1
// (or the edges as given), area = |e1 x e2| / 2; shading records (three
// normals, area, material id) and uvs.
// A face with a non-finite coordinate sets *bad (the builds bin by centroid
// and must not see NaN or infinity).
__global__ void k_pack_faces(const float* __restrict__ pos, const float* __restrict__ nor,
                             const float* __restrict__ uv, const uint32_t* __restrict__ mid, uint32_t n, bool edges,
                             float* __restrict__ v1, float* __restrict__ e1, float* __restrict__ e2,
                             float4* __restrict__ shade, float4* __restrict__ uvs, uint32_t* bad) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float* p = pos + 9ull * i;
        float a[3], b[3];
        bool finite = true;
        for (int k = 0; k < 3; ++k) {
            a[k] = edges ? p[3 + k] : p[3 + k] - p[k];
            b[k] = edges ? p[6 + k] : p[6 + k] - p[k];
            finite = finite && isfinite(p[k]) && isfinite(p[k] + a[k]) && isfinite(p[k] + b[k]) &&
                     isfinite(a[k]) && isfinite(b[k]);
            v1[3ull * i + k] = p[k];
            e1[3ull * i + k] = a[k];
            e2[3ull * i + k] = b[k];
        }
        if (!finite) atomicMin(bad, i);
        const float cx = a[1] * b[2] - a[2] * b[1], cy = a[2] * b[0] - a[0] * b[2], cz = a[0] * b[1] - a[1] * b[0];
        const float area = sqrtf(cx * cx + cy * cy + cz * cz) / 2.0f;
        const float* nn = nor + 9ull * i;
        shade[3ull * i + 0] = make_float4(nn[0], nn[1], nn[2], nn[3]);
        shade[3ull * i + 1] = make_float4(nn[4], nn[5], nn[6], nn[7]);
        shade[3ull * i + 2] = make_float4(nn[8], area, __uint_as_float(mid[i]), 0.f);
        if (uv) {
            const float* t = uv + 6ull * i;
            uvs[2ull * i + 0] = make_float4(t[0], t[1], t[2], t[3]);
            uvs[2ull * i + 1] = make_float4(t[4], t[5], 0.f, 0.f);
        } else {
            uvs[2ull * i + 0] = uvs[2ull * i + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
}

// Texels to float4: linear floats as given, or RGBA8 through the 8-bit to
// float table stbi_loadf applies; alpha dropped.
__global__ void k_pack_texels(const float* __restrict__ rgb, const uchar4* __restrict__ rgba8,
                              const float* __restrict__ table, uint64_t total, float4* __restrict__ out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
        if (rgba8) {
            const uchar4 c = rgba8[i];
            out[i] = make_float4(table[c.x], table[c.y], table[c.z], 0.f);
        } else {
            out[i] = make_float4(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2], 0.f);
        }
    }
}

// Face area on the host, in k_pack_faces' operation order.
static float face_area(const crt_scene_desc* d, uint32_t f, float e1[3], float e2[3]) {
    const bool edges = (d->flags & CRT_SCENE_EDGES) != 0;
    const float* p = d->positions + 9ull * f;
    for (int k = 0; k < 3; ++k) {
        e1[k] = edges ? p[3 + k] : p[3 + k] - p[k];
        e2[k] = edges ? p[6 + k] : p[6 + k] - p[k];
    }
    const float cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2],
                cz = e1[0] * e2[1] - e1[1] * e2[0];
    return sqrtf(cx * cx + cy * cy + cz * cz) / 2.0f;
}

template <typename T>
static int upload_raw(DevBuf& b, const T* p, size_t count) {
    cudaError_t e = b.alloc(count ? count * sizeof(T) : 16);
    if (e != cudaSuccess) return cuda_error(e, "cudaMalloc");
    if (count) {
        e = cudaMemcpy(b.p, p, count * sizeof(T), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_error(e, "cudaMemcpy");
    }
    return CRT_OK;
}

// Materials (createMaterialsData, parallel_renderer.cu:252-279) with the
// emission scaling ka = Ka * 3 * lightsArea (scene.cpp:163,177).
static std::vector<float4> pack_materials(const crt_material* ms, uint32_t n, float lights_area,
                                          bool ka_scaled) {
    std::vector<float4> mats(4ull * n);
    for (uint32_t m = 0; m < n; ++m) {
        const crt_material& M = ms[m];
        float ka[3];
        for (int k = 0; k < 3; ++k) ka[k] = ka_scaled ? M.ka[k] : (M.ka[k] * 3.0f) * lights_area;
        mats[4 * m + 0] = f4(M.kd[0], M.kd[1], M.kd[2], bits((int32_t)M.texture));
        mats[4 * m + 1] = f4(ka[0], ka[1], ka[2], bits((int32_t)M.bsdf));
        mats[4 * m + 2] = f4(M.ks[0], M.ks[1], M.ks[2], M.ns);
        mats[4 * m + 3] = f4(M.ni, M.diffuse, 0.f, 0.f);
    }
    return mats;
}

}  // namespace
}  // namespace crt

using namespace crt;

extern "C" {

int crt_api_version(void) { return CRT_API_VERSION; }

const char* crt_last_error(void) { return g_last_error.c_str(); }

int crt_camera_from_json(float fov_deg, float focal_length, float fstop, const float eye[3],
                         const float view_dir[3], const float up[3], uint32_t width,
                         uint32_t height, crt_camera* out) {
    // CameraJsonLoader::getCamera (src/context/json_loader.cpp:26-48), in FP32
    // with the same double-precision degree conversion.
    if (!eye || !view_dir || !up || !out || width == 0 || height == 0)
        return set_error(CRT_ERR_INVALID, "crt_camera_from_json: bad argument");
    auto norm = [](const float* v, float* o) {
        float n = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        o[0] = v[0] / n; o[1] = v[1] / n; o[2] = v[2] / n;
    };
    out->xpixels = (int32_t)width;
    out->ypixels = (int32_t)height;
    out->fov = tanf((float)((double)(fov_deg * 0.5f) * 3.14159265358979323846 / 180.0));
    for (int k = 0; k < 3; ++k) out->eye[k] = eye[k];
    out->focus = sqrtf(view_dir[0] * view_dir[0] + view_dir[1] * view_dir[1] + view_dir[2] * view_dir[2]);
    norm(view_dir, out->dir);
    norm(up, out->up);
    float r[3] = {out->dir[1] * out->up[2] - out->dir[2] * out->up[1],
                  out->dir[2] * out->up[0] - out->dir[0] * out->up[2],
                  out->dir[0] * out->up[1] - out->dir[1] * out->up[0]};
    norm(r, out->right);
    out->aperture = focal_length / fstop;
    out->aspect = (float)width / (float)height;
    return CRT_OK;
}

int crt_scene_create(const crt_scene_desc* d, crt_scene* out) {
    if (!d || !out) return set_error(CRT_ERR_INVALID, "crt_scene_create: null argument");
    *out = nullptr;
    const uint32_t n = d->num_triangles;
    if (n == 0 || !d->positions || !d->normals || !d->material_ids)
        return set_error(CRT_ERR_INVALID, "scene needs triangles, normals and material ids");
    if (d->num_materials == 0 || !d->materials)
        return set_error(CRT_ERR_INVALID, "scene has no materials");
    if (n >= (1u << 31)) return set_error(CRT_ERR_LIMIT, "more than 2^31 triangles");
    for (uint32_t i = 0; i < n; ++i)
        if (d->material_ids[i] >= d->num_materials)
            return set_error(CRT_ERR_INVALID, "material id out of range at face " + std::to_string(i));
    for (uint32_t m = 0; m < d->num_materials; ++m) {
        int t = d->materials[m].texture;
        if (t != CRT_NO_TEXTURE && (t < 0 || (uint32_t)t >= d->num_textures))
            return set_error(CRT_ERR_INVALID, "texture index out of range in material " + std::to_string(m));
        if (d->materials[m].bsdf < 0 || d->materials[m].bsdf > CRT_BSDF_EMISSIVE)
            return set_error(CRT_ERR_INVALID, "unknown bsdf in material " + std::to_string(m));
    }
    if (d->num_textures && (!d->texture_dims || (!d->texels && !d->texels_rgba8)))
        return set_error(CRT_ERR_INVALID, "textures need dims and texels");
    if (d->node_format > CRT_NODES_F32) return set_error(CRT_ERR_INVALID, "unknown node format");
    if (d->flags & ~(uint32_t)(CRT_SCENE_EDGES | CRT_SCENE_KA_SCALED))
        return set_error(CRT_ERR_INVALID, "unknown scene flag");
    if (d->builder > CRT_BVH_GPU) return set_error(CRT_ERR_INVALID, "unknown BVH builder");
    if (d->bvh_width != 0 && d->bvh_width != 4 && d->bvh_width != 8)
        return set_error(CRT_ERR_INVALID, "bvh_width must be 4 or 8");

    auto t0 = std::chrono::steady_clock::now();
    crt_scene s = new crt_scene_s();

    // Light list (scene.cpp:148-160) and total light area (scene.cpp:167-173),
    // with each light's geometry as Scene::loadTriangles computes it.
    if (d->num_lights) {
        if (!d->light_indices) { delete s; return set_error(CRT_ERR_INVALID, "light_indices is null"); }
        for (uint32_t i = 0; i < d->num_lights; ++i) {
            if (d->light_indices[i] >= n) { delete s; return set_error(CRT_ERR_INVALID, "light index out of range"); }
            s->lights.push_back(d->light_indices[i]);
        }
    } else {
        for (uint32_t i = 0; i < n; ++i)
            if (d->materials[d->material_ids[i]].bsdf == CRT_BSDF_EMISSIVE) s->lights.push_back(i);
    }
    if (s->lights.empty()) {
        delete s;
        return set_error(CRT_ERR_INVALID, "scene has no emissive triangles (light sampling needs one)");
    }
    std::vector<float4> lgeo(3 * s->lights.size());
    float lights_area = 0;
    for (size_t i = 0; i < s->lights.size(); ++i) {
        const uint32_t f = s->lights[i];
        float e1[3], e2[3];
        const float area = face_area(d, f, e1, e2);
        const float* p = d->positions + 9ull * f;
        lgeo[3 * i + 0] = f4(p[0], p[1], p[2], bits(f));
        lgeo[3 * i + 1] = f4(e1[0], e1[1], e1[2], area);
        lgeo[3 * i + 2] = f4(e2[0], e2[1], e2[2], bits(d->material_ids[f]));
        lights_area += area;
    }
    // Textures flattened in order, then as many zero texels as the last
    // texture is wide (texture_store.cpp:68-70).
    std::vector<uint2> dims;
    std::vector<uint32_t> offs;
    uint64_t total = 0;
    for (uint32_t t = 0; t < d->num_textures; ++t) {
        uint32_t w = d->texture_dims[2 * t], h = d->texture_dims[2 * t + 1];
        if (w == 0 || h == 0) { delete s; return set_error(CRT_ERR_INVALID, "empty texture"); }
        dims.push_back(make_uint2(w, h));
        offs.push_back((uint32_t)total);
        total += (uint64_t)w * h;
        if (total >= (1ull << 31)) { delete s; return set_error(CRT_ERR_LIMIT, "texture data too large"); }
    }
    const uint64_t pad = d->num_textures ? dims.back().x : 0;
    // Host-side validation is complete; from here on a device is needed.
    cudaError_t dev_err = cudaGetDevice(&s->device);
    if (dev_err != cudaSuccess) { delete s; return cuda_error(dev_err, "cudaGetDevice"); }

    const uint32_t width = d->bvh_width ? d->bvh_width : 8u;
    s->builder = d->builder;
    const bool f32 = d->node_format == CRT_NODES_F32;
    // Both encodings go to the device (the FP32 one only while child indices
    // fit 24 bits); each render picks one.
    s->default_f32 = f32;
    s->n_mats = d->num_materials;
    s->ka_scaled = (d->flags & CRT_SCENE_KA_SCALED) != 0;

    // The caller's arrays go up as they are; one kernel forms the triangle,
    // shading and uv records there.
    int st = CRT_OK;
    {
        DevBuf dpos, dnor, duv, dmid, dv1, de1, de2;
        if ((st = upload_raw(dpos, d->positions, 9ull * n)) || (st = upload_raw(dnor, d->normals, 9ull * n)) ||
            (d->uvs && (st = upload_raw(duv, d->uvs, 6ull * n))) || (st = upload_raw(dmid, d->material_ids, n))) {
            delete s;
            return st;
        }
        DevBuf dbad;
        cudaError_t e = dbad.alloc(4);
        if (e == cudaSuccess) e = cudaMemset(dbad.p, 0xFF, 4);   // lowest bad face, or UINT32_MAX
        if (e == cudaSuccess) e = dv1.alloc(12ull * n);
        if (e == cudaSuccess) e = de1.alloc(12ull * n);
        if (e == cudaSuccess) e = de2.alloc(12ull * n);
        if (e == cudaSuccess) e = s->shade.alloc(48ull * n);
        if (e == cudaSuccess) e = s->uvs.alloc(32ull * n);
        if (e != cudaSuccess) { delete s; return cuda_error(e, "cudaMalloc"); }
        const uint32_t grid = (uint32_t)std::min<uint64_t>((n + 255) / 256, 4096);
        k_pack_faces<<<grid, 256>>>(dpos.as<float>(), dnor.as<float>(), d->uvs ? duv.as<float>() : nullptr,
                                    dmid.as<uint32_t>(), n, (d->flags & CRT_SCENE_EDGES) != 0, dv1.as<float>(),
                                    de1.as<float>(), de2.as<float>(), s->shade.as<float4>(), s->uvs.as<float4>(),
                                    dbad.as<uint32_t>());
        e = cudaGetLastError();
        uint32_t bad_face = UINT32_MAX;
        if (e == cudaSuccess) e = cudaMemcpy(&bad_face, dbad.p, 4, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) { delete s; return cuda_error(e, "k_pack_faces"); }
        if (bad_face != UINT32_MAX) {
            delete s;
            return set_error(CRT_ERR_INVALID, "non-finite vertex coordinate in face " + std::to_string(bad_face));
        }
        if (s->builder == CRT_BVH_GPU) {
            st = build_on_device(s, dv1.as<float>(), de1.as<float>(), de2.as<float>(), n, width);
        } else {
            std::vector<float> v1(3ull * n), e1(3ull * n), e2(3ull * n);
            e = cudaMemcpy(v1.data(), dv1.p, 12ull * n, cudaMemcpyDeviceToHost);
            if (e == cudaSuccess) e = cudaMemcpy(e1.data(), de1.p, 12ull * n, cudaMemcpyDeviceToHost);
            if (e == cudaSuccess) e = cudaMemcpy(e2.data(), de2.p, 12ull * n, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) { delete s; return cuda_error(e, "cudaMemcpy"); }
            st = build_and_install(s, v1, e1, e2, n, width);
        }
        if (st != CRT_OK) { delete s; return st; }
    }
    {   // texels: floats or RGBA8 bytes up, float4 records formed on the device
        DevBuf raw, table;
        cudaError_t e = s->texels.alloc(16ull * (total + pad) + (total + pad == 0 ? 16 : 0));
        if (e == cudaSuccess && pad) e = cudaMemset(s->texels.as<float4>() + total, 0, 16ull * pad);
        if (e != cudaSuccess) { delete s; return cuda_error(e, "texels"); }
        if (total) {
            if (d->texels_rgba8) {
                if ((st = upload_raw(raw, d->texels_rgba8, 4ull * total)) ||
                    (st = upload_raw(table, stb_texel_table(), 256))) {
                    delete s;
                    return st;
                }
            } else if ((st = upload_raw(raw, d->texels, 3ull * total))) {
                delete s;
                return st;
            }
            const uint32_t grid = (uint32_t)std::min<uint64_t>((total + 255) / 256, 4096);
            k_pack_texels<<<grid, 256>>>(d->texels_rgba8 ? nullptr : raw.as<float>(),
                                         d->texels_rgba8 ? raw.as<uchar4>() : nullptr, table.as<float>(), total,
                                         s->texels.as<float4>());
            e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaDeviceSynchronize();
            if (e != cudaSuccess) { delete s; return cuda_error(e, "k_pack_texels"); }
        }
    }
    const std::vector<float4> mats =
        pack_materials(d->materials, d->num_materials, lights_area, (d->flags & CRT_SCENE_KA_SCALED) != 0);
    if ((st = upload(s->mats, mats)) || (st = upload(s->light_geo, lgeo)) || (st = upload(s->tex_dims, dims)) ||
        (st = upload(s->tex_offsets, offs))) {
        delete s;
        return st;
    }
    cudaError_t e = s->error.alloc(16);
    if (e == cudaSuccess) e = cudaMemset(s->error.p, 0, 16);
    if (e != cudaSuccess) { delete s; return cuda_error(e, "error word"); }

    DevScene& D = s->dev;
    D.shade = s->shade.as<float4>();
    D.uvs = s->uvs.as<float4>();
    D.mats = s->mats.as<float4>();
    D.light_geo = s->light_geo.as<float4>();
    D.texels = s->texels.as<float4>();
    D.tex_dims = s->tex_dims.as<uint2>();
    D.tex_offsets = s->tex_offsets.as<uint32_t>();
    D.tex_total = (uint32_t)(total + pad);
    D.n_lights = (uint32_t)s->lights.size();
    D.lights_area = lights_area;
    D.n_faces = n;
    D.max_visits = kMaxNodeVisits;
    D.error = s->error.as<uint32_t>();

    crt_scene_info& I = s->info;
    I.num_triangles = n;
    I.num_lights = D.n_lights;
    I.num_materials = d->num_materials;
    I.num_textures = d->num_textures;
    I.shading_bytes = 80ull * n;   // 3 + 2 float4 per face
    I.texture_bytes = 16ull * (total + pad);
    I.lights_area = lights_area;
    I.build_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    *out = s;
    return CRT_OK;
}

int crt_scene_destroy(crt_scene s) {
    delete s;
    return CRT_OK;
}

int crt_scene_set_visit_limit(crt_scene s, uint32_t max_visits) {
    if (!s) return set_error(CRT_ERR_INVALID, "crt_scene_set_visit_limit: null scene");
    CRT_CUDA(cudaDeviceSynchronize());   // passes already queued keep their limit
    if (max_visits > kVisitCeiling) return set_error(CRT_ERR_LIMIT, "crt_scene_set_visit_limit: at most 2^30 visits");
    s->dev.max_visits = max_visits ? max_visits : kMaxNodeVisits;
    ++s->generation;   // render handles re-capture their wave graphs with it
    return CRT_OK;
}

int crt_scene_clear_errors(crt_scene s) {
    if (!s) return set_error(CRT_ERR_INVALID, "crt_scene_clear_errors: null scene");
    CRT_CUDA(cudaDeviceSynchronize());
    CRT_CUDA(cudaMemset(s->error.p, 0, 16));
    return CRT_OK;
}

static_assert(ERR_WATCHDOG == CRT_SCENE_ERR_WATCHDOG && ERR_STACK == CRT_SCENE_ERR_STACK,
              "device error bits and their public names");

int crt_scene_errors(crt_scene s, void* stream, uint32_t* bits) {
    if (!s || !bits) return set_error(CRT_ERR_INVALID, "crt_scene_errors: null argument");
    uint32_t w = 0;
    CRT_CUDA(cudaMemcpyAsync(&w, s->error.p, 4, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    CRT_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    *bits = w & (CRT_SCENE_ERR_WATCHDOG | CRT_SCENE_ERR_STACK);
    return CRT_OK;
}

int crt_scene_set_materials(crt_scene s, const crt_material* materials, uint32_t n) {
    if (!s || !materials) return set_error(CRT_ERR_INVALID, "crt_scene_set_materials: null argument");
    if (n != s->n_mats) return set_error(CRT_ERR_INVALID, "crt_scene_set_materials: material count differs");
    for (uint32_t m = 0; m < n; ++m) {
        const int t = materials[m].texture;
        if (t != CRT_NO_TEXTURE && (t < 0 || (uint32_t)t >= s->info.num_textures))
            return set_error(CRT_ERR_INVALID, "texture index out of range in material " + std::to_string(m));
        if (materials[m].bsdf < 0 || materials[m].bsdf > CRT_BSDF_EMISSIVE)
            return set_error(CRT_ERR_INVALID, "unknown bsdf in material " + std::to_string(m));
    }
    const std::vector<float4> mats = pack_materials(materials, n, s->info.lights_area, s->ka_scaled);
    CRT_CUDA(cudaSetDevice(s->device));
    CRT_CUDA(cudaDeviceSynchronize());   // no queued pass may read a half-written table
    CRT_CUDA(cudaMemcpy(s->mats.p, mats.data(), mats.size() * sizeof(float4), cudaMemcpyHostToDevice));
    return CRT_OK;
}

int crt_scene_set_bvh_width(crt_scene s, uint32_t width) {
    if (!s) return set_error(CRT_ERR_INVALID, "crt_scene_set_bvh_width: null scene");
    if (width != 4 && width != 8) return set_error(CRT_ERR_INVALID, "bvh_width must be 4 or 8");
    if (width == s->info.bvh_width) return CRT_OK;
    const auto t0 = std::chrono::steady_clock::now();
    CRT_CUDA(cudaSetDevice(s->device));
    if (int st = ensure_host_bvh(s)) return st;
    // the triangle records hold each face's v1, e1, e2 exactly as built
    const uint32_t n = s->info.num_triangles;
    std::vector<float> v1(3ull * n), e1(3ull * n), e2(3ull * n);
    for (const TriRecord& r : s->bvh.tris) {
        const uint32_t f = r.face;
        for (int k = 0; k < 3; ++k) {
            v1[3ull * f + k] = r.v1[k];
            e1[3ull * f + k] = r.e1[k];
            e2[3ull * f + k] = r.e2[k];
        }
    }
    CRT_CUDA(cudaDeviceSynchronize());   // nothing may still read the old nodes
    int st = build_and_install(s, v1, e1, e2, n, width);
    if (st != CRT_OK) return st;
    s->info.build_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return CRT_OK;
}

int crt_scene_get_info(crt_scene s, crt_scene_info* out) {
    if (!s || !out) return set_error(CRT_ERR_INVALID, "crt_scene_get_info: null argument");
    *out = s->info;
    return CRT_OK;
}

int crt_scene_export_bvh(crt_scene s, void* nodes, void* triangles) {
    if (!s) return set_error(CRT_ERR_INVALID, "crt_scene_export_bvh: null scene");
    CRT_CUDA(cudaSetDevice(s->device));
    if (int st = ensure_host_bvh(s)) return st;
    if (nodes) std::memcpy(nodes, s->bvh.nodes.data(), s->bvh.nodes.size() * sizeof(Bvh8Node));
    if (triangles) std::memcpy(triangles, s->bvh.tris.data(), s->bvh.tris.size() * sizeof(TriRecord));
    return CRT_OK;
}

int crt_bvh_build_host(const float* positions, uint32_t n, uint32_t bvh_width, uint32_t* num_nodes,
                       uint32_t* max_depth, void* nodes, void* triangles) {
    if (!positions || n == 0) return set_error(CRT_ERR_INVALID, "crt_bvh_build_host: no triangles");
    if (bvh_width != 0 && bvh_width != 4 && bvh_width != 8)
        return set_error(CRT_ERR_INVALID, "bvh_width must be 4 or 8");
    std::vector<float> v1(3ull * n), e1(3ull * n), e2(3ull * n);
    for (uint32_t i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) {
            const float* p = positions + 9ull * i;
            v1[3 * i + k] = p[k];
            e1[3 * i + k] = p[3 + k] - p[k];
            e2[3 * i + k] = p[6 + k] - p[k];
        }
    Bvh8 b;
    const char* msg = nullptr;
    if (!build_bvh8(v1.data(), e1.data(), e2.data(), n, (uint32_t)kMaxLevels, b, &msg,
                    bvh_width ? (int)bvh_width : 8))
        return set_error(CRT_ERR_LIMIT, msg ? msg : "BVH build failed");
    if (num_nodes) *num_nodes = (uint32_t)b.nodes.size();
    if (max_depth) *max_depth = b.max_depth;
    if (nodes) std::memcpy(nodes, b.nodes.data(), b.nodes.size() * sizeof(Bvh8Node));
    if (triangles) std::memcpy(triangles, b.tris.data(), b.tris.size() * sizeof(TriRecord));
    return CRT_OK;
}

}  // extern "C"
