// render.cu -- progressive rendering: the plain megakernel (drop-in for the
// reference's renderKernel, src/renderer/parallel_renderer.cu:318-342), the
// output resolve, and the crt_render_* C ABI.  The wavefront form lives in
// wavefront.cu and shares the path state machine below.
#include "crt_internal.h"
#include "render_common.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace crt {

int grid_for(uint32_t n, int block, int per_sm);
int wavefront_pass(crt_render r, const std::vector<ViewWork>& work);
int wavefront_profile_pass(crt_render r, const std::vector<ViewWork>& work, crt_stage_profile* out);
int wavefront_adjoint(crt_render r, const std::vector<ViewWork>& work, const float4* adj, float* gkd, float* gka,
                      uint32_t flags);

constexpr int kMegaBlock = 128;         // 16 x 8 pixel tile, warps of 8 x 4
constexpr uint32_t kMegaSppPerLaunch = 4;

// One thread per pixel; samples [spp0, spp0 + nspp) are added to the FP32
// accumulator in sample order, so the sums equal the reference's per-pass
// accumulation (`p_imgBuffer[idx] += color`, parallel_renderer.cu:340).
template <bool F32>
// Register cap of the megakernel (the whole path lives in registers):
// measured 80 best against 64, 96 and the uncapped 128.
#ifndef CRT_MEGA_REGS
#define CRT_MEGA_REGS 80
#endif
__global__ void __maxnreg__(F32 ? CRT_MEGA_REGS + 16 : CRT_MEGA_REGS) mega_kernel(RenderParams P) {
    __shared__ uint2 stack_sh[kStackShared * kMegaBlock];
    Stack st;
    st.setup(stack_sh, kMegaBlock, kStackShared);
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t x = blockIdx.x * 16u + (warp & 1u) * 8u + (lane & 7u);
    const uint32_t y = blockIdx.y * 8u + (warp >> 1) * 4u + (lane >> 3);
    uint32_t n_ext = 0, n_shadow = 0;
    if (x < P.width && y < P.height) {
        const uint32_t pixel = y * P.width + x;
        float4 acc = P.accum[pixel];
        for (uint32_t s = 0; s < P.nspp; ++s) {
            const float3 c = sample_path<F32>(P, (int)x, (int)y, pixel, P.spp0 + s, st, n_ext, n_shadow);
            acc.x = acc.x + c.x;
            acc.y = acc.y + c.y;
            acc.z = acc.z + c.z;
        }
        P.accum[pixel] = acc;
    }
    count_rays(P.ray_counts, n_ext, n_shadow);
}

// float3ToUchar4 (renderer.h:149-156) of sum / spp, then the host-side
// gammaCorrectPixel (renderer.cu:495-504) as a 256-entry table.
__global__ void resolve_kernel(const float4* __restrict__ accum, uint32_t n, float spp,
                               const uint8_t* __restrict__ lut, uchar4* __restrict__ out) {
    __shared__ uint8_t L[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) L[i] = lut[i];
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 a = accum[i];
        const float vx = a.x / spp, vy = a.y / spp, vz = a.z / spp;
        const uint32_t qx = (uint32_t)((vx > 1.0f ? 1.0f : vx) * 255.f);
        const uint32_t qy = (uint32_t)((vy > 1.0f ? 1.0f : vy) * 255.f);
        const uint32_t qz = (uint32_t)((vz > 1.0f ? 1.0f : vz) * 255.f);
        out[i] = make_uchar4(L[qx & 255u], L[qy & 255u], L[qz & 255u], 255u);
    }
}

// renderKernel's device-side image: float3ToUchar4 of the average, no gamma.
__global__ void average_u8_kernel(const float4* __restrict__ accum, uint32_t n, float spp,
                                  uchar4* __restrict__ out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 a = accum[i];
        const float vx = a.x / spp, vy = a.y / spp, vz = a.z / spp;
        out[i] = make_uchar4((unsigned char)((vx > 1.0f ? 1.0f : vx) * 255.f),
                             (unsigned char)((vy > 1.0f ? 1.0f : vy) * 255.f),
                             (unsigned char)((vz > 1.0f ? 1.0f : vz) * 255.f), 255u);
    }
}

__global__ void unpack_accum_kernel(const float4* __restrict__ accum, uint32_t n, float* __restrict__ out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 a = accum[i];
        out[3ull * i] = a.x;
        out[3ull * i + 1] = a.y;
        out[3ull * i + 2] = a.z;
    }
}

Camera to_device_camera(const crt_camera& c) {
    Camera d;
    d.eye = make_float3(c.eye[0], c.eye[1], c.eye[2]);
    d.dir = make_float3(c.dir[0], c.dir[1], c.dir[2]);
    d.up = make_float3(c.up[0], c.up[1], c.up[2]);
    d.right = make_float3(c.right[0], c.right[1], c.right[2]);
    d.fov = c.fov;
    d.aspect = c.aspect;
    d.aperture = c.aperture;
    d.focus = c.focus;
    d.xpixels = c.xpixels;
    d.ypixels = c.ypixels;
    return d;
}

RenderParams make_params(crt_render r, uint32_t view, uint32_t spp0, uint32_t nspp) {
    const ViewState& V = r->views[view];
    RenderParams P;
    P.S = r->scene->view(uses_f32_nodes(r));
    P.cam = V.cam;
    P.accum = r->accum.as<float4>() + V.pix_off;
    P.width = V.width;
    P.height = V.height;
    P.seed = r->opts.seed;
    P.view = V.view_id;
    P.spp0 = spp0;
    P.nspp = nspp;
    P.max_depth = r->opts.max_depth;
    P.ray_counts = r->ray_counts.as<unsigned long long>();
    P.ka_scale = 3.0f * r->scene->dev.lights_area;
    return P;
}

int check_device_error(crt_render r) {
    uint32_t err = 0;
    CRT_CUDA(cudaMemcpyAsync(&err, r->scene->error.p, 4, cudaMemcpyDeviceToHost, r->stream));
    CRT_CUDA(cudaStreamSynchronize(r->stream));
    if (err & ERR_WATCHDOG) return set_error(CRT_ERR_WATCHDOG, "traversal exceeded its node-visit limit");
    if (err & ERR_STACK) return set_error(CRT_ERR_WATCHDOG, "traversal stack overflow");
    return CRT_OK;
}

// Copies the view table (cameras, sizes, accumulator offsets) to the device.
static int upload_views(crt_render r) {
    std::vector<DevView> t(r->views.size());
    for (size_t v = 0; v < t.size(); ++v) {
        const ViewState& V = r->views[v];
        t[v].cam = V.cam;
        t[v].width = V.width;
        t[v].height = V.height;
        t[v].view_id = V.view_id;
        t[v].pix_off = V.pix_off;
    }
    CRT_CUDA(cudaMemcpyAsync(r->view_table.p, t.data(), t.size() * sizeof(DevView), cudaMemcpyHostToDevice,
                             r->stream));
    CRT_CUDA(cudaStreamSynchronize(r->stream));
    return CRT_OK;
}

// A render handle over `views` (pixel offsets assigned here).
static int create_render(crt_scene s, std::vector<ViewState> views, const crt_render_options* opts,
                         crt_render* out) {
    *out = nullptr;
    crt_render_options o;
    if (opts) o = *opts;
    else crt_render_options_default(&o);
    if (int st = check_render_options(o)) return st;
    uint64_t total = 0;
    for (ViewState& V : views) {
        V.pix_off = (uint32_t)total;
        total += (uint64_t)V.width * V.height;
    }
    if (total >= (1ull << 31)) return set_error(CRT_ERR_LIMIT, "views hold 2^31 pixels or more");
    crt_render r = new crt_render_s();
    r->scene = s;
    r->views = std::move(views);
    r->opts = o;
    cudaError_t e = cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) r->own_stream = true;
    if (e == cudaSuccess) e = r->accum.alloc(total * sizeof(float4));
    if (e == cudaSuccess) e = cudaMemsetAsync(r->accum.p, 0, total * sizeof(float4), r->stream);
    if (e == cudaSuccess) e = r->ray_counts.alloc(2 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemsetAsync(r->ray_counts.p, 0, 2 * sizeof(unsigned long long), r->stream);
    if (e == cudaSuccess) e = r->view_table.alloc(r->views.size() * sizeof(DevView));
    // gammaCorrectPixel (renderer.cu:495-504) runs on the host in the
    // reference; the same powf per byte value gives the table.
    uint8_t lut[256];
    const float inv_gamma = 1.f / 2.2f;
    for (int v = 0; v < 256; ++v) lut[v] = (uint8_t)(powf((float)v * 1.f / 255.f, inv_gamma) * 255.f);
    if (e == cudaSuccess) e = r->lut.alloc(256);
    if (e == cudaSuccess) e = cudaMemcpyAsync(r->lut.p, lut, 256, cudaMemcpyHostToDevice, r->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(r->stream);
    int st = e == cudaSuccess ? upload_views(r) : cuda_error(e, "crt_render_create");
    if (st != CRT_OK) {
        if (r->own_stream) cudaStreamDestroy(r->stream);
        r->stream = nullptr;
        delete r;
        return st;
    }
    *out = r;
    return CRT_OK;
}

// Renders work[v] of every view: the wavefront form as one stream of waves
// over all views, the megakernel as one launch sequence per view.
static int run_pass(crt_render r, const std::vector<ViewWork>& work, crt_stage_profile* prof) {
    bool any = false;
    for (size_t v = 0; v < work.size(); ++v) {
        if ((uint64_t)work[v].spp0 + work[v].nspp >= (1ull << 32))
            return set_error(CRT_ERR_LIMIT, "sample counter overflow");
        any = any || work[v].nspp;
    }
    if (!any) return CRT_OK;
    if (prof) {
        if (int st = wavefront_profile_pass(r, work, prof)) return st;
    } else if (r->opts.mode == CRT_MODE_WAVEFRONT) {
        if (int st = wavefront_pass(r, work)) return st;
    } else {
        const bool f32 = uses_f32_nodes(r);
        for (uint32_t v = 0; v < (uint32_t)work.size(); ++v) {
            const ViewState& V = r->views[v];
            const dim3 grid((V.width + 15) / 16, (V.height + 7) / 8);
            for (uint32_t done = 0; done < work[v].nspp;) {
                const uint32_t k = std::min(work[v].nspp - done, kMegaSppPerLaunch);
                const RenderParams P = make_params(r, v, work[v].spp0 + done, k);
                if (f32) mega_kernel<true><<<grid, kMegaBlock, 0, r->stream>>>(P);
                else mega_kernel<false><<<grid, kMegaBlock, 0, r->stream>>>(P);
                done += k;
            }
        }
        CRT_CUDA(cudaGetLastError());
    }
    for (size_t v = 0; v < work.size(); ++v) r->views[v].samples_rendered += work[v].nspp;
    return CRT_OK;
}

static std::vector<ViewWork> uniform_work(crt_render r, uint32_t n_spp) {
    std::vector<ViewWork> w;
    for (const ViewState& V : r->views) w.push_back({V.next_sample(), n_spp});
    return w;
}

static int resolve_view(crt_render r, uint32_t v, uint8_t* host_rgba) {
    const ViewState& V = r->views[v];
    if (V.samples_rendered == 0) return set_error(CRT_ERR_INVALID, "no samples rendered");
    const uint32_t n = V.npix();
    DevBuf out;
    CRT_CUDA(out.alloc((size_t)n * 4));
    resolve_kernel<<<grid_for(n, 256, 8), 256, 0, r->stream>>>(r->accum.as<float4>() + V.pix_off, n,
                                                              (float)V.samples_rendered,
                                                              r->lut.as<uint8_t>(), out.as<uchar4>());
    CRT_CUDA(cudaGetLastError());
    CRT_CUDA(cudaMemcpyAsync(host_rgba, out.p, (size_t)n * 4, cudaMemcpyDeviceToHost, r->stream));
    CRT_CUDA(cudaStreamSynchronize(r->stream));
    return check_device_error(r);
}

static int accum_view(crt_render r, uint32_t v, float* host_rgb) {
    const ViewState& V = r->views[v];
    const uint32_t n = V.npix();
    DevBuf out;
    CRT_CUDA(out.alloc((size_t)n * 12));
    unpack_accum_kernel<<<grid_for(n, 256, 8), 256, 0, r->stream>>>(r->accum.as<float4>() + V.pix_off, n,
                                                                   out.as<float>());
    CRT_CUDA(cudaGetLastError());
    CRT_CUDA(cudaMemcpyAsync(host_rgb, out.p, (size_t)n * 12, cudaMemcpyDeviceToHost, r->stream));
    CRT_CUDA(cudaStreamSynchronize(r->stream));
    return check_device_error(r);
}

}  // namespace crt

using namespace crt;

extern "C" {

void crt_render_options_default(crt_render_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->max_depth = 6;           // c_maxBounces (renderer.cu:25,33)
    o->seed = 1234;             // the reference's curand seed (parallel_renderer.cu:315)
    o->view_id = 0;
    o->mode = CRT_MODE_MEGAKERNEL;
    o->block_size = 0;
    o->wave_paths = 0;
    o->node_format = -1;        // the scene's default encoding
    o->top_nodes = 9;           // the tree's top two levels staged in shared memory (+1% at 1080p)
}

int crt_render_create(crt_scene s, const crt_camera* cam, uint32_t width, uint32_t height,
                      const crt_render_options* opts, crt_render* out) {
    if (!s || !cam || !out) return set_error(CRT_ERR_INVALID, "crt_render_create: null argument");
    if (width == 0 || height == 0 || (uint64_t)width * height >= (1ull << 31))
        return set_error(CRT_ERR_INVALID, "crt_render_create: bad image size");
    std::vector<ViewState> views(1);
    views[0].cam = to_device_camera(*cam);
    views[0].width = width;
    views[0].height = height;
    views[0].view_id = opts ? opts->view_id : 0;
    return create_render(s, std::move(views), opts, out);
}

int crt_batch_create(crt_scene s, const crt_view* views, uint32_t num_views, const crt_render_options* opts,
                     crt_render* out) {
    if (!s || !views || !out) return set_error(CRT_ERR_INVALID, "crt_batch_create: null argument");
    if (num_views == 0 || num_views > CRT_MAX_VIEWS)
        return set_error(CRT_ERR_LIMIT, "crt_batch_create: num_views must be in [1, CRT_MAX_VIEWS]");
    std::vector<ViewState> vs(num_views);
    for (uint32_t v = 0; v < num_views; ++v) {
        const crt_view& d = views[v];
        if (d.width == 0 || d.height == 0 || (uint64_t)d.width * d.height >= (1ull << 31))
            return set_error(CRT_ERR_INVALID, "crt_batch_create: bad image size in view " + std::to_string(v));
        vs[v].cam = to_device_camera(d.camera);
        vs[v].width = d.width;
        vs[v].height = d.height;
        vs[v].spp = d.spp;
        vs[v].view_id = d.view_id;
    }
    return create_render(s, std::move(vs), opts, out);
}

int crt_render_destroy(crt_render r) {
    if (!r) return CRT_OK;
    if (r->stream) cudaStreamSynchronize(r->stream);
    if (r->own_stream) cudaStreamDestroy(r->stream);
    r->stream = nullptr;   // the handle's destructor must not touch it
    delete r;
    return CRT_OK;
}

int crt_render_set_stream(crt_render r, void* stream) {
    if (!r) return set_error(CRT_ERR_INVALID, "null render");
    CRT_CUDA(cudaStreamSynchronize(r->stream));
    if (r->own_stream) cudaStreamDestroy(r->stream);
    r->stream = (cudaStream_t)stream;
    r->own_stream = false;
    return CRT_OK;
}

int crt_render_set_camera(crt_render r, const crt_camera* cam) {
    if (!r || !cam) return set_error(CRT_ERR_INVALID, "null argument");
    CRT_CUDA(cudaStreamSynchronize(r->stream));   // every wave set joins this stream
    r->views[0].cam = to_device_camera(*cam);
    return upload_views(r);   // the wave kernels read cameras from the view table
}

int crt_render_pass(crt_render r, uint32_t n_spp) {
    if (!r) return set_error(CRT_ERR_INVALID, "null render");
    if (n_spp == 0) return CRT_OK;
    return run_pass(r, uniform_work(r, n_spp), nullptr);
}

int crt_batch_render(crt_render r) {
    if (!r) return set_error(CRT_ERR_INVALID, "null render");
    std::vector<ViewWork> w;
    for (const ViewState& V : r->views) w.push_back({V.next_sample(), V.spp});
    return run_pass(r, w, nullptr);
}

int crt_render_profile_pass(crt_render r, uint32_t n_spp, crt_stage_profile* out) {
    if (!r || !out) return set_error(CRT_ERR_INVALID, "null argument");
    if (r->opts.mode != CRT_MODE_WAVEFRONT)
        return set_error(CRT_ERR_UNSUPPORTED, "stage profiling needs a wavefront handle");
    std::memset(out, 0, sizeof(*out));
    if (n_spp == 0) return CRT_OK;
    return run_pass(r, uniform_work(r, n_spp), out);
}

int crt_render_adjoint(crt_render r, uint32_t spp0, uint32_t n_spp, const float* d_adjoint, float* d_grad_kd,
                       float* d_grad_ka, uint32_t flags) {
    if (!r || !d_adjoint || !d_grad_kd || !d_grad_ka) return set_error(CRT_ERR_INVALID, "crt_render_adjoint: null argument");
    if (((uintptr_t)d_adjoint & 15u) != 0) return set_error(CRT_ERR_INVALID, "d_adjoint must be 16-byte aligned");
    if (n_spp == 0) return CRT_OK;
    if ((uint64_t)spp0 + n_spp >= (1ull << 32)) return set_error(CRT_ERR_LIMIT, "sample index overflow");
    std::vector<ViewWork> work(r->views.size(), ViewWork{spp0, n_spp});
    if (flags & ~(uint32_t)CRT_ADJOINT_EXACT_ROULETTE) return set_error(CRT_ERR_INVALID, "unknown adjoint flag");
    return wavefront_adjoint(r, work, reinterpret_cast<const float4*>(d_adjoint), d_grad_kd, d_grad_ka, flags);
}

int crt_render_samples_rendered(crt_render r, uint32_t* out) {
    if (!r || !out) return set_error(CRT_ERR_INVALID, "null argument");
    *out = r->views[0].samples_rendered;
    return CRT_OK;
}

int crt_render_view_info(crt_render r, uint32_t view, crt_view* desc, uint32_t* samples_rendered,
                         uint32_t* pixel_offset) {
    if (!r) return set_error(CRT_ERR_INVALID, "null render");
    if (view >= r->views.size()) return set_error(CRT_ERR_INVALID, "view index out of range");
    const ViewState& V = r->views[view];
    if (desc) {
        std::memset(desc, 0, sizeof(*desc));
        desc->width = V.width;
        desc->height = V.height;
        desc->spp = V.spp;
        desc->view_id = V.view_id;
    }
    if (samples_rendered) *samples_rendered = V.samples_rendered;
    if (pixel_offset) *pixel_offset = V.pix_off;
    return CRT_OK;
}

int crt_render_synchronize(crt_render r) {
    if (!r) return set_error(CRT_ERR_INVALID, "null render");
    CRT_CUDA(cudaStreamSynchronize(r->stream));
    return check_device_error(r);
}

int crt_render_resolve(crt_render r, uint8_t* host_rgba) {
    if (!r || !host_rgba) return set_error(CRT_ERR_INVALID, "null argument");
    return resolve_view(r, 0, host_rgba);
}

int crt_render_view_resolve(crt_render r, uint32_t view, uint8_t* host_rgba) {
    if (!r || !host_rgba) return set_error(CRT_ERR_INVALID, "null argument");
    if (view >= r->views.size()) return set_error(CRT_ERR_INVALID, "view index out of range");
    return resolve_view(r, view, host_rgba);
}

int crt_render_resolve_device(crt_render r, void* d_rgba) {
    if (!r || !d_rgba) return set_error(CRT_ERR_INVALID, "null argument");
    const ViewState& V = r->views[0];
    if (V.samples_rendered == 0) return set_error(CRT_ERR_INVALID, "no samples rendered");
    const uint32_t n = V.npix();
    average_u8_kernel<<<grid_for(n, 256, 8), 256, 0, r->stream>>>(r->accum.as<float4>() + V.pix_off, n,
                                                                 (float)V.samples_rendered, (uchar4*)d_rgba);
    CRT_CUDA(cudaGetLastError());
    return CRT_OK;
}

int crt_render_resolve_async(crt_render r, uint8_t* host_rgba) {
    if (!r || !host_rgba) return set_error(CRT_ERR_INVALID, "null argument");
    const ViewState& V = r->views[0];
    if (V.samples_rendered == 0) return set_error(CRT_ERR_INVALID, "no samples rendered");
    const uint32_t n = V.npix();
    if (r->staging.bytes < (size_t)n * 4) CRT_CUDA(r->staging.alloc((size_t)n * 4));
    resolve_kernel<<<grid_for(n, 256, 8), 256, 0, r->stream>>>(r->accum.as<float4>() + V.pix_off, n,
                                                              (float)V.samples_rendered,
                                                              r->lut.as<uint8_t>(), r->staging.as<uchar4>());
    CRT_CUDA(cudaGetLastError());
    CRT_CUDA(cudaMemcpyAsync(host_rgba, r->staging.p, (size_t)n * 4, cudaMemcpyDeviceToHost, r->stream));
    return CRT_OK;
}

__global__ void pack_accum_kernel(const float* __restrict__ in, uint32_t n, float4* __restrict__ accum) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        accum[i] = make_float4(in[3ull * i], in[3ull * i + 1], in[3ull * i + 2], 0.f);
}

int crt_render_load_accum(crt_render r, uint32_t view, const float* host_rgb, uint32_t samples,
                          uint32_t first_sample) {
    if (!r || !host_rgb) return set_error(CRT_ERR_INVALID, "null argument");
    if (view >= r->views.size()) return set_error(CRT_ERR_INVALID, "view index out of range");
    if ((uint64_t)first_sample + samples >= (1ull << 32)) return set_error(CRT_ERR_LIMIT, "sample index overflow");
    ViewState& V = r->views[view];
    const uint32_t n = V.npix();
    DevBuf tmp;
    CRT_CUDA(tmp.alloc((size_t)n * 12));
    CRT_CUDA(cudaMemcpyAsync(tmp.p, host_rgb, (size_t)n * 12, cudaMemcpyHostToDevice, r->stream));
    pack_accum_kernel<<<grid_for(n, 256, 8), 256, 0, r->stream>>>(tmp.as<float>(), n, r->accum.as<float4>() + V.pix_off);
    CRT_CUDA(cudaGetLastError());
    CRT_CUDA(cudaStreamSynchronize(r->stream));
    V.first_sample = first_sample;
    V.samples_rendered = samples;
    return CRT_OK;
}

int crt_render_accum(crt_render r, float* host_rgb) {
    if (!r || !host_rgb) return set_error(CRT_ERR_INVALID, "null argument");
    return accum_view(r, 0, host_rgb);
}

int crt_render_view_accum(crt_render r, uint32_t view, float* host_rgb) {
    if (!r || !host_rgb) return set_error(CRT_ERR_INVALID, "null argument");
    if (view >= r->views.size()) return set_error(CRT_ERR_INVALID, "view index out of range");
    return accum_view(r, view, host_rgb);
}

int crt_render_accum_device(crt_render r, float** d_rgb) {
    if (!r || !d_rgb) return set_error(CRT_ERR_INVALID, "null argument");
    *d_rgb = r->accum.as<float>();   // [pixels of every view][4]: rgb + unused
    return CRT_OK;
}

int crt_render_reset(crt_render r) {
    if (!r) return set_error(CRT_ERR_INVALID, "null render");
    CRT_CUDA(cudaMemsetAsync(r->accum.p, 0, r->accum.bytes, r->stream));
    CRT_CUDA(cudaMemsetAsync(r->ray_counts.p, 0, r->ray_counts.bytes, r->stream));
    for (ViewState& V : r->views) V.first_sample = V.samples_rendered = 0;
    return CRT_OK;
}

int crt_render_restart(crt_render r, uint32_t first_sample) {
    if (!r) return set_error(CRT_ERR_INVALID, "null render");
    CRT_CUDA(cudaMemsetAsync(r->accum.p, 0, r->accum.bytes, r->stream));
    CRT_CUDA(cudaMemsetAsync(r->ray_counts.p, 0, r->ray_counts.bytes, r->stream));
    for (ViewState& V : r->views) {
        V.first_sample = first_sample;
        V.samples_rendered = 0;
    }
    return CRT_OK;
}

int crt_render_ray_counts(crt_render r, uint64_t* ext, uint64_t* shadow) {
    if (!r) return set_error(CRT_ERR_INVALID, "null render");
    unsigned long long c[2] = {0, 0};
    CRT_CUDA(cudaMemcpyAsync(c, r->ray_counts.p, sizeof(c), cudaMemcpyDeviceToHost, r->stream));
    CRT_CUDA(cudaStreamSynchronize(r->stream));
    if (ext) *ext = c[0];
    if (shadow) *shadow = c[1];
    return CRT_OK;
}

}  // extern "C"
