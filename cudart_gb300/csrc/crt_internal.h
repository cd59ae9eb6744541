// crt_internal.h -- host-side structures shared by the library's
// translation units (not part of the public ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/crt_gb300.h"
#include "bvh8.h"
#include "crt_device.cuh"

namespace crt {

// Thread-local error message behind crt_last_error().
int set_error(int status, const std::string& msg);
int cuda_error(cudaError_t e, const char* what);

#define CRT_CUDA(call)                                      \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_error(e_, #call); \
    } while (0)

// Owning device buffer.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    ~DevBuf() { if (p) cudaFree(p); }
    cudaError_t alloc(size_t n) {
        if (p) { cudaFree(p); p = nullptr; }
        bytes = n;
        return n ? cudaMalloc(&p, n) : cudaSuccess;
    }
    template <typename T> T* as() const { return static_cast<T*>(p); }
};

}  // namespace crt

struct crt_scene_s {
    int device = 0;
    crt::Bvh8 bvh;                  // host copy (export / statistics)
    crt::DevBuf nodes, fnodes, tris, shade, uvs, mats, light_geo, texels, tex_dims, tex_offsets, error;
    crt::DevScene dev{};
    crt_scene_info info{};
    std::vector<uint32_t> lights;   // face indices in pick order
};

// Wavefront path-state buffers (see render.cu).
struct WaveBuffers {
    uint32_t capacity = 0;
    crt::DevBuf ray_o, ray_d, mask, color, hit, path_id, queue_a, queue_b, shadow, counters, waves, prof;
};

namespace crt {
void destroy_wave_graph(void* g);
}

struct crt_render_s {
    crt_scene scene = nullptr;
    crt::Camera cam{};
    uint32_t width = 0, height = 0;
    crt_render_options opts{};
    uint32_t samples_rendered = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    crt::DevBuf accum, lut, ray_counts;
    WaveBuffers wave;
    void* wave_graph = nullptr;     // instantiated wave sequence (wavefront.cu)
    ~crt_render_s() { crt::destroy_wave_graph(wave_graph); }
};
