// crt_internal.h -- host-side structures shared by the library's
// translation units (not part of the public ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <utility>
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
    void swap(DevBuf& o) {
        std::swap(p, o.p);
        std::swap(bytes, o.bytes);
    }
};

}  // namespace crt

struct crt_scene_s {
    int device = 0;
    crt::Bvh8 bvh;                  // host copy (export / statistics)
    crt::DevBuf nodes, fnodes, tris, shade, uvs, mats, light_geo, texels, tex_dims, tex_offsets, error;
    crt::DevScene dev{};            // both node encodings uploaded
    bool default_f32 = false;       // encoding renders use unless told otherwise
    uint32_t n_mats = 0;
    bool ka_scaled = false;         // materials were given with the emission scaling applied
    uint32_t builder = 0;           // crt_bvh_builder
    bool host_bvh = true;           // `bvh` holds the device BVH (the GPU build fills it on demand)
    uint32_t generation = 0;        // bumped whenever the BVH buffers are replaced
    crt_scene_info info{};

    // Device view with the FP32 or the quantised nodes.
    crt::DevScene view(bool f32) const {
        crt::DevScene d = dev;
        if (!f32) d.fnodes = nullptr;
        return d;
    }
    std::vector<uint32_t> lights;   // face indices in pick order
};

// Wavefront path-state buffers (wavefront.cu).
struct WaveBuffers {
    uint32_t capacity = 0;
    uint32_t seg_capacity = 0;      // wave segments the segs buffer holds
    bool octant = false;            // queues hold 8 octant regions
    crt::DevBuf ray_o, color, hit, queue_a, queue_b, shadow, shadow_q, counters, waves, segs, prof;
    crt::DevBuf adj_L, adj_W, adj_shadow, adj_hist;   // adjoint replay state, allocated on first use
};

// One independent set of wavefront buffers with its own stream and captured
// wave graph; several sets run waves concurrently (wavefront.cu).
struct WaveSet {
    WaveBuffers buf;
    cudaStream_t stream = nullptr;
    cudaEvent_t acc_done = nullptr;   // recorded after this set's latest accumulate
    void* graph = nullptr;
    void* adj_graph = nullptr;        // adjoint wave body, captured for adj_key's pointers
    const void* adj_key[3] = {nullptr, nullptr, nullptr};
    uint32_t adj_flags = 0;
};

namespace crt {
int build_bvh_gpu(const float* d_v1, const float* d_e1, const float* d_e2, uint32_t n, uint32_t max_levels,
                  int max_children, DevBuf& nodes_out, DevBuf& fnodes_out, DevBuf& tris_out, uint32_t* num_nodes,
                  uint32_t* max_depth, bool* fnodes_ok, cudaStream_t s);
void destroy_wave_sets(struct ::crt_render_s* r);
void drop_wave_graphs(struct ::crt_render_s* r);
}

// One camera view of a render; its image is pixels
// [pix_off, pix_off + width * height) of the render's accumulator.
struct ViewState {
    crt::Camera cam{};
    uint32_t width = 0, height = 0;
    uint32_t spp = 0;               // samples per pixel one batch render adds
    uint32_t view_id = 0;           // Philox counter word
    uint32_t pix_off = 0;
    uint32_t first_sample = 0;      // sample index the accumulator starts at
    uint32_t samples_rendered = 0;  // samples in the accumulator
    uint32_t npix() const { return width * height; }
    uint32_t next_sample() const { return first_sample + samples_rendered; }
};

// Samples [spp0, spp0 + nspp) of one view, rendered by a pass.
struct ViewWork {
    uint32_t spp0, nspp;
};

struct crt_render_s {
    crt_scene scene = nullptr;
    std::vector<ViewState> views;   // a single render has one; a batch many
    crt_render_options opts{};
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    crt::DevBuf accum, lut, ray_counts, view_table, staging;
    std::vector<WaveSet> sets;
    uint32_t scene_generation = 0;  // scene BVH the captured wave graphs point at
    cudaEvent_t pass_start = nullptr;
    uint32_t graph_epoch = 0;       // bumped whenever a set's wave graph is captured
    void* pass_graph = nullptr;     // a whole pass as one graph (wavefront.cu), or null
    uint64_t pass_key = 0;          // waves, sets and epoch it was built for
    ~crt_render_s() { crt::destroy_wave_sets(this); }
};

namespace crt {

// Node encoding a render traverses: its option, else the scene's default.
inline bool uses_f32_nodes(const crt_scene_s* s, int32_t node_format) {
    if (!s->dev.fnodes) return false;
    return node_format < 0 ? s->default_f32 : node_format == CRT_NODES_F32;
}
inline bool uses_f32_nodes(const crt_render_s* r) { return uses_f32_nodes(r->scene, r->opts.node_format); }

// Traversal launch shape of a wavefront render.
inline uint32_t traversal_block(const crt_render_options& o) { return o.block_size ? o.block_size : 128u; }
inline uint32_t traversal_stack(const crt_render_options& o) { return o.stack_depth ? o.stack_depth : 8u; }
inline uint32_t queue_chunk(const crt_render_options& o) { return o.queue_chunk ? o.queue_chunk : 32u; }
inline uint32_t refill_busy(const crt_render_options& o) { return o.refill_busy ? o.refill_busy : 31u; }
inline uint32_t staged_nodes(const crt_scene_s* s, const crt_render_options& o) {
    return o.top_nodes < s->info.num_nodes ? o.top_nodes : s->info.num_nodes;
}

// Default paths in flight per wave set: about 16 samples of every pixel of
// the handle's views, rounded up to a power of two in [2^16, 2^25] (32M paths
// at 1080p, 4.7 GB of path state per set).  Longer waves balance the thin
// late bounces of one wave against the heavy early bounces of the next;
// measured on the 1080p frame with the window sort and 4 sets: 16M paths
// 1,170, 32M 1,195 Msamples/s (before the sort: 4M 890, 8M 906, 16M 915,
// 32M 919).
inline uint32_t default_wave_paths(uint64_t pixels) {
    const uint64_t want = pixels * 16;
    uint32_t cap = 1u << 16;
    while (cap < want && cap < (1u << 25)) cap <<= 1;
    return cap;
}

// Checks the fields every render entry point shares; CRT_OK or an error.
inline int check_render_options(const crt_render_options& o) {
    if (o.max_depth == 0 || o.max_depth > 1024) return set_error(CRT_ERR_INVALID, "max_depth must be in [1, 1024]");
    if (o.mode > CRT_MODE_WAVEFRONT) return set_error(CRT_ERR_INVALID, "unknown mode");
    if (o.block_size != 0 && o.block_size != 64 && o.block_size != 128 && o.block_size != 256)
        return set_error(CRT_ERR_INVALID, "block_size must be 0, 64, 128 or 256");
    if (o.stack_depth != 0 && (o.stack_depth < 4 || o.stack_depth > (uint32_t)kStackSharedMax))
        return set_error(CRT_ERR_INVALID, "stack_depth must be 0 or in [4, 32]");
    if (o.node_format < -1 || o.node_format > CRT_NODES_F32) return set_error(CRT_ERR_INVALID, "unknown node format");
    if (o.wave_sets > 8) return set_error(CRT_ERR_INVALID, "wave_sets must be in [0, 8]");
    if (o.queue_chunk != 0 && o.queue_chunk != 32 && o.queue_chunk != 64 && o.queue_chunk != 128 &&
        o.queue_chunk != 256)
        return set_error(CRT_ERR_INVALID, "queue_chunk must be 0, 32, 64, 128 or 256");
    if (o.top_nodes > 128) return set_error(CRT_ERR_INVALID, "top_nodes must be in [0, 128]");
    if (o.refill_busy > 31) return set_error(CRT_ERR_INVALID, "refill_busy must be in [0, 31]");
    if (o.flags & ~(uint32_t)(CRT_FLAG_LANE_REFILL | CRT_FLAG_SPLIT_LEAF | CRT_FLAG_OCTANT_QUEUES |
                              CRT_FLAG_SERIAL_SHADOW | CRT_FLAG_NO_WINDOW_SORT))
        return set_error(CRT_ERR_INVALID, "unknown render flag");
    return CRT_OK;
}

}  // namespace crt
