// trace.cu -- batched closest-hit queries (crt_trace_closest) and the
// instrumented traversal that counts node visits and triangle tests per ray.
//
// Replaces intersectBVH (src/renderer/renderer.cu:283-330) for batches of
// arbitrary rays.  One thread per ray, 128-thread blocks, grid-stride loop
// over a grid that is a multiple of the SM count.
#include "crt_internal.h"

namespace crt {

constexpr int kTraceBlock = 128;

template <bool COUNT, bool F32>
__global__ void __launch_bounds__(kTraceBlock) trace_closest_kernel(DevScene S, const float4* __restrict__ rays,
                                                                    uint32_t n, int32_t* __restrict__ out_face,
                                                                    float* __restrict__ out_t,
                                                                    float2* __restrict__ out_uv,
                                                                    uint32_t* __restrict__ out_nodes,
                                                                    uint32_t* __restrict__ out_tris) {
    __shared__ uint2 stack_sh[kStackShared * kTraceBlock];
    Stack st;
    st.setup(stack_sh, kTraceBlock, kStackShared);
    for (uint32_t i = blockIdx.x * kTraceBlock + threadIdx.x; i < n; i += gridDim.x * kTraceBlock) {
        const float4 a = rays[2ull * i], b = rays[2ull * i + 1];
        Hit h;
        h.t = b.w;
        h.face = -1;
        h.u = h.v = 0.f;
        TraversalStats ts{0, 0};
        traverse<false, COUNT, F32>(S, xyz(a), xyz(b), a.w, h, -1, st, &ts);
        if (COUNT) {
            out_nodes[i] = ts.nodes;
            out_tris[i] = ts.tris;
        } else {
            out_face[i] = h.face;
            out_t[i] = h.face >= 0 ? h.t : FLT_MAX;
            if (out_uv) out_uv[i] = make_float2(h.u, h.v);
        }
    }
}

// Gather ceiling: every thread fetches `loads` records of `rec16` float4s at
// indices from its own LCG (independent of the loaded data, so many fetches
// are in flight), through L2 only (.cg) or through L1 as the traversal's
// __ldg fetches go (.nc).  The XOR of what was read goes to sink[thread] so
// that no load is dropped.
template <bool L1>
__global__ void __launch_bounds__(256) gather_kernel(const float4* __restrict__ base, uint64_t records,
                                                     uint32_t rec16, uint32_t loads,
                                                     uint32_t* __restrict__ sink) {
    const uint32_t tid = blockIdx.x * 256u + threadIdx.x;
    uint32_t state = tid * 2654435761u + 12345u;
    uint32_t acc = 0;
    for (uint32_t k = 0; k < loads; ++k) {
        state = state * 1664525u + 1013904223u;
        const uint64_t r = ((uint64_t)state * records) >> 32;   // < records
        const float4* p = base + r * rec16;
#pragma unroll 4
        for (uint32_t j = 0; j < rec16; ++j) {
            const float4 v = L1 ? __ldg(p + j) : __ldcg(p + j);
            acc ^= __float_as_uint(v.x) ^ __float_as_uint(v.y) ^ __float_as_uint(v.z) ^ __float_as_uint(v.w);
        }
    }
    sink[tid] = acc;
}

int grid_for(uint32_t n, int block, int per_sm) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    uint64_t need = (n + (uint64_t)block - 1) / block;
    uint64_t cap = (uint64_t)sms * per_sm;
    return (int)(need < cap ? (need ? need : 1) : cap);
}

}  // namespace crt

using namespace crt;

extern "C" {

int crt_trace_closest(crt_scene s, const float* d_rays, uint32_t n, int32_t* d_index, float* d_t,
                      float* d_uv, void* stream) {
    if (!s || (!d_rays && n) || (n && (!d_index || !d_t)))
        return set_error(CRT_ERR_INVALID, "crt_trace_closest: null argument");
    if (n == 0) return CRT_OK;
    if (((uintptr_t)d_rays & 15u) != 0) return set_error(CRT_ERR_INVALID, "rays must be 16-byte aligned");
    auto k = s->default_f32 ? trace_closest_kernel<false, true> : trace_closest_kernel<false, false>;
    k<<<grid_for(n, kTraceBlock, 16), kTraceBlock, 0, (cudaStream_t)stream>>>(
        s->view(s->default_f32), (const float4*)d_rays, n, d_index, d_t, (float2*)d_uv, nullptr, nullptr);
    CRT_CUDA(cudaGetLastError());
    return CRT_OK;
}

int crt_trace_counts(crt_scene s, const float* d_rays, uint32_t n, uint32_t* d_nodes, uint32_t* d_tris,
                     void* stream) {
    if (!s || (n && (!d_rays || !d_nodes || !d_tris)))
        return set_error(CRT_ERR_INVALID, "crt_trace_counts: null argument");
    if (n == 0) return CRT_OK;
    if (((uintptr_t)d_rays & 15u) != 0) return set_error(CRT_ERR_INVALID, "rays must be 16-byte aligned");
    auto k = s->default_f32 ? trace_closest_kernel<true, true> : trace_closest_kernel<true, false>;
    k<<<grid_for(n, kTraceBlock, 16), kTraceBlock, 0, (cudaStream_t)stream>>>(
        s->view(s->default_f32), (const float4*)d_rays, n, nullptr, nullptr, nullptr, d_nodes, d_tris);
    CRT_CUDA(cudaGetLastError());
    return CRT_OK;
}

int crt_measure_gather(const void* d_buf, uint64_t bytes, uint32_t record_bytes, uint32_t n_threads,
                       uint32_t loads_per_thread, uint32_t flags, uint32_t* d_sink, void* stream) {
    if (!d_buf || !d_sink) return set_error(CRT_ERR_INVALID, "crt_measure_gather: null argument");
    if (((uintptr_t)d_buf & 15u) != 0) return set_error(CRT_ERR_INVALID, "buffer must be 16-byte aligned");
    if (record_bytes == 0 || record_bytes % 16 != 0 || record_bytes > 4096)
        return set_error(CRT_ERR_INVALID, "record_bytes must be a multiple of 16 in [16, 4096]");
    const uint64_t records = bytes / record_bytes;
    if (records == 0 || records > 0xFFFFFFFFull)
        return set_error(CRT_ERR_INVALID, "buffer must hold between 1 and 2^32-1 records");
    if (n_threads == 0 || n_threads % 256 != 0)
        return set_error(CRT_ERR_INVALID, "n_threads must be a positive multiple of 256");
    if (flags & ~CRT_GATHER_L1) return set_error(CRT_ERR_INVALID, "crt_measure_gather: unknown flag");
    auto k = (flags & CRT_GATHER_L1) ? gather_kernel<true> : gather_kernel<false>;
    k<<<n_threads / 256, 256, 0, (cudaStream_t)stream>>>((const float4*)d_buf, records, record_bytes / 16,
                                                          loads_per_thread, d_sink);
    CRT_CUDA(cudaGetLastError());
    return CRT_OK;
}

}  // extern "C"
