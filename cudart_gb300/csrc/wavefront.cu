// wavefront.cu -- the wavefront form of the path tracer.
//
// A pass is cut into waves of at most `capacity` paths (a pixel range x a
// sample range).  One wave runs
//
//   generate -> { extend -> shade -> shadow -> flip } x max_depth -> accumulate
//
// * generate:   camera rays for every path of the wave (queue = all paths)
// * extend:     persistent closest-hit kernel; warps fetch 32 queue entries at
//               a time from a global counter
// * shade:      one bounce of the estimator (render_common.cuh); surviving
//               paths and shadow requests are appended to the next queues
//               with __ballot_sync / __popc warp-aggregated atomics
// * shadow:     persistent any-hit kernel; a visible light adds the request's
//               contribution to the path colour
// * flip:       one thread swaps the queue counters for the next bounce
// * accumulate: adds each pixel's per-sample colours in sample order, so the
//               FP32 sums equal the megakernel's bit for bit
//
// Queue lengths live in device memory, so the whole wave is launched without
// host synchronisation and is captured once as a CUDA graph; the graph reads
// its wave descriptor through a device-side wave counter.
#include "crt_internal.h"
#include "render_common.cuh"

#include <algorithm>
#include <vector>

namespace crt {

int grid_for(uint32_t n, int block, int per_sm);
RenderParams make_params(crt_render r, uint32_t spp0, uint32_t nspp);

constexpr int kWaveBlock = 128;
constexpr uint32_t kDefaultCapacity = 1u << 22;
constexpr uint32_t kMaxWaves = 1u << 16;   // descriptors uploaded per chunk

enum Counter : uint32_t {
    C_QUEUE0 = 0,       // length of queue 0
    C_QUEUE1 = 1,       // length of queue 1
    C_SHADOW = 2,       // shadow requests this bounce
    C_FETCH_EXT = 3,    // extend work counter
    C_FETCH_SHD = 4,    // shadow work counter
    C_CUR = 5,          // which extension queue is current (0/1)
    C_WAVE = 6,         // wave index within the pass
    C_COUNT = 8
};

struct WaveParams {
    RenderParams R;
    float4* st_o;       // o.xyz, pixel
    float4* st_d;       // d.xyz, sample
    float4* st_c;       // color.xyz, rng draws
    float4* st_m;       // mask.xyz, prev | bounce << 8
    float4* hit;        // t, face, u, v
    uint32_t* queue[2];
    float4* shadow;     // 3 float4 per request
    uint32_t* counters;
    const uint4* waves; // pixel0, pixel1, sample0, sample1
};

CRT_D uint4 wave_desc(const WaveParams& W) { return W.waves[W.counters[C_WAVE]]; }

CRT_D void store_state(const WaveParams& W, uint32_t i, const PathState& ps, const Ray& ray, uint32_t pixel,
                       uint32_t sample) {
    W.st_o[i] = make_float4(ray.o.x, ray.o.y, ray.o.z, __uint_as_float(pixel));
    W.st_d[i] = make_float4(ray.d.x, ray.d.y, ray.d.z, __uint_as_float(sample));
    W.st_c[i] = make_float4(ps.color.x, ps.color.y, ps.color.z, __uint_as_float(ps.rng.n));
    W.st_m[i] = make_float4(ps.mask.x, ps.mask.y, ps.mask.z, __uint_as_float((uint32_t)ps.prev | (ps.bounce << 8)));
}

// Warp-aggregated append: returns the slot for this lane (if `want`).
CRT_D uint32_t warp_append(uint32_t* counter, bool want) {
    const uint32_t active = __activemask();
    const uint32_t ballot = __ballot_sync(active, want);
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t leader = __ffs(active) - 1;
    uint32_t base = 0;
    if (lane == leader && ballot) base = atomicAdd(counter, __popc(ballot));
    base = __shfl_sync(active, base, leader);
    return base + __popc(ballot & ((1u << lane) - 1u));
}

__global__ void __launch_bounds__(kWaveBlock) wf_generate(WaveParams W) {
    const uint4 wd = wave_desc(W);
    const uint32_t np = wd.y - wd.x, n = np * (wd.w - wd.z);
    const uint32_t cur = W.counters[C_CUR];
    for (uint32_t i = blockIdx.x * kWaveBlock + threadIdx.x; i < n; i += gridDim.x * kWaveBlock) {
        const uint32_t pixel = wd.x + i % np, sample = wd.z + i / np;
        PathState ps;
        Ray ray;
        begin_path(W.R, pixel % W.R.width, pixel / W.R.width, pixel, sample, ps, ray);
        store_state(W, i, ps, ray, pixel, sample);
        W.queue[cur][i] = i;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        W.counters[cur] = n;
        W.counters[cur ^ 1u] = 0;
        W.counters[C_SHADOW] = 0;
        W.counters[C_FETCH_EXT] = 0;
        W.counters[C_FETCH_SHD] = 0;
    }
}

__global__ void __launch_bounds__(kWaveBlock) wf_extend(WaveParams W) {
    __shared__ uint2 stack_sh[kStackShared * kWaveBlock];
    Stack st;
    st.sh = stack_sh + threadIdx.x;
    st.stride = kWaveBlock;
    const uint32_t cur = W.counters[C_CUR];
    const uint32_t n = W.counters[cur];
    const uint32_t* q = W.queue[cur];
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t rays = 0;
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&W.counters[C_FETCH_EXT], 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= n) break;
        const uint32_t i = base + lane;
        if (i < n) {
            const uint32_t path = q[i];
            const float4 o = W.st_o[path], d = W.st_d[path];
            Hit h;
            h.t = FLT_MAX;
            h.face = -1;
            h.u = h.v = 0.f;
            traverse<false, false>(W.R.S, xyz(o), xyz(d), kEps, h, -1, st, nullptr);
            W.hit[path] = make_float4(h.t, __int_as_float(h.face), h.u, h.v);
            ++rays;
        }
    }
    count_rays(W.R.ray_counts, rays, 0);
}

__global__ void __launch_bounds__(kWaveBlock) wf_shade(WaveParams W) {
    const uint32_t cur = W.counters[C_CUR];
    const uint32_t n = W.counters[cur];
    const uint32_t* q = W.queue[cur];
    uint32_t* qn = W.queue[cur ^ 1u];
    const uint32_t end = (n + 31u) & ~31u;   // whole warps stay converged for the ballots
    for (uint32_t i = blockIdx.x * kWaveBlock + threadIdx.x; i < end; i += gridDim.x * kWaveBlock) {
        bool alive = false, want_shadow = false;
        uint32_t path = 0;
        ShadowReq sr;
        sr.valid = false;
        if (i < n) {
            path = q[i];
            const float4 o = W.st_o[path], d = W.st_d[path], c = W.st_c[path], m = W.st_m[path];
            const float4 hv = W.hit[path];
            const uint32_t pixel = __float_as_uint(o.w), sample = __float_as_uint(d.w);
            const uint32_t pb = __float_as_uint(m.w);
            PathState ps;
            ps.color = xyz(c);
            ps.mask = xyz(m);
            ps.prev = (int)(pb & 0xFFu);
            ps.bounce = pb >> 8;
            ps.rng.init(W.R.seed, W.R.view, pixel, sample, __float_as_uint(c.w));
            Ray ray;
            ray.o = xyz(o);
            ray.d = xyz(d);
            Hit h;
            h.t = hv.x;
            h.face = __float_as_int(hv.y);
            h.u = hv.z;
            h.v = hv.w;
            if (h.face < 0) {
                shade_miss(ps);
            } else {
                alive = shade_hit(W.R, ps, ray, h, sr) && ps.bounce < W.R.max_depth;
                want_shadow = sr.valid;
            }
            store_state(W, path, ps, ray, pixel, sample);
        }
        const uint32_t slot = warp_append(&W.counters[cur ^ 1u], alive);
        if (alive) qn[slot] = path;
        const uint32_t ss = warp_append(&W.counters[C_SHADOW], want_shadow);
        if (want_shadow) {
            float4* e = W.shadow + 3ull * ss;
            e[0] = make_float4(sr.o.x, sr.o.y, sr.o.z, __uint_as_float(path));
            e[1] = make_float4(sr.d.x, sr.d.y, sr.d.z, sr.t_light);
            e[2] = make_float4(sr.contrib.x, sr.contrib.y, sr.contrib.z, __uint_as_float(sr.light_face));
        }
    }
}

__global__ void __launch_bounds__(kWaveBlock) wf_shadow(WaveParams W) {
    __shared__ uint2 stack_sh[kStackShared * kWaveBlock];
    Stack st;
    st.sh = stack_sh + threadIdx.x;
    st.stride = kWaveBlock;
    const uint32_t n = W.counters[C_SHADOW];
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t rays = 0;
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&W.counters[C_FETCH_SHD], 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= n) break;
        const uint32_t i = base + lane;
        if (i < n) {
            const float4* e = W.shadow + 3ull * i;
            const float4 a = e[0], b = e[1], c = e[2];
            ShadowReq sr;
            sr.o = xyz(a);
            sr.d = xyz(b);
            sr.t_light = b.w;
            sr.light_face = __float_as_uint(c.w);
            ++rays;
            if (!occluded(W.R.S, sr, st)) {
                const uint32_t path = __float_as_uint(a.w);
                float4 col = W.st_c[path];
                col.x = col.x + c.x;
                col.y = col.y + c.y;
                col.z = col.z + c.z;
                W.st_c[path] = col;
            }
        }
    }
    count_rays(W.R.ray_counts, 0, rays);
}

__global__ void wf_flip(WaveParams W) {
    const uint32_t cur = W.counters[C_CUR];
    W.counters[cur] = 0;
    W.counters[C_CUR] = cur ^ 1u;
    W.counters[C_SHADOW] = 0;
    W.counters[C_FETCH_EXT] = 0;
    W.counters[C_FETCH_SHD] = 0;
}

__global__ void __launch_bounds__(256) wf_accumulate(WaveParams W) {
    const uint4 wd = wave_desc(W);
    const uint32_t np = wd.y - wd.x, ns = wd.w - wd.z;
    for (uint32_t i = blockIdx.x * 256 + threadIdx.x; i < np; i += gridDim.x * 256) {
        float4 acc = W.R.accum[wd.x + i];
        for (uint32_t s = 0; s < ns; ++s) {
            const float4 c = W.st_c[s * np + i];
            acc.x = acc.x + c.x;
            acc.y = acc.y + c.y;
            acc.z = acc.z + c.z;
        }
        W.R.accum[wd.x + i] = acc;
    }
}

__global__ void wf_next_wave(WaveParams W) { W.counters[C_WAVE] += 1; }

int persistent_grid(const void* kernel, int block, size_t smem) {
    int dev = 0, sms = 1, per = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, block, smem);
    return sms * (per > 0 ? per : 1);
}

}  // namespace crt

using namespace crt;

struct WaveGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    ~WaveGraph() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
    }
};

namespace crt {

static int ensure_wave_buffers(crt_render r) {
    WaveBuffers& B = r->wave;
    uint32_t cap = r->opts.wave_paths ? r->opts.wave_paths : kDefaultCapacity;
    if (B.capacity == cap) return CRT_OK;
    B.capacity = cap;
    const size_t c = cap;
    CRT_CUDA(B.ray_o.alloc(c * 16));
    CRT_CUDA(B.ray_d.alloc(c * 16));
    CRT_CUDA(B.color.alloc(c * 16));
    CRT_CUDA(B.mask.alloc(c * 16));
    CRT_CUDA(B.hit.alloc(c * 16));
    CRT_CUDA(B.queue_a.alloc(c * 4));
    CRT_CUDA(B.queue_b.alloc(c * 4));
    CRT_CUDA(B.shadow.alloc(c * 48));
    CRT_CUDA(B.counters.alloc(C_COUNT * 4));
    CRT_CUDA(cudaMemsetAsync(B.counters.p, 0, C_COUNT * 4, r->stream));
    CRT_CUDA(B.waves.alloc(kMaxWaves * sizeof(uint4)));
    destroy_wave_graph(r->wave_graph);   // captured launches hold the old buffers
    r->wave_graph = nullptr;
    return CRT_OK;
}

static WaveParams wave_params(crt_render r) {
    WaveBuffers& B = r->wave;
    WaveParams W;
    W.R = make_params(r, 0, 0);
    W.st_o = B.ray_o.as<float4>();
    W.st_d = B.ray_d.as<float4>();
    W.st_c = B.color.as<float4>();
    W.st_m = B.mask.as<float4>();
    W.hit = B.hit.as<float4>();
    W.queue[0] = B.queue_a.as<uint32_t>();
    W.queue[1] = B.queue_b.as<uint32_t>();
    W.shadow = B.shadow.as<float4>();
    W.counters = B.counters.as<uint32_t>();
    W.waves = B.waves.as<uint4>();
    return W;
}

struct WaveGrids {
    int gen, ext, shd, acc;
};

// Grid sizes are queried before a capture starts.
static WaveGrids wave_grids(uint32_t capacity) {
    WaveGrids g;
    g.gen = grid_for(capacity, kWaveBlock, 16);
    g.ext = persistent_grid((const void*)wf_extend, kWaveBlock, 0);
    g.shd = persistent_grid((const void*)wf_shadow, kWaveBlock, 0);
    g.acc = grid_for(capacity, 256, 8);
    return g;
}

// Enqueue one wave; captured into the handle's graph.
static void enqueue_wave(const WaveParams& W, const WaveGrids& G, uint32_t max_depth, cudaStream_t s) {
    const int g_gen = G.gen, g_ext = G.ext, g_shd = G.shd;
    wf_generate<<<g_gen, kWaveBlock, 0, s>>>(W);
    for (uint32_t b = 0; b < max_depth; ++b) {
        wf_extend<<<g_ext, kWaveBlock, 0, s>>>(W);
        wf_shade<<<g_gen, kWaveBlock, 0, s>>>(W);
        wf_shadow<<<g_shd, kWaveBlock, 0, s>>>(W);
        wf_flip<<<1, 1, 0, s>>>(W);
    }
    wf_accumulate<<<G.acc, 256, 0, s>>>(W);
    wf_next_wave<<<1, 1, 0, s>>>(W);
}

int wavefront_pass(crt_render r, uint32_t spp0, uint32_t nspp) {
    int st = ensure_wave_buffers(r);
    if (st != CRT_OK) return st;
    WaveBuffers& B = r->wave;
    const uint32_t npix = r->width * r->height;
    // Wave descriptors: whole sample layers when the image fits, else
    // pixel ranges of one sample each.
    std::vector<uint4> waves;
    if (npix <= B.capacity) {
        const uint32_t layers = B.capacity / npix;
        for (uint32_t s = 0; s < nspp; s += layers)
            waves.push_back(make_uint4(0, npix, spp0 + s, spp0 + std::min(nspp, s + layers)));
    } else {
        for (uint32_t s = 0; s < nspp; ++s)
            for (uint32_t p = 0; p < npix; p += B.capacity)
                waves.push_back(make_uint4(p, std::min(npix, p + B.capacity), spp0 + s, spp0 + s + 1));
    }
    // The wave's launch sequence is captured once per handle and replayed.
    WaveGraph* g = static_cast<WaveGraph*>(r->wave_graph);
    if (!g) {
        g = new WaveGraph();
        r->wave_graph = g;
        const WaveParams W = wave_params(r);
        const WaveGrids G = wave_grids(B.capacity);
        CRT_CUDA(cudaGetLastError());
        CRT_CUDA(cudaStreamBeginCapture(r->stream, cudaStreamCaptureModeThreadLocal));
        enqueue_wave(W, G, r->opts.max_depth, r->stream);
        cudaError_t e = cudaStreamEndCapture(r->stream, &g->graph);
        if (e != cudaSuccess) return cuda_error(e, "capture wave graph");
        CRT_CUDA(cudaGraphInstantiate(&g->exec, g->graph, 0));
    }
    const uint32_t zero[2] = {0, 0};
    for (size_t w0 = 0; w0 < waves.size(); w0 += kMaxWaves) {
        const size_t nw = std::min<size_t>(kMaxWaves, waves.size() - w0);
        CRT_CUDA(cudaMemcpyAsync(B.waves.p, waves.data() + w0, nw * sizeof(uint4), cudaMemcpyHostToDevice,
                                 r->stream));
        // C_CUR and C_WAVE restart at zero for each chunk of descriptors
        CRT_CUDA(cudaMemcpyAsync(B.counters.as<uint32_t>() + C_CUR, zero, 8, cudaMemcpyHostToDevice, r->stream));
        for (size_t w = 0; w < nw; ++w) CRT_CUDA(cudaGraphLaunch(g->exec, r->stream));
    }
    return CRT_OK;
}

void destroy_wave_graph(void* g) { delete static_cast<WaveGraph*>(g); }

}  // namespace crt
