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
#include <mutex>
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
    C_FETCH_CNT = 7,    // work counter of the profiling count kernels
    C_COUNT = 8
};

// Profiling totals: extension rays, nodes, triangles; shadow rays, nodes, triangles.
enum ProfileCounter : uint32_t { P_EXT_RAYS, P_EXT_NODES, P_EXT_TRIS, P_SHD_RAYS, P_SHD_NODES, P_SHD_TRIS, P_COUNT };

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
    unsigned long long* prof;   // ProfileCounter totals (profiling pass only)
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

// Persistent work loop shared by the extend and shadow kernels.  REFILL: a
// lane whose ray finished takes the next queue entry at once (warp-local
// pool, one global atomic per 32 entries).  Otherwise a warp takes 32 entries
// and runs all of them to completion before taking more.  Job supplies
// start(i) (initialise the lane's traversal for queue entry i), step() and
// finish().
template <bool REFILL, class Job>
CRT_D void persistent_loop(uint32_t n, uint32_t* fetch, Job& job) {
    if (REFILL) {
        bool active = false;
        WarpPool pool;
        pool.init();
        for (;;) {
            const uint32_t i = pool.take(!active, fetch, n);
            if (i != UINT32_MAX) {
                job.start(i);
                active = true;
            }
            if (!__any_sync(0xFFFFFFFFu, active)) break;
            if (active && job.step()) {
                job.finish();
                active = false;
            }
        }
    } else {
        const uint32_t lane = threadIdx.x & 31u;
        for (;;) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(fetch, 32u);
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (base >= n) break;
            if (base + lane < n) {
                job.start(base + lane);
                while (!job.step()) {
                }
                job.finish();
            }
        }
    }
}

template <bool WHOLE_LEAF, bool F32>
struct ExtendJob {
    const WaveParams& W;
    const uint32_t* q;
    Stack& st;
    Traversal<false, false, WHOLE_LEAF, F32> T;
    uint32_t path = 0, rays = 0;

    CRT_D ExtendJob(const WaveParams& W_, const uint32_t* q_, Stack& st_) : W(W_), q(q_), st(st_) {}
    CRT_D void start(uint32_t i) {
        path = q[i];
        T.init(xyz(W.st_o[path]), xyz(W.st_d[path]), kEps, FLT_MAX, -1, st);
    }
    CRT_D bool step() { return T.step(W.R.S, st, nullptr); }
    CRT_D void finish() {
        W.hit[path] = make_float4(T.h.t, __int_as_float(T.h.face), T.h.u, T.h.v);
        ++rays;
    }
};

template <bool REFILL, bool WHOLE_LEAF, bool F32>
__global__ void __launch_bounds__(kWaveBlock) wf_extend(WaveParams W) {
    __shared__ uint2 stack_sh[kStackShared * kWaveBlock];
    Stack st;
    st.sh = stack_sh + threadIdx.x;
    st.stride = kWaveBlock;
    const uint32_t cur = W.counters[C_CUR];
    ExtendJob<WHOLE_LEAF, F32> job(W, W.queue[cur], st);
    persistent_loop<REFILL>(W.counters[cur], &W.counters[C_FETCH_EXT], job);
    count_rays(W.R.ray_counts, job.rays, 0);
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

template <bool WHOLE_LEAF, bool F32>
struct ShadowJob {
    const WaveParams& W;
    Stack& st;
    Traversal<true, false, WHOLE_LEAF, F32> T;
    uint32_t entry = 0, rays = 0;

    CRT_D ShadowJob(const WaveParams& W_, Stack& st_) : W(W_), st(st_) {}
    CRT_D void start(uint32_t i) {
        entry = i;
        const float4* e = W.shadow + 3ull * i;
        const float4 b = e[1];
        T.init(xyz(e[0]), xyz(b), kEps, b.w, (int32_t)__float_as_uint(e[2].w), st);
    }
    CRT_D bool step() { return T.step(W.R.S, st, nullptr); }
    // a visible light adds the request's contribution to the path colour
    CRT_D void finish() {
        ++rays;
        if (T.occluded) return;
        const float4* e = W.shadow + 3ull * entry;
        const uint32_t path = __float_as_uint(e[0].w);
        const float4 c = e[2];
        float4 col = W.st_c[path];
        col.x = col.x + c.x;
        col.y = col.y + c.y;
        col.z = col.z + c.z;
        W.st_c[path] = col;
    }
};

template <bool REFILL, bool WHOLE_LEAF, bool F32>
__global__ void __launch_bounds__(kWaveBlock) wf_shadow(WaveParams W) {
    __shared__ uint2 stack_sh[kStackShared * kWaveBlock];
    Stack st;
    st.sh = stack_sh + threadIdx.x;
    st.stride = kWaveBlock;
    ShadowJob<WHOLE_LEAF, F32> job(W, st);
    persistent_loop<REFILL>(W.counters[C_SHADOW], &W.counters[C_FETCH_SHD], job);
    count_rays(W.R.ray_counts, 0, job.rays);
}

using WaveKernel = void (*)(WaveParams);

// Kernel variants by the CRT_FLAG_* traversal-scheduling flags and the
// scene's node format.
template <bool F32>
static WaveKernel extend_kernel_f(uint32_t flags) {
    const bool refill = flags & CRT_FLAG_LANE_REFILL, whole = !(flags & CRT_FLAG_SPLIT_LEAF);
    if (refill) return whole ? wf_extend<true, true, F32> : wf_extend<true, false, F32>;
    return whole ? wf_extend<false, true, F32> : wf_extend<false, false, F32>;
}

template <bool F32>
static WaveKernel shadow_kernel_f(uint32_t flags) {
    const bool refill = flags & CRT_FLAG_LANE_REFILL, whole = !(flags & CRT_FLAG_SPLIT_LEAF);
    if (refill) return whole ? wf_shadow<true, true, F32> : wf_shadow<true, false, F32>;
    return whole ? wf_shadow<false, true, F32> : wf_shadow<false, false, F32>;
}

static WaveKernel extend_kernel(uint32_t flags, bool f32) {
    return f32 ? extend_kernel_f<true>(flags) : extend_kernel_f<false>(flags);
}

static WaveKernel shadow_kernel(uint32_t flags, bool f32) {
    return f32 ? shadow_kernel_f<true>(flags) : shadow_kernel_f<false>(flags);
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

__global__ void wf_reset_count_fetch(WaveParams W) { W.counters[C_FETCH_CNT] = 0; }

CRT_D void add_profile(unsigned long long* p, uint32_t rays, uint32_t nodes, uint32_t tris) {
    const uint32_t r = __reduce_add_sync(0xFFFFFFFFu, rays);
    const uint32_t n = __reduce_add_sync(0xFFFFFFFFu, nodes);
    const uint32_t t = __reduce_add_sync(0xFFFFFFFFu, tris);
    if ((threadIdx.x & 31u) == 0) {
        atomicAdd(p, (unsigned long long)r);
        atomicAdd(p + 1, (unsigned long long)n);
        atomicAdd(p + 2, (unsigned long long)t);
    }
}

// Counting re-runs (profiling only): the same traversals as wf_extend /
// wf_shadow over the same queue entries, tallying node visits and triangle
// tests instead of writing results.
template <bool F32>
__global__ void __launch_bounds__(kWaveBlock) wf_extend_count(WaveParams W) {
    __shared__ uint2 stack_sh[kStackShared * kWaveBlock];
    Stack st;
    st.sh = stack_sh + threadIdx.x;
    st.stride = kWaveBlock;
    const uint32_t cur = W.counters[C_CUR];
    const uint32_t n = W.counters[cur];
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t rays = 0;
    TraversalStats ts{0, 0};
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&W.counters[C_FETCH_CNT], 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= n) break;
        const uint32_t i = base + lane;
        if (i < n) {
            const uint32_t path = W.queue[cur][i];
            Hit h;
            h.t = FLT_MAX;
            h.face = -1;
            h.u = h.v = 0.f;
            traverse<false, true, F32>(W.R.S, xyz(W.st_o[path]), xyz(W.st_d[path]), kEps, h, -1, st, &ts);
            ++rays;
        }
    }
    add_profile(W.prof + P_EXT_RAYS, rays, ts.nodes, ts.tris);
}

template <bool F32>
__global__ void __launch_bounds__(kWaveBlock) wf_shadow_count(WaveParams W) {
    __shared__ uint2 stack_sh[kStackShared * kWaveBlock];
    Stack st;
    st.sh = stack_sh + threadIdx.x;
    st.stride = kWaveBlock;
    const uint32_t n = W.counters[C_SHADOW];
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t rays = 0;
    TraversalStats ts{0, 0};
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&W.counters[C_FETCH_CNT], 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= n) break;
        const uint32_t i = base + lane;
        if (i < n) {
            const float4* e = W.shadow + 3ull * i;
            const float4 b = e[1], c = e[2];
            Hit h;
            h.t = b.w;
            h.face = (int32_t)__float_as_uint(c.w);
            h.u = h.v = 0.f;
            traverse<true, true, F32>(W.R.S, xyz(e[0]), xyz(b), kEps, h, h.face, st, &ts);
            ++rays;
        }
    }
    add_profile(W.prof + P_SHD_RAYS, rays, ts.nodes, ts.tris);
}

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
    CRT_CUDA(B.prof.alloc(P_COUNT * sizeof(unsigned long long)));
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
    W.prof = B.prof.as<unsigned long long>();
    return W;
}

struct WaveGrids {
    int gen, ext, shd, acc;
    WaveKernel extend, shadow, extend_count, shadow_count;
};

// Kernel choice and grid sizes, queried before a capture starts.
static WaveGrids wave_grids(uint32_t capacity, uint32_t flags, bool f32) {
    WaveGrids g;
    g.extend = extend_kernel(flags, f32);
    g.shadow = shadow_kernel(flags, f32);
    g.extend_count = f32 ? wf_extend_count<true> : wf_extend_count<false>;
    g.shadow_count = f32 ? wf_shadow_count<true> : wf_shadow_count<false>;
    g.gen = grid_for(capacity, kWaveBlock, 16);
    g.ext = persistent_grid((const void*)g.extend, kWaveBlock, 0);
    g.shd = persistent_grid((const void*)g.shadow, kWaveBlock, 0);
    g.acc = grid_for(capacity, 256, 8);
    return g;
}

// Enqueue one wave; captured into the handle's graph.
static void enqueue_wave(const WaveParams& W, const WaveGrids& G, uint32_t max_depth, cudaStream_t s) {
    wf_generate<<<G.gen, kWaveBlock, 0, s>>>(W);
    for (uint32_t b = 0; b < max_depth; ++b) {
        G.extend<<<G.ext, kWaveBlock, 0, s>>>(W);
        wf_shade<<<G.gen, kWaveBlock, 0, s>>>(W);
        G.shadow<<<G.shd, kWaveBlock, 0, s>>>(W);
        wf_flip<<<1, 1, 0, s>>>(W);
    }
    wf_accumulate<<<G.acc, 256, 0, s>>>(W);
    wf_next_wave<<<1, 1, 0, s>>>(W);
}

// Wave descriptors: whole sample layers when the image fits, else pixel
// ranges of one sample each.
static std::vector<uint4> make_waves(uint32_t npix, uint32_t capacity, uint32_t spp0, uint32_t nspp) {
    std::vector<uint4> waves;
    if (npix <= capacity) {
        const uint32_t layers = capacity / npix;
        for (uint32_t s = 0; s < nspp; s += layers)
            waves.push_back(make_uint4(0, npix, spp0 + s, spp0 + std::min(nspp, s + layers)));
    } else {
        for (uint32_t s = 0; s < nspp; ++s)
            for (uint32_t p = 0; p < npix; p += capacity)
                waves.push_back(make_uint4(p, std::min(npix, p + capacity), spp0 + s, spp0 + s + 1));
    }
    return waves;
}

// Uploads one chunk of descriptors and restarts C_CUR / C_WAVE at zero.
static int upload_waves(crt_render r, const std::vector<uint4>& waves, size_t w0, size_t nw) {
    WaveBuffers& B = r->wave;
    const uint32_t zero[2] = {0, 0};
    CRT_CUDA(cudaMemcpyAsync(B.waves.p, waves.data() + w0, nw * sizeof(uint4), cudaMemcpyHostToDevice,
                             r->stream));
    CRT_CUDA(cudaMemcpyAsync(B.counters.as<uint32_t>() + C_CUR, zero, 8, cudaMemcpyHostToDevice, r->stream));
    return CRT_OK;
}

int wavefront_pass(crt_render r, uint32_t spp0, uint32_t nspp) {
    int st = ensure_wave_buffers(r);
    if (st != CRT_OK) return st;
    WaveBuffers& B = r->wave;
    const std::vector<uint4> waves = make_waves(r->width * r->height, B.capacity, spp0, nspp);
    // The wave's launch sequence is captured once per handle and replayed.
    WaveGraph* g = static_cast<WaveGraph*>(r->wave_graph);
    if (!g) {
        g = new WaveGraph();
        r->wave_graph = g;
        const WaveParams W = wave_params(r);
        const WaveGrids G = wave_grids(B.capacity, r->opts.flags, r->scene->dev.fnodes != nullptr);
        CRT_CUDA(cudaGetLastError());
        // Captured on a private stream: the caller's stream may be the legacy
        // default stream, which cannot be captured.  The graph is launched on
        // the caller's stream below.
        cudaStream_t cap = nullptr;
        CRT_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            enqueue_wave(W, G, r->opts.max_depth, cap);
            e = cudaStreamEndCapture(cap, &g->graph);
        }
        cudaStreamDestroy(cap);
        if (e != cudaSuccess) return cuda_error(e, "capture wave graph");
        CRT_CUDA(cudaGraphInstantiate(&g->exec, g->graph, 0));
    }
    for (size_t w0 = 0; w0 < waves.size(); w0 += kMaxWaves) {
        const size_t nw = std::min<size_t>(kMaxWaves, waves.size() - w0);
        if ((st = upload_waves(r, waves, w0, nw)) != CRT_OK) return st;
        for (size_t w = 0; w < nw; ++w) CRT_CUDA(cudaGraphLaunch(g->exec, r->stream));
    }
    return CRT_OK;
}

// Same launch sequence as enqueue_wave(), one kernel at a time with CUDA
// events around each launch, plus untimed counting re-runs of each traversal.
int wavefront_profile_pass(crt_render r, uint32_t spp0, uint32_t nspp, crt_stage_profile* out) {
    int st = ensure_wave_buffers(r);
    if (st != CRT_OK) return st;
    WaveBuffers& B = r->wave;
    const std::vector<uint4> waves = make_waves(r->width * r->height, B.capacity, spp0, nspp);
    const WaveParams W = wave_params(r);
    const WaveGrids G = wave_grids(B.capacity, r->opts.flags, r->scene->dev.fnodes != nullptr);
    CRT_CUDA(cudaMemsetAsync(B.prof.p, 0, B.prof.bytes, r->stream));
    cudaEvent_t e0, e1;
    CRT_CUDA(cudaEventCreate(&e0));
    CRT_CUDA(cudaEventCreate(&e1));
    cudaStream_t s = r->stream;
    cudaError_t err = cudaSuccess;
    auto timed = [&](int stage, auto launch) {
        if (err != cudaSuccess) return;
        cudaEventRecord(e0, s);
        launch();
        cudaEventRecord(e1, s);
        err = cudaEventSynchronize(e1);
        if (err == cudaSuccess) err = cudaGetLastError();
        float ms = 0.f;
        if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
        out->ms[stage] += ms;
        out->launches[stage] += 1;
    };
    for (size_t w0 = 0; w0 < waves.size() && err == cudaSuccess; w0 += kMaxWaves) {
        const size_t nw = std::min<size_t>(kMaxWaves, waves.size() - w0);
        if ((st = upload_waves(r, waves, w0, nw)) != CRT_OK) break;
        for (size_t w = 0; w < nw; ++w) {
            timed(0, [&] { wf_generate<<<G.gen, kWaveBlock, 0, s>>>(W); });
            for (uint32_t b = 0; b < r->opts.max_depth; ++b) {
                timed(1, [&] { G.extend<<<G.ext, kWaveBlock, 0, s>>>(W); });
                wf_reset_count_fetch<<<1, 1, 0, s>>>(W);
                G.extend_count<<<G.ext, kWaveBlock, 0, s>>>(W);
                timed(2, [&] { wf_shade<<<G.gen, kWaveBlock, 0, s>>>(W); });
                timed(3, [&] { G.shadow<<<G.shd, kWaveBlock, 0, s>>>(W); });
                wf_reset_count_fetch<<<1, 1, 0, s>>>(W);
                G.shadow_count<<<G.shd, kWaveBlock, 0, s>>>(W);
                timed(5, [&] { wf_flip<<<1, 1, 0, s>>>(W); });
            }
            timed(4, [&] { wf_accumulate<<<G.acc, 256, 0, s>>>(W); });
            timed(5, [&] { wf_next_wave<<<1, 1, 0, s>>>(W); });
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != CRT_OK) return st;
    if (err != cudaSuccess) return cuda_error(err, "profiled wavefront pass");
    unsigned long long c[P_COUNT];
    CRT_CUDA(cudaMemcpyAsync(c, B.prof.p, sizeof(c), cudaMemcpyDeviceToHost, s));
    CRT_CUDA(cudaStreamSynchronize(s));
    out->extension_rays += c[P_EXT_RAYS];
    out->extension_nodes += c[P_EXT_NODES];
    out->extension_tris += c[P_EXT_TRIS];
    out->shadow_rays += c[P_SHD_RAYS];
    out->shadow_nodes += c[P_SHD_NODES];
    out->shadow_tris += c[P_SHD_TRIS];
    return CRT_OK;
}

void destroy_wave_graph(void* g) { delete static_cast<WaveGraph*>(g); }

// ---------------------------------------------------------------------------
// Allocation-free tile renders (crt_render_tile_noalloc).
//
// Some callers cannot allocate device memory at render time: a host
// application that owns every device allocation through its own pool (a
// plugin inside a DCC tool or game engine), or a latency-sensitive loop that
// must not pay for cudaMalloc / cudaFree and the synchronisation they imply.
// For them the wavefront kernels can run on a fixed scratch area that lives
// in this file as a static device array: every GPU that loads the library
// holds kNoAllocBytes (about 8.5 MiB) of it until the process exits.  The
// caller brings the inputs (a scene) and the output (an accumulator); the
// paths in flight, queues, counters and the wave descriptor use the scratch.
// ---------------------------------------------------------------------------
Camera to_device_camera(const crt_camera& c);

constexpr uint32_t kNoAllocPaths = CRT_NOALLOC_MAX_PATHS;
constexpr size_t kNoAllocOff[] = {
    0,                                  // ray_o    16 B per path
    16ull * kNoAllocPaths,              // ray_d
    32ull * kNoAllocPaths,              // color
    48ull * kNoAllocPaths,              // mask
    64ull * kNoAllocPaths,              // hit
    80ull * kNoAllocPaths,              // queue 0  4 B per path
    84ull * kNoAllocPaths,              // queue 1
    88ull * kNoAllocPaths,              // shadow requests 48 B per path
    136ull * kNoAllocPaths,             // counters (C_COUNT words), then the wave descriptor
    136ull * kNoAllocPaths + 256,       // ray counts (2 x u64)
};
constexpr size_t kNoAllocBytes = 136ull * kNoAllocPaths + 512;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Device address of the scratch on each device, looked up once per device.
static std::mutex g_noalloc_mutex;
static void* g_noalloc_addr[64] = {};

static int noalloc_scratch(void** out) {
    int dev = 0;
    CRT_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_error(CRT_ERR_LIMIT, "device ordinal above 63");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        // the array's host-side name is only a handle: the kernels need the
        // device address, which belongs to the current device
        CRT_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return CRT_OK;
}

// Starts a call: clears the counters and ray counts and installs the wave
// descriptor (everything that must start at zero; path state is always
// written before it is read).
__global__ void wf_noalloc_begin(WaveParams W, uint4 wave) {
    for (int i = 0; i < C_COUNT; ++i) W.counters[i] = 0;
    W.R.ray_counts[0] = W.R.ray_counts[1] = 0;
    const_cast<uint4*>(W.waves)[0] = wave;
}

}  // namespace crt

using namespace crt;

extern "C" int crt_render_tile_noalloc(crt_scene scene, const crt_camera* camera, uint32_t width,
                                       uint32_t height, const crt_render_options* opts, uint32_t pixel0,
                                       uint32_t pixel_count, uint32_t spp0, uint32_t nspp, float* d_accum,
                                       void* stream) {
    if (!scene || !camera || !d_accum) return set_error(CRT_ERR_INVALID, "crt_render_tile_noalloc: null argument");
    if (width == 0 || height == 0 || (uint64_t)width * height >= (1ull << 31))
        return set_error(CRT_ERR_INVALID, "crt_render_tile_noalloc: bad image size");
    if (pixel_count == 0 || nspp == 0) return CRT_OK;
    if ((uint64_t)pixel0 + pixel_count > (uint64_t)width * height)
        return set_error(CRT_ERR_INVALID, "crt_render_tile_noalloc: pixel range outside the image");
    if ((uint64_t)pixel_count * nspp > kNoAllocPaths)
        return set_error(CRT_ERR_LIMIT, "crt_render_tile_noalloc: pixel_count * nspp exceeds "
                                        "CRT_NOALLOC_MAX_PATHS (65536 paths in flight)");
    if ((uint64_t)spp0 + nspp >= (1ull << 32)) return set_error(CRT_ERR_LIMIT, "sample index overflow");
    if (((uintptr_t)d_accum & 15u) != 0) return set_error(CRT_ERR_INVALID, "d_accum must be 16-byte aligned");
    crt_render_options o;
    if (opts) o = *opts;
    else crt_render_options_default(&o);
    if (o.max_depth == 0 || o.max_depth > 1024) return set_error(CRT_ERR_INVALID, "max_depth must be in [1, 1024]");
    void* base = nullptr;
    int st = noalloc_scratch(&base);
    if (st != CRT_OK) return st;
    unsigned char* b = static_cast<unsigned char*>(base);
    WaveParams W;
    RenderParams& R = W.R;
    R.S = scene->dev;
    R.cam = to_device_camera(*camera);
    R.accum = reinterpret_cast<float4*>(d_accum);
    R.width = width;
    R.height = height;
    R.seed = o.seed;
    R.view = o.view_id;
    R.spp0 = spp0;
    R.nspp = nspp;
    R.max_depth = o.max_depth;
    R.ray_counts = reinterpret_cast<unsigned long long*>(b + kNoAllocOff[9]);
    W.st_o = reinterpret_cast<float4*>(b + kNoAllocOff[0]);
    W.st_d = reinterpret_cast<float4*>(b + kNoAllocOff[1]);
    W.st_c = reinterpret_cast<float4*>(b + kNoAllocOff[2]);
    W.st_m = reinterpret_cast<float4*>(b + kNoAllocOff[3]);
    W.hit = reinterpret_cast<float4*>(b + kNoAllocOff[4]);
    W.queue[0] = reinterpret_cast<uint32_t*>(b + kNoAllocOff[5]);
    W.queue[1] = reinterpret_cast<uint32_t*>(b + kNoAllocOff[6]);
    W.shadow = reinterpret_cast<float4*>(b + kNoAllocOff[7]);
    W.counters = reinterpret_cast<uint32_t*>(b + kNoAllocOff[8]);
    W.waves = reinterpret_cast<const uint4*>(b + kNoAllocOff[8] + 64);
    W.prof = nullptr;
    const WaveGrids G = wave_grids(kNoAllocPaths, o.flags, scene->dev.fnodes != nullptr);
    cudaStream_t s = (cudaStream_t)stream;
    wf_noalloc_begin<<<1, 1, 0, s>>>(W, make_uint4(pixel0, pixel0 + pixel_count, spp0, spp0 + nspp));
    wf_generate<<<G.gen, kWaveBlock, 0, s>>>(W);
    for (uint32_t k = 0; k < o.max_depth; ++k) {
        G.extend<<<G.ext, kWaveBlock, 0, s>>>(W);
        wf_shade<<<G.gen, kWaveBlock, 0, s>>>(W);
        G.shadow<<<G.shd, kWaveBlock, 0, s>>>(W);
        wf_flip<<<1, 1, 0, s>>>(W);
    }
    wf_accumulate<<<G.acc, 256, 0, s>>>(W);
    CRT_CUDA(cudaGetLastError());
    return CRT_OK;
}
