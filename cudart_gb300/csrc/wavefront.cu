// wavefront.cu -- the wavefront form of the path tracer.
//
// A pass is cut into waves of at most `capacity` paths.  A wave is a list of
// segments, each a pixel range x a sample range of one view (a single render
// has one view; a batch many), and holds each pixel of a view at most once.
// One wave runs
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
RenderParams make_params(crt_render r, uint32_t view, uint32_t spp0, uint32_t nspp);

constexpr int kWaveBlock = 128;            // generate / shade / counting kernels
constexpr int kTraversalBlockMax = 256;    // extend / shadow: block size chosen at launch
// Register cap of the traversal kernels: fewer registers, more resident
// warps to hide the dependent node loads (measured: 56 beats 64, 48 and 40).
#ifndef CRT_TRAVERSAL_REGS
#define CRT_TRAVERSAL_REGS 56
#endif
// FP32 planes: 56 as well since the window sort (+0.6% on the 1080p frame,
// +1.1% on the mixed scene over 64, 16 bytes of spill; 72 loses 2-3%).
#ifndef CRT_TRAVERSAL_REGS_F32
#define CRT_TRAVERSAL_REGS_F32 56
#endif
constexpr uint32_t kDefaultWaveSets = 4;   // measured: 4 x 32M-path sets +1.2% over 3 at 1080p
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
    C_OCT0 = 8,         // octant-binned queues: entries per octant of queue 0 (8 words)
    C_OCT1 = 16,        //                       and of queue 1 (8 words)
    C_COUNT = 24
};

// Profiling totals: extension rays, nodes, triangles; shadow rays, nodes, triangles.
// Visits to the staged top nodes: P_EXT_TOP, P_SHD_TOP.
enum ProfileCounter : uint32_t {
    P_EXT_RAYS, P_EXT_NODES, P_EXT_TRIS, P_SHD_RAYS, P_SHD_NODES, P_SHD_TRIS, P_EXT_TOP, P_SHD_TOP, P_COUNT
};

// Pixels [p0, p1) x samples [s0, s1) of view `view`: path slot0 +
// seg_slot(k, s) carries sample s0 + s of the k-th pixel of the range
// (seg_pixel); the segment's pixels are entries [pix0, pix0 + p1 - p0) of
// the wave's accumulate range.
struct WaveSeg {
    uint32_t view, p0, p1, s0, s1, slot0, pix0;
    uint32_t band;   // nonzero: the range is whole bands of this many pixels (4 rows of a view whose width is a
                     // multiple of 8), walked in 8x4 tiles of 2x2 quads, each quad's samples together
};

// The k-th pixel of a segment's range: row order, or on whole 4-row bands
// 8x4 tiles left to right, each as eight 2x2 quads, so a warp's paths start
// from one tile or quad (closer rays than a 32-pixel row).  A bijection on
// [p0, p1) either way, shared by the path generator and the accumulator.
CRT_D uint32_t seg_pixel(const WaveSeg& sg, uint32_t k) {
    if (!sg.band) return sg.p0 + k;
    const uint32_t b = k / sg.band, r = k - b * sg.band, w = sg.band >> 2;
    // within a tile, 2x2 quads: u = quad * 4 + pixel of the quad
    const uint32_t u = r & 31u, qd = u >> 2, q = u & 3u;
    const uint32_t x = ((r >> 5) << 3) | ((qd & 3u) << 1) | (q & 1u), y = ((qd >> 2) << 1) | (q >> 1);
    return sg.p0 + b * sg.band + y * w + x;
}

// Path slot (from the segment's slot0) of sample s of the k-th pixel, and
// back.  Row-order segments hold whole sample layers one after another;
// tiled segments hold each 2x2 quad's samples together (4 pixels x ns
// samples), so the 32 paths of a warp start from nearly the same camera
// rays (measured +5.6% on the 1080p frame over sample layers of 8x4 tiles,
// +1.2% on the mixed scene).
CRT_D uint32_t seg_slot(const WaveSeg& sg, uint32_t k, uint32_t s) {
    const uint32_t ns = sg.s1 - sg.s0;
    return sg.band ? (k >> 2) * 4u * ns + s * 4u + (k & 3u) : s * (sg.p1 - sg.p0) + k;
}
CRT_D void seg_slot_inv(const WaveSeg& sg, uint32_t j, uint32_t& k, uint32_t& s) {
    const uint32_t ns = sg.s1 - sg.s0, np = sg.p1 - sg.p0;
    if (sg.band) {
        const uint32_t g = j / (4u * ns), r = j - g * 4u * ns;
        s = r >> 2;
        k = g * 4u + (r & 3u);
    } else {
        s = j / np;
        k = j - s * np;
    }
}

// Path state word (mask record .w): previous bsdf (8 bits), bounce (11
// bits), view.
constexpr uint32_t kBounceShift = 8, kViewShift = 19;

// A path's state is two 32-byte records, each moved with one 256-bit access
// (a warp whose paths are scattered issues half the load and store
// instructions of four 16-byte arrays):
//   st_od[2i], st_od[2i+1]: o.xyz, pixel within its view | d.xyz, sample
//   st_cm[2i], st_cm[2i+1]: color.xyz, rng draws | mask.xyz, state word
CRT_D void ld_pair(const float4* p, float4& a, float4& b) {
    asm volatile("ld.global.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
                 : "l"(p));
}
CRT_D void st_pair(float4* p, float4 a, float4 b) {
    asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "f"(a.x), "f"(a.y),
                 "f"(a.z), "f"(a.w), "f"(b.x), "f"(b.y), "f"(b.z), "f"(b.w)
                 : "memory");
}

struct WaveParams {
    RenderParams R;     // scene, seed, depth, ray counts; R.accum = all views
    const DevView* views;
    float4* st_od;      // per path (32-byte aligned pairs): o.xyz, pixel | d.xyz, sample
    float4* st_cm;      // color.xyz, rng draws | mask.xyz, prev | bounce << 8 | view << 19
    float4* hit;        // t, face, u, v
    uint32_t* queue[2];
    float4* shadow;     // 3 float4 per request
    uint32_t* shadow_q; // window sort: request slots (= queue entries) in traversal order, else null
    uint32_t* counters;
    const uint4* waves; // first segment, segments, paths, accumulate entries
    const WaveSeg* segs;
    unsigned long long* prof;   // ProfileCounter totals (profiling pass only)
    int stack_depth;            // traversal stack entries in shared memory
    uint32_t queue_chunk;       // queue entries a warp claims per fetch (batch mode)
    uint32_t top_nodes;         // BVH nodes staged in shared memory by extend / shadow
    uint32_t refill_busy;       // lane refill: busy lanes at or below which idle lanes refill
    // adjoint replay only
    const float4* adj;          // d(objective)/d(radiance sum), per pixel of every view
    float4* st_L;               // radiance of each path's primal trace
    float4* st_W;               // adjoint weight of each path's pixel
    float4* shd_grad;           // per shadow request: w * d contrib / d ka, light material
    float* grad_kd;             // [n_mats][3], added to
    float* grad_ka;             // [n_mats][3], added to
    uint32_t n_mats;
    uint16_t* adj_hist;         // exact roulette: [capacity][kHistMax] kd-factor materials
    bool adj_exact;
    // octant-binned extension queues: queue q holds 8 regions of `capacity`
    // entries, region k the paths whose next ray points into octant k
    bool octant;
    uint32_t capacity;
};

// Queue entries read back in region order (octant 0 first), keeping each
// region's order.  `pre` is the prefix of the 8 region counts, in shared
// memory; without octant binning a queue is one region.
struct QueueView {
    const uint32_t* q;
    const uint32_t* pre;   // [9], or null
    uint32_t cap;
    CRT_D uint32_t at(uint32_t i) const {
        if (!pre) return q[i];
        uint32_t k = 0;
        while (i >= pre[k + 1]) ++k;
        return q[(size_t)k * cap + (i - pre[k])];
    }
};

// Builds the region prefix of queue `which` in shared memory (one block).
CRT_D QueueView queue_view(const WaveParams& W, uint32_t which, uint32_t* pre_sh) {
    QueueView v{W.queue[which], nullptr, W.capacity};
    if (!W.octant) return v;
    if (threadIdx.x == 0) {
        uint32_t s = 0;
        pre_sh[0] = 0;
        for (int k = 0; k < 8; ++k) {
            s += W.counters[(which ? C_OCT1 : C_OCT0) + k];
            pre_sh[k + 1] = s;
        }
    }
    __syncthreads();
    v.pre = pre_sh;
    return v;
}

// Exact-roulette bookkeeping per path, kept in st_W.w: history length
// (bits 0-4); history length and channel at the previous applied roulette
// (5-9, 10-11); a surviving roulette not yet applied (flag 19) with its
// history length and channel (12-16, 17-18).
constexpr uint32_t kHistMax = 16;
CRT_D uint32_t hist_len(uint32_t meta) { return meta & 31u; }
CRT_D uint32_t hist_prev_len(uint32_t meta) { return (meta >> 5) & 31u; }
CRT_D uint32_t hist_prev_channel(uint32_t meta) { return (meta >> 10) & 3u; }
CRT_D uint32_t hist_pend_len(uint32_t meta) { return (meta >> 12) & 31u; }
CRT_D uint32_t hist_pend_channel(uint32_t meta) { return (meta >> 17) & 3u; }
constexpr uint32_t kHistPending = 1u << 19;

// ---------------------------------------------------------------------------
// Adjoint (path-replay backpropagation) helpers.  Gradients are summed per
// block in shared memory, [n_mats][6] = kd rgb, ka rgb; within a warp the
// lanes adding to the same material are summed first, so each warp issues
// one shared atomic per material and channel.
// ---------------------------------------------------------------------------
CRT_D void warp_add_grad(float* acc, uint32_t key, uint32_t off, float3 v) {
    const uint32_t active = __activemask();
    const uint32_t peers = __match_any_sync(active, key);
    float3 s = f3(0.f, 0.f, 0.f);
    for (uint32_t rest = active; rest; rest &= rest - 1u) {
        const int j = __ffs(rest) - 1;
        const float x = __shfl_sync(active, v.x, j);
        const float y = __shfl_sync(active, v.y, j);
        const float z = __shfl_sync(active, v.z, j);
        if ((peers >> j) & 1u) s = s + f3(x, y, z);
    }
    if ((int)(threadIdx.x & 31u) == __ffs(peers) - 1) {
        float* a = acc + 6u * key + off;
        atomicAdd(a, s.x);
        atomicAdd(a + 1, s.y);
        atomicAdd(a + 2, s.z);
    }
}

CRT_D void zero_grad_block(float* acc, uint32_t n_mats) {
    for (uint32_t i = threadIdx.x; i < 6u * n_mats; i += blockDim.x) acc[i] = 0.f;
    __syncthreads();
}

CRT_D void flush_grad_block(const WaveParams& W, const float* acc) {
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < 6u * W.n_mats; i += blockDim.x) {
        const float v = acc[i];
        if (v == 0.f) continue;
        const uint32_t m = i / 6u, k = i % 6u;
        atomicAdd(k < 3u ? W.grad_kd + 3u * m + k : W.grad_ka + 3u * m + (k - 3u), v);
    }
}

CRT_D float channel(float3 v, uint32_t c) { return c == 0 ? v.x : c == 1 ? v.y : v.z; }
CRT_D float3 in_channel(uint32_t c, float x) { return f3(c == 0 ? x : 0.f, c == 1 ? x : 0.f, c == 2 ? x : 0.f); }

// The shade_hit hooks of the replay (see NoGrad): w is the adjoint weight of
// the path's pixel, total the radiance its primal trace returned.
struct WaveGrad {
    static constexpr bool kActive = true;
    float* acc;
    float3 w, total;
    const DevScene* S = nullptr;   // exact roulette only: kd of history entries
    uint16_t* hist = nullptr;      // this path's history, or null (constant survival probability)
    uint32_t meta = 0;
    CRT_D void emission(uint32_t m, float3 d) { warp_add_grad(acc, m, 3, w * d); }
    CRT_D void albedo(uint32_t m, float3 kd, float3 color) {
        const float3 rest = total - color;
        const float3 g = f3(kd.x != 0.f ? w.x * rest.x / kd.x : 0.f, kd.y != 0.f ? w.y * rest.y / kd.y : 0.f,
                            kd.z != 0.f ? w.z * rest.z / kd.z : 0.f);
        warp_add_grad(acc, m, 0, g);
        if (hist && hist_len(meta) < kHistMax) {
            hist[hist_len(meta)] = (uint16_t)m;
            ++meta;
        }
    }
    // After a surviving roulette the throughput is mask / mask[c] (c the
    // channel max_component picks): every later term gets -1/kd[c] per kd
    // factor so far, in channel c, replacing the previous roulette's
    // correction.  "Later" starts after this vertex's light sample, which the
    // shadow kernel adds after shade, so the correction is recorded here and
    // applied at the path's next shade (a path that ends first adds nothing
    // later, and its correction is zero).
    CRT_D void roulette(float3 mask, float3) {
        if (!hist) return;
        const uint32_t c01 = mask.x > mask.y ? 0u : 1u;
        const float v01 = mask.x > mask.y ? mask.x : mask.y;
        const uint32_t c = v01 > mask.z ? c01 : 2u;
        meta = (meta & 0xFFFu) | (hist_len(meta) << 12) | (c << 17) | kHistPending;
    }
    // The pending roulette correction, with `color` the radiance the path
    // had gathered by the end of that roulette's vertex.
    CRT_D void apply_pending(float3 color) {
        if (!hist || !(meta & kHistPending)) return;
        const float3 rest = total - color;
        const float s = w.x * rest.x + w.y * rest.y + w.z * rest.z;
        const uint32_t n = hist_pend_len(meta), c = hist_pend_channel(meta);
        const uint32_t pn = hist_prev_len(meta), pc = hist_prev_channel(meta);
        for (uint32_t i = 0; i < n; ++i) {
            const uint32_t m = hist[i];
            const float k = channel(load_material(*S, m).kd, c);
            warp_add_grad(acc, m, 0, in_channel(c, k != 0.f ? -s / k : 0.f));
        }
        for (uint32_t i = 0; i < pn; ++i) {
            const uint32_t m = hist[i];
            const float k = channel(load_material(*S, m).kd, pc);
            warp_add_grad(acc, m, 0, in_channel(pc, k != 0.f ? s / k : 0.f));
        }
        meta = hist_len(meta) | (n << 5) | (c << 10);
    }
};

CRT_D uint4 wave_desc(const WaveParams& W) { return W.waves[W.counters[C_WAVE]]; }

CRT_D void store_state(const WaveParams& W, uint32_t i, const PathState& ps, const Ray& ray, uint32_t pixel,
                       uint32_t sample, uint32_t view) {
    st_pair(W.st_od + 2ull * i, make_float4(ray.o.x, ray.o.y, ray.o.z, __uint_as_float(pixel)),
            make_float4(ray.d.x, ray.d.y, ray.d.z, __uint_as_float(sample)));
    const uint32_t word = (uint32_t)ps.prev | (ps.bounce << kBounceShift) | (view << kViewShift);
    st_pair(W.st_cm + 2ull * i, make_float4(ps.color.x, ps.color.y, ps.color.z, __uint_as_float(ps.rng.n)),
            make_float4(ps.mask.x, ps.mask.y, ps.mask.z, __uint_as_float(word)));
}

// The segment of a wave holding entry i: the last of segs[0, n) whose
// start (slot0, or pix0 when by_pixel) is <= i.
CRT_D uint32_t find_segment(const WaveSeg* segs, uint32_t n, uint32_t i, bool by_pixel) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        const uint32_t start = by_pixel ? segs[mid].pix0 : segs[mid].slot0;
        if (start <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Warp-aggregated append into one of `nkeys` regions: the lanes that want
// region `key` share one atomic on counters[key]; returns this lane's slot in
// it.
CRT_D uint32_t warp_append_keyed(uint32_t* counters, bool want, uint32_t key, uint32_t nkeys = 8u) {
    const uint32_t active = __activemask();
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t peers = __match_any_sync(active, want ? key : nkeys) & __ballot_sync(active, want);
    uint32_t base = 0;
    const int leader = __ffs(peers) - 1;
    if (want && (int)lane == leader) base = atomicAdd(counters + key, __popc(peers));
    // every lane reads its group leader's base (lanes without work read their own)
    base = __shfl_sync(active, base, want ? leader : (int)lane);
    return base + __popc(peers & ((1u << lane) - 1u));
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

// REPLAY: the adjoint's second trace; each slot first keeps the radiance its
// primal trace left in its colour and picks up its pixel's adjoint weight.
template <bool REPLAY>
__global__ void __launch_bounds__(kWaveBlock) wf_generate(WaveParams W) {
    const uint4 wd = wave_desc(W);
    const WaveSeg* segs = W.segs + wd.x;
    const uint32_t n = wd.z;
    const uint32_t cur = W.counters[C_CUR];
    for (uint32_t i = blockIdx.x * kWaveBlock + threadIdx.x; i < n; i += gridDim.x * kWaveBlock) {
        const WaveSeg sg = segs[find_segment(segs, wd.y, i, false)];
        uint32_t k, s;
        seg_slot_inv(sg, i - sg.slot0, k, s);
        const uint32_t pixel = seg_pixel(sg, k), sample = sg.s0 + s;
        const DevView& V = W.views[sg.view];
        if (REPLAY) {
            W.st_L[i] = W.st_cm[2ull * i];
            float4 a = W.adj[V.pix_off + pixel];
            a.w = __uint_as_float(0u);   // exact-roulette history: empty
            W.st_W[i] = a;
        }
        PathState ps;
        Ray ray;
        begin_path(V.cam, W.R.seed, V.view_id, pixel % V.width, pixel / V.width, pixel, sample, ps, ray);
        store_state(W, i, ps, ray, pixel, sample, sg.view);
        W.queue[cur][i] = i;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        W.counters[cur] = n;
        W.counters[cur ^ 1u] = 0;
        if (W.octant)   // camera rays: one region, in pixel order
            for (int k = 0; k < 8; ++k) {
                W.counters[(cur ? C_OCT1 : C_OCT0) + k] = k == 0 ? n : 0u;
                W.counters[(cur ? C_OCT0 : C_OCT1) + k] = 0;
            }
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
CRT_D void persistent_loop(uint32_t n, uint32_t* fetch, uint32_t chunk, uint32_t refill_busy, Job& job) {
    if (REFILL) {
        // idle lanes take new entries together, once at most `refill_busy`
        // lanes of the warp are still busy (31: as soon as one is idle)
        bool active = false;
        WarpPool pool;
        pool.init();
        for (;;) {
            if ((uint32_t)__popc(__ballot_sync(0xFFFFFFFFu, active)) <= refill_busy) {
                const uint32_t i = pool.take(!active, fetch, n);
                if (i != UINT32_MAX) {
                    job.start(i);
                    active = true;
                }
                if (!__any_sync(0xFFFFFFFFu, active)) break;
            }
            if (active && job.step()) {
                job.finish();
                active = false;
            }
        }
    } else {
        // each warp claims `chunk` entries (a multiple of 32) per atomic
        const uint32_t lane = threadIdx.x & 31u;
        for (;;) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(fetch, chunk);
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (base >= n) break;
            const uint32_t end = min(base + chunk, n);
            for (uint32_t i = base + lane; i < end; i += 32u) {
                job.start(i);
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
    QueueView q;
    Stack& st;
    Traversal<false, false, WHOLE_LEAF, F32> T;
    uint32_t path = 0, rays = 0;

    CRT_D ExtendJob(const WaveParams& W_, QueueView q_, Stack& st_) : W(W_), q(q_), st(st_) {}
    CRT_D void start(uint32_t i) {
        path = q.at(i);
        float4 o, d;
        ld_pair(W.st_od + 2ull * path, o, d);
        T.init(xyz(o), xyz(d), kEps, FLT_MAX, -1, st, W.R.S.max_visits);
    }
    CRT_D bool step() { return T.step(W.R.S, st, nullptr); }
    CRT_D void finish() {
        W.hit[path] = make_float4(T.h.t, __int_as_float(T.h.face), T.h.u, T.h.v);
        ++rays;
    }
};

// Copies the first W.top_nodes nodes to the start of dynamic shared memory
// and returns where the stacks begin (TOP = false: no staging at all).
template <bool F32, bool TOP>
CRT_D uint2* stage_top_nodes(const WaveParams& W) {
    if (!TOP) return reinterpret_cast<uint2*>(crt_top_nodes);
    const uint32_t n = W.top_nodes * (F32 ? 13u : 5u);
    const float4* src = F32 ? W.R.S.fnodes : W.R.S.nodes;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) crt_top_nodes[i] = ldg(src + i);
    __syncthreads();
    return reinterpret_cast<uint2*>(crt_top_nodes + n);
}

template <bool REFILL, bool WHOLE_LEAF, bool F32, bool TOP>
__global__ void __maxnreg__(F32 ? CRT_TRAVERSAL_REGS_F32 : CRT_TRAVERSAL_REGS) wf_extend(WaveParams W) {
    uint2* stacks = stage_top_nodes<F32, TOP>(W);
    Stack st;
    st.setup(stacks, blockDim.x, W.stack_depth, TOP ? W.top_nodes : 0u);
    const uint32_t cur = W.counters[C_CUR];
    __shared__ uint32_t pre_sh[9];
    ExtendJob<WHOLE_LEAF, F32> job(W, queue_view(W, cur, pre_sh), st);
    persistent_loop<REFILL>(W.counters[cur], &W.counters[C_FETCH_EXT], W.queue_chunk, W.refill_busy, job);
    count_rays(W.R.ray_counts, job.rays, 0);
}

// One bounce of queue entry i (< n): loads the path, shades its hit (or
// miss), stores the path back and reports whether it continues, its shadow
// request and its next direction.  ADJ: the adjoint replay, the same bounce
// with gradient hooks summed into grad_sh.
template <bool ADJ>
CRT_D void shade_entry(const WaveParams& W, const QueueView& q, uint32_t i, float* grad_sh, uint32_t& path,
                       bool& alive, ShadowReq& sr, float3& dir) {
    path = q.at(i);
    float4 o, d, c, m;
    ld_pair(W.st_od + 2ull * path, o, d);
    ld_pair(W.st_cm + 2ull * path, c, m);
    const float4 hv = W.hit[path];
    const uint32_t pixel = __float_as_uint(o.w), sample = __float_as_uint(d.w);
    const uint32_t pb = __float_as_uint(m.w);
    const uint32_t view = pb >> kViewShift;
    PathState ps;
    ps.color = xyz(c);
    ps.mask = xyz(m);
    ps.prev = (int)(pb & 0xFFu);
    ps.bounce = (pb >> kBounceShift) & ((1u << (kViewShift - kBounceShift)) - 1u);
    ps.rng.init(W.R.seed, W.views[view].view_id, pixel, sample, __float_as_uint(c.w));
    Ray ray;
    ray.o = xyz(o);
    ray.d = xyz(d);
    Hit h;
    h.t = hv.x;
    h.face = __float_as_int(hv.y);
    h.u = hv.z;
    h.v = hv.w;
    if (ADJ) {
        const float4 wv = W.st_W[path];
        WaveGrad g{grad_sh, xyz(wv), xyz(W.st_L[path])};
        if (W.adj_exact) {
            g.S = &W.R.S;
            g.hist = W.adj_hist + (size_t)path * kHistMax;
            g.meta = __float_as_uint(wv.w);
            g.apply_pending(ps.color);
        }
        if (h.face < 0) {
            shade_miss(ps);
        } else {
            alive = shade_hit(W.R, ps, ray, h, sr, &g) && ps.bounce < W.R.max_depth;
        }
        if (W.adj_exact) W.st_W[path].w = __uint_as_float(g.meta);
    } else if (h.face < 0) {
        shade_miss(ps);
    } else {
        alive = shade_hit(W.R, ps, ray, h, sr) && ps.bounce < W.R.max_depth;
    }
    store_state(W, path, ps, ray, pixel, sample, view);
    dir = ray.d;
}

template <bool ADJ>
CRT_D void write_shadow_request(const WaveParams& W, uint32_t ss, uint32_t path, const ShadowReq& sr) {
    float4* e = W.shadow + 3ull * ss;
    e[0] = make_float4(sr.o.x, sr.o.y, sr.o.z, __uint_as_float(path));
    e[1] = make_float4(sr.d.x, sr.d.y, sr.d.z, sr.t_light);
    e[2] = make_float4(sr.contrib.x, sr.contrib.y, sr.contrib.z, __uint_as_float(sr.light_face));
    if (ADJ) {
        const float3 w = xyz(W.st_W[path]) * sr.dcontrib;
        W.shd_grad[ss] = make_float4(w.x, w.y, w.z, __uint_as_float(sr.light_mat));
    }
}

CRT_D uint32_t octant_of(float3 d) {
    return (signbit(d.x) ? 1u : 0u) | (signbit(d.y) ? 2u : 0u) | (signbit(d.z) ? 4u : 0u);
}

// Window sort: the block shades kSortWin consecutive queue entries, then
// places its surviving paths in the next extension queue grouped by
// direction bin and its shadow requests grouped by light face, so that a
// traversal warp takes rays that start near one another (the window's
// entries come from one region of the image) and head the same way, or go
// to the same light.  The order of queue entries changes no result.
// Binning 0: octant x dominant axis (24 bins); N > 0: an N x N grid over the
// octahedral map of the sphere.  A window entry packs (bin, rank in bin)
// into 16 bits.  Measured (1080p and mixed scenes, FP32 nodes, against no
// sort): 24 bins +13.6% / +7.8%, 5 x 5 +15.4% / +7.1%, 7 x 7 +16.2% / +7.4%;
// windows of 2048 entries lost 2-4% to 1024.
#ifndef CRT_SORT_ITERS
#define CRT_SORT_ITERS 8
#endif
#ifndef CRT_SORT_BINNING
#define CRT_SORT_BINNING 7
#endif
constexpr uint32_t kSortIters = CRT_SORT_ITERS, kSortWin = kWaveBlock * kSortIters;
constexpr uint32_t kSortBinsUsed = CRT_SORT_BINNING == 0 ? 24u : CRT_SORT_BINNING * CRT_SORT_BINNING;
constexpr uint32_t kSortBins = kSortBinsUsed <= 32u ? 32u : 64u;    // one or two bins per lane in the scan
constexpr uint32_t kRankBits = kSortWin <= 1024u ? 10u : 11u;
static_assert(kSortBinsUsed <= 64u && kSortWin <= 2048u &&
                  (((kSortBinsUsed - 1u) << kRankBits) | (kSortWin - 1u)) < 0xFFFFu,
              "window sort packing: a (bin, rank) pair must fit 16 bits below the empty mark");

CRT_D uint32_t direction_bin(float3 d) {
    if (CRT_SORT_BINNING == 0) {
        const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
        const uint32_t dom = (ax >= ay && ax >= az) ? 0u : (ay >= az ? 1u : 2u);
        return octant_of(d) * 3u + dom;
    }
    // octahedral map: the sphere onto the square [-1, 1]^2
    const float l1 = fabsf(d.x) + fabsf(d.y) + fabsf(d.z);
    float px = d.x / l1, py = d.y / l1;
    if (d.z < 0.f) {
        const float qx = (1.f - fabsf(py)) * (px >= 0.f ? 1.f : -1.f);
        const float qy = (1.f - fabsf(px)) * (py >= 0.f ? 1.f : -1.f);
        px = qx;
        py = qy;
    }
    const float N = (float)CRT_SORT_BINNING;
    const uint32_t ix = min((uint32_t)CRT_SORT_BINNING - 1u, (uint32_t)fmaxf(0.f, (px + 1.f) * 0.5f * N));
    const uint32_t iy = min((uint32_t)CRT_SORT_BINNING - 1u, (uint32_t)fmaxf(0.f, (py + 1.f) * 0.5f * N));
    return iy * (uint32_t)CRT_SORT_BINNING + ix;
}

// Register cap of the shade kernel: measured 64 slightly ahead of uncapped.
#ifndef CRT_SHADE_REGS
#define CRT_SHADE_REGS 64
#endif
// ADJ: the adjoint replay, dynamic shared memory [n_mats][6] floats.
// SORT: window sort of both output queues (W.shadow_q set, no octant queues).
template <bool ADJ, bool SORT>
__global__ void __maxnreg__(ADJ ? CRT_SHADE_REGS + 32 : CRT_SHADE_REGS) wf_shade(WaveParams W) {
    extern __shared__ float grad_sh[];
    if (ADJ) zero_grad_block(grad_sh, W.n_mats);
    const uint32_t cur = W.counters[C_CUR];
    const uint32_t n = W.counters[cur];
    __shared__ uint32_t pre_sh[9];
    const QueueView q = queue_view(W, cur, pre_sh);
    uint32_t* qn = W.queue[cur ^ 1u];
    if (!SORT) {
        const uint32_t end = (n + 31u) & ~31u;   // whole warps stay converged for the ballots
        for (uint32_t i = blockIdx.x * kWaveBlock + threadIdx.x; i < end; i += gridDim.x * kWaveBlock) {
            bool alive = false;
            uint32_t path = 0;
            ShadowReq sr;
            sr.valid = false;
            float3 dir = f3(0.f, 0.f, 0.f);
            if (i < n) shade_entry<ADJ>(W, q, i, grad_sh, path, alive, sr, dir);
            if (W.octant) {
                const uint32_t oct = octant_of(dir);
                const uint32_t slot = warp_append_keyed(&W.counters[cur ? C_OCT0 : C_OCT1], alive, oct);
                if (alive) qn[(size_t)oct * W.capacity + slot] = path;
            } else {
                const uint32_t slot = warp_append(&W.counters[cur ^ 1u], alive);
                if (alive) qn[slot] = path;
            }
            const uint32_t ss = warp_append(&W.counters[C_SHADOW], sr.valid);
            if (sr.valid) write_shadow_request<ADJ>(W, ss, path, sr);
        }
    } else {
        // per window entry: (bin << kRankBits | rank in bin) of its surviving
        // path and of its shadow request, or 0xFFFF.  A request is stored at
        // the slot of its queue entry (one per path and bounce at most), and
        // the shadow queue lists the slots in bin order.
        constexpr uint32_t kNone = 0xFFFFu, kRankMask = (1u << kRankBits) - 1u;
        __shared__ uint16_t s_ext[kSortWin], s_shd[kSortWin];
        __shared__ uint32_t s_cnt[2 * kSortBins];
        for (uint32_t w0 = blockIdx.x * kSortWin; w0 < n; w0 += gridDim.x * kSortWin) {
            for (uint32_t k = threadIdx.x; k < 2 * kSortBins; k += kWaveBlock) s_cnt[k] = 0;
            __syncthreads();
            for (uint32_t it = 0; it < kSortIters; ++it) {
                const uint32_t j = it * kWaveBlock + threadIdx.x, i = w0 + j;
                bool alive = false;
                uint32_t path = 0;
                ShadowReq sr;
                sr.valid = false;
                float3 dir = f3(0.f, 0.f, 0.f);
                if (i < n) shade_entry<ADJ>(W, q, i, grad_sh, path, alive, sr, dir);
                const uint32_t ek = alive ? direction_bin(dir) : 0u;
                const uint32_t sk = sr.valid ? (sr.light_face % kSortBinsUsed) : 0u;
                const uint32_t er = warp_append_keyed(s_cnt, alive, ek, kSortBins);
                const uint32_t sn = warp_append_keyed(s_cnt + kSortBins, sr.valid, sk, kSortBins);
                if (sr.valid) write_shadow_request<ADJ>(W, i, path, sr);
                s_ext[j] = alive ? (uint16_t)((ek << kRankBits) | er) : (uint16_t)kNone;
                s_shd[j] = sr.valid ? (uint16_t)((sk << kRankBits) | sn) : (uint16_t)kNone;
            }
            __syncthreads();
            if (threadIdx.x < 32) {
                // exclusive scans of both bin counts (kSortBins / 32 bins per
                // lane), offset by the window's places in the two queues (one
                // atomic each)
                constexpr uint32_t kPer = kSortBins / 32u;
                const uint32_t lane = threadIdx.x;
                uint32_t e[kPer], sh[kPer], et = 0, st = 0;
#pragma unroll
                for (uint32_t k = 0; k < kPer; ++k) {
                    e[k] = s_cnt[lane * kPer + k];
                    sh[k] = s_cnt[kSortBins + lane * kPer + k];
                    et += e[k];
                    st += sh[k];
                }
                uint32_t ei = et, si = st;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t a = __shfl_up_sync(0xFFFFFFFFu, ei, o), b = __shfl_up_sync(0xFFFFFFFFu, si, o);
                    if ((int)lane >= o) {
                        ei += a;
                        si += b;
                    }
                }
                uint32_t eb = 0, sb = 0;
                if (lane == 31) {
                    if (ei) eb = atomicAdd(&W.counters[cur ^ 1u], ei);
                    if (si) sb = atomicAdd(&W.counters[C_SHADOW], si);
                }
                eb = __shfl_sync(0xFFFFFFFFu, eb, 31) + ei - et;
                sb = __shfl_sync(0xFFFFFFFFu, sb, 31) + si - st;
#pragma unroll
                for (uint32_t k = 0; k < kPer; ++k) {
                    s_cnt[lane * kPer + k] = eb;
                    s_cnt[kSortBins + lane * kPer + k] = sb;
                    eb += e[k];
                    sb += sh[k];
                }
            }
            __syncthreads();
            for (uint32_t it = 0; it < kSortIters; ++it) {
                const uint32_t j = it * kWaveBlock + threadIdx.x, i = w0 + j;
                const uint32_t e = s_ext[j], sh = s_shd[j];
                if (e != kNone) qn[s_cnt[e >> kRankBits] + (e & kRankMask)] = q.at(i);
                if (sh != kNone) W.shadow_q[s_cnt[kSortBins + (sh >> kRankBits)] + (sh & kRankMask)] = i;
            }
            __syncthreads();   // the next window reuses the shared arrays
        }
    }
    if (ADJ) flush_grad_block(W, grad_sh);
}

template <bool WHOLE_LEAF, bool F32, bool ADJ = false>
struct ShadowJob {
    const WaveParams& W;
    Stack& st;
    float* grad;        // ADJ: the block's gradient sums
    Traversal<true, false, WHOLE_LEAF, F32> T;
    uint32_t entry = 0, rays = 0;

    CRT_D ShadowJob(const WaveParams& W_, Stack& st_, float* grad_ = nullptr) : W(W_), st(st_), grad(grad_) {}
    CRT_D void start(uint32_t i) {
        entry = W.shadow_q ? W.shadow_q[i] : i;
        const float4* e = W.shadow + 3ull * entry;
        const float4 b = e[1];
        T.init(xyz(e[0]), xyz(b), kEps, b.w, (int32_t)__float_as_uint(e[2].w), st, W.R.S.max_visits);
    }
    CRT_D bool step() { return T.step(W.R.S, st, nullptr); }
    // a visible light adds the request's contribution to the path colour
    CRT_D void finish() {
        ++rays;
        if (T.occluded) return;
        const float4* e = W.shadow + 3ull * entry;
        const uint32_t path = __float_as_uint(e[0].w);
        const float4 c = e[2];
        float4 col = W.st_cm[2ull * path];
        col.x = col.x + c.x;
        col.y = col.y + c.y;
        col.z = col.z + c.z;
        W.st_cm[2ull * path] = col;
        if (ADJ) {
            const float4 g = W.shd_grad[entry];
            warp_add_grad(grad, __float_as_uint(g.w), 3, xyz(g));
        }
    }
};

// The adjoint replay's shadow rays (batch fetch, whole leaves): as wf_shadow,
// and a visible light adds d objective / d (light material ka).  Dynamic
// shared memory: the traversal stacks, then [n_mats][6] gradient floats.
template <bool F32>
__global__ void __maxnreg__(F32 ? CRT_TRAVERSAL_REGS_F32 : CRT_TRAVERSAL_REGS) wf_shadow_adj(WaveParams W) {
    uint2* stacks = stage_top_nodes<F32, true>(W);
    float* grad = reinterpret_cast<float*>(stacks + (size_t)blockDim.x * W.stack_depth);
    zero_grad_block(grad, W.n_mats);
    Stack st;
    st.setup(stacks, blockDim.x, W.stack_depth, W.top_nodes);
    ShadowJob<true, F32, true> job(W, st, grad);
    persistent_loop<false>(W.counters[C_SHADOW], &W.counters[C_FETCH_SHD], W.queue_chunk, 31u, job);
    count_rays(W.R.ray_counts, 0, job.rays);
    flush_grad_block(W, grad);
}

template <bool REFILL, bool WHOLE_LEAF, bool F32, bool TOP>
__global__ void __maxnreg__(F32 ? CRT_TRAVERSAL_REGS_F32 : CRT_TRAVERSAL_REGS) wf_shadow(WaveParams W) {
    uint2* stacks = stage_top_nodes<F32, TOP>(W);
    Stack st;
    st.setup(stacks, blockDim.x, W.stack_depth, TOP ? W.top_nodes : 0u);
    ShadowJob<WHOLE_LEAF, F32> job(W, st);
    persistent_loop<REFILL>(W.counters[C_SHADOW], &W.counters[C_FETCH_SHD], W.queue_chunk, W.refill_busy, job);
    count_rays(W.R.ray_counts, 0, job.rays);
}

using WaveKernel = void (*)(WaveParams);

// Kernel variants by the CRT_FLAG_* traversal-scheduling flags, the node
// format and whether top nodes are staged in shared memory.
template <bool F32, bool TOP>
static WaveKernel extend_kernel_f(uint32_t flags) {
    const bool refill = flags & CRT_FLAG_LANE_REFILL, whole = !(flags & CRT_FLAG_SPLIT_LEAF);
    if (refill) return whole ? wf_extend<true, true, F32, TOP> : wf_extend<true, false, F32, TOP>;
    return whole ? wf_extend<false, true, F32, TOP> : wf_extend<false, false, F32, TOP>;
}

template <bool F32, bool TOP>
static WaveKernel shadow_kernel_f(uint32_t flags) {
    const bool refill = flags & CRT_FLAG_LANE_REFILL, whole = !(flags & CRT_FLAG_SPLIT_LEAF);
    if (refill) return whole ? wf_shadow<true, true, F32, TOP> : wf_shadow<true, false, F32, TOP>;
    return whole ? wf_shadow<false, true, F32, TOP> : wf_shadow<false, false, F32, TOP>;
}

static WaveKernel extend_kernel(uint32_t flags, bool f32, bool top) {
    if (f32) return top ? extend_kernel_f<true, true>(flags) : extend_kernel_f<true, false>(flags);
    return top ? extend_kernel_f<false, true>(flags) : extend_kernel_f<false, false>(flags);
}

static WaveKernel shadow_kernel(uint32_t flags, bool f32, bool top) {
    if (f32) return top ? shadow_kernel_f<true, true>(flags) : shadow_kernel_f<true, false>(flags);
    return top ? shadow_kernel_f<false, true>(flags) : shadow_kernel_f<false, false>(flags);
}

__global__ void wf_flip(WaveParams W) {
    const uint32_t cur = W.counters[C_CUR];
    W.counters[cur] = 0;
    if (W.octant) {
        uint32_t total = 0;
        for (int k = 0; k < 8; ++k) {
            W.counters[(cur ? C_OCT1 : C_OCT0) + k] = 0;
            total += W.counters[(cur ? C_OCT0 : C_OCT1) + k];
        }
        W.counters[cur ^ 1u] = total;
    }
    W.counters[C_CUR] = cur ^ 1u;
    W.counters[C_SHADOW] = 0;
    W.counters[C_FETCH_EXT] = 0;
    W.counters[C_FETCH_SHD] = 0;
}

// wf_flip in two halves, for waves whose shadow traversal of bounce b runs
// beside the extension traversal of bounce b + 1: the extension queues
// switch before extend(b + 1), the shadow counters reset after shadow(b).
__global__ void wf_flip_ext(WaveParams W) {
    const uint32_t cur = W.counters[C_CUR];
    W.counters[cur] = 0;
    if (W.octant) {
        uint32_t total = 0;
        for (int k = 0; k < 8; ++k) {
            W.counters[(cur ? C_OCT1 : C_OCT0) + k] = 0;
            total += W.counters[(cur ? C_OCT0 : C_OCT1) + k];
        }
        W.counters[cur ^ 1u] = total;
    }
    W.counters[C_CUR] = cur ^ 1u;
    W.counters[C_FETCH_EXT] = 0;
}

__global__ void wf_flip_shadow(WaveParams W) {
    W.counters[C_SHADOW] = 0;
    W.counters[C_FETCH_SHD] = 0;
}

__global__ void __launch_bounds__(256) wf_accumulate(WaveParams W) {
    const uint4 wd = wave_desc(W);
    const WaveSeg* segs = W.segs + wd.x;
    for (uint32_t i = blockIdx.x * 256 + threadIdx.x; i < wd.w; i += gridDim.x * 256) {
        const WaveSeg sg = segs[find_segment(segs, wd.y, i, true)];
        const uint32_t ns = sg.s1 - sg.s0, k = i - sg.pix0;
        float4* a = W.R.accum + W.views[sg.view].pix_off + seg_pixel(sg, k);
        float4 acc = *a;
        for (uint32_t s = 0; s < ns; ++s) {
            const float4 c = W.st_cm[2ull * (sg.slot0 + seg_slot(sg, k, s))];
            acc.x = acc.x + c.x;
            acc.y = acc.y + c.y;
            acc.z = acc.z + c.z;
        }
        *a = acc;
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

CRT_D void add_top(unsigned long long* p, uint32_t top) {
    const uint32_t t = __reduce_add_sync(0xFFFFFFFFu, top);
    if ((threadIdx.x & 31u) == 0 && t) atomicAdd(p, (unsigned long long)t);
}

// Counting re-runs (profiling only): the same traversals as wf_extend /
// wf_shadow over the same queue entries, tallying node visits and triangle
// tests instead of writing results.
template <bool F32>
__global__ void __launch_bounds__(kWaveBlock) wf_extend_count(WaveParams W) {
    __shared__ uint2 stack_sh[kStackShared * kWaveBlock];
    Stack st;
    st.setup(stack_sh, kWaveBlock, kStackShared);
    const uint32_t cur = W.counters[C_CUR];
    const uint32_t n = W.counters[cur];
    __shared__ uint32_t pre_sh[9];
    const QueueView q = queue_view(W, cur, pre_sh);
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t rays = 0;
    TraversalStats ts{0, 0, 0, W.top_nodes};
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&W.counters[C_FETCH_CNT], 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= n) break;
        const uint32_t i = base + lane;
        if (i < n) {
            const uint32_t path = q.at(i);
            Hit h;
            h.t = FLT_MAX;
            h.face = -1;
            h.u = h.v = 0.f;
            float4 o, d;
            ld_pair(W.st_od + 2ull * path, o, d);
            traverse<false, true, F32>(W.R.S, xyz(o), xyz(d), kEps, h, -1, st, &ts);
            ++rays;
        }
    }
    add_profile(W.prof + P_EXT_RAYS, rays, ts.nodes, ts.tris);
    add_top(W.prof + P_EXT_TOP, ts.top);
}

template <bool F32>
__global__ void __launch_bounds__(kWaveBlock) wf_shadow_count(WaveParams W) {
    __shared__ uint2 stack_sh[kStackShared * kWaveBlock];
    Stack st;
    st.setup(stack_sh, kWaveBlock, kStackShared);
    const uint32_t n = W.counters[C_SHADOW];
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t rays = 0;
    TraversalStats ts{0, 0, 0, W.top_nodes};
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&W.counters[C_FETCH_CNT], 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= n) break;
        const uint32_t i = base + lane;
        if (i < n) {
            const float4* e = W.shadow + 3ull * (W.shadow_q ? W.shadow_q[i] : i);
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
    add_top(W.prof + P_SHD_TOP, ts.top);
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

static void drop_set_graphs(WaveSet& s) {
    delete static_cast<WaveGraph*>(s.graph);
    delete static_cast<WaveGraph*>(s.adj_graph);
    s.graph = s.adj_graph = nullptr;
}

static void destroy_set(WaveSet& s) {
    if (s.stream) cudaStreamSynchronize(s.stream);
    drop_set_graphs(s);
    if (s.acc_done) cudaEventDestroy(s.acc_done);
    if (s.stream) cudaStreamDestroy(s.stream);
    s.acc_done = nullptr;
    s.stream = nullptr;
}

static void drop_pass_graph(crt_render r) {
    delete static_cast<WaveGraph*>(r->pass_graph);
    r->pass_graph = nullptr;
    r->pass_key = 0;
}

// Callers have synchronised the handle's stream (which may be gone already:
// crt_render_destroy destroys its own stream before the handle).
void destroy_wave_sets(crt_render r) {
    drop_pass_graph(r);
    for (WaveSet& s : r->sets) destroy_set(s);
    r->sets.clear();
    if (r->pass_start) cudaEventDestroy(r->pass_start);
    r->pass_start = nullptr;
}

// Captured launches hold the camera, stream-independent buffers and
// options of the moment; they are re-captured on the next pass.
void drop_wave_graphs(crt_render r) {
    if (r->stream) cudaStreamSynchronize(r->stream);
    drop_pass_graph(r);
    for (WaveSet& s : r->sets) {
        if (s.stream) cudaStreamSynchronize(s.stream);
        drop_set_graphs(s);
    }
}

// Window sort of the shade kernel's output queues: on unless turned off by
// CRT_FLAG_NO_WINDOW_SORT or replaced by octant-binned extension queues.
static bool window_sort(uint32_t flags) {
    return !(flags & (CRT_FLAG_NO_WINDOW_SORT | CRT_FLAG_OCTANT_QUEUES));
}

static int alloc_set(WaveSet& S, uint32_t cap, bool octant) {
    WaveBuffers& B = S.buf;
    B.capacity = cap;
    B.octant = octant;
    const size_t c = cap;
    CRT_CUDA(B.ray_o.alloc(c * 32));    // o | d pairs
    CRT_CUDA(B.color.alloc(c * 32));    // color | mask pairs
    CRT_CUDA(B.hit.alloc(c * 16));
    CRT_CUDA(B.queue_a.alloc(c * 4 * (octant ? 8 : 1)));
    CRT_CUDA(B.queue_b.alloc(c * 4 * (octant ? 8 : 1)));
    CRT_CUDA(B.shadow.alloc(c * 48));
    CRT_CUDA(B.shadow_q.alloc(c * 4));
    CRT_CUDA(B.counters.alloc(C_COUNT * 4));
    CRT_CUDA(cudaMemset(B.counters.p, 0, C_COUNT * 4));
    CRT_CUDA(B.waves.alloc(kMaxWaves * sizeof(uint4)));
    B.seg_capacity = kMaxWaves;
    CRT_CUDA(B.segs.alloc((size_t)B.seg_capacity * sizeof(WaveSeg)));
    CRT_CUDA(B.prof.alloc(P_COUNT * sizeof(unsigned long long)));
    CRT_CUDA(cudaStreamCreateWithFlags(&S.stream, cudaStreamNonBlocking));
    CRT_CUDA(cudaEventCreateWithFlags(&S.acc_done, cudaEventDisableTiming));
    return CRT_OK;
}

// `count` wave sets of the handle's capacity (reallocated when either changes).
static int ensure_wave_sets(crt_render r, uint32_t count) {
    uint64_t pixels = 0;
    for (const ViewState& V : r->views) pixels += V.npix();
    const uint32_t cap = r->opts.wave_paths ? r->opts.wave_paths : default_wave_paths(pixels);
    const bool octant = (r->opts.flags & CRT_FLAG_OCTANT_QUEUES) != 0;
    if (r->sets.size() == count && r->sets[0].buf.capacity == cap && r->sets[0].buf.octant == octant) return CRT_OK;
    CRT_CUDA(cudaStreamSynchronize(r->stream));
    destroy_wave_sets(r);
    CRT_CUDA(cudaEventCreateWithFlags(&r->pass_start, cudaEventDisableTiming));
    r->sets.resize(count);
    for (WaveSet& s : r->sets) {
        int st = alloc_set(s, cap, octant);
        if (st != CRT_OK) {
            destroy_wave_sets(r);
            return st;
        }
    }
    return CRT_OK;
}

// Room for n segments in a set's table; a larger table invalidates the
// set's captured graph, which holds the old address.
static int ensure_segments(WaveSet& set, size_t n) {
    WaveBuffers& B = set.buf;
    if (n <= B.seg_capacity) return CRT_OK;
    if (n > (size_t)UINT32_MAX) return set_error(CRT_ERR_LIMIT, "too many wave segments");
    CRT_CUDA(cudaStreamSynchronize(set.stream));
    drop_set_graphs(set);
    B.seg_capacity = (uint32_t)std::max<size_t>(n, 2ull * B.seg_capacity);
    CRT_CUDA(B.segs.alloc((size_t)B.seg_capacity * sizeof(WaveSeg)));
    return CRT_OK;
}

static WaveParams wave_params(crt_render r, WaveSet& set) {
    WaveBuffers& B = set.buf;
    WaveParams W{};
    W.R = make_params(r, 0, 0, 0);
    W.R.accum = r->accum.as<float4>();   // every view; segments add their offsets
    W.views = r->view_table.as<DevView>();
    W.st_od = B.ray_o.as<float4>();
    W.st_cm = B.color.as<float4>();
    W.hit = B.hit.as<float4>();
    W.queue[0] = B.queue_a.as<uint32_t>();
    W.queue[1] = B.queue_b.as<uint32_t>();
    W.shadow = B.shadow.as<float4>();
    W.counters = B.counters.as<uint32_t>();
    W.waves = B.waves.as<uint4>();
    W.segs = B.segs.as<WaveSeg>();
    W.prof = B.prof.as<unsigned long long>();
    W.stack_depth = (int)traversal_stack(r->opts);
    W.queue_chunk = queue_chunk(r->opts);
    W.top_nodes = staged_nodes(r->scene, r->opts);
    W.refill_busy = refill_busy(r->opts);
    W.octant = B.octant;
    W.shadow_q = window_sort(r->opts.flags) ? B.shadow_q.as<uint32_t>() : nullptr;
    W.capacity = B.capacity;
    return W;
}

struct WaveGrids {
    int gen, ext, shd, acc, cnt;
    int tblock;          // extend / shadow threads per block
    size_t tsmem;        // their dynamic shared memory (traversal stacks)
    WaveKernel extend, shadow, extend_count, shadow_count;
    WaveKernel shade, shade_adj;   // forward and adjoint-replay bounce (window sort or not)
};


// Kernel choice and launch shapes, queried before a capture starts.
static WaveGrids wave_grids(uint32_t capacity, uint32_t flags, bool f32, uint32_t block, uint32_t depth,
                            uint32_t top_nodes) {
    WaveGrids g;
    g.extend = extend_kernel(flags, f32, top_nodes > 0);
    g.shadow = shadow_kernel(flags, f32, top_nodes > 0);
    g.extend_count = f32 ? wf_extend_count<true> : wf_extend_count<false>;
    g.shadow_count = f32 ? wf_shadow_count<true> : wf_shadow_count<false>;
    const bool sort = window_sort(flags);
    g.shade = sort ? wf_shade<false, true> : wf_shade<false, false>;
    g.shade_adj = sort ? wf_shade<true, true> : wf_shade<true, false>;
    g.tblock = (int)block;
    g.tsmem = (size_t)top_nodes * (f32 ? sizeof(Bvh8FloatNode) : sizeof(Bvh8Node)) + (size_t)block * depth * sizeof(uint2);
    cudaFuncSetAttribute((const void*)g.extend, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.tsmem);
    cudaFuncSetAttribute((const void*)g.shadow, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.tsmem);
    g.gen = grid_for(capacity, kWaveBlock, 16);
    g.ext = persistent_grid((const void*)g.extend, g.tblock, g.tsmem);
    g.shd = persistent_grid((const void*)g.shadow, g.tblock, g.tsmem);
    g.cnt = persistent_grid((const void*)g.extend_count, kWaveBlock, 0);
    g.acc = grid_for(capacity, 256, 8);
    return g;
}

static WaveGrids wave_grids(crt_render r, uint32_t capacity) {
    return wave_grids(capacity, r->opts.flags, uses_f32_nodes(r), traversal_block(r->opts), traversal_stack(r->opts),
                      staged_nodes(r->scene, r->opts));
}

// Enqueue the body of one wave (generation and every bounce); captured into
// a wave set's graph.  The accumulate and wave-advance kernels follow it
// outside the graph so that accumulates of concurrent sets can be ordered.
//
// With `s2` (and two events), bounce b's shadow traversal is a branch of its
// own: it starts after shade(b) and runs beside the queue switch and
// extend(b + 1); shade(b + 1) -- which appends new shadow requests and reads
// the path colours shadow(b) adds to -- waits for it.  The two traversals
// touch disjoint state (hit records vs colours and the shadow queue), and
// as persistent kernels each fills the tail of the other.
static void enqueue_wave_body(const WaveParams& W, const WaveGrids& G, uint32_t max_depth, cudaStream_t s,
                              cudaStream_t s2 = nullptr, cudaEvent_t shaded = nullptr,
                              cudaEvent_t shadowed = nullptr) {
    wf_generate<false><<<G.gen, kWaveBlock, 0, s>>>(W);
    for (uint32_t b = 0; b < max_depth; ++b) {
        G.extend<<<G.ext, G.tblock, G.tsmem, s>>>(W);
        if (!s2) {
            G.shade<<<G.gen, kWaveBlock, 0, s>>>(W);
            G.shadow<<<G.shd, G.tblock, G.tsmem, s>>>(W);
            wf_flip<<<1, 1, 0, s>>>(W);
            continue;
        }
        if (b > 0) {
            cudaStreamWaitEvent(s, shadowed, 0);   // shadow(b - 1) is done
            wf_flip_shadow<<<1, 1, 0, s>>>(W);
        }
        G.shade<<<G.gen, kWaveBlock, 0, s>>>(W);
        cudaEventRecord(shaded, s);
        cudaStreamWaitEvent(s2, shaded, 0);
        G.shadow<<<G.shd, G.tblock, G.tsmem, s2>>>(W);
        cudaEventRecord(shadowed, s2);
        wf_flip_ext<<<1, 1, 0, s>>>(W);
    }
    if (s2) {
        cudaStreamWaitEvent(s, shadowed, 0);   // the branch rejoins before the wave ends
        wf_flip_shadow<<<1, 1, 0, s>>>(W);
    }
}

// The waves of a pass, as descriptors {first segment, segments, paths,
// accumulate entries} over one segment list.
struct WavePlan {
    std::vector<uint4> waves;
    std::vector<WaveSeg> segs;
};

// Packs every view's work into waves of at most `capacity` paths.  Views are
// taken in order; each view adds at most one segment to a wave -- whole
// sample layers when the rest of its image fits, else a pixel range of one
// sample -- so no pixel appears twice in a wave, and each pixel's samples
// arrive in sample order wave after wave.  A lone view packs exactly like the
// single-image rule: whole layers while the image fits, else pixel ranges.
static WavePlan make_waves(const crt_render_s* r, const std::vector<ViewWork>& work, uint32_t capacity) {
    struct Pending {
        uint32_t view, npix, s, end, p;   // next sample s (of [s, end)), next pixel p of that sample
    };
    std::vector<Pending> pend;
    for (uint32_t v = 0; v < (uint32_t)work.size(); ++v)
        if (work[v].nspp)
            pend.push_back({v, r->views[v].npix(), work[v].spp0, work[v].spp0 + work[v].nspp, 0});
    WavePlan plan;
    size_t first = 0;   // first view with work left
    while (first < pend.size()) {
        const uint32_t seg0 = (uint32_t)plan.segs.size();
        uint32_t used = 0, pixels = 0;
        for (size_t j = first; j < pend.size() && used < capacity; ++j) {
            Pending& P = pend[j];
            if (P.s >= P.end) continue;
            const uint32_t room = capacity - used;
            WaveSeg g{};
            g.view = P.view;
            g.slot0 = used;
            g.pix0 = pixels;
            if (P.p == 0 && P.npix <= room) {
                const uint32_t k = std::min(room / P.npix, P.end - P.s);
                g.p0 = 0;
                g.p1 = P.npix;
                g.s0 = P.s;
                g.s1 = P.s + k;
                used += k * P.npix;
                P.s += k;
            } else {
                const uint32_t take = std::min(P.npix - P.p, room);
                g.p0 = P.p;
                g.p1 = P.p + take;
                g.s0 = P.s;
                g.s1 = P.s + 1;
                used += take;
                P.p += take;
                if (P.p == P.npix) {
                    P.p = 0;
                    P.s += 1;
                }
            }
            // whole 4-row bands walk in 8x4 tiles of 2x2 quads (measured:
            // tiles +3.2% on the 1080p frame and +1.2% on the mixed scene over
            // rows, the quads' samples together another +5.6% / +1.2%)
            const uint32_t vw = r->views[P.view].width, band = 4u * vw;
            if (vw % 8u == 0 && g.p0 % band == 0 && (g.p1 - g.p0) % band == 0) g.band = band;
            pixels += g.p1 - g.p0;
            plan.segs.push_back(g);
        }
        plan.waves.push_back(make_uint4(seg0, (uint32_t)plan.segs.size() - seg0, used, pixels));
        while (first < pend.size() && pend[first].s >= pend[first].end) ++first;
    }
    return plan;
}

// Waves [w0, w1) of a plan, taking every `stride`-th one, with their
// segments rebased to a table of their own.
static void slice_waves(const WavePlan& plan, size_t w0, size_t w1, size_t stride, std::vector<uint4>& waves,
                        std::vector<WaveSeg>& segs) {
    waves.clear();
    segs.clear();
    for (size_t w = w0; w < w1; w += stride) {
        uint4 d = plan.waves[w];
        const uint32_t base = (uint32_t)segs.size();
        segs.insert(segs.end(), plan.segs.begin() + d.x, plan.segs.begin() + d.x + d.y);
        d.x = base;
        waves.push_back(d);
    }
}

// Uploads a set's descriptors (at most kMaxWaves) and segments on `s` and
// restarts its C_CUR / C_WAVE at zero.
static int upload_waves(WaveSet& set, const std::vector<uint4>& waves, const std::vector<WaveSeg>& segs,
                        cudaStream_t s) {
    WaveBuffers& B = set.buf;
    const uint32_t zero[2] = {0, 0};
    CRT_CUDA(cudaMemcpyAsync(B.waves.p, waves.data(), waves.size() * sizeof(uint4), cudaMemcpyHostToDevice, s));
    CRT_CUDA(cudaMemcpyAsync(B.segs.p, segs.data(), segs.size() * sizeof(WaveSeg), cudaMemcpyHostToDevice, s));
    CRT_CUDA(cudaMemcpyAsync(B.counters.as<uint32_t>() + C_CUR, zero, 8, cudaMemcpyHostToDevice, s));
    return CRT_OK;
}

static int capture_set_graph(crt_render r, WaveSet& set) {
    if (set.graph) return CRT_OK;
    WaveGraph* g = new WaveGraph();
    set.graph = g;
    ++r->graph_epoch;   // a whole-pass graph built from the old one is stale
    const WaveParams W = wave_params(r, set);
    const WaveGrids G = wave_grids(r, set.buf.capacity);
    CRT_CUDA(cudaGetLastError());
    // Captured on a private stream (and a second one for the shadow
    // branches); launched on the set's stream.
    const bool overlap = (r->opts.flags & CRT_FLAG_SERIAL_SHADOW) == 0;
    cudaStream_t cap = nullptr, cap2 = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    CRT_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaError_t e = cudaSuccess;
    if (overlap) {
        e = cudaStreamCreateWithFlags(&cap2, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        enqueue_wave_body(W, G, r->opts.max_depth, cap, cap2, ev[0], ev[1]);
        e = cudaStreamEndCapture(cap, &g->graph);
    }
    for (cudaEvent_t x : ev)
        if (x) cudaEventDestroy(x);
    if (cap2) cudaStreamDestroy(cap2);
    cudaStreamDestroy(cap);
    if (e != cudaSuccess) return cuda_error(e, "capture wave graph");
    CRT_CUDA(cudaGraphInstantiate(&g->exec, g->graph, 0));
    return CRT_OK;
}

// A whole pass as one graph: wave w is a copy of set (w % K)'s wave graph,
// after that set's previous wave has advanced its wave counter; its
// accumulate follows its body and the previous wave's accumulate (any set),
// so pixels add their samples in sample order, as the stream schedule below
// does, and the bodies of consecutive waves on different sets overlap.  The
// handle replays it with one launch per pass while the number of waves, the
// sets and their wave graphs stay the same (the wave descriptors are data:
// each pass uploads its own).
// Passes of more waves (tiny waves or huge passes) keep the per-wave stream
// launches: a graph of ~45 nodes per wave would take long to instantiate.
constexpr size_t kMaxPassGraphWaves = 1024;

static int build_pass_graph(crt_render r, size_t n_waves, uint32_t K) {
    WaveGraph* pg = new WaveGraph();
    r->pass_graph = pg;
    CRT_CUDA(cudaGraphCreate(&pg->graph, 0));
    const WaveGrids G = wave_grids(r, r->sets[0].buf.capacity);
    std::vector<cudaGraphNode_t> last(K, nullptr);
    cudaGraphNode_t prev_acc = nullptr;
    for (size_t w = 0; w < n_waves; ++w) {
        const uint32_t k = (uint32_t)(w % K);
        WaveSet& s = r->sets[k];
        WaveParams W = wave_params(r, s);
        cudaGraphNode_t body = nullptr, acc = nullptr, next = nullptr;
        CRT_CUDA(cudaGraphAddChildGraphNode(&body, pg->graph, last[k] ? &last[k] : nullptr, last[k] ? 1 : 0,
                                            static_cast<WaveGraph*>(s.graph)->graph));
        void* args[] = {&W};
        cudaKernelNodeParams kp{};
        kp.func = (void*)wf_accumulate;
        kp.gridDim = dim3((unsigned)G.acc);
        kp.blockDim = dim3(256);
        kp.kernelParams = args;
        const cudaGraphNode_t acc_deps[2] = {body, prev_acc};
        CRT_CUDA(cudaGraphAddKernelNode(&acc, pg->graph, acc_deps, prev_acc ? 2 : 1, &kp));
        kp.func = (void*)wf_next_wave;
        kp.gridDim = dim3(1);
        kp.blockDim = dim3(1);
        CRT_CUDA(cudaGraphAddKernelNode(&next, pg->graph, &acc, 1, &kp));
        last[k] = next;
        prev_acc = acc;
    }
    CRT_CUDA(cudaGraphInstantiate(&pg->exec, pg->graph, 0));
    return CRT_OK;
}

// A pass: wave w runs on set w % K.  Each set's stream replays its graph for
// the wave body, then waits for the previous wave's accumulate (on whichever
// set ran it) before accumulating, so every pixel adds its samples in sample
// order while the bodies of consecutive waves overlap: one wave's thin late
// bounces share the GPU with the next wave's heavy first bounces.
int wavefront_pass(crt_render r, const std::vector<ViewWork>& work) {
    const uint32_t K = r->opts.wave_sets ? r->opts.wave_sets : kDefaultWaveSets;
    int st = ensure_wave_sets(r, K);
    if (st != CRT_OK) return st;
    const uint32_t cap = r->sets[0].buf.capacity;
    const WavePlan plan = make_waves(r, work, cap);
    if (r->scene_generation != r->scene->generation) {   // the scene's BVH was rebuilt
        drop_wave_graphs(r);
        r->scene_generation = r->scene->generation;
    }
    const size_t chunk = (size_t)kMaxWaves * K;
    std::vector<uint4> mine;
    std::vector<WaveSeg> segs;
    // segment tables large enough for every chunk before any graph is captured
    for (size_t c0 = 0; c0 < plan.waves.size(); c0 += chunk)
        for (uint32_t k = 0; k < K; ++k) {
            slice_waves(plan, c0 + k, std::min(plan.waves.size(), c0 + chunk), K, mine, segs);
            if ((st = ensure_segments(r->sets[k], segs.size())) != CRT_OK) return st;
        }
    for (WaveSet& s : r->sets)
        if ((st = capture_set_graph(r, s)) != CRT_OK) return st;
    if (plan.waves.size() <= std::min<size_t>(chunk, kMaxPassGraphWaves)) {
        // one upload of wave descriptors covers the pass: queue it and the
        // whole pass as one graph on the handle's stream
        for (uint32_t k = 0; k < K; ++k) {
            slice_waves(plan, k, plan.waves.size(), K, mine, segs);
            if (!mine.empty() && (st = upload_waves(r->sets[k], mine, segs, r->stream))) return st;
        }
        const uint64_t key = ((uint64_t)plan.waves.size() << 40) ^ ((uint64_t)K << 32) ^ r->graph_epoch;
        if (!r->pass_graph || r->pass_key != key) {
            drop_pass_graph(r);
            if ((st = build_pass_graph(r, plan.waves.size(), K)) != CRT_OK) return st;
            r->pass_key = key;
        }
        CRT_CUDA(cudaGraphLaunch(static_cast<WaveGraph*>(r->pass_graph)->exec, r->stream));
        return CRT_OK;
    }
    // the sets start after everything already queued on the handle's stream
    CRT_CUDA(cudaEventRecord(r->pass_start, r->stream));
    for (WaveSet& s : r->sets) CRT_CUDA(cudaStreamWaitEvent(s.stream, r->pass_start, 0));
    const WaveGrids G = wave_grids(r, cap);
    int prev = -1;
    for (size_t c0 = 0; c0 < plan.waves.size(); c0 += chunk) {
        const size_t c1 = std::min(plan.waves.size(), c0 + chunk);
        for (uint32_t k = 0; k < K; ++k) {
            slice_waves(plan, c0 + k, c1, K, mine, segs);
            if (!mine.empty() && (st = upload_waves(r->sets[k], mine, segs, r->sets[k].stream))) return st;
        }
        for (size_t w = c0; w < c1; ++w) {
            const int k = (int)(w % K);
            WaveSet& s = r->sets[k];
            const WaveParams W = wave_params(r, s);
            CRT_CUDA(cudaGraphLaunch(static_cast<WaveGraph*>(s.graph)->exec, s.stream));
            if (prev >= 0) CRT_CUDA(cudaStreamWaitEvent(s.stream, r->sets[prev].acc_done, 0));
            wf_accumulate<<<G.acc, 256, 0, s.stream>>>(W);
            wf_next_wave<<<1, 1, 0, s.stream>>>(W);
            CRT_CUDA(cudaEventRecord(s.acc_done, s.stream));
            prev = k;
        }
    }
    CRT_CUDA(cudaGetLastError());
    // the handle's stream continues after every set's last accumulate
    for (WaveSet& s : r->sets) CRT_CUDA(cudaStreamWaitEvent(r->stream, s.acc_done, 0));
    return CRT_OK;
}

// ---------------------------------------------------------------------------
// Adjoint pass (crt_render_adjoint): every wave is traced twice from the same
// Philox counters -- the primal trace leaves each path's radiance in st_c,
// then the replay re-runs the path and turns each event into gradient terms
// (WaveGrad) -- so nothing per vertex is stored.
// ---------------------------------------------------------------------------
static int ensure_adjoint_buffers(WaveSet& set, bool exact) {
    WaveBuffers& B = set.buf;
    const size_t c = B.capacity;
    if (!B.adj_L.p) {
        CRT_CUDA(B.adj_L.alloc(c * 16));
        CRT_CUDA(B.adj_W.alloc(c * 16));
        CRT_CUDA(B.adj_shadow.alloc(c * 16));
    }
    if (exact && !B.adj_hist.p) CRT_CUDA(B.adj_hist.alloc(c * kHistMax * sizeof(uint16_t)));
    return CRT_OK;
}

struct AdjointGrids {
    int shd;
    size_t shade_smem, shadow_smem;
    WaveKernel shadow;
};

static AdjointGrids adjoint_grids(crt_render r, const WaveGrids& G) {
    AdjointGrids a;
    const size_t gsm = (size_t)6 * r->scene->n_mats * sizeof(float);
    a.shade_smem = gsm;
    a.shadow_smem = G.tsmem + gsm;
    a.shadow = uses_f32_nodes(r) ? wf_shadow_adj<true> : wf_shadow_adj<false>;
    cudaFuncSetAttribute((const void*)a.shadow, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)a.shadow_smem);
    cudaFuncSetAttribute((const void*)G.shade_adj, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)a.shade_smem);
    a.shd = persistent_grid((const void*)a.shadow, G.tblock, a.shadow_smem);
    return a;
}

static WaveParams adjoint_params(crt_render r, WaveSet& set, const float4* adj, float* gkd, float* gka,
                                 uint32_t flags) {
    WaveParams W = wave_params(r, set);
    W.adj_exact = (flags & CRT_ADJOINT_EXACT_ROULETTE) != 0;
    W.adj_hist = set.buf.adj_hist.as<uint16_t>();
    W.adj = adj;
    W.st_L = set.buf.adj_L.as<float4>();
    W.st_W = set.buf.adj_W.as<float4>();
    W.shd_grad = set.buf.adj_shadow.as<float4>();
    W.grad_kd = gkd;
    W.grad_ka = gka;
    W.n_mats = r->scene->n_mats;
    return W;
}

static int capture_adjoint_graph(crt_render r, WaveSet& set, const float4* adj, float* gkd, float* gka,
                                 uint32_t flags) {
    if (set.adj_graph && set.adj_key[0] == adj && set.adj_key[1] == gkd && set.adj_key[2] == gka &&
        set.adj_flags == flags)
        return CRT_OK;
    delete static_cast<WaveGraph*>(set.adj_graph);
    WaveGraph* g = new WaveGraph();
    set.adj_graph = g;
    set.adj_key[0] = adj;
    set.adj_key[1] = gkd;
    set.adj_key[2] = gka;
    set.adj_flags = flags;
    const WaveParams W = adjoint_params(r, set, adj, gkd, gka, flags);
    const WaveGrids G = wave_grids(r, set.buf.capacity);
    const AdjointGrids A = adjoint_grids(r, G);
    CRT_CUDA(cudaGetLastError());
    cudaStream_t cap = nullptr;
    CRT_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        enqueue_wave_body(W, G, r->opts.max_depth, cap);     // primal trace
        wf_generate<true><<<G.gen, kWaveBlock, 0, cap>>>(W);  // replay
        for (uint32_t b = 0; b < r->opts.max_depth; ++b) {
            G.extend<<<G.ext, G.tblock, G.tsmem, cap>>>(W);
            G.shade_adj<<<G.gen, kWaveBlock, A.shade_smem, cap>>>(W);
            A.shadow<<<A.shd, G.tblock, A.shadow_smem, cap>>>(W);
            wf_flip<<<1, 1, 0, cap>>>(W);
        }
        e = cudaStreamEndCapture(cap, &g->graph);
    }
    cudaStreamDestroy(cap);
    if (e != cudaSuccess) return cuda_error(e, "capture adjoint graph");
    CRT_CUDA(cudaGraphInstantiate(&g->exec, g->graph, 0));
    return CRT_OK;
}

// Waves run on the K sets round-robin, concurrently: gradient sums need no
// ordering (their atomic adds commute up to rounding).
int wavefront_adjoint(crt_render r, const std::vector<ViewWork>& work, const float4* adj, float* gkd,
                      float* gka, uint32_t flags) {
    if ((size_t)6 * r->scene->n_mats * sizeof(float) > 24u * 1024u)
        return set_error(CRT_ERR_LIMIT, "the adjoint supports at most 1024 materials");
    const bool exact = (flags & CRT_ADJOINT_EXACT_ROULETTE) != 0;
    if (exact && r->opts.max_depth > kHistMax)
        return set_error(CRT_ERR_LIMIT, "CRT_ADJOINT_EXACT_ROULETTE supports max_depth <= 16");
    const uint32_t K = r->opts.wave_sets ? r->opts.wave_sets : kDefaultWaveSets;
    int st = ensure_wave_sets(r, K);
    if (st != CRT_OK) return st;
    for (WaveSet& s : r->sets)
        if ((st = ensure_adjoint_buffers(s, exact)) != CRT_OK) return st;
    const uint32_t cap = r->sets[0].buf.capacity;
    const WavePlan plan = make_waves(r, work, cap);
    if (r->scene_generation != r->scene->generation) {
        drop_wave_graphs(r);
        r->scene_generation = r->scene->generation;
    }
    const size_t chunk = (size_t)kMaxWaves * K;
    std::vector<uint4> mine;
    std::vector<WaveSeg> segs;
    for (size_t c0 = 0; c0 < plan.waves.size(); c0 += chunk)
        for (uint32_t k = 0; k < K; ++k) {
            slice_waves(plan, c0 + k, std::min(plan.waves.size(), c0 + chunk), K, mine, segs);
            if ((st = ensure_segments(r->sets[k], segs.size())) != CRT_OK) return st;
        }
    for (WaveSet& s : r->sets)
        if ((st = capture_adjoint_graph(r, s, adj, gkd, gka, flags)) != CRT_OK) return st;
    CRT_CUDA(cudaEventRecord(r->pass_start, r->stream));
    for (WaveSet& s : r->sets) CRT_CUDA(cudaStreamWaitEvent(s.stream, r->pass_start, 0));
    for (size_t c0 = 0; c0 < plan.waves.size(); c0 += chunk) {
        const size_t c1 = std::min(plan.waves.size(), c0 + chunk);
        for (uint32_t k = 0; k < K; ++k) {
            slice_waves(plan, c0 + k, c1, K, mine, segs);
            if (!mine.empty() && (st = upload_waves(r->sets[k], mine, segs, r->sets[k].stream))) return st;
        }
        for (size_t w = c0; w < c1; ++w) {
            WaveSet& s = r->sets[w % K];
            CRT_CUDA(cudaGraphLaunch(static_cast<WaveGraph*>(s.adj_graph)->exec, s.stream));
            wf_next_wave<<<1, 1, 0, s.stream>>>(wave_params(r, s));
        }
    }
    CRT_CUDA(cudaGetLastError());
    for (WaveSet& s : r->sets) {
        CRT_CUDA(cudaEventRecord(s.acc_done, s.stream));
        CRT_CUDA(cudaStreamWaitEvent(r->stream, s.acc_done, 0));
    }
    return CRT_OK;
}

// Same launch sequence as a wave graph, one kernel at a time with CUDA
// events around each launch, plus untimed counting re-runs of each traversal.
// The profile pass runs its waves one after another on set 0, on the
// handle's stream (after any earlier pass has joined it).
int wavefront_profile_pass(crt_render r, const std::vector<ViewWork>& work, crt_stage_profile* out) {
    int st = ensure_wave_sets(r, r->opts.wave_sets ? r->opts.wave_sets : kDefaultWaveSets);
    if (st != CRT_OK) return st;
    WaveSet& set0 = r->sets[0];
    WaveBuffers& B = set0.buf;
    const WavePlan plan = make_waves(r, work, B.capacity);
    std::vector<uint4> mine;
    std::vector<WaveSeg> segs;
    for (size_t w0 = 0; w0 < plan.waves.size(); w0 += kMaxWaves) {
        slice_waves(plan, w0, std::min(plan.waves.size(), w0 + kMaxWaves), 1, mine, segs);
        if ((st = ensure_segments(set0, segs.size())) != CRT_OK) return st;
    }
    const WaveParams W = wave_params(r, set0);
    const WaveGrids G = wave_grids(r, B.capacity);
    CRT_CUDA(cudaMemsetAsync(B.prof.p, 0, B.prof.bytes, r->stream));
    cudaEvent_t e0, e1;
    CRT_CUDA(cudaEventCreate(&e0));
    CRT_CUDA(cudaEventCreate(&e1));
    cudaStream_t s = r->stream;
    cudaError_t err = cudaSuccess;
    auto timed = [&](int stage, auto launch) -> float {
        if (err != cudaSuccess) return 0.f;
        cudaEventRecord(e0, s);
        launch();
        cudaEventRecord(e1, s);
        err = cudaEventSynchronize(e1);
        if (err == cudaSuccess) err = cudaGetLastError();
        float ms = 0.f;
        if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
        out->ms[stage] += ms;
        out->launches[stage] += 1;
        return ms;
    };
    // queue lengths (device counters) read after the stage that consumes them
    auto counter = [&](uint32_t idx) -> uint32_t {
        uint32_t v = 0;
        if (err == cudaSuccess) err = cudaMemcpy(&v, B.counters.as<uint32_t>() + idx, 4, cudaMemcpyDeviceToHost);
        return v;
    };
    for (size_t w0 = 0; w0 < plan.waves.size() && err == cudaSuccess; w0 += kMaxWaves) {
        slice_waves(plan, w0, std::min(plan.waves.size(), w0 + kMaxWaves), 1, mine, segs);
        if ((st = upload_waves(set0, mine, segs, s)) != CRT_OK) break;
        for (size_t w = 0; w < mine.size(); ++w) {
            timed(0, [&] { wf_generate<false><<<G.gen, kWaveBlock, 0, s>>>(W); });
            for (uint32_t b = 0; b < r->opts.max_depth; ++b) {
                const uint32_t bb = b < 15 ? b : 15;
                out->extend_ms_by_bounce[bb] += timed(1, [&] { G.extend<<<G.ext, G.tblock, G.tsmem, s>>>(W); });
                out->extend_rays_by_bounce[bb] += counter(counter(C_CUR));
                wf_reset_count_fetch<<<1, 1, 0, s>>>(W);
                G.extend_count<<<G.cnt, kWaveBlock, 0, s>>>(W);
                timed(2, [&] { G.shade<<<G.gen, kWaveBlock, 0, s>>>(W); });
                out->shadow_ms_by_bounce[bb] += timed(3, [&] { G.shadow<<<G.shd, G.tblock, G.tsmem, s>>>(W); });
                out->shadow_rays_by_bounce[bb] += counter(C_SHADOW);
                wf_reset_count_fetch<<<1, 1, 0, s>>>(W);
                G.shadow_count<<<G.cnt, kWaveBlock, 0, s>>>(W);
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
    out->extension_top_nodes += c[P_EXT_TOP];
    out->shadow_top_nodes += c[P_SHD_TOP];
    return CRT_OK;
}


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
    0,                                  // o | d pairs   32 B per path (two slices)
    16ull * kNoAllocPaths,
    32ull * kNoAllocPaths,              // color | mask pairs   32 B per path
    48ull * kNoAllocPaths,
    64ull * kNoAllocPaths,              // hit
    80ull * kNoAllocPaths,              // queue 0  4 B per path
    84ull * kNoAllocPaths,              // queue 1
    88ull * kNoAllocPaths,              // shadow requests 48 B per path
    136ull * kNoAllocPaths,             // counters (C_COUNT words)
    136ull * kNoAllocPaths + 128,       // wave descriptor (uint4)
    136ull * kNoAllocPaths + 160,       // its one segment (WaveSeg)
    136ull * kNoAllocPaths + 192,       // ray counts (2 x u64)
    136ull * kNoAllocPaths + 256,       // the view (DevView)
};
constexpr size_t kNoAllocBytes = 136ull * kNoAllocPaths + 512;
static_assert(sizeof(WaveSeg) == 32 && sizeof(DevView) <= 256 && C_COUNT * 4 <= 128, "no-alloc scratch layout");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Device address of the scratch on each device, looked up once per device.
// The address belongs to the device's primary context; a cudaDeviceReset
// would unload the module and leave it stale (documented in the header: the
// entry point is not used again after a reset).
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

// Starts a call: clears the counters and ray counts (everything that must
// start at zero; path state is always written before it is read) and
// installs the view, the wave's one segment and its descriptor.
__global__ void wf_noalloc_begin(WaveParams W, uint4 wave, WaveSeg seg, DevView view) {
    for (int i = 0; i < C_COUNT; ++i) W.counters[i] = 0;
    W.R.ray_counts[0] = W.R.ray_counts[1] = 0;
    const_cast<uint4*>(W.waves)[0] = wave;
    const_cast<WaveSeg*>(W.segs)[0] = seg;
    const_cast<DevView*>(W.views)[0] = view;
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
    if (int st = check_render_options(o)) return st;
    // an error left by earlier work belongs to its caller: report it without
    // clearing it, and launch nothing, so the final check sees only ours
    if (cudaError_t pending = cudaPeekAtLastError())
        return set_error(CRT_ERR_CUDA, std::string("crt_render_tile_noalloc: CUDA error pending from "
                                                   "earlier work: ") + cudaGetErrorString(pending));
    void* base = nullptr;
    int st = noalloc_scratch(&base);
    if (st != CRT_OK) return st;
    unsigned char* b = static_cast<unsigned char*>(base);
    WaveParams W{};
    RenderParams& R = W.R;
    const bool f32 = uses_f32_nodes(scene, o.node_format);
    R.S = scene->view(f32);
    R.cam = to_device_camera(*camera);
    R.accum = reinterpret_cast<float4*>(d_accum);
    R.width = width;
    R.height = height;
    R.seed = o.seed;
    R.view = o.view_id;
    R.spp0 = spp0;
    R.nspp = nspp;
    R.max_depth = o.max_depth;
    R.ka_scale = 3.0f * scene->dev.lights_area;
    R.ray_counts = reinterpret_cast<unsigned long long*>(b + kNoAllocOff[11]);
    W.views = reinterpret_cast<const DevView*>(b + kNoAllocOff[12]);
    W.st_od = reinterpret_cast<float4*>(b + kNoAllocOff[0]);   // with [1]: 32 B per path
    W.st_cm = reinterpret_cast<float4*>(b + kNoAllocOff[2]);   // with [3]: 32 B per path
    W.hit = reinterpret_cast<float4*>(b + kNoAllocOff[4]);
    W.queue[0] = reinterpret_cast<uint32_t*>(b + kNoAllocOff[5]);
    W.queue[1] = reinterpret_cast<uint32_t*>(b + kNoAllocOff[6]);
    W.shadow = reinterpret_cast<float4*>(b + kNoAllocOff[7]);
    W.counters = reinterpret_cast<uint32_t*>(b + kNoAllocOff[8]);
    W.waves = reinterpret_cast<const uint4*>(b + kNoAllocOff[9]);
    W.segs = reinterpret_cast<const WaveSeg*>(b + kNoAllocOff[10]);
    W.prof = nullptr;
    W.stack_depth = (int)traversal_stack(o);
    W.queue_chunk = queue_chunk(o);
    W.top_nodes = staged_nodes(scene, o);
    W.refill_busy = refill_busy(o);
    W.octant = false;   // the scratch holds single-region queues
    W.capacity = kNoAllocPaths;
    const WaveGrids G = wave_grids(kNoAllocPaths, o.flags, f32, traversal_block(o), W.stack_depth, W.top_nodes);
    cudaStream_t s = (cudaStream_t)stream;
    DevView view;
    view.cam = R.cam;
    view.width = width;
    view.height = height;
    view.view_id = o.view_id;
    view.pix_off = 0;
    const WaveSeg seg{0, pixel0, pixel0 + pixel_count, spp0, spp0 + nspp, 0, 0, 0};
    wf_noalloc_begin<<<1, 1, 0, s>>>(W, make_uint4(0, 1, pixel_count * nspp, pixel_count), seg, view);
    wf_generate<false><<<G.gen, kWaveBlock, 0, s>>>(W);
    for (uint32_t k = 0; k < o.max_depth; ++k) {
        G.extend<<<G.ext, G.tblock, G.tsmem, s>>>(W);
        wf_shade<false, false><<<G.gen, kWaveBlock, 0, s>>>(W);
        G.shadow<<<G.shd, G.tblock, G.tsmem, s>>>(W);
        wf_flip<<<1, 1, 0, s>>>(W);
    }
    wf_accumulate<<<G.acc, 256, 0, s>>>(W);
    CRT_CUDA(cudaGetLastError());
    return CRT_OK;
}
