// tune.cu -- the autotuner: picks the wavefront launch options for one
// scene, camera and image size by timing short renders of that workload.
//
// The reference fixes its launch shape at compile time (16x16 blocks, one
// thread per pixel, renderer.cu:543-551) and has nothing to tune.  Here the
// options that change speed but never the image -- node encoding, traversal
// block size, shared-memory stack depth, queue entries claimed per fetch,
// wave sets in flight, paths per wave, lane refill and its threshold, top BVH
// nodes staged in shared memory, and the BVH's width --
// are searched by coordinate descent: each axis in turn is swept with the
// others held, and a value is adopted when it beats the current best by more
// than the noise margin.  Every candidate renders the same samples (a fresh
// handle from sample 0), timed with CUDA events on the handle's stream after
// one untimed pass that allocates and captures its wave graphs.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <map>
#include <tuple>

#include "crt_internal.h"

namespace crt {
namespace {

constexpr float kAdoptMargin = 0.02f;   // a candidate must be 2 % faster to move the search

using Key = std::tuple<int32_t, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t,
                       uint32_t>;

Key key_of(const crt_render_options& o, uint32_t bvh_width) {
    return Key(o.node_format, o.block_size, o.stack_depth, o.queue_chunk, o.wave_sets, o.wave_paths,
               o.flags, o.top_nodes, o.refill_busy, bvh_width);
}

struct Tuner {
    crt_scene scene;
    crt_camera cam;
    uint32_t width, height;
    crt_tune_params P;
    std::map<Key, float> seen;   // measured ms per sample per pixel
    uint32_t candidates = 0;

    // Path-state bytes of a candidate: 140 bytes per path per wave set (two
    // 32-byte state records, the hit, two queue words, one shadow request and
    // its shadow-queue word), plus 56 more with octant-binned queues.
    uint64_t wave_bytes(const crt_render_options& o) const {
        const uint64_t paths = o.wave_paths ? o.wave_paths : default_wave_paths((uint64_t)width * height);
        const uint64_t sets = o.wave_sets ? o.wave_sets : 4u;
        return paths * sets * ((o.flags & CRT_FLAG_OCTANT_QUEUES) ? 196ull : 140ull);
    }

    // ms per sample per pixel of `o`, or a negative value when the candidate
    // cannot run (too much memory, a failed allocation): it is then skipped.
    float measure(const crt_render_options& o) {
        const Key k = key_of(o, scene->info.bvh_width);
        auto it = seen.find(k);
        if (it != seen.end()) return it->second;
        float best = -1.f;
        if (wave_bytes(o) <= P.max_wave_bytes) best = time_candidate(o);
        seen[k] = best;
        ++candidates;
        return best;
    }

    float time_candidate(const crt_render_options& o) {
        crt_render r = nullptr;
        if (crt_render_create(scene, &cam, width, height, &o, &r) != CRT_OK) return -1.f;
        float best = -1.f;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        bool ok = cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess;
        ok = ok && crt_render_pass(r, P.trial_spp) == CRT_OK && cudaStreamSynchronize(r->stream) == cudaSuccess;
        for (uint32_t i = 0; ok && i < P.repeats; ++i) {
            ok = cudaEventRecord(e0, r->stream) == cudaSuccess && crt_render_pass(r, P.trial_spp) == CRT_OK &&
                 cudaEventRecord(e1, r->stream) == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess;
            float ms = 0.f;
            ok = ok && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess;
            if (ok) {
                const float per = ms / (float)P.trial_spp;
                best = best < 0.f ? per : std::min(best, per);
            }
        }
        if (!ok) {
            best = -1.f;
            cudaGetLastError();   // an allocation failure is not sticky; clear it
        }
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        crt_render_destroy(r);
        return best;
    }

    // One coordinate-descent sweep from `cur` (time `t`); returns the time of
    // the options left in `cur`.
    float sweep(crt_render_options& cur, float t) {
        struct Axis {
            uint32_t crt_render_options::*field;
            std::vector<uint32_t> values;
        };
        const bool f32_ok = scene->dev.fnodes != nullptr;
        // node format first: it changes what every other axis measures
        if (f32_ok) {
            for (int32_t nf : {(int32_t)CRT_NODES_Q8, (int32_t)CRT_NODES_F32}) {
                if (nf == cur.node_format) continue;
                crt_render_options c = cur;
                c.node_format = nf;
                const float tc = measure(c);
                if (tc > 0.f && tc < t * (1.f - kAdoptMargin)) {
                    cur = c;
                    t = tc;
                }
            }
        }
        const Axis axes[] = {
            {&crt_render_options::block_size, {64, 128, 256}},
            {&crt_render_options::stack_depth, {8, 12, 16, 24}},
            {&crt_render_options::wave_sets, {1, 2, 3, 4}},
            {&crt_render_options::wave_paths, {1u << 21, 1u << 22, 1u << 23, 1u << 24, 1u << 25}},
            {&crt_render_options::queue_chunk, {32, 64, 128}},
            {&crt_render_options::top_nodes, {0, 9, 73}},
        };
        for (const Axis& a : axes) {
            for (uint32_t v : a.values) {
                if (cur.*a.field == v) continue;
                crt_render_options c = cur;
                c.*a.field = v;
                const float tc = measure(c);
                if (tc > 0.f && tc < t * (1.f - kAdoptMargin)) {
                    cur = c;
                    t = tc;
                }
            }
        }
        // queue order: octant-binned queues, and the shade kernel's window sort
        for (uint32_t f : {(uint32_t)CRT_FLAG_OCTANT_QUEUES, (uint32_t)CRT_FLAG_NO_WINDOW_SORT}) {
            crt_render_options c = cur;
            c.flags ^= f;
            const float tc = measure(c);
            if (tc > 0.f && tc < t * (1.f - kAdoptMargin)) {
                cur = c;
                t = tc;
            }
        }
        // scheduling: batch fetch, or lane refill at a busy-lane threshold
        const uint32_t sched[][2] = {{0u, 31u}, {CRT_FLAG_LANE_REFILL, 31u}, {CRT_FLAG_LANE_REFILL, 20u},
                                     {CRT_FLAG_LANE_REFILL, 12u}};
        for (const auto& sv : sched) {
            const uint32_t flags = (cur.flags & ~(uint32_t)CRT_FLAG_LANE_REFILL) | sv[0];
            if (flags == cur.flags && sv[1] == cur.refill_busy) continue;
            crt_render_options c = cur;
            c.flags = flags;
            c.refill_busy = sv[1];
            const float tc = measure(c);
            if (tc > 0.f && tc < t * (1.f - kAdoptMargin)) {
                cur = c;
                t = tc;
            }
        }
        return t;
    }

    float descend(crt_render_options& cur) {
        float t = measure(cur);
        if (t < 0.f) return t;
        for (uint32_t round = 0; round < P.rounds; ++round) {
            const float before = t;
            t = sweep(cur, t);
            if (!(t < before)) break;   // a full sweep moved nothing
        }
        return t;
    }
};

// Spells out the defaults so that equal options compare equal as keys.
crt_render_options explicit_options(const crt_render_options& in, const crt_scene_s* s, uint64_t pixels) {
    crt_render_options o = in;
    o.mode = CRT_MODE_WAVEFRONT;
    o.block_size = traversal_block(o);
    o.stack_depth = traversal_stack(o);
    o.queue_chunk = queue_chunk(o);
    o.refill_busy = refill_busy(o);
    if (!o.wave_sets) o.wave_sets = 4;
    if (!o.wave_paths) o.wave_paths = default_wave_paths(pixels);
    o.node_format = uses_f32_nodes(s, o.node_format) ? CRT_NODES_F32 : CRT_NODES_Q8;
    return o;
}

}  // namespace
}  // namespace crt

using namespace crt;

extern "C" {

void crt_tune_params_default(crt_tune_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->trial_spp = 8;
    p->repeats = 3;
    p->rounds = 2;
    p->tune_bvh_width = 1;
    p->max_wave_bytes = 32ull << 30;
}

int crt_autotune(crt_scene scene, const crt_camera* camera, uint32_t width, uint32_t height,
                 const crt_render_options* start, const crt_tune_params* params, crt_tune_result* out) {
    if (!scene || !camera || !out) return set_error(CRT_ERR_INVALID, "crt_autotune: null argument");
    if (width == 0 || height == 0 || (uint64_t)width * height >= (1ull << 31))
        return set_error(CRT_ERR_INVALID, "crt_autotune: bad image size");
    crt_tune_params P;
    crt_tune_params_default(&P);
    if (params) {
        if (params->trial_spp) P.trial_spp = params->trial_spp;
        if (params->repeats) P.repeats = params->repeats;
        if (params->rounds) P.rounds = params->rounds;
        P.tune_bvh_width = params->tune_bvh_width;
        if (params->max_wave_bytes) P.max_wave_bytes = params->max_wave_bytes;
    }
    crt_render_options o;
    if (start) o = *start;
    else crt_render_options_default(&o);
    if (int st = check_render_options(o)) return st;
    const auto t0 = std::chrono::steady_clock::now();

    Tuner T{scene, *camera, width, height, P};
    crt_render_options best = explicit_options(o, scene, (uint64_t)width * height);
    const float t_start = T.measure(best);
    if (t_start < 0.f)
        return set_error(CRT_ERR_CUDA, std::string("crt_autotune: the starting options do not run: ") +
                                           crt_last_error());
    float t_best = T.descend(best);
    uint32_t best_width = scene->info.bvh_width;
    if (P.tune_bvh_width) {
        const uint32_t other = best_width == 8 ? 4u : 8u;
        if (int st = crt_scene_set_bvh_width(scene, other)) return st;
        crt_render_options alt = best;
        if (alt.node_format == CRT_NODES_F32 && !scene->dev.fnodes) alt.node_format = CRT_NODES_Q8;
        const float t_alt = T.descend(alt);
        if (t_alt > 0.f && t_alt < t_best * (1.f - kAdoptMargin)) {
            best = alt;
            t_best = t_alt;
            best_width = other;
        } else if (int st = crt_scene_set_bvh_width(scene, best_width)) {
            return st;
        }
    }
    std::memset(out, 0, sizeof(*out));
    out->options = best;
    out->bvh_width = best_width;
    out->candidates = T.candidates;
    out->ms_per_spp = t_best;
    out->start_ms_per_spp = t_start;
    out->tune_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return CRT_OK;
}

}  // extern "C"
