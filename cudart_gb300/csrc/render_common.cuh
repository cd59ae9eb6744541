// render_common.cuh -- the per-sample path state machine shared by the
// megakernel and the wavefront stages.  It restates samplePixel
// (src/renderer/renderer.cu:119-262) one bounce at a time:
//
//   closest hit -> shade_hit() -> [shadow test -> color += contribution]
//
// shade_hit() performs everything the reference does for one bounce after
// its intersectBVH call (emission on camera/specular hits, BSDF choice,
// light sampling, Russian roulette) and returns the direct-light term as a
// shadow request.  Adding the request's contribution after the occlusion
// test gives the same float additions in the same order as the reference:
// Russian roulette only rescales `mask`, never `color`.
#pragma once

#include "crt_device.cuh"

namespace crt {

struct RenderParams {
    DevScene S;
    Camera cam;
    float4* accum;
    uint32_t width, height;
    uint64_t seed;
    uint32_t view;
    uint32_t spp0, nspp;
    uint32_t max_depth;
    unsigned long long* ray_counts;   // [0] extension rays, [1] shadow rays
    float ka_scale;                   // d(stored emission)/d(material ka) = 3 * lights area
};

// One camera view of a render as the wavefront kernels see it: its image
// is pixels [pix_off, pix_off + width * height) of the render's accumulator.
struct DevView {
    Camera cam;
    uint32_t width, height;
    uint32_t view_id;    // Philox counter word
    uint32_t pix_off;
};

struct PathState {
    float3 color, mask;
    int prev;            // bsdf of the previous bounce
    uint32_t bounce;
    Rng rng;
};

struct ShadowReq {
    bool valid;
    float3 o, d;
    float t_light;
    uint32_t light_face;
    float3 contrib;      // mask * directLighting if the light is visible
    float3 dcontrib;     // adjoint only: d contrib / d (light material ka), per channel
    uint32_t light_mat;  // adjoint only
};

// Gradient hooks of shade_hit.  The forward estimator uses NoGrad (every
// hook compiles away); the adjoint replay passes a policy that turns each
// event into gradient contributions (path-replay backpropagation):
// * emission(m, d): the path just added mask * ka_m / lights_area;
//   d = d(that term)/d(material ka), channel-wise;
// * albedo(m, kd, color): a diffuse vertex of untextured material m is about
//   to multiply the throughput by kd; everything the path adds from here on
//   (its total minus `color`, the radiance so far) carries one factor kd.
// * roulette(mask, color): the path survived Russian roulette and is about
//   to divide its throughput by max_component(mask).  By default the
//   survival probability counts as a constant (the hook does nothing); the
//   exact mode differentiates that division as well.
struct NoGrad {
    static constexpr bool kActive = false;
    CRT_D void emission(uint32_t, float3) {}
    CRT_D void albedo(uint32_t, float3, float3) {}
    CRT_D void roulette(float3, float3) {}
};

CRT_D void begin_path(const Camera& cam, uint64_t seed, uint32_t view, uint32_t x, uint32_t y, uint32_t pixel,
                      uint32_t sample, PathState& ps, Ray& ray) {
    ps.rng.init(seed, view, pixel, sample);
    ray = camera_ray(cam, (int)x, (int)y, ps.rng);
    ps.color = f3(0.f, 0.f, 0.f);
    ps.mask = f3(1.f, 1.f, 1.f);
    ps.prev = DIFFUSE;
    ps.bounce = 0;
}

// Miss: the skybox term (renderer.cu:145-151).
CRT_D void shade_miss(PathState& ps) {
    ps.color = ps.color + ps.mask * f3(0.0f, 0.025f, 0.05f);
}

// One bounce after a hit.  Updates ps and `ray` (the next extension ray)
// and returns whether the path continues (Russian roulette, renderer.cu:252-259).
template <class G = NoGrad>
CRT_D bool shade_hit(const RenderParams& P, PathState& ps, Ray& ray, const Hit& h, ShadowReq& sr, G* g = nullptr) {
    const DevScene& S = P.S;
    sr.valid = false;
    const Shading sh = load_shading(S, (uint32_t)h.face);
    const Material m = load_material(S, sh.material);
    if (ps.bounce == 0 || ps.prev == SPECULAR || ps.prev == REFRACTIVE) {
        ps.color = ps.color + ps.mask * m.ka * (1.f / S.lights_area);
        if (G::kActive) g->emission(sh.material, ps.mask * P.ka_scale * (1.f / S.lights_area));
    }
    const float3 normal = shading_normal(sh, h.u, h.v);
    const float3 position = ray.o + ray.d * h.t + normal * kEps2;
    const float3 out_dir = normalize(ray.d);
    // EMISSIVE and MICROFACET set no new direction; the reference then keeps
    // interaction.inputDirection, i.e. the current ray direction after the
    // first bounce and the zero vector on the camera hit (renderer.cu:132,247).
    float3 in_dir = ps.bounce == 0 ? f3(0.f, 0.f, 0.f) : ray.d;
    int bsdf = m.bsdf;
    if (bsdf == DIFFSPEC) {                                       // renderer.cu:171-181
        const float p = m.diffuse;
        if (ps.rng.next() < p) { bsdf = DIFFUSE; ps.mask = ps.mask * (1.0f / p); }
        else { bsdf = SPECULAR; ps.mask = ps.mask * (1.0f / (1.0f - p)); }
    }
    if (bsdf == REFRACTIVE) {                                     // renderer.cu:183-205
        const Fresnel f = fresnel(out_dir, normal, m.ni);
        if (f.pr == 1.0f) {
            bsdf = SPECULAR;
        } else {
            const float Pr = 0.25f + .5f * f.pr;
            const float RP = f.pr / Pr;
            const float TP = f.pt / (1.f - Pr);
            if (ps.rng.next() > 0.25f) {
                in_dir = f.tdir;
                ps.mask = ps.mask * m.ks * TP;
            } else {
                ps.mask = ps.mask * RP;
                bsdf = SPECULAR;
            }
        }
    }
    if (bsdf == DIFFUSE) {                                        // renderer.cu:207-236
        in_dir = diffuse_direction(normal, ps.rng);
        const float cosw = dot(in_dir, normal);
        float3 kd = m.kd;
        if (m.tex != kNoTexture) {
            const float4 uv01 = ldg(S.uvs + 2ull * h.face), uv2 = ldg(S.uvs + 2ull * h.face + 1);
            const float w = 1.f - h.u - h.v;
            const float tu = uv01.x * w + uv01.z * h.u + uv2.x * h.v;
            const float tv = uv01.y * w + uv01.w * h.u + uv2.y * h.v;
            kd = sample_texture(S, m.tex, tu, tv);
        } else if (G::kActive) {
            g->albedo(sh.material, kd, ps.color);
        }
        ps.mask = ps.mask * (kd * cosw) / 0.5f;
        const LightGeo L = load_light(S, pick_light(S, ps.rng.next()));
        if ((uint32_t)h.face != L.face) {                          // estimateDirectLighting
            const float3 ro = position + normal * kEps;
            const float pu = ps.rng.next();
            const float pv = ps.rng.next();
            const float3 sd = normalize(light_point(L, pu, pv) - position);
            float lu = 0.f, lv = 0.f;
            const float tl = mt_intersect(ro, sd, L.v1, L.e1, L.e2, lu, lv);
            if (tl != FLT_MAX) {
                const float3 lcolor = xyz(ldg(S.mats + 4ull * L.material + 1));
                sr.valid = true;
                sr.o = ro;
                sr.d = sd;
                sr.t_light = tl;
                sr.light_face = L.face;
                const float wgt = light_weight(S, L, tl, lu, lv, sd);
                sr.contrib = ps.mask * (f3(0.f, 0.f, 0.f) + lcolor * wgt);
                if (G::kActive) {
                    sr.dcontrib = ps.mask * (P.ka_scale * wgt);
                    sr.light_mat = L.material;
                }
            }
        }
    }
    if (bsdf == SPECULAR) {                                       // renderer.cu:238-243
        in_dir = out_dir - normal * dot(out_dir, normal) * 2.f;
        ps.mask = ps.mask * m.ks / 1.0f;
    }
    ps.prev = bsdf;
    ray.o = position + in_dir * kEps;
    ray.d = in_dir;
    const uint32_t b = ps.bounce++;
    if (b >= 3) {
        const float p = max_component(ps.mask);
        if (ps.rng.next() > p) return false;
        if (G::kActive) g->roulette(ps.mask, ps.color);
        ps.mask = ps.mask / p;
    }
    return true;
}

template <bool F32>
CRT_D bool occluded(const DevScene& S, const ShadowReq& sr, Stack& st) {
    Hit h;
    h.t = sr.t_light;
    h.face = (int32_t)sr.light_face;
    h.u = h.v = 0.f;
    return traverse<true, false, F32>(S, sr.o, sr.d, kEps, h, (int32_t)sr.light_face, st, nullptr);
}

template <bool F32>
CRT_D float3 sample_path(const RenderParams& P, int x, int y, uint32_t pixel, uint32_t sample, Stack& st,
                         uint32_t& n_ext, uint32_t& n_shadow) {
    PathState ps;
    Ray ray;
    begin_path(P.cam, P.seed, P.view, (uint32_t)x, (uint32_t)y, pixel, sample, ps, ray);
    for (uint32_t bounce = 0; bounce < P.max_depth; ++bounce) {
        Hit h;
        h.t = FLT_MAX;
        h.face = -1;
        h.u = h.v = 0.f;
        ++n_ext;
        traverse<false, false, F32>(P.S, ray.o, ray.d, kEps, h, -1, st, nullptr);
        if (h.face < 0) {
            shade_miss(ps);
            break;
        }
        ShadowReq sr;
        const bool alive = shade_hit(P, ps, ray, h, sr);
        if (sr.valid) {
            ++n_shadow;
            if (!occluded<F32>(P.S, sr, st)) ps.color = ps.color + sr.contrib;
        }
        if (!alive) break;
    }
    return ps.color;
}

CRT_D void count_rays(unsigned long long* counts, uint32_t ext, uint32_t shadow) {
    const uint32_t e = __reduce_add_sync(0xFFFFFFFFu, ext);
    const uint32_t s = __reduce_add_sync(0xFFFFFFFFu, shadow);
    if ((threadIdx.x & 31u) == 0) {
        if (e) atomicAdd(counts, (unsigned long long)e);
        if (s) atomicAdd(counts + 1, (unsigned long long)s);
    }
}

}  // namespace crt
