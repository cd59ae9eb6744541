// crt_device.cuh -- device code shared by the closest-hit, megakernel,
// wavefront and adjoint kernels (sm_103a).
//
// Arithmetic contract: every translation unit that includes this header is
// compiled with -fmad=false, so each float multiply and add rounds
// separately exactly like the reference's host pass; the slab tests use
// explicit fmaf() where fusing is wanted.  Division and square root are
// IEEE round-to-nearest (no fast-math).
#pragma once

#include <cfloat>
#include <cstdint>
#include <cuda_runtime.h>

namespace crt {

#define CRT_D __device__ __forceinline__

constexpr float kEps = 0.00001f;      // EPSILON   (src/include/geometry.h:9)
constexpr float kEps2 = 0.000005f;    // EPSILON_2 (src/include/geometry.h:10)
constexpr int kNoTexture = -1;

enum Bsdf : int { DIFFUSE = 0, SPECULAR = 1, DIFFSPEC = 2, MICROFACET = 3, REFRACTIVE = 4, EMISSIVE = 5 };

// Traversal stack: kStackShared entries per thread in shared memory, then
// kStackLocal more in local memory (touched only by very deep trees).
constexpr int kStackShared = 16;
constexpr int kStackLocal = 48;
constexpr int kMaxLevels = kStackShared + kStackLocal;
constexpr uint32_t kMaxNodeVisits = 1u << 20;   // watchdog per traversal

enum ErrorBits : uint32_t { ERR_WATCHDOG = 1u, ERR_STACK = 2u };

// ---------------------------------------------------------------------------
// Device view of a scene (all arrays in HBM, 16-byte aligned).
// ---------------------------------------------------------------------------
struct DevScene {
    const float4* nodes;       // 5 float4 per 8-wide node
    const float4* tris;        // 3 float4 per record (leaf order)
    const float4* shade;       // 3 float4 per face: n1.xyz n2.x | n2.yz n3.xy | n3.z area mat 0
    const float4* uvs;         // 2 float4 per face: uv1 uv2 | uv3 0 0
    const float4* mats;        // 4 float4 per material: kd tex | ka bsdf | ks ns | ni diffuse 0 0
    const float4* light_geo;   // 3 float4 per light: v1 face | e1 area | e2 material
    const float4* texels;      // rgb0 per texel, with the zero padding
    const uint2* tex_dims;
    const uint32_t* tex_offsets;
    uint32_t tex_total;
    uint32_t n_lights;
    float lights_area;
    uint32_t n_faces;
    uint32_t* error;           // ErrorBits, sticky
};

struct Camera {
    float3 eye, dir, up, right;
    float fov, aspect, aperture, focus;
    int xpixels, ypixels;
};

// ---------------------------------------------------------------------------
// float3 helpers in the reference's operation order (src/include/linalg.h)
// ---------------------------------------------------------------------------
CRT_D float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
CRT_D float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
CRT_D float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
CRT_D float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
CRT_D float3 operator*(float3 a, float b) { return f3(a.x * b, a.y * b, a.z * b); }
CRT_D float3 operator/(float3 a, float b) { return f3(a.x / b, a.y / b, a.z / b); }
CRT_D float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
CRT_D float3 cross(float3 a, float3 b) {
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
CRT_D float3 normalize(float3 v) {
    float n = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
    return f3(v.x / n, v.y / n, v.z / n);
}
CRT_D float max_component(float3 v) { float m = v.x > v.y ? v.x : v.y; return m > v.z ? m : v.z; }
CRT_D float3 xyz(float4 v) { return f3(v.x, v.y, v.z); }

template <typename T>
CRT_D T ldg(const T* p) { return __ldg(p); }

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11) and the per-sample stream.
// Key = seed; counter = (draw / 4, sample, pixel, view).  A draw is
// (x >> 8) * 2^-24 in [0, 1).
// ---------------------------------------------------------------------------
CRT_D uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}

struct Rng {
    uint2 key;
    uint32_t sample, pixel, view;
    uint32_t n;          // draws consumed
    uint4 buf;

    CRT_D void init(uint64_t seed, uint32_t view_, uint32_t pixel_, uint32_t sample_, uint32_t n0 = 0) {
        key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
        sample = sample_;
        pixel = pixel_;
        view = view_;
        n = n0;
        if (n & 3u) buf = philox4x32_10(make_uint4(n >> 2, sample, pixel, view), key);
    }
    // Sampler::getNextFloat (src/renderer/renderer.cu:72-78).
    CRT_D float next() {
        uint32_t lane = n & 3u;
        if (lane == 0) buf = philox4x32_10(make_uint4(n >> 2, sample, pixel, view), key);
        uint32_t x = lane == 0 ? buf.x : (lane == 1 ? buf.y : (lane == 2 ? buf.z : buf.w));
        ++n;
        return (float)(x >> 8) * 0x1p-24f;
    }
};

// ---------------------------------------------------------------------------
// Moller-Trumbore, Triangle::intersect (src/geometry/geometry.cu:38-65), in
// the reference's operation order with explicitly rounded operations, so t,
// u, v are bit-identical to the CPU path.  Returns FLT_MAX on a miss.
// ---------------------------------------------------------------------------
CRT_D float mt_intersect(float3 o, float3 d, float3 v1, float3 e1, float3 e2, float& ou, float& ov) {
    float px = __fsub_rn(__fmul_rn(d.y, e2.z), __fmul_rn(d.z, e2.y));
    float py = __fsub_rn(__fmul_rn(d.z, e2.x), __fmul_rn(d.x, e2.z));
    float pz = __fsub_rn(__fmul_rn(d.x, e2.y), __fmul_rn(d.y, e2.x));
    float det = __fadd_rn(__fadd_rn(__fmul_rn(e1.x, px), __fmul_rn(e1.y, py)), __fmul_rn(e1.z, pz));
    if (fabsf(det) < kEps) return FLT_MAX;
    float inv_det = __frcp_rn(det);
    float tx = __fsub_rn(o.x, v1.x), ty = __fsub_rn(o.y, v1.y), tz = __fsub_rn(o.z, v1.z);
    float u = __fmul_rn(__fadd_rn(__fadd_rn(__fmul_rn(tx, px), __fmul_rn(ty, py)), __fmul_rn(tz, pz)), inv_det);
    if (u < 0.f || u > 1.f) return FLT_MAX;
    float qx = __fsub_rn(__fmul_rn(ty, e1.z), __fmul_rn(tz, e1.y));
    float qy = __fsub_rn(__fmul_rn(tz, e1.x), __fmul_rn(tx, e1.z));
    float qz = __fsub_rn(__fmul_rn(tx, e1.y), __fmul_rn(ty, e1.x));
    float v = __fmul_rn(__fadd_rn(__fadd_rn(__fmul_rn(d.x, qx), __fmul_rn(d.y, qy)), __fmul_rn(d.z, qz)), inv_det);
    if (v < 0.f || __fadd_rn(u, v) > 1.f) return FLT_MAX;
    float t = __fmul_rn(__fadd_rn(__fadd_rn(__fmul_rn(e2.x, qx), __fmul_rn(e2.y, qy)), __fmul_rn(e2.z, qz)), inv_det);
    if (t > kEps) { ou = u; ov = v; return t; }
    return FLT_MAX;
}

// ---------------------------------------------------------------------------
// 8-wide BVH traversal.
// ---------------------------------------------------------------------------
struct Hit {
    float t;
    int32_t face;
    float u, v;
};

struct TraversalStats {
    uint32_t nodes, tris;
};

// Per-thread stack: shared-memory part (stride = threads per block) and a
// local-memory overflow part.
struct Stack {
    uint2* sh;
    uint32_t stride;
    int sp;
    uint2 spill[kStackLocal];

    CRT_D void push(uint2 e) {
        if (sp < kStackShared) sh[sp * stride] = e;
        else spill[sp - kStackShared] = e;
        ++sp;
    }
    CRT_D uint2 pop() {
        --sp;
        return sp < kStackShared ? sh[sp * stride] : spill[sp - kStackShared];
    }
};

CRT_D float safe_rcp(float d) {
    float a = fabsf(d);
    return 1.0f / copysignf(a > 0x1p-80f ? a : 0x1p-80f, d);
}

CRT_D float byte_as_float(uint32_t word, uint32_t sel) {
    // 0x4B0000bb is 2^23 + bb; subtracting 2^23 gives bb exactly.
    return __uint_as_float(__byte_perm(word, 0x4B000000u, sel)) - 8388608.0f;
}

// Mode CLOSEST: nearest hit with lowest-face tie rule, h.t starts at tmax.
// Mode OCCLUDED: returns true as soon as a face other than `target` is hit
// with t < h.t, or t == h.t and face < target (exactly the faces that
// would make the closest hit differ from `target`).
template <bool OCCLUDED, bool COUNT>
CRT_D bool traverse(const DevScene& S, float3 o, float3 d, float tmin, Hit& h, int32_t target,
                    Stack& st, TraversalStats* stats) {
    const float ix = safe_rcp(d.x), iy = safe_rcp(d.y), iz = safe_rcp(d.z);
    const uint32_t oct = (signbit(d.x) ? 1u : 0u) | (signbit(d.y) ? 2u : 0u) | (signbit(d.z) ? 4u : 0u);
    // near/far plane selection per axis: negative direction enters at the hi plane
    const bool nx = oct & 1u, ny = oct & 2u, nz = oct & 4u;
    uint2 grp = make_uint2(0u, ((1u << oct) << 8) | 1u);   // root = slot 0 of a virtual parent
    st.sp = 0;
    uint32_t visits = 0;
    for (;;) {
        uint32_t hits = grp.y >> 8;
        if (hits == 0) {
            if (st.sp == 0) break;
            grp = st.pop();
            continue;
        }
        const uint32_t k = __ffs(hits) - 1;
        hits &= hits - 1;
        const uint32_t imask = grp.y & 0xFFu;
        const uint32_t slot = k ^ oct;
        const uint32_t node = grp.x + __popc(imask & ((1u << slot) - 1u));
        if (hits) {
            if (st.sp >= kMaxLevels) { atomicOr(S.error, ERR_STACK); break; }
            st.push(make_uint2(grp.x, (hits << 8) | imask));
        }
        if (++visits > kMaxNodeVisits) { atomicOr(S.error, ERR_WATCHDOG); break; }
        if (COUNT) stats->nodes++;

        const float4* np = S.nodes + 5ull * node;
        const float4 n0 = ldg(np), n1 = ldg(np + 1), n2 = ldg(np + 2), n3 = ldg(np + 3), n4 = ldg(np + 4);
        const uint32_t ebits = __float_as_uint(n0.w);
        const float sx = __uint_as_float((ebits & 0xFFu) << 23) * ix;
        const float sy = __uint_as_float(((ebits >> 8) & 0xFFu) << 23) * iy;
        const float sz = __uint_as_float(((ebits >> 16) & 0xFFu) << 23) * iz;
        const float ax = (n0.x - o.x) * ix, ay = (n0.y - o.y) * iy, az = (n0.z - o.z) * iz;
        const uint32_t child_imask = ebits >> 24;
        const uint32_t child_base = __float_as_uint(n1.x), tri_base = __float_as_uint(n1.y);
        const uint32_t meta_lo = __float_as_uint(n1.z), meta_hi = __float_as_uint(n1.w);
        // quantised planes: lo x|y|z in n2.xy n2.zw n3.xy, hi x|y|z in n3.zw n4.xy n4.zw
        const uint32_t nlx0 = __float_as_uint(nx ? n3.z : n2.x), nlx1 = __float_as_uint(nx ? n3.w : n2.y);
        const uint32_t flx0 = __float_as_uint(nx ? n2.x : n3.z), flx1 = __float_as_uint(nx ? n2.y : n3.w);
        const uint32_t nly0 = __float_as_uint(ny ? n4.x : n2.z), nly1 = __float_as_uint(ny ? n4.y : n2.w);
        const uint32_t fly0 = __float_as_uint(ny ? n2.z : n4.x), fly1 = __float_as_uint(ny ? n2.w : n4.y);
        const uint32_t nlz0 = __float_as_uint(nz ? n4.z : n3.x), nlz1 = __float_as_uint(nz ? n4.w : n3.y);
        const uint32_t flz0 = __float_as_uint(nz ? n3.x : n4.z), flz1 = __float_as_uint(nz ? n3.y : n4.w);
        const float tfar_cap = h.t;
        uint32_t child_hits = 0, tri_mask = 0;
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            const uint32_t meta = ((s < 4 ? meta_lo : meta_hi) >> (8 * (s & 3))) & 0xFFu;
            const uint32_t sel = (uint32_t)(s & 3) | 0x7540u;
            const float tnx = fmaf(byte_as_float(s < 4 ? nlx0 : nlx1, sel), sx, ax);
            const float tfx = fmaf(byte_as_float(s < 4 ? flx0 : flx1, sel), sx, ax);
            const float tny = fmaf(byte_as_float(s < 4 ? nly0 : nly1, sel), sy, ay);
            const float tfy = fmaf(byte_as_float(s < 4 ? fly0 : fly1, sel), sy, ay);
            const float tnz = fmaf(byte_as_float(s < 4 ? nlz0 : nlz1, sel), sz, az);
            const float tfz = fmaf(byte_as_float(s < 4 ? flz0 : flz1, sel), sz, az);
            const float tnear = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, tmin));
            const float tfar = fminf(fminf(tfx, tfy), fminf(tfz, tfar_cap));
            if (meta != 0u && tnear <= tfar) {
                if (child_imask & (1u << s)) child_hits |= 1u << (s ^ oct);
                else tri_mask |= ((1u << (meta >> 5)) - 1u) << (meta & 31u);
            }
        }
        grp = make_uint2(child_base, (child_hits << 8) | child_imask);
        while (tri_mask) {
            const uint32_t b = __ffs(tri_mask) - 1;
            tri_mask &= tri_mask - 1;
            const float4* tp = S.tris + 3ull * (tri_base + b);
            const float4 a = ldg(tp), e1 = ldg(tp + 1), e2 = ldg(tp + 2);
            if (COUNT) stats->tris++;
            float u, v;
            const float t = mt_intersect(o, d, xyz(a), xyz(e1), xyz(e2), u, v);
            const int32_t face = (int32_t)__float_as_uint(a.w);
            if (t == FLT_MAX || !(t > tmin)) continue;
            if (OCCLUDED) {
                if (face != target && (t < h.t || (t == h.t && face < target))) return true;
            } else if (t < h.t || (t == h.t && h.face >= 0 && face < h.face)) {
                h.t = t;
                h.face = face;
                h.u = u;
                h.v = v;
            }
        }
    }
    return false;
}

// ---------------------------------------------------------------------------
// Estimator pieces (src/renderer/renderer.cu:119-262 and helpers)
// ---------------------------------------------------------------------------
struct Material {
    float3 kd, ka, ks;
    float ns, ni, diffuse;
    int bsdf, tex;
};

CRT_D Material load_material(const DevScene& S, uint32_t m) {
    const float4* p = S.mats + 4ull * m;
    float4 a = ldg(p), b = ldg(p + 1), c = ldg(p + 2), d = ldg(p + 3);
    Material r;
    r.kd = xyz(a); r.tex = __float_as_int(a.w);
    r.ka = xyz(b); r.bsdf = __float_as_int(b.w);
    r.ks = xyz(c); r.ns = c.w;
    r.ni = d.x; r.diffuse = d.y;
    return r;
}

struct Shading {
    float3 n1, n2, n3;
    float area;
    uint32_t material;
};

CRT_D Shading load_shading(const DevScene& S, uint32_t face) {
    const float4* p = S.shade + 3ull * face;
    float4 a = ldg(p), b = ldg(p + 1), c = ldg(p + 2);
    Shading s;
    s.n1 = xyz(a);
    s.n2 = f3(a.w, b.x, b.y);
    s.n3 = f3(b.z, b.w, c.x);
    s.area = c.y;
    s.material = __float_as_uint(c.z);
    return s;
}

// Triangle::getNormal (src/geometry/geometry.cu:67-71).
CRT_D float3 shading_normal(const Shading& s, float u, float v) {
    float w = 1.f - u - v;
    return normalize(s.n1 * w + s.n2 * u + s.n3 * v);
}

// sampleTexture, host branch (src/renderer/renderer.cu:92-115): bilinear at
// (u*W, v*H) without a half-texel offset or wrap; neighbours at i+1 / j+1
// read the next texel of the flattened array, which ends in zero padding.
CRT_D float3 sample_texture(const DevScene& S, int tex, float u, float v) {
    const uint2 dim = ldg(S.tex_dims + tex);
    const uint32_t off = ldg(S.tex_offsets + tex);
    const uint32_t avail = S.tex_total - off;
    const float pu = u * (float)dim.x;
    const float pv = v * (float)dim.y;
    const uint32_t i = (uint32_t)truncf(pu);
    const uint32_t j = (uint32_t)truncf(pv);
    const float fu = floorf(pu), fv = floorf(pv), cu = ceilf(pu), cv = ceilf(pv);
    const uint32_t ia = j * dim.x + i + 1, ib = j * dim.x + i;
    const uint32_t ic = (j + 1) * dim.x + i + 1, id = (j + 1) * dim.x + i;
    const float4* p = S.texels + off;
    const float3 z = f3(0.f, 0.f, 0.f);
    const float3 ta = ia < avail ? xyz(ldg(p + ia)) : z, tb = ib < avail ? xyz(ldg(p + ib)) : z;
    const float3 tc = ic < avail ? xyz(ldg(p + ic)) : z, td = id < avail ? xyz(ldg(p + id)) : z;
    const float3 a1 = ta * (pu - fu);
    const float3 a2 = tb * (cu - pu);
    const float3 b1 = tc * (pu - fu);
    const float3 b2 = td * (cu - pu);
    return (a1 + a2) * (cv - pv) + (b1 + b2) * (pv - fv);
}

struct Ray {
    float3 o, d;
};

// tentFilter + Camera::computeCameraRay (src/geometry/camera.cu:13-57).
CRT_D Ray camera_ray(const Camera& c, int i, int j, Rng& rng) {
    const float r1 = 2.f * rng.next();
    const float r2 = 2.f * rng.next();
    const float dx = r1 < 1.f ? sqrtf(r1) - 1.f : 1.f - sqrtf(2.f - r1);
    const float dy = r2 < 1.f ? sqrtf(r2) - 1.f : 1.f - sqrtf(2.f - r2);
    // (float)((double)a - 0.5) equals the float subtraction: a - 0.5 is exact in double
    const float ni = (((float)i + dx) / (float)c.xpixels) - 0.5f;
    const float nj = 0.5f - (((float)j + dy) / (float)c.ypixels);
    float3 dir = c.dir;
    float3 origin = c.eye;
    dir = dir + c.right * c.fov * c.aspect * ni;
    dir = dir + c.up * c.fov * nj;
    if (c.aperture > 0.0f) {
        const float q1 = (float)((double)rng.next() - 3.14159265358979323846);
        const float q2 = rng.next() - 0.5f;
        float s, co;
        sincosf(q1, &s, &co);
        const float rj = co * q2 * c.aperture;
        const float uj = s * q2 * c.aperture;
        origin = origin + (c.right * rj + c.up * uj);
        const float3 focal = c.eye + dir * c.focus;
        dir = focal - origin;
    }
    Ray r;
    r.o = origin;
    r.d = normalize(dir);
    return r;
}

// Diffuse direction of sampleDiffuseBSDF (src/renderer/renderer.cu:375-402).
CRT_D float3 diffuse_direction(float3 normal, Rng& rng) {
    const float r1 = (float)(6.283185307179586 * (double)rng.next());   // 2 * M_PI * xi
    const float r2 = rng.next();
    const float r2sq = sqrtf(r2);
    const float3 w = normal;
    const float3 u = normalize(cross(fabsf(w.x) > 0.1f ? f3(0.f, 1.f, 0.f) : f3(1.f, 0.f, 0.f), w));
    const float3 v = cross(w, u);
    float s, c;
    sincosf(r1, &s, &c);
    return normalize(u * c * r2sq + v * s * r2sq + w * sqrtf(1.f - r2));
}

struct Fresnel {
    float pr, pt;
    float3 tdir;
};

// getFresnelReflectance (src/renderer/renderer.cu:464-493), including its
// R0 = (etai - etat)^2 / (etat + etai) * (etat + etai) grouping.
CRT_D Fresnel fresnel(float3 incident, float3 normal, float ior) {
    float cosi = dot(incident, normal);
    float etai = 1.f, etat = ior;
    float3 n = normal;
    if (cosi < 0.0f) cosi = -cosi;
    else { float tmp = etai; etai = etat; etat = tmp; n = normal * -1.0f; }
    const float eta = etai / etat;
    const float k = 1.f - eta * eta * (1.f - cosi * cosi);
    Fresnel f;
    f.tdir = f3(0.f, 0.f, 0.f);
    if (k < 0.f) { f.pr = 1.0f; f.pt = 0.0f; return f; }
    f.tdir = incident * eta + n * (eta * cosi - sqrtf(k));
    const float R0 = (etai - etat) * (etai - etat) / (etat + etai) * (etat + etai);
    const float c = 1.f - dot(f.tdir, normal);
    const float Re = R0 + (1.f - R0) * c * c * c * c * c;
    f.pr = Re;
    f.pt = 1.f - Re;
    return f;
}

struct LightGeo {
    float3 v1, e1, e2;
    float area;
    uint32_t face, material;
};

CRT_D LightGeo load_light(const DevScene& S, uint32_t i) {
    const float4* p = S.light_geo + 3ull * i;
    float4 a = ldg(p), b = ldg(p + 1), c = ldg(p + 2);
    LightGeo l;
    l.v1 = xyz(a); l.face = __float_as_uint(a.w);
    l.e1 = xyz(b); l.area = b.w;
    l.e2 = xyz(c); l.material = __float_as_uint(c.w);
    return l;
}

// Light pick of samplePixel (src/renderer/renderer.cu:218-219).
CRT_D uint32_t pick_light(const DevScene& S, float xi) {
    const float rn = xi * ((float)S.n_lights - .00001f);
    uint32_t li = (uint32_t)truncf(rn);
    return li < S.n_lights ? li : S.n_lights - 1;
}

// Triangle::getRandomPointOn (src/geometry/geometry.cu:73-80).
CRT_D float3 light_point(const LightGeo& l, float pu, float pv) {
    if (pu + pv >= 1.0f) { pu = 1.0f - pu; pv = 1.0f - pv; }
    return l.v1 + l.e1 * pu + l.e2 * pv;
}

// Contribution of estimateDirectLighting after a successful shadow test
// (src/renderer/renderer.cu:436-443): ka_light * A |cos| / (d^2 A_total).
CRT_D float3 light_contribution(const DevScene& S, const LightGeo& l, float3 lcolor, float t,
                                float lu, float lv, float3 dir) {
    const Shading ls = load_shading(S, l.face);
    const float d2 = t * t;
    const float cost = fabsf(dot(shading_normal(ls, lu, lv), dir * -1.0f));
    const float wgt = l.area / (d2 * S.lights_area) * cost;
    return f3(0.f, 0.f, 0.f) + lcolor * wgt;
}

}  // namespace crt
