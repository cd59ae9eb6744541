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

// Traversal stack: the first entries of each thread's stack live in shared
// memory (kStackShared by default, or the launch's chosen depth, at most
// kStackSharedMax), the rest in local memory, which only very deep trees
// touch.  A traversal never holds more than kMaxLevels entries.
constexpr int kStackShared = 16;
constexpr int kStackSharedMax = 32;
constexpr int kMaxLevels = 64;
constexpr uint32_t kMaxNodeVisits = 1u << 20;   // default watchdog per traversal
constexpr uint32_t kVisitCeiling = 1u << 30;    // largest limit; the counter starts at ceiling - limit

enum ErrorBits : uint32_t { ERR_WATCHDOG = 1u, ERR_STACK = 2u };

// ---------------------------------------------------------------------------
// Device view of a scene (all arrays in HBM, 16-byte aligned).
// ---------------------------------------------------------------------------
struct DevScene {
    const float4* nodes;       // 5 float4 per 8-wide node (8-bit quantised planes)
    const float4* fnodes;      // 13 float4 per node with FP32 planes, or null
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
    uint32_t max_visits;       // node visits a traversal may make (watchdog), <= kVisitCeiling
    uint32_t* error;           // ErrorBits, sticky until crt_scene_clear_errors
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

// Counting traversals: node visits, triangle tests, and visits to the first
// top_limit nodes (those a staging kernel holds in shared memory).
struct TraversalStats {
    uint32_t nodes, tris;
    uint32_t top = 0, top_limit = 0;
};

// Dynamic shared memory of the traversal kernels that stage the top of the
// BVH: the first n_top nodes (BFS order: the shallowest levels, which every
// ray visits) copied from HBM at kernel start, then the stacks.
extern __shared__ float4 crt_top_nodes[];

// Per-thread stack: shared-memory part (stride = threads per block) and a
// local-memory overflow part.  It also carries how many top nodes the
// launching kernel staged in shared memory (0: none).
struct Stack {
    uint2* sh;           // this thread's first shared entry; entries are `stride` apart
    uint32_t stride;     // threads per block
    int depth;           // entries kept in shared memory
    int sp;
    uint32_t n_top = 0;  // nodes [0, n_top) are in crt_top_nodes
    uint2 spill[kMaxLevels];

    CRT_D void setup(uint2* base, uint32_t threads, int shared_depth, uint32_t staged_nodes = 0) {
        sh = base + threadIdx.x;
        stride = threads;
        depth = shared_depth;
        sp = 0;
        n_top = staged_nodes;
    }
    CRT_D void push(uint2 e) {
        if (sp < depth) sh[sp * stride] = e;
        else spill[sp - depth] = e;
        ++sp;
    }
    CRT_D uint2 pop() {
        --sp;
        return sp < depth ? sh[sp * stride] : spill[sp - depth];
    }
};

CRT_D float safe_rcp(float d) {
    float a = fabsf(d);
    return 1.0f / copysignf(a > 0x1p-80f ? a : 0x1p-80f, d);
}

// Three-input min / max (PTX ISA 8.8, sm_100 and later): one instruction each.
CRT_D float max3f(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
CRT_D float min3f(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Bit s of m moves to bit s ^ oct (8-bit masks).
CRT_D uint32_t permute_octant(uint32_t m, uint32_t oct) {
    if (oct & 1u) m = ((m & 0x55u) << 1) | ((m & 0xAAu) >> 1);
    if (oct & 2u) m = ((m & 0x33u) << 2) | ((m & 0xCCu) >> 2);
    if (oct & 4u) m = ((m & 0x0Fu) << 4) | ((m & 0xF0u) >> 4);
    return m;
}

CRT_D float byte_as_float(uint32_t word, uint32_t sel) {
    // 0x4B0000bb is 2^23 + bb; subtracting 2^23 gives bb exactly.
    return __uint_as_float(__byte_perm(word, 0x4B000000u, sel)) - 8388608.0f;
}

// Resumable traversal of one ray.  step() visits one node (popping the
// stack first when the current group is exhausted) and tests the triangles
// of the leaves it hits; it returns true when the ray is finished.  Kernels
// that keep a lane busy with a new ray as soon as its old one finishes drive
// step() directly; traverse() runs a ray to completion.
//
// Mode CLOSEST: nearest hit with the lowest-face tie rule, h.t starts at tmax.
// Mode OCCLUDED: finishes as soon as a face other than `target` is hit with
// t < h.t, or t == h.t and face < target (exactly the faces that would make
// the closest hit differ from `target`); `occluded` is then true.
template <bool OCCLUDED, bool COUNT, bool WHOLE_LEAF = true, bool F32 = false>
struct Traversal {
    float3 o, d;
    float ix, iy, iz, tmin;
    uint32_t oct;
    uint2 grp;          // child base, (visit-order hit mask << 8) | internal mask
    uint32_t tri_base;  // triangles of the last visited node still to test
    uint32_t tri_mask;
    uint32_t visits;
    int32_t target;
    bool occluded;
    Hit h;

    // max_visits: the scene's watchdog limit (DevScene::max_visits); the
    // counter starts at kVisitCeiling - max_visits so that every visit
    // compares against a constant.
    CRT_D void init(float3 o_, float3 d_, float tmin_, float tmax, int32_t target_, Stack& st,
                    uint32_t max_visits) {
        o = o_;
        d = d_;
        ix = safe_rcp(d.x);
        iy = safe_rcp(d.y);
        iz = safe_rcp(d.z);
        tmin = tmin_;
        oct = (signbit(d.x) ? 1u : 0u) | (signbit(d.y) ? 2u : 0u) | (signbit(d.z) ? 4u : 0u);
        grp = make_uint2(0u, ((1u << oct) << 8) | 1u);   // root = slot 0 of a virtual parent
        tri_base = tri_mask = 0;
        visits = kVisitCeiling - max_visits;
        target = target_;
        occluded = false;
        h.t = tmax;
        h.face = -1;
        h.u = h.v = 0.f;
        st.sp = 0;
    }

    // One pending triangle test.  Returns true if it ends an occlusion query.
    CRT_D bool test_triangle(const DevScene& S, TraversalStats* stats) {
        const uint32_t b = __ffs(tri_mask) - 1;
        tri_mask &= tri_mask - 1;
        const float4* tp = S.tris + 3ull * (tri_base + b);
        const float4 a = ldg(tp), e1 = ldg(tp + 1), e2 = ldg(tp + 2);
        if (COUNT) stats->tris++;
        float u, v;
        const float t = mt_intersect(o, d, xyz(a), xyz(e1), xyz(e2), u, v);
        const int32_t face = (int32_t)__float_as_uint(a.w);
        if (t == FLT_MAX || !(t > tmin)) return false;
        if (OCCLUDED) {
            if (face != target && (t < h.t || (t == h.t && face < target))) {
                occluded = true;
                return true;
            }
        } else if (t < h.t || (t == h.t && h.face >= 0 && face < h.face)) {
            h.t = t;
            h.face = face;
            h.u = u;
            h.v = v;
        }
        return false;
    }

    // One unit of work: the next pending triangle of the last visited node,
    // else one node visit.  Lanes of a warp that are testing triangles and
    // lanes that are visiting nodes each do one unit per step, so a leaf
    // with many triangles does not hold the other lanes back.
    // With WHOLE_LEAF a step is one node visit followed by all of its
    // triangle tests.
    CRT_D bool step(const DevScene& S, Stack& st, TraversalStats* stats) {
        if (WHOLE_LEAF) {
            if (visit(S, st, stats)) return true;
            while (tri_mask)
                if (test_triangle(S, stats)) return true;
            return false;
        }
        if (tri_mask) return test_triangle(S, stats);
        return visit(S, st, stats);
    }

    // Slab tests of the 8 children of an 80-byte node: planes are 8-bit
    // offsets from the node origin in units of a power-of-two scale.
    CRT_D void test_children_q8(const DevScene& S, uint32_t node, uint32_t n_top, uint32_t& child_base,
                                uint32_t& child_imask, uint32_t& tri_base_new, uint32_t& meta_lo,
                                uint32_t& meta_hi, uint32_t& hitmask) const {
        float4 n0, n1, n2, n3, n4;
        if (node < n_top) {
            const float4* sp = crt_top_nodes + 5u * node;
            n0 = sp[0]; n1 = sp[1]; n2 = sp[2]; n3 = sp[3]; n4 = sp[4];
        } else {
            const float4* np = S.nodes + 5ull * node;
            n0 = ldg(np); n1 = ldg(np + 1); n2 = ldg(np + 2); n3 = ldg(np + 3); n4 = ldg(np + 4);
        }
        const uint32_t ebits = __float_as_uint(n0.w);
        const float sx = __uint_as_float((ebits & 0xFFu) << 23) * ix;
        const float sy = __uint_as_float(((ebits >> 8) & 0xFFu) << 23) * iy;
        const float sz = __uint_as_float(((ebits >> 16) & 0xFFu) << 23) * iz;
        const float ax = (n0.x - o.x) * ix, ay = (n0.y - o.y) * iy, az = (n0.z - o.z) * iz;
        child_imask = ebits >> 24;
        child_base = __float_as_uint(n1.x);
        tri_base_new = __float_as_uint(n1.y);
        meta_lo = __float_as_uint(n1.z);
        meta_hi = __float_as_uint(n1.w);
        // quantised planes: lo x|y|z in n2.xy n2.zw n3.xy, hi x|y|z in n3.zw n4.xy n4.zw;
        // a negative direction enters a slab at its hi plane
        const bool nx = oct & 1u, ny = oct & 2u, nz = oct & 4u;
        const uint32_t nlx0 = __float_as_uint(nx ? n3.z : n2.x), nlx1 = __float_as_uint(nx ? n3.w : n2.y);
        const uint32_t flx0 = __float_as_uint(nx ? n2.x : n3.z), flx1 = __float_as_uint(nx ? n2.y : n3.w);
        const uint32_t nly0 = __float_as_uint(ny ? n4.x : n2.z), nly1 = __float_as_uint(ny ? n4.y : n2.w);
        const uint32_t fly0 = __float_as_uint(ny ? n2.z : n4.x), fly1 = __float_as_uint(ny ? n2.w : n4.y);
        const uint32_t nlz0 = __float_as_uint(nz ? n4.z : n3.x), nlz1 = __float_as_uint(nz ? n4.w : n3.y);
        const uint32_t flz0 = __float_as_uint(nz ? n3.x : n4.z), flz1 = __float_as_uint(nz ? n3.y : n4.w);
        const float tfar_cap = h.t;
        hitmask = 0;
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            const uint32_t sel = (uint32_t)(s & 3) | 0x7540u;
            const float tnx = fmaf(byte_as_float(s < 4 ? nlx0 : nlx1, sel), sx, ax);
            const float tfx = fmaf(byte_as_float(s < 4 ? flx0 : flx1, sel), sx, ax);
            const float tny = fmaf(byte_as_float(s < 4 ? nly0 : nly1, sel), sy, ay);
            const float tfy = fmaf(byte_as_float(s < 4 ? fly0 : fly1, sel), sy, ay);
            const float tnz = fmaf(byte_as_float(s < 4 ? nlz0 : nlz1, sel), sz, az);
            const float tfz = fmaf(byte_as_float(s < 4 ? flz0 : flz1, sel), sz, az);
            const float tnear = max3f(tnx, tny, fmaxf(tnz, tmin));
            const float tfar = min3f(tfx, tfy, fminf(tfz, tfar_cap));
            hitmask |= (tnear <= tfar ? 1u : 0u) << s;
        }
    }

    // Slab tests of the 8 children of a 208-byte node with FP32 planes:
    // t = plane * (1/d) - o * (1/d) in one fused multiply-add per plane.
    CRT_D void test_children_f32(const DevScene& S, uint32_t node, uint32_t n_top, uint32_t& child_base,
                                 uint32_t& child_imask, uint32_t& tri_base_new, uint32_t& meta_lo,
                                 uint32_t& meta_hi, uint32_t& hitmask) const {
        const bool staged = node < n_top;
        const float4* np = S.fnodes + 13ull * node;
        const float4* sp = crt_top_nodes + 13u * node;
        auto load = [&](int i) { return staged ? sp[i] : ldg(np + i); };
        const float4 hd = load(12);
        const uint32_t cbi = __float_as_uint(hd.x);
        child_base = cbi & 0xFFFFFFu;
        child_imask = cbi >> 24;
        tri_base_new = __float_as_uint(hd.y);
        meta_lo = __float_as_uint(hd.z);
        meta_hi = __float_as_uint(hd.w);
        // planes: lo x, y, z at float4 0-1, 2-3, 4-5; hi x, y, z at 6-7, 8-9, 10-11
        const int nxo = (oct & 1u) ? 6 : 0, nyo = (oct & 2u) ? 8 : 2, nzo = (oct & 4u) ? 10 : 4;
        const float ox = -o.x * ix, oy = -o.y * iy, oz = -o.z * iz;
        const float tfar_cap = h.t;
        hitmask = 0;
#pragma unroll
        for (int half = 0; half < 2; ++half) {   // slots 4*half .. 4*half+3
            const float4 nxv = load(nxo + half), fxv = load((6 - nxo) + half);
            const float4 nyv = load(nyo + half), fyv = load((10 - nyo) + half);
            const float4 nzv = load(nzo + half), fzv = load((14 - nzo) + half);
            const float nxs[4] = {nxv.x, nxv.y, nxv.z, nxv.w}, fxs[4] = {fxv.x, fxv.y, fxv.z, fxv.w};
            const float nys[4] = {nyv.x, nyv.y, nyv.z, nyv.w}, fys[4] = {fyv.x, fyv.y, fyv.z, fyv.w};
            const float nzs[4] = {nzv.x, nzv.y, nzv.z, nzv.w}, fzs[4] = {fzv.x, fzv.y, fzv.z, fzv.w};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float tnear = max3f(fmaf(nxs[j], ix, ox), fmaf(nys[j], iy, oy), fmaxf(fmaf(nzs[j], iz, oz), tmin));
                const float tfar = min3f(fmaf(fxs[j], ix, ox), fmaf(fys[j], iy, oy), fminf(fmaf(fzs[j], iz, oz), tfar_cap));
                hitmask |= (tnear <= tfar ? 1u : 0u) << (4 * half + j);
            }
        }
    }

    // Visits the next node: pops the stack first when the current group is
    // exhausted; returns true when nothing is left.
    CRT_D bool visit(const DevScene& S, Stack& st, TraversalStats* stats) {
        uint32_t hits = grp.y >> 8;
        if (hits == 0) {
            if (st.sp == 0) return true;
            grp = st.pop();
            hits = grp.y >> 8;
        }
        const uint32_t k = __ffs(hits) - 1;
        hits &= hits - 1;
        const uint32_t imask = grp.y & 0xFFu;
        const uint32_t slot = k ^ oct;
        const uint32_t node = grp.x + __popc(imask & ((1u << slot) - 1u));
        if (hits) {
            if (st.sp >= kMaxLevels) { atomicOr(S.error, ERR_STACK); return true; }
            st.push(make_uint2(grp.x, (hits << 8) | imask));
        }
        if (++visits > kVisitCeiling) { atomicOr(S.error, ERR_WATCHDOG); return true; }
        if (COUNT) {
            stats->nodes++;
            if (node < stats->top_limit) stats->top++;
        }

        uint32_t child_base, child_imask, tri_base_new, meta_lo, meta_hi, hitmask;
        if (F32) test_children_f32(S, node, st.n_top, child_base, child_imask, tri_base_new, meta_lo, meta_hi, hitmask);
        else test_children_q8(S, node, st.n_top, child_base, child_imask, tri_base_new, meta_lo, meta_hi, hitmask);
        // Empty slots hold inverted boxes and never hit; a leaf's meta byte
        // gives its triangle count (bits 5-6) and offset (bits 0-4).
        uint32_t leaves = hitmask & ~child_imask;
        uint32_t tri_mask_new = 0;
        while (leaves) {
            const uint32_t s = __ffs(leaves) - 1;
            leaves &= leaves - 1;
            const uint32_t meta = ((s < 4 ? meta_lo : meta_hi) >> (8 * (s & 3))) & 0xFFu;
            tri_mask_new |= ((1u << (meta >> 5)) - 1u) << (meta & 31u);
        }
        const uint32_t child_hits = permute_octant(hitmask & child_imask, oct);
        grp = make_uint2(child_base, (child_hits << 8) | child_imask);
        tri_base = tri_base_new;
        tri_mask = tri_mask_new;
        return false;
    }
};

template <bool OCCLUDED, bool COUNT, bool F32 = false>
CRT_D bool traverse(const DevScene& S, float3 o, float3 d, float tmin, Hit& h, int32_t target,
                    Stack& st, TraversalStats* stats) {
    Traversal<OCCLUDED, COUNT, true, F32> T;
    T.init(o, d, tmin, h.t, target, st, S.max_visits);
    while (!T.step(S, st, stats)) {
    }
    if (!OCCLUDED) h = T.h;
    return T.occluded;
}

// Warp-local pool of queue entries for persistent kernels: lanes whose ray
// finished take the next entries at once, and the warp claims 32 more from
// the global counter only when the pool runs dry.
struct WarpPool {
    uint32_t next, end;      // warp-uniform
    bool exhausted;

    CRT_D void init() { next = end = 0; exhausted = false; }

    // Returns the queue index for this lane (or UINT32_MAX) when `want`.
    CRT_D uint32_t take(bool want, uint32_t* counter, uint32_t n) {
        const uint32_t lane = threadIdx.x & 31u;
        const uint32_t need = __ballot_sync(0xFFFFFFFFu, want);
        if (!need || exhausted) return UINT32_MAX;
        const uint32_t k = __popc(need);
        const uint32_t rank = __popc(need & ((1u << lane) - 1u));
        const uint32_t have = end - next;
        uint32_t mine = UINT32_MAX;
        if (want && rank < have) mine = next + rank;
        if (k <= have) {
            next += k;
        } else {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(counter, 32u);
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (base >= n) {
                exhausted = true;
                next = end;
            } else {
                const uint32_t chunk_end = base + 32u < n ? base + 32u : n;
                if (want && rank >= have && base + (rank - have) < chunk_end) mine = base + (rank - have);
                const uint32_t used = k - have;
                next = base + used < chunk_end ? base + used : chunk_end;
                end = chunk_end;
            }
        }
        return mine;
    }
};

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
// Geometry weight of a light sample: the contribution is lcolor * weight.
CRT_D float light_weight(const DevScene& S, const LightGeo& l, float t, float lu, float lv, float3 dir) {
    const Shading ls = load_shading(S, l.face);
    const float d2 = t * t;
    const float cost = fabsf(dot(shading_normal(ls, lu, lv), dir * -1.0f));
    return l.area / (d2 * S.lights_area) * cost;
}

CRT_D float3 light_contribution(const DevScene& S, const LightGeo& l, float3 lcolor, float t,
                                float lu, float lv, float3 dir) {
    return f3(0.f, 0.f, 0.f) + lcolor * light_weight(S, l, t, lu, lv, dir);
}

}  // namespace crt
