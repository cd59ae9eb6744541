// bvh_gpu.cu -- GPU build of the 8-wide (or 4-wide) quantised BVH.
//
// Binary hierarchy by parallel locally-ordered clustering (PLOC: Meister and
// Bittner, "Parallel Locally-Ordered Clustering for Bounding Volume
// Hierarchy Construction", IEEE TVCG 2018): triangles sorted by 63-bit
// Morton codes of their centroids start as clusters; every iteration each
// cluster finds, among the clusters within kRadius (3) places of it in
// Morton order, the one whose merged box has the least surface area; mutual
// nearest neighbours merge (the merged cluster keeps the left one's place),
// and the list is compacted.  Then the host build's collapse and encoding
// (bvh8.cpp) run level by level: each wide node takes the children the
// collapse chose, assigns them to slots by octant, and quantises their boxes
// outward on a power-of-two grid.  The collapse is
// the host build's SAH-optimal dynamic programme (Ylitie et al., HPG 2017),
// computed bottom-up on the device; it also picks the leaf slots (subtrees
// of at most 3 triangles).  Node and triangle layouts
// are the host build's, so the traversal kernels and every query result are
// unchanged; only the tree differs, and with it the nodes a ray visits.
//
// Triangle boxes get the host build's conservative margin (2^-15 of the
// largest coordinate magnitude, computed in FP64 and rounded outward).
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <climits>
#include <chrono>
#include <vector>

#include "crt_internal.h"

namespace crt {
namespace {

constexpr uint32_t kSlotTrisMax = 3;  // triangles a leaf slot holds (3-bit count)
constexpr float kTriCost = 0.5f;      // the collapse's cost model, as the host build's
constexpr int kBlock = 256;
// PLOC search radius (clusters on each side).  With the SAH-optimal
// collapse a small radius traces best (C3 / C2, Msamples/s at 64 spp:
// r2 877 / 386, r3 882 / 391, r4 866 / 394, r8 850 / 397, r16 827 / 389,
// r32 809 / 390; the host SAH tree: 888 / 375).
constexpr int kRadius = 3;

struct GBox {
    float lo[3], hi[3];
};

// Binary nodes: internal nodes at 0..n-2 (the root at 0, created last),
// triangle i of the sorted order at n-1+i.  `count` is the node's number of
// triangles; a leaf's `first` is its sorted position.
struct GNode {
    GBox box;
    int32_t left, right, parent;
    uint32_t first, count;
};

// Decisions of the SAH-optimal collapse for one binary node (as DpCollapse
// in bvh8.cpp): as one slot, a leaf slot or a wide node; as a wide node,
// the slots of its left child; with at most i slots, those of the left
// child (0: as with i - 1).
struct GDec {
    uint8_t leaf, wk;
    uint8_t split[9];
    uint8_t pad;
};

// Children of one wide node, in the order the collapse picked them.
struct GWide {
    int32_t nch;
    int32_t ch[8];
    int32_t slot_of[8];
};

__device__ __forceinline__ uint32_t float_order(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float order_float(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}
__device__ __forceinline__ float half_area(const GBox& b) {
    const float dx = fmaxf(b.hi[0] - b.lo[0], 0.f), dy = fmaxf(b.hi[1] - b.lo[1], 0.f),
                dz = fmaxf(b.hi[2] - b.lo[2], 0.f);
    return dx * dy + dy * dz + dz * dx;
}
__device__ __forceinline__ void grow(GBox& a, const GBox& b) {
    for (int k = 0; k < 3; ++k) {
        a.lo[k] = fminf(a.lo[k], b.lo[k]);
        a.hi[k] = fmaxf(a.hi[k], b.hi[k]);
    }
}

// Largest coordinate magnitude, as order-preserving bits of a positive float.
__global__ void k_max_abs(const float* __restrict__ v1, const float* __restrict__ e1, const float* __restrict__ e2,
                          uint32_t n3, uint32_t* out) {
    float m = 0.f;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += gridDim.x * blockDim.x) {
        const float a = v1[i];
        m = fmaxf(m, fmaxf(fabsf(a), fmaxf(fabsf(a + e1[i]), fabsf(a + e2[i]))));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
    if ((threadIdx.x & 31u) == 0) atomicMax(out, __float_as_uint(m));
}

// Conservative triangle boxes and centroids exactly as the host build forms
// them (FP64 bounds minus / plus the margin, rounded outward to FP32), and
// the centroid bounds.
__global__ void k_tri_boxes(const float* __restrict__ v1, const float* __restrict__ e1, const float* __restrict__ e2,
                            uint32_t n, float margin, GBox* __restrict__ tbox, float* __restrict__ cent,
                            uint32_t* __restrict__ cbounds) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        GBox b;
        for (int k = 0; k < 3; ++k) {
            const double a = v1[3ull * t + k];
            const double bb = a + (double)e1[3ull * t + k];
            const double c = a + (double)e2[3ull * t + k];
            const double lo = fmin(a, fmin(bb, c)) - (double)margin, hi = fmax(a, fmax(bb, c)) + (double)margin;
            float flo = __double2float_rn(lo), fhi = __double2float_rn(hi);
            if ((double)flo > lo) flo = nextafterf(flo, -FLT_MAX);
            if ((double)fhi < hi) fhi = nextafterf(fhi, FLT_MAX);
            b.lo[k] = flo;
            b.hi[k] = fhi;
            const float cc = 0.5f * (flo + fhi);
            cent[3ull * t + k] = cc;
            atomicMin(&cbounds[k], float_order(cc));
            atomicMax(&cbounds[3 + k], float_order(cc));
        }
        tbox[t] = b;
    }
}

// Spreads the low 21 bits of x to every third bit of a 63-bit code.
__device__ __forceinline__ uint64_t spread21(uint64_t x) {
    x &= 0x1FFFFFull;
    x = (x | (x << 32)) & 0x1F00000000FFFFull;
    x = (x | (x << 16)) & 0x1F0000FF0000FFull;
    x = (x | (x << 8)) & 0x100F00F00F00F00Full;
    x = (x | (x << 4)) & 0x10C30C30C30C30C3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

// 63-bit Morton codes (21 bits per axis) of the centroids.
__global__ void k_morton(const float* __restrict__ cent, uint32_t n, const uint32_t* __restrict__ cbounds,
                         uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    // one scale for all axes (the centroid bounds' largest extent): Morton
    // cells are cubes, so a flat axis does not get the same weight in the
    // curve as the wide ones
    float lo[3];
    const float top = (float)((1u << 21) - 1u);
    float ext = 0.f;
    for (int k = 0; k < 3; ++k) {
        lo[k] = order_float(cbounds[k]);
        ext = fmaxf(ext, order_float(cbounds[3 + k]) - lo[k]);
    }
    const float sc = ext > 0.f ? top / ext : 0.f;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        uint64_t q[3];
        for (int k = 0; k < 3; ++k) {
            const float f = (cent[3ull * t + k] - lo[k]) * sc;
            q[k] = (uint64_t)fminf(fmaxf(f, 0.f), top);
        }
        keys[t] = (spread21(q[0]) << 2) | (spread21(q[1]) << 1) | spread21(q[2]);
        vals[t] = t;
    }
}

__global__ void k_leaves(const GBox* __restrict__ tbox, const uint32_t* __restrict__ perm, int n,
                         GNode* __restrict__ nodes) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    GNode& lf = nodes[n - 1 + i];
    lf.box = tbox[perm[i]];
    lf.left = lf.right = -1;
    lf.first = (uint32_t)i;
    lf.count = 1;
}

// PLOC nearest neighbour: for cluster i of m (in Morton order), the cluster
// j within kRadius places whose merged box has the least half area.  Pairs
// are ordered by (area, |i - j|, min(i, j) odd, min(i, j)): a total order on
// unordered pairs, so the best pair overall is always mutual and every
// iteration merges; among equal boxes (2k, 2k + 1) pair up, so even a scene
// of identical triangles halves its clusters every iteration.
__global__ void k_ploc_nn(const int32_t* __restrict__ clusters, int m, const GNode* __restrict__ nodes,
                          int32_t* __restrict__ nn, int n, uint32_t* err) {
    __shared__ GBox tile[kBlock + 2 * kRadius];
    const int b0 = blockIdx.x * kBlock;
    const int lo = max(0, b0 - kRadius), hi = min(m, b0 + kBlock + kRadius);   // [lo, hi) staged
    for (int k = lo + (int)threadIdx.x; k < hi; k += kBlock) {
        const int32_t c = clusters[k];
        if (c < 0 || c > 2 * n - 2) {   // never expected; keeps the read in bounds
            atomicOr(err, 1u);
            tile[k - lo] = GBox{{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
        } else {
            tile[k - lo] = nodes[c].box;
        }
    }
    __syncthreads();
    const int i = b0 + (int)threadIdx.x;
    if (i >= m) return;
    const GBox bi = tile[i - lo];
    float best = FLT_MAX;
    int bj = -1, bdist = INT_MAX, bodd = 1, bmin = INT_MAX;
    const int j0 = max(0, i - kRadius), j1 = min(m - 1, i + kRadius);
    for (int j = j0; j <= j1; ++j) {
        if (j == i) continue;
        GBox u = bi;
        grow(u, tile[j - lo]);
        const float d = half_area(u);
        const int dist = abs(i - j), mn = min(i, j), odd = mn & 1;
        const bool better =
            d < best || (d == best && (dist < bdist || (dist == bdist && (odd < bodd || (odd == bodd && mn < bmin)))));
        if (better) {
            best = d;
            bj = j;
            bdist = dist;
            bodd = odd;
            bmin = mn;
        }
    }
    nn[i] = bj;
}

// Merge flags, packed for one 64-bit scan: high word = cluster survives
// (kept or merged into), low word = a new node is created here.
__global__ void k_ploc_flags(const int32_t* __restrict__ nn, int m, uint64_t* __restrict__ flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int j = nn[i];
    const bool mutual = j >= 0 && j < m && nn[j] == i;
    const bool create = mutual && i < j;
    const bool survive = !mutual || i < j;
    flags[i] = ((uint64_t)survive << 32) | (uint64_t)create;
}

__global__ void k_ploc_init(int32_t* __restrict__ clusters, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) clusters[i] = n - 1 + i;   // every triangle is a cluster
}

// Creates the merged nodes (ids counting down from `next_id`) and writes the
// compacted cluster list.
__global__ void k_ploc_merge(const int32_t* __restrict__ clusters, const int32_t* __restrict__ nn, int m,
                             const uint64_t* __restrict__ scan, int32_t next_id, GNode* __restrict__ nodes,
                             int32_t* __restrict__ out, int n, uint32_t* err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int j = nn[i];
    const bool mutual = j >= 0 && j < m && nn[j] == i;
    if (mutual && i > j) return;   // merged into cluster j
    const uint64_t sc = scan[i];
    const uint32_t pos = (uint32_t)(sc >> 32);
    int32_t id = clusters[i];
    if (mutual) {
        id = next_id - (int32_t)(uint32_t)(sc & 0xFFFFFFFFull);
        const int32_t l = clusters[i], r = clusters[j];
        if (id < 0 || id > n - 2 || l < 0 || r < 0 || l > 2 * n - 2 || r > 2 * n - 2) {
            atomicOr(err, 1u);   // never expected; keeps every write in bounds
            return;
        }
        GNode nd;
        nd.box = nodes[l].box;
        grow(nd.box, nodes[r].box);
        nd.left = l;
        nd.right = r;
        nd.parent = -1;
        nd.first = 0;
        nd.count = nodes[l].count + nodes[r].count;
        nodes[id] = nd;
        nodes[l].parent = id;
        nodes[r].parent = id;
    }
    if (pos >= (uint32_t)m) {
        atomicOr(err, 1u);
        return;
    }
    out[pos] = id;
}

// C(x, 1..W) of the collapse, from the children's costs (cost[8 * node + i - 1]).
__device__ void dp_node(int32_t x, const GNode& nd, const float* L, const float* R, int W, float* C, GDec& d) {
    const float A = half_area(nd.box);
    const float leafc = nd.count <= kSlotTrisMax ? kTriCost * A * (float)nd.count : FLT_MAX;
    float D[9];
    uint8_t K[9];
    for (int i = 2; i <= W; ++i) {
        D[i] = FLT_MAX;
        K[i] = 1;
        for (int k = 1; k < i; ++k) {
            const float c = L[k - 1] + R[i - k - 1];
            if (c < D[i]) {
                D[i] = c;
                K[i] = (uint8_t)k;
            }
        }
    }
    const float wide = A + D[W];
    d.leaf = leafc <= wide;
    d.wk = K[W];
    C[0] = d.leaf ? leafc : wide;
    d.split[1] = 0;
    for (int i = 2; i <= W; ++i) {
        if (D[i] < C[i - 2]) {
            C[i - 1] = D[i];
            d.split[i] = K[i];
        } else {
            C[i - 1] = C[i - 2];
            d.split[i] = 0;
        }
    }
}

__global__ void k_dp_leaves(int n, const GNode* __restrict__ nodes, int W, float* __restrict__ cost,
                            GDec* __restrict__ dec) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int x = n - 1 + i;
    const float c = kTriCost * half_area(nodes[x].box) * (float)nodes[x].count;
    for (int k = 0; k < W; ++k) cost[8ull * x + k] = c;
    GDec d;
    memset(&d, 0, sizeof(d));
    d.leaf = 1;
    dec[x] = d;
}

// Bottom-up: the second child to finish computes its parent.
__global__ void k_dp_up(int n, const GNode* __restrict__ nodes, int W, float* cost, GDec* __restrict__ dec,
                        uint32_t* flags, uint32_t* err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int p = nodes[n - 1 + i].parent;
    for (int climbed = 0; p >= 0; ++climbed) {
        if (p > n - 2 || climbed >= n) {   // never expected; ends the climb
            atomicOr(err, 8u);
            return;
        }
        __threadfence();
        if (atomicAdd(&flags[p], 1u) == 0) return;   // the sibling subtree is not done yet
        __threadfence();
        const GNode nd = nodes[p];
        if (nd.left < 0 || nd.right < 0 || nd.left > 2 * n - 2 || nd.right > 2 * n - 2) {
            atomicOr(err, 8u);
            return;
        }
        float L[8], R[8], C[8];
        for (int k = 0; k < W; ++k) {
            L[k] = __ldcg(&cost[8ull * nd.left + k]);
            R[k] = __ldcg(&cost[8ull * nd.right + k]);
        }
        GDec d;
        memset(&d, 0, sizeof(d));
        dp_node(p, nd, L, R, W, C, d);
        for (int k = 0; k < W; ++k) __stcg(&cost[8ull * p + k], C[k]);
        dec[p] = d;
        p = nd.parent;
    }
}

__device__ __forceinline__ bool wide_slot(const GDec* dec, int32_t x) { return dec[x].leaf == 0; }

// One wide node per thread: the collapse's children, slots by octant.
__global__ void k_choose(const int32_t* __restrict__ front, uint32_t F, const GNode* __restrict__ nodes,
                         const GDec* __restrict__ dec, int max_children, GWide* __restrict__ recs,
                         uint32_t* __restrict__ cnt_int, uint32_t* __restrict__ cnt_tri, int n, uint32_t* err) {
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= F) return;
    const int32_t x = front[f];
    GWide w;
    int nch = 0;
    if (!wide_slot(dec, x)) {
        w.ch[nch++] = x;                      // a root of at most 3 triangles
    } else {
        // expand (node, slots) pairs left to right, as DpCollapse::expand
        int32_t sn[16];
        int sb[16];
        int sp = 0;
        sn[sp] = nodes[x].right;
        sb[sp++] = max_children - dec[x].wk;
        sn[sp] = nodes[x].left;
        sb[sp++] = dec[x].wk;
        while (sp > 0) {
            const int32_t y = sn[--sp];
            int i = sb[sp];
            if (y < 0 || y > 2 * n - 2 || i < 1 || i > max_children) { atomicOr(err, 16u); break; }
            while (i > 1 && dec[y].split[i] == 0) --i;
            if (i == 1) {
                if (nch < max_children) w.ch[nch++] = y;
                else { atomicOr(err, 16u); break; }
            } else {
                const int k = dec[y].split[i];
                if (sp + 2 > 16 || k < 1 || k >= i) { atomicOr(err, 16u); break; }
                sn[sp] = nodes[y].right;
                sb[sp++] = i - k;
                sn[sp] = nodes[y].left;
                sb[sp++] = k;
            }
        }
    }
    w.nch = nch;
    GBox nb;
    for (int k = 0; k < 3; ++k) { nb.lo[k] = FLT_MAX; nb.hi[k] = -FLT_MAX; }
    for (int c = 0; c < nch; ++c) grow(nb, nodes[w.ch[c]].box);
    float pc[3];
    for (int k = 0; k < 3; ++k) pc[k] = 0.5f * (nb.lo[k] + nb.hi[k]);
    bool used_slot[8] = {false, false, false, false, false, false, false, false};
    bool placed[8] = {false, false, false, false, false, false, false, false};
    for (int round = 0; round < nch; ++round) {
        float best = -FLT_MAX;
        int bc = -1, bs = -1;
        for (int c = 0; c < nch; ++c) {
            if (placed[c]) continue;
            const GBox& cb = nodes[w.ch[c]].box;
            float dd[3];
            for (int k = 0; k < 3; ++k) dd[k] = 0.5f * (cb.lo[k] + cb.hi[k]) - pc[k];
            for (int s = 0; s < 8; ++s) {
                if (used_slot[s]) continue;
                const float sc = ((s & 1) ? dd[0] : -dd[0]) + ((s & 2) ? dd[1] : -dd[1]) + ((s & 4) ? dd[2] : -dd[2]);
                if (sc > best) { best = sc; bc = c; bs = s; }
            }
        }
        placed[bc] = true;
        used_slot[bs] = true;
        w.slot_of[bc] = bs;
    }
    uint32_t ni = 0, nt = 0;
    for (int c = 0; c < nch; ++c) {
        if (wide_slot(dec, w.ch[c])) ++ni;
        else nt += nodes[w.ch[c]].count;
    }
    recs[f] = w;
    cnt_int[f] = ni;
    cnt_tri[f] = nt;
}

__device__ int scale_exponent_d(double ext) {
    if (!(ext > 0.0)) return -126;
    int k;
    const double m = frexp(ext / 255.0, &k);
    const int e = (m == 0.5) ? k - 1 : k;
    return max(-126, min(127, e));
}

// Encodes the wide nodes of one level (the host build's encoding), writes
// the next level's frontier and the triangle records of the leaf slots.
__global__ void k_emit(const GWide* __restrict__ recs, uint32_t F, uint32_t level_base, uint32_t next_base,
                       uint32_t tri_level_base, const uint32_t* __restrict__ int_off,
                       const uint32_t* __restrict__ tri_off, const GNode* __restrict__ nodes,
                       const GDec* __restrict__ dec, const uint32_t* __restrict__ perm, const float* __restrict__ v1,
                       const float* __restrict__ e1, const float* __restrict__ e2, Bvh8Node* __restrict__ out,
                       Bvh8FloatNode* __restrict__ fout, TriRecord* __restrict__ tris, int32_t* __restrict__ next_front,
                       uint32_t n_tris, uint32_t cap_nodes, uint32_t* err) {
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= F) return;
    if (level_base + f >= cap_nodes) {
        atomicOr(err, 2u);
        return;
    }
    const GWide w = recs[f];
    int child_at[8];
    for (int s = 0; s < 8; ++s) child_at[s] = -1;
    for (int c = 0; c < w.nch; ++c) child_at[w.slot_of[c]] = c;
    GBox nb;
    for (int k = 0; k < 3; ++k) { nb.lo[k] = FLT_MAX; nb.hi[k] = -FLT_MAX; }
    for (int c = 0; c < w.nch; ++c) grow(nb, nodes[w.ch[c]].box);
    Bvh8Node node;
    memset(&node, 0, sizeof(node));
    Bvh8FloatNode fnode;
    memset(&fnode, 0, sizeof(fnode));
    node.px = nb.lo[0];
    node.py = nb.lo[1];
    node.pz = nb.lo[2];
    int e[3];
    for (int k = 0; k < 3; ++k) e[k] = scale_exponent_d((double)nb.hi[k] - (double)nb.lo[k]);
    node.ex = (uint8_t)(e[0] + 127);
    node.ey = (uint8_t)(e[1] + 127);
    node.ez = (uint8_t)(e[2] + 127);
    node.child_base = next_base + int_off[f];
    node.tri_base = tri_level_base + tri_off[f];
    uint32_t tri_o = 0, int_o = 0;
    for (int s = 0; s < 8; ++s) {
        const int c = child_at[s];
        if (c < 0) {
            for (int k = 0; k < 3; ++k) {
                node.qlo[k][s] = 255;
                node.qhi[k][s] = 0;
                fnode.lo[k][s] = FLT_MAX;
                fnode.hi[k][s] = -FLT_MAX;
            }
            continue;
        }
        const GNode& cn = nodes[w.ch[c]];
        for (int k = 0; k < 3; ++k) {
            fnode.lo[k][s] = cn.box.lo[k];
            fnode.hi[k][s] = cn.box.hi[k];
            const double step = ldexp(1.0, e[k]);
            const double lo = floor(((double)cn.box.lo[k] - (double)nb.lo[k]) / step);
            const double hi = ceil(((double)cn.box.hi[k] - (double)nb.lo[k]) / step);
            node.qlo[k][s] = (uint8_t)fmax(0.0, fmin(255.0, lo));
            node.qhi[k][s] = (uint8_t)fmax(0.0, fmin(255.0, hi));
        }
        if (wide_slot(dec, w.ch[c])) {
            node.imask |= (uint8_t)(1u << s);
            node.meta[s] = 0x80;
            const uint32_t k = int_off[f] + int_o++;
            if (next_base + k < cap_nodes) next_front[k] = w.ch[c];
            else atomicOr(err, 2u);
        } else {
            node.meta[s] = (uint8_t)((cn.count << 5) | tri_o);
            // the subtree's triangles, left to right (at most kSlotTrisMax)
            uint32_t pos[kSlotTrisMax];
            uint32_t np = 0;
            int32_t stack[2 * kSlotTrisMax];
            int sp = 0;
            stack[sp++] = w.ch[c];
            while (sp > 0) {
                const int32_t x = stack[--sp];
                if (x < 0 || x > 2 * (int32_t)n_tris - 2) { atomicOr(err, 4u); break; }
                const GNode& g = nodes[x];
                if (g.left < 0) {
                    if (np < kSlotTrisMax) pos[np++] = g.first;
                    else atomicOr(err, 4u);
                } else if (sp + 2 <= 2 * (int)kSlotTrisMax) {
                    stack[sp++] = g.right;
                    stack[sp++] = g.left;
                } else {
                    atomicOr(err, 4u);
                    break;
                }
            }
            if (np != cn.count) atomicOr(err, 4u);
            for (uint32_t i = 0; i < np; ++i) {
                const uint32_t t = perm[pos[i]];
                TriRecord r;
                for (int k = 0; k < 3; ++k) {
                    r.v1[k] = v1[3ull * t + k];
                    r.e1[k] = e1[3ull * t + k];
                    r.e2[k] = e2[3ull * t + k];
                }
                r.face = t;
                r.pad1 = r.pad2 = 0.f;
                if (node.tri_base + tri_o + i < n_tris) tris[node.tri_base + tri_o + i] = r;
                else atomicOr(err, 4u);
            }
            tri_o += np;
        }
    }
    out[level_base + f] = node;
    fnode.child_base_imask = node.child_base | ((uint32_t)node.imask << 24);
    fnode.tri_base = node.tri_base;
    memcpy(fnode.meta, node.meta, 8);
    fout[level_base + f] = fnode;
}

uint32_t blocks(uint64_t n) { return (uint32_t)std::max<uint64_t>(1, (n + kBlock - 1) / kBlock); }

}  // namespace

// Builds the BVH of n triangles (device arrays v1/e1/e2, [n][3]) into nodes,
// fnodes and tris (device, allocated here); fills max_depth and the node
// count.  Returns CRT_OK or an error with its message set.
int build_bvh_gpu(const float* d_v1, const float* d_e1, const float* d_e2, uint32_t n, uint32_t max_levels,
                  int max_children, DevBuf& nodes_out, DevBuf& fnodes_out, DevBuf& tris_out, uint32_t* num_nodes,
                  uint32_t* max_depth, bool* fnodes_ok, cudaStream_t s) {
    if (n == 0) return set_error(CRT_ERR_INVALID, "scene has no triangles");
    if (n >= (1u << 30)) return set_error(CRT_ERR_LIMIT, "GPU BVH build: at most 2^30 triangles");
    DevBuf maxbits, tbox, cent, cbounds, keys, vals, keys2, perm, gnodes, tmp, errbuf;
    CRT_CUDA(errbuf.alloc(4));
    CRT_CUDA(cudaMemsetAsync(errbuf.p, 0, 4, s));
    uint32_t* err = errbuf.as<uint32_t>();
    CRT_CUDA(maxbits.alloc(4));
    CRT_CUDA(cudaMemsetAsync(maxbits.p, 0, 4, s));
    k_max_abs<<<blocks(3ull * n) < 1024 ? blocks(3ull * n) : 1024, kBlock, 0, s>>>(d_v1, d_e1, d_e2, 3 * n,
                                                                                  maxbits.as<uint32_t>());
    uint32_t mb = 0;
    CRT_CUDA(cudaMemcpyAsync(&mb, maxbits.p, 4, cudaMemcpyDeviceToHost, s));
    CRT_CUDA(cudaStreamSynchronize(s));
    float maxabs;
    std::memcpy(&maxabs, &mb, 4);
    const float margin = (float)std::ldexp(std::max(1.0, (double)maxabs), -15);

    CRT_CUDA(tbox.alloc((size_t)n * sizeof(GBox)));
    CRT_CUDA(cent.alloc((size_t)n * 12));
    CRT_CUDA(cbounds.alloc(24));
    const uint32_t init[6] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u};
    CRT_CUDA(cudaMemcpyAsync(cbounds.p, init, 24, cudaMemcpyHostToDevice, s));
    k_tri_boxes<<<std::min<uint32_t>(blocks(n), 4096), kBlock, 0, s>>>(d_v1, d_e1, d_e2, n, margin, tbox.as<GBox>(),
                                                                        cent.as<float>(), cbounds.as<uint32_t>());
    CRT_CUDA(keys.alloc((size_t)n * 8));
    CRT_CUDA(vals.alloc((size_t)n * 4));
    CRT_CUDA(keys2.alloc((size_t)n * 8));
    CRT_CUDA(perm.alloc((size_t)n * 4));
    k_morton<<<std::min<uint32_t>(blocks(n), 4096), kBlock, 0, s>>>(cent.as<float>(), n, cbounds.as<uint32_t>(),
                                                                     keys.as<uint64_t>(), vals.as<uint32_t>());
    size_t tmp_bytes = 0;
    CRT_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys.as<uint64_t>(), keys2.as<uint64_t>(),
                                             vals.as<uint32_t>(), perm.as<uint32_t>(), (int)n, 0, 63, s));
    CRT_CUDA(tmp.alloc(tmp_bytes));
    CRT_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tmp_bytes, keys.as<uint64_t>(), keys2.as<uint64_t>(),
                                             vals.as<uint32_t>(), perm.as<uint32_t>(), (int)n, 0, 63, s));
    const int ni = (int)n;
    CRT_CUDA(gnodes.alloc((size_t)(2 * n - 1) * sizeof(GNode)));
    CRT_CUDA(cudaMemsetAsync(gnodes.p, 0xFF, gnodes.bytes, s));   // every parent / child index starts at -1
    GNode* gn = gnodes.as<GNode>();
    k_leaves<<<blocks(n), kBlock, 0, s>>>(tbox.as<GBox>(), perm.as<uint32_t>(), ni, gn);
    int32_t root = (int32_t)n - 1;   // a lone triangle is its own root
    if (n > 1) {
        // PLOC iterations over the cluster list (Morton order), ping-ponged
        DevBuf cl_a, cl_b, nnb, fl, scan, ploc_tmp;
        CRT_CUDA(cl_a.alloc((size_t)n * 4));
        CRT_CUDA(cl_b.alloc((size_t)n * 4));
        CRT_CUDA(nnb.alloc((size_t)n * 4));
        CRT_CUDA(fl.alloc((size_t)(n + 1) * 8));
        CRT_CUDA(scan.alloc((size_t)(n + 1) * 8));
        k_ploc_init<<<blocks(n), kBlock, 0, s>>>(cl_a.as<int32_t>(), ni);
        size_t ploc_bytes = 0;
        CRT_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, ploc_bytes, fl.as<uint64_t>(), scan.as<uint64_t>(),
                                               (int)n + 1, s));
        CRT_CUDA(ploc_tmp.alloc(ploc_bytes));
        int32_t* cur = cl_a.as<int32_t>();
        int32_t* nxt = cl_b.as<int32_t>();
        uint32_t m = n;
        int32_t next_id = (int32_t)n - 2;
        for (uint32_t iter = 0; m > 1; ++iter) {
            if (iter >= n) return set_error(CRT_ERR_CUDA, "GPU BVH build: clustering did not converge");
            k_ploc_nn<<<blocks(m), kBlock, 0, s>>>(cur, (int)m, gn, nnb.as<int32_t>(), ni, err);
            k_ploc_flags<<<blocks(m), kBlock, 0, s>>>(nnb.as<int32_t>(), (int)m, fl.as<uint64_t>());
            CRT_CUDA(cudaMemsetAsync(fl.as<uint64_t>() + m, 0, 8, s));
            CRT_CUDA(cub::DeviceScan::ExclusiveSum(ploc_tmp.p, ploc_bytes, fl.as<uint64_t>(), scan.as<uint64_t>(),
                                                   (int)m + 1, s));
            k_ploc_merge<<<blocks(m), kBlock, 0, s>>>(cur, nnb.as<int32_t>(), (int)m, scan.as<uint64_t>(), next_id,
                                                      gn, nxt, ni, err);
            uint64_t total = 0;
            CRT_CUDA(cudaMemcpyAsync(&total, scan.as<uint64_t>() + m, 8, cudaMemcpyDeviceToHost, s));
            CRT_CUDA(cudaStreamSynchronize(s));
            const uint32_t survivors = (uint32_t)(total >> 32), merges = (uint32_t)(total & 0xFFFFFFFFull);
            if (merges == 0 || survivors + merges != m || (int64_t)next_id + 1 < (int64_t)merges)
                return set_error(CRT_ERR_CUDA, "GPU BVH build: inconsistent clustering step");
            m = survivors;
            next_id -= (int32_t)merges;
            std::swap(cur, nxt);
        }
        CRT_CUDA(cudaMemcpyAsync(&root, cur, 4, cudaMemcpyDeviceToHost, s));
        CRT_CUDA(cudaStreamSynchronize(s));
        if (root != 0 || next_id != -1) return set_error(CRT_ERR_CUDA, "GPU BVH build: clustering left no single root");
    }
    // the collapse's costs and decisions, bottom-up
    DevBuf dp_cost, dp_dec, dp_flags;
    CRT_CUDA(dp_cost.alloc((size_t)(2 * n - 1) * 8 * sizeof(float)));
    CRT_CUDA(dp_dec.alloc((size_t)(2 * n - 1) * sizeof(GDec)));
    CRT_CUDA(dp_flags.alloc((size_t)n * 4));
    CRT_CUDA(cudaMemsetAsync(dp_flags.p, 0, (size_t)n * 4, s));
    k_dp_leaves<<<blocks(n), kBlock, 0, s>>>(ni, gn, max_children, dp_cost.as<float>(), dp_dec.as<GDec>());
    k_dp_up<<<blocks(n), kBlock, 0, s>>>(ni, gn, max_children, dp_cost.as<float>(), dp_dec.as<GDec>(),
                                         dp_flags.as<uint32_t>(), err);
    const GDec* dec = dp_dec.as<GDec>();
    CRT_CUDA(cudaGetLastError());
    {   // the collapse follows child links: stop here if any were not set
        uint32_t e = 0;
        CRT_CUDA(cudaMemcpyAsync(&e, err, 4, cudaMemcpyDeviceToHost, s));
        CRT_CUDA(cudaStreamSynchronize(s));
        if (e) return set_error(CRT_ERR_CUDA, "GPU BVH build: inconsistent hierarchy (" + std::to_string(e) + ")");
    }

    // ---- collapse level by level -------------------------------------------
    const uint32_t cap_nodes = n;   // a wide node holds >= 1 triangle of its own subtree
    CRT_CUDA(nodes_out.alloc((size_t)cap_nodes * sizeof(Bvh8Node)));
    CRT_CUDA(fnodes_out.alloc((size_t)cap_nodes * sizeof(Bvh8FloatNode)));
    CRT_CUDA(tris_out.alloc((size_t)n * sizeof(TriRecord)));
    DevBuf front_a, front_b, recs, cnt_int, cnt_tri, off_int, off_tri, scan_tmp;
    CRT_CUDA(front_a.alloc((size_t)cap_nodes * 4));
    CRT_CUDA(front_b.alloc((size_t)cap_nodes * 4));
    CRT_CUDA(recs.alloc((size_t)cap_nodes * sizeof(GWide)));
    CRT_CUDA(cnt_int.alloc((size_t)cap_nodes * 4 + 4));
    CRT_CUDA(cnt_tri.alloc((size_t)cap_nodes * 4 + 4));
    CRT_CUDA(off_int.alloc((size_t)cap_nodes * 4 + 4));
    CRT_CUDA(off_tri.alloc((size_t)cap_nodes * 4 + 4));
    size_t scan_bytes = 0;
    CRT_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, cnt_int.as<uint32_t>(), off_int.as<uint32_t>(),
                                           (int)cap_nodes + 1, s));
    CRT_CUDA(scan_tmp.alloc(scan_bytes));
    CRT_CUDA(cudaMemcpyAsync(front_a.p, &root, 4, cudaMemcpyHostToDevice, s));
    uint32_t F = 1, level_base = 0, tri_base = 0, depth = 0;
    int32_t* cur = front_a.as<int32_t>();
    int32_t* nxt = front_b.as<int32_t>();
    while (F > 0) {
        if (++depth > max_levels) return set_error(CRT_ERR_LIMIT, "BVH deeper than the traversal stack allows");
        k_choose<<<blocks(F), kBlock, 0, s>>>(cur, F, gn, dec, max_children, recs.as<GWide>(), cnt_int.as<uint32_t>(),
                                              cnt_tri.as<uint32_t>(), ni, err);
        // exclusive sums over F + 1 entries: the last is each level's total
        CRT_CUDA(cudaMemsetAsync(cnt_int.as<uint32_t>() + F, 0, 4, s));
        CRT_CUDA(cudaMemsetAsync(cnt_tri.as<uint32_t>() + F, 0, 4, s));
        CRT_CUDA(cub::DeviceScan::ExclusiveSum(scan_tmp.p, scan_bytes, cnt_int.as<uint32_t>(), off_int.as<uint32_t>(),
                                               (int)F + 1, s));
        CRT_CUDA(cub::DeviceScan::ExclusiveSum(scan_tmp.p, scan_bytes, cnt_tri.as<uint32_t>(), off_tri.as<uint32_t>(),
                                               (int)F + 1, s));
        const uint32_t next_base = level_base + F;
        k_emit<<<blocks(F), kBlock, 0, s>>>(recs.as<GWide>(), F, level_base, next_base, tri_base,
                                            off_int.as<uint32_t>(), off_tri.as<uint32_t>(), gn, dec, perm.as<uint32_t>(),
                                            d_v1, d_e1, d_e2, nodes_out.as<Bvh8Node>(), fnodes_out.as<Bvh8FloatNode>(),
                                            tris_out.as<TriRecord>(), nxt, n, cap_nodes, err);
        uint32_t totals[2];
        CRT_CUDA(cudaMemcpyAsync(&totals[0], off_int.as<uint32_t>() + F, 4, cudaMemcpyDeviceToHost, s));
        CRT_CUDA(cudaMemcpyAsync(&totals[1], off_tri.as<uint32_t>() + F, 4, cudaMemcpyDeviceToHost, s));
        CRT_CUDA(cudaStreamSynchronize(s));
        CRT_CUDA(cudaGetLastError());
        level_base = next_base;
        tri_base += totals[1];
        F = totals[0];
        if (level_base + F > cap_nodes) return set_error(CRT_ERR_LIMIT, "GPU BVH node count overflow");
        std::swap(cur, nxt);
    }
    uint32_t errbits = 0;
    CRT_CUDA(cudaMemcpyAsync(&errbits, err, 4, cudaMemcpyDeviceToHost, s));
    CRT_CUDA(cudaStreamSynchronize(s));
    if (errbits) return set_error(CRT_ERR_CUDA, "GPU BVH build: inconsistent tree (" + std::to_string(errbits) + ")");
    if (tri_base != n) return set_error(CRT_ERR_CUDA, "GPU BVH lost triangles");
    *num_nodes = level_base;
    *max_depth = depth;
    *fnodes_ok = level_base <= (1u << 24);
    return CRT_OK;
}

}  // namespace crt
