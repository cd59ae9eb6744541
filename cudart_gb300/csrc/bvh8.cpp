// bvh8.cpp -- host build of the 8-wide quantised BVH (see bvh8.h).
#include "bvh8.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <future>
#include <thread>

namespace crt {
namespace {

struct Box {
    float lo[3], hi[3];
    void reset() {
        for (int k = 0; k < 3; ++k) { lo[k] = FLT_MAX; hi[k] = -FLT_MAX; }
    }
    void grow(const Box& b) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], b.lo[k]);
            hi[k] = std::max(hi[k], b.hi[k]);
        }
    }
    float half_area() const {
        float dx = std::max(hi[0] - lo[0], 0.f), dy = std::max(hi[1] - lo[1], 0.f),
              dz = std::max(hi[2] - lo[2], 0.f);
        return dx * dy + dy * dz + dz * dx;
    }
};

struct Node2 {
    Box box;
    int32_t left = -1, right = -1;   // children (internal)
    uint32_t first = 0, count = 0;   // leaf range into the index array (count > 0)
};

constexpr int kBins = 32;
constexpr uint32_t kLeafMax = 3;          // the reference's maxTrisInNode (bvh.cpp:62)
constexpr uint32_t kParallelMin = 1u << 15;

struct Builder {
    const Box* tbox;
    const float* cent;     // [n][3]
    uint32_t* idx;

    // Binned SAH split of idx[start, end); returns mid (start < mid < end).
    uint32_t split(uint32_t start, uint32_t end, const Box& cb) const {
        float best_cost = FLT_MAX;
        int best_axis = -1, best_bin = 0;
        for (int ax = 0; ax < 3; ++ax) {
            float ext = cb.hi[ax] - cb.lo[ax];
            if (!(ext > 0.f)) continue;
            float scale = kBins / ext;
            Box bb[kBins];
            uint32_t cnt[kBins] = {0};
            for (int b = 0; b < kBins; ++b) bb[b].reset();
            for (uint32_t i = start; i < end; ++i) {
                uint32_t t = idx[i];
                int b = std::min(kBins - 1, (int)((cent[3 * t + ax] - cb.lo[ax]) * scale));
                b = std::max(b, 0);
                cnt[b]++;
                bb[b].grow(tbox[t]);
            }
            float left_area[kBins];
            uint32_t left_cnt[kBins];
            Box acc;
            acc.reset();
            uint32_t c = 0;
            for (int b = 0; b < kBins; ++b) {
                acc.grow(bb[b]);
                c += cnt[b];
                left_area[b] = acc.half_area();
                left_cnt[b] = c;
            }
            acc.reset();
            c = 0;
            for (int b = kBins - 1; b > 0; --b) {
                acc.grow(bb[b]);
                c += cnt[b];
                if (left_cnt[b - 1] == 0 || c == 0) continue;
                float cost = left_area[b - 1] * left_cnt[b - 1] + acc.half_area() * c;
                if (cost < best_cost) { best_cost = cost; best_axis = ax; best_bin = b - 1; }
            }
        }
        if (best_axis < 0) return start + (end - start) / 2;   // coincident centroids
        float scale = kBins / (cb.hi[best_axis] - cb.lo[best_axis]);
        float lo = cb.lo[best_axis];
        uint32_t* mid = std::partition(idx + start, idx + end, [&](uint32_t t) {
            int b = std::min(kBins - 1, (int)((cent[3 * t + best_axis] - lo) * scale));
            return std::max(b, 0) <= best_bin;
        });
        uint32_t m = (uint32_t)(mid - idx);
        if (m == start || m == end) m = start + (end - start) / 2;
        return m;
    }

    // Builds idx[start, end) into `out`; returns the subtree root index.
    int32_t build(uint32_t start, uint32_t end, std::vector<Node2>& out, int par_depth) const {
        Box nb, cb;
        nb.reset();
        cb.reset();
        for (uint32_t i = start; i < end; ++i) {
            uint32_t t = idx[i];
            nb.grow(tbox[t]);
            for (int k = 0; k < 3; ++k) {
                cb.lo[k] = std::min(cb.lo[k], cent[3 * t + k]);
                cb.hi[k] = std::max(cb.hi[k], cent[3 * t + k]);
            }
        }
        int32_t me = (int32_t)out.size();
        out.emplace_back();
        out[me].box = nb;
        if (end - start <= kLeafMax) {
            out[me].first = start;
            out[me].count = end - start;
            return me;
        }
        uint32_t mid = split(start, end, cb);
        if (par_depth > 0 && end - start >= kParallelMin) {
            std::vector<Node2> lv;
            auto fut = std::async(std::launch::async, [&] { return build(start, mid, lv, par_depth - 1); });
            std::vector<Node2> rv;
            int32_t rr = build(mid, end, rv, par_depth - 1);
            int32_t lr = fut.get();
            int32_t lbase = (int32_t)out.size();
            for (Node2 n : lv) {
                if (n.count == 0) { n.left += lbase; n.right += lbase; }
                out.push_back(n);
            }
            int32_t rbase = (int32_t)out.size();
            for (Node2 n : rv) {
                if (n.count == 0) { n.left += rbase; n.right += rbase; }
                out.push_back(n);
            }
            out[me].left = lbase + lr;
            out[me].right = rbase + rr;
        } else {
            int32_t l = build(start, mid, out, 0);
            int32_t r = build(mid, end, out, 0);
            out[me].left = l;
            out[me].right = r;
        }
        return me;
    }
};

// Smallest e with ext <= 255 * 2^e, clamped to the normal float range.
int scale_exponent(double ext) {
    if (!(ext > 0.0)) return -126;
    int k;
    double m = std::frexp(ext / 255.0, &k);   // ext/255 = m * 2^k, m in [0.5, 1)
    int e = (m == 0.5) ? k - 1 : k;
    return std::max(-126, std::min(127, e));
}

}  // namespace

bool build_bvh8(const float* v1, const float* e1, const float* e2, uint32_t n,
                uint32_t max_levels, Bvh8& out, const char** msg, int max_children) {
    if (max_children != 4 && max_children != 8) { *msg = "BVH width must be 4 or 8"; return false; }
    if (n == 0) { *msg = "scene has no triangles"; return false; }
    // Margin: 2^-15 of the largest coordinate magnitude (at least 2^-15).
    double scale = 1.0;
    for (uint64_t i = 0; i < 3ull * n; ++i) {
        scale = std::max(scale, (double)std::fabs(v1[i]));
        scale = std::max(scale, (double)std::fabs(v1[i] + e1[i]));
        scale = std::max(scale, (double)std::fabs(v1[i] + e2[i]));
    }
    const float margin = (float)std::ldexp(scale, -15);
    std::vector<Box> tbox(n);
    std::vector<float> cent(3ull * n);
    for (uint32_t t = 0; t < n; ++t) {
        for (int k = 0; k < 3; ++k) {
            double a = v1[3 * t + k];
            double b = a + (double)e1[3 * t + k];
            double c = a + (double)e2[3 * t + k];
            double lo = std::min(a, std::min(b, c)), hi = std::max(a, std::max(b, c));
            tbox[t].lo[k] = (float)(lo - margin);
            tbox[t].hi[k] = (float)(hi + margin);
            if ((double)tbox[t].lo[k] > lo - margin) tbox[t].lo[k] = std::nextafter(tbox[t].lo[k], -FLT_MAX);
            if ((double)tbox[t].hi[k] < hi + margin) tbox[t].hi[k] = std::nextafter(tbox[t].hi[k], FLT_MAX);
            cent[3 * t + k] = 0.5f * (tbox[t].lo[k] + tbox[t].hi[k]);
        }
    }
    std::vector<uint32_t> idx(n);
    for (uint32_t i = 0; i < n; ++i) idx[i] = i;
    Builder b{tbox.data(), cent.data(), idx.data()};
    std::vector<Node2> n2;
    n2.reserve(2ull * n);
    unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    int par_depth = 0;
    while ((1u << par_depth) < hw * 2 && par_depth < 8) ++par_depth;
    int32_t root = b.build(0, n, n2, par_depth);

    // ---- collapse to 8-wide, breadth first --------------------------------
    struct Item { int32_t n2; uint32_t depth; };
    std::vector<Item> queue;
    queue.push_back({root, 1});
    out.nodes.clear();
    out.tris.clear();
    out.tris.reserve(n);
    out.max_depth = 0;
    out.margin = margin;
    out.fnodes.clear();
    out.fnodes_ok = true;
    out.nodes.resize(1);
    for (size_t qi = 0; qi < queue.size(); ++qi) {
        const Item it = queue[qi];
        out.max_depth = std::max(out.max_depth, it.depth);
        if (it.depth > max_levels) { *msg = "BVH deeper than the traversal stack allows"; return false; }
        int32_t ch[8];
        int nch = 0;
        if (n2[it.n2].count > 0) {
            ch[nch++] = it.n2;                 // single-leaf root
        } else {
            ch[nch++] = n2[it.n2].left;
            ch[nch++] = n2[it.n2].right;
            while (nch < max_children) {
                int best = -1;
                float area = -1.f;
                for (int c = 0; c < nch; ++c)
                    if (n2[ch[c]].count == 0 && n2[ch[c]].box.half_area() > area) {
                        area = n2[ch[c]].box.half_area();
                        best = c;
                    }
                if (best < 0) break;
                int32_t x = ch[best];
                ch[best] = n2[x].left;
                ch[nch++] = n2[x].right;
            }
        }
        // node box and slot assignment by octant
        Box nb;
        nb.reset();
        for (int c = 0; c < nch; ++c) nb.grow(n2[ch[c]].box);
        float pc[3];
        for (int k = 0; k < 3; ++k) pc[k] = 0.5f * (nb.lo[k] + nb.hi[k]);
        int slot_of[8];
        bool used_slot[8] = {false}, placed[8] = {false};
        for (int round = 0; round < nch; ++round) {
            float best = -FLT_MAX;
            int bc = -1, bs = -1;
            for (int c = 0; c < nch; ++c) {
                if (placed[c]) continue;
                const Box& cb = n2[ch[c]].box;
                float d[3];
                for (int k = 0; k < 3; ++k) d[k] = 0.5f * (cb.lo[k] + cb.hi[k]) - pc[k];
                for (int s = 0; s < 8; ++s) {
                    if (used_slot[s]) continue;
                    float sc = ((s & 1) ? d[0] : -d[0]) + ((s & 2) ? d[1] : -d[1]) + ((s & 4) ? d[2] : -d[2]);
                    if (sc > best) { best = sc; bc = c; bs = s; }
                }
            }
            placed[bc] = true;
            used_slot[bs] = true;
            slot_of[bc] = bs;
        }
        int child_at[8];
        for (int s = 0; s < 8; ++s) child_at[s] = -1;
        for (int c = 0; c < nch; ++c) child_at[slot_of[c]] = ch[c];

        Bvh8Node node;
        std::memset(&node, 0, sizeof(node));
        Bvh8FloatNode fnode;
        std::memset(&fnode, 0, sizeof(fnode));
        node.px = nb.lo[0];
        node.py = nb.lo[1];
        node.pz = nb.lo[2];
        int e[3];
        for (int k = 0; k < 3; ++k) e[k] = scale_exponent((double)nb.hi[k] - (double)nb.lo[k]);
        node.ex = (uint8_t)(e[0] + 127);
        node.ey = (uint8_t)(e[1] + 127);
        node.ez = (uint8_t)(e[2] + 127);
        node.child_base = (uint32_t)out.nodes.size();
        node.tri_base = (uint32_t)out.tris.size();
        uint32_t tri_off = 0;
        for (int s = 0; s < 8; ++s) {
            int32_t c = child_at[s];
            if (c < 0) {
                // empty slot: inverted box (lo plane above hi plane) never hits
                for (int k = 0; k < 3; ++k) {
                    node.qlo[k][s] = 255;
                    node.qhi[k][s] = 0;
                    fnode.lo[k][s] = FLT_MAX;
                    fnode.hi[k][s] = -FLT_MAX;
                }
                continue;
            }
            const Node2& cn = n2[c];
            for (int k = 0; k < 3; ++k) {
                fnode.lo[k][s] = cn.box.lo[k];
                fnode.hi[k][s] = cn.box.hi[k];
            }
            for (int k = 0; k < 3; ++k) {
                double step = std::ldexp(1.0, e[k]);
                double lo = std::floor(((double)cn.box.lo[k] - (double)nb.lo[k]) / step);
                double hi = std::ceil(((double)cn.box.hi[k] - (double)nb.lo[k]) / step);
                node.qlo[k][s] = (uint8_t)std::max(0.0, std::min(255.0, lo));
                node.qhi[k][s] = (uint8_t)std::max(0.0, std::min(255.0, hi));
            }
            if (cn.count == 0) {
                node.imask |= (uint8_t)(1u << s);
                node.meta[s] = 0x80;
                queue.push_back({c, it.depth + 1});
            } else {
                node.meta[s] = (uint8_t)((cn.count << 5) | tri_off);
                for (uint32_t i = 0; i < cn.count; ++i) {
                    uint32_t t = idx[cn.first + i];
                    TriRecord r;
                    for (int k = 0; k < 3; ++k) {
                        r.v1[k] = v1[3 * t + k];
                        r.e1[k] = e1[3 * t + k];
                        r.e2[k] = e2[3 * t + k];
                    }
                    r.face = t;
                    r.pad1 = r.pad2 = 0.f;
                    out.tris.push_back(r);
                }
                tri_off += cn.count;
            }
        }
        out.nodes.resize(out.nodes.size() + __builtin_popcount(node.imask));
        out.nodes[qi] = node;
        if (node.child_base >= (1u << 24)) out.fnodes_ok = false;   // 24-bit child index
        fnode.child_base_imask = node.child_base | ((uint32_t)node.imask << 24);
        fnode.tri_base = node.tri_base;
        std::memcpy(fnode.meta, node.meta, 8);
        out.fnodes.resize(out.nodes.size());
        out.fnodes[qi] = fnode;
    }
    *msg = nullptr;
    return true;
}

}  // namespace crt
