// bvh8.cpp -- host build of the 8-wide quantised BVH (see bvh8.h).
#include "bvh8.h"

#include <algorithm>
#include <array>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <future>
#include <memory>
#include <mutex>
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
    int32_t left, right;     // children; -1 for a leaf
    uint32_t first, count;   // range of the index array the node covers
};

constexpr int kBins = 32;
constexpr uint32_t kSmallMax = 32;        // ranges up to this size get an exact SAH sweep
// The binary build goes down to single triangles; the collapse to wide nodes
// is SAH-optimal by dynamic programming over that tree (Ylitie, Karras and
// Laine, "Efficient Incoherent Ray Traversal on GPUs Through Compressed Wide
// BVHs", HPG 2017) and also decides which subtrees of at most 3 triangles
// become leaf slots.  The triangle test costs 0.5 of a wide-node visit in
// the cost model (0.2 / 0.3 / 0.5 / 1.0 measured on C2 and C3: 0.5 fastest).
// Against the earlier greedy collapse (open the largest-area child, leaves
// of 2) it traces 4% faster with 37% fewer nodes.
constexpr uint32_t kLeafMax = 1;
constexpr uint32_t kSlotTrisMax = 3;   // triangles a leaf slot holds (3-bit count)
constexpr float kTriCost = 0.5f;
constexpr uint32_t kParallelMin = 1u << 15;

struct Builder {
    const Box* tbox;
    const float* cent;     // [n][3]
    uint32_t* idx;
    unsigned hw_threads;

    // Bins of idx[s, e) along every axis with a positive centroid extent.
    struct Bins {
        Box bb[3][kBins];
        uint32_t cnt[3][kBins];
        void reset() {
            for (int ax = 0; ax < 3; ++ax)
                for (int b = 0; b < kBins; ++b) {
                    bb[ax][b].reset();
                    cnt[ax][b] = 0;
                }
        }
        void merge(const Bins& o) {
            for (int ax = 0; ax < 3; ++ax)
                for (int b = 0; b < kBins; ++b) {
                    bb[ax][b].grow(o.bb[ax][b]);
                    cnt[ax][b] += o.cnt[ax][b];
                }
        }
    };

    // One axis at a time: each pass streams idx[s, e) once.
    void bin_range(uint32_t s, uint32_t e, const Box& cb, const float scale[3], Bins& B) const {
        for (int ax = 0; ax < 3; ++ax) {
            if (!(scale[ax] > 0.f)) continue;
            const float lo = cb.lo[ax], sc = scale[ax];
            Box* bb = B.bb[ax];
            uint32_t* cnt = B.cnt[ax];
            for (uint32_t i = s; i < e; ++i) {
                const uint32_t t = idx[i];
                int b = std::min(kBins - 1, (int)((cent[3 * t + ax] - lo) * sc));
                b = std::max(b, 0);
                cnt[b]++;
                bb[b].grow(tbox[t]);
            }
        }
    }

    // Binned SAH split of idx[start, end); returns mid (start < mid < end).
    // Large ranges are binned by several threads; boxes merge by min / max
    // and counts by sums, so the split does not depend on the thread count.
    // Exact SAH split of a small range: per axis, sort by centroid and sweep
    // every split position (cheaper than 32 bins per axis, and exact).
    uint32_t split_small(uint32_t start, uint32_t end) const {
        const uint32_t n = end - start;
        uint32_t order[3][kSmallMax];
        float right_area[kSmallMax];
        float best_cost = FLT_MAX;
        int best_axis = -1;
        uint32_t best_pos = 0;
        for (int ax = 0; ax < 3; ++ax) {
            uint32_t* o = order[ax];
            for (uint32_t i = 0; i < n; ++i) o[i] = idx[start + i];
            // insertion sort by centroid, ties by triangle index (deterministic)
            for (uint32_t i = 1; i < n; ++i) {
                const uint32_t t = o[i];
                const float c = cent[3 * t + ax];
                uint32_t j = i;
                while (j > 0 && (cent[3 * o[j - 1] + ax] > c || (cent[3 * o[j - 1] + ax] == c && o[j - 1] > t))) {
                    o[j] = o[j - 1];
                    --j;
                }
                o[j] = t;
            }
            Box acc;
            acc.reset();
            for (uint32_t i = n; i-- > 1;) {
                acc.grow(tbox[o[i]]);
                right_area[i] = acc.half_area();
            }
            acc.reset();
            for (uint32_t i = 1; i < n; ++i) {
                acc.grow(tbox[o[i - 1]]);
                const float cost = acc.half_area() * i + right_area[i] * (n - i);
                if (cost < best_cost) { best_cost = cost; best_axis = ax; best_pos = i; }
            }
        }
        if (best_axis < 0) return start + n / 2;
        for (uint32_t i = 0; i < n; ++i) idx[start + i] = order[best_axis][i];
        return start + best_pos;
    }

    uint32_t split(uint32_t start, uint32_t end, const Box& cb) const {
        if (end - start <= kSmallMax) return split_small(start, end);
        float scale[3];
        for (int ax = 0; ax < 3; ++ax) {
            const float ext = cb.hi[ax] - cb.lo[ax];
            scale[ax] = ext > 0.f ? kBins / ext : 0.f;
        }
        Bins B;
        B.reset();
        const uint32_t n = end - start;
        const unsigned parts = n >= (1u << 16) ? std::min<unsigned>(hw_threads, n >> 15) : 1u;
        if (parts > 1) {
            std::vector<Bins> part(parts);
            std::vector<std::thread> pool;
            for (unsigned p = 0; p < parts; ++p) {
                const uint32_t s = start + (uint32_t)((uint64_t)n * p / parts);
                const uint32_t e = start + (uint32_t)((uint64_t)n * (p + 1) / parts);
                pool.emplace_back([&, p, s, e] {
                    part[p].reset();
                    bin_range(s, e, cb, scale, part[p]);
                });
            }
            for (std::thread& t : pool) t.join();
            for (const Bins& q : part) B.merge(q);
        } else {
            bin_range(start, end, cb, scale, B);
        }
        float best_cost = FLT_MAX;
        int best_axis = -1, best_bin = 0;
        for (int ax = 0; ax < 3; ++ax) {
            if (!(scale[ax] > 0.f)) continue;
            float left_area[kBins];
            uint32_t left_cnt[kBins];
            Box acc;
            acc.reset();
            uint32_t c = 0;
            for (int b = 0; b < kBins; ++b) {
                acc.grow(B.bb[ax][b]);
                c += B.cnt[ax][b];
                left_area[b] = acc.half_area();
                left_cnt[b] = c;
            }
            acc.reset();
            c = 0;
            for (int b = kBins - 1; b > 0; --b) {
                acc.grow(B.bb[ax][b]);
                c += B.cnt[ax][b];
                if (left_cnt[b - 1] == 0 || c == 0) continue;
                float cost = left_area[b - 1] * left_cnt[b - 1] + acc.half_area() * c;
                if (cost < best_cost) { best_cost = cost; best_axis = ax; best_bin = b - 1; }
            }
        }
        if (best_axis < 0) return start + (end - start) / 2;   // coincident centroids
        const float sc = scale[best_axis];
        const float lo = cb.lo[best_axis];
        uint32_t* mid = std::partition(idx + start, idx + end, [&](uint32_t t) {
            int b = std::min(kBins - 1, (int)((cent[3 * t + best_axis] - lo) * sc));
            return std::max(b, 0) <= best_bin;
        });
        uint32_t m = (uint32_t)(mid - idx);
        if (m == start || m == end) m = start + (end - start) / 2;
        return m;
    }

    // Bounds of the triangles and of the centroids of idx[s, e).
    void bounds(uint32_t s, uint32_t e, Box& nb, Box& cb) const {
        for (uint32_t i = s; i < e; ++i) {
            uint32_t t = idx[i];
            nb.grow(tbox[t]);
            for (int k = 0; k < 3; ++k) {
                cb.lo[k] = std::min(cb.lo[k], cent[3 * t + k]);
                cb.hi[k] = std::max(cb.hi[k], cent[3 * t + k]);
            }
        }
    }

    // Builds idx[start, end) at nodes[slot]: a subtree of m primitives owns
    // slots [slot, slot + 2m - 1) (a binary tree has at most 2m - 1 nodes),
    // so subtrees built in parallel write disjoint ranges of one array.
    void build(uint32_t start, uint32_t end, Node2* nodes, uint32_t slot, int par_depth) const {
        Box nb, cb;
        nb.reset();
        cb.reset();
        const uint32_t parts = end - start >= (1u << 16) ? std::min<unsigned>(hw_threads, (end - start) >> 15) : 1u;
        if (parts > 1) {   // min / max merge exactly, in any order
            std::vector<Box> pn(parts), pc(parts);
            std::vector<std::thread> pool;
            for (uint32_t p = 0; p < parts; ++p) {
                pn[p].reset();
                pc[p].reset();
                const uint32_t s = start + (uint32_t)((uint64_t)(end - start) * p / parts);
                const uint32_t e = start + (uint32_t)((uint64_t)(end - start) * (p + 1) / parts);
                pool.emplace_back([&, p, s, e] { bounds(s, e, pn[p], pc[p]); });
            }
            for (std::thread& t : pool) t.join();
            for (uint32_t p = 0; p < parts; ++p) {
                nb.grow(pn[p]);
                cb.grow(pc[p]);
            }
        } else {
            bounds(start, end, nb, cb);
        }
        Node2& me = nodes[slot];
        me.box = nb;
        me.first = start;
        me.count = end - start;
        if (end - start <= kLeafMax) {
            me.left = me.right = -1;
            return;
        }
        const uint32_t mid = split(start, end, cb);
        const uint32_t lslot = slot + 1, rslot = slot + 2 * (mid - start);
        me.left = (int32_t)lslot;
        me.right = (int32_t)rslot;
        if (par_depth > 0 && end - start >= kParallelMin) {
            auto fut = std::async(std::launch::async, [&] { build(start, mid, nodes, lslot, par_depth - 1); });
            build(mid, end, nodes, rslot, par_depth - 1);
            fut.get();
        } else {
            build(start, mid, nodes, lslot, 0);
            build(mid, end, nodes, rslot, 0);
        }
    }
};

// Runs f(begin, end) over [0, n) split across the hardware threads.
template <class F>
void parallel_for(size_t n, F f) {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    if (n < 8192 || hw == 1) {
        f(size_t(0), n);
        return;
    }
    const size_t chunk = (n + hw - 1) / hw;
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < hw; ++t) {
        const size_t b = t * chunk, e = std::min(n, b + chunk);
        if (b >= e) break;
        pool.emplace_back(f, b, e);
    }
    for (std::thread& t : pool) t.join();
}

// Smallest e with ext <= 255 * 2^e, clamped to the normal float range.
int scale_exponent(double ext) {
    if (!(ext > 0.0)) return -126;
    int k;
    double m = std::frexp(ext / 255.0, &k);   // ext/255 = m * 2^k, m in [0.5, 1)
    int e = (m == 0.5) ? k - 1 : k;
    return std::max(-126, std::min(127, e));
}

}  // namespace

// SAH-optimal collapse of a binary tree into nodes of at most W children
// (Ylitie et al. 2017, section 4): with C(x, i) the least SAH cost of the
// subtree of x as at most i slots,
//   C(x, 1) = min(c_tri * A(x) * N(x)  [x a leaf slot, N(x) <= 3],
//                 A(x) + D(x, W)       [x a wide node]),
//   C(x, i) = min(C(x, i - 1), D(x, i)),  D(x, i) = min_k C(l, k) + C(r, i - k),
// computed bottom-up (subtrees in parallel); the decisions then give each
// wide node its children.
struct DpCollapse {
    struct Dec {
        uint8_t leaf;        // as one slot: a leaf slot (else a wide node)
        uint8_t wk;          // as a wide node: slots of the left child
        uint8_t split[9];    // with at most i slots (i >= 2): slots of the left child, 0 = as with i - 1
    };
    using Costs = std::array<float, 9>;
    const Node2* n2;
    std::vector<Dec> dec;
    int W;
    float ctri;

    Costs run(int32_t x, int par_depth) {
        const Node2& nd = n2[x];
        const float A = nd.box.half_area();
        const float leafc = nd.count <= kSlotTrisMax ? ctri * A * (float)nd.count : FLT_MAX;
        Dec& d = dec[x];
        Costs C;
        C[0] = 0.f;
        if (nd.left < 0) {
            for (int i = 1; i <= W; ++i) {
                C[i] = leafc;
                d.split[i] = 0;
            }
            d.leaf = 1;
            d.wk = 0;
            return C;
        }
        Costs L, R;
        if (par_depth > 0 && nd.count >= kParallelMin) {
            auto fut = std::async(std::launch::async, [&] { return run(nd.left, par_depth - 1); });
            R = run(nd.right, par_depth - 1);
            L = fut.get();
        } else {
            L = run(nd.left, 0);
            R = run(nd.right, 0);
        }
        float D[9];
        uint8_t K[9];
        for (int i = 2; i <= W; ++i) {
            D[i] = FLT_MAX;
            K[i] = 1;
            for (int k = 1; k < i; ++k) {
                const float c = L[k] + R[i - k];
                if (c < D[i]) {
                    D[i] = c;
                    K[i] = (uint8_t)k;
                }
            }
        }
        const float wide = A + D[W];
        d.leaf = leafc <= wide;
        d.wk = K[W];
        C[1] = d.leaf ? leafc : wide;
        d.split[1] = 0;
        for (int i = 2; i <= W; ++i) {
            if (D[i] < C[i - 1]) {
                C[i] = D[i];
                d.split[i] = K[i];
            } else {
                C[i] = C[i - 1];
                d.split[i] = 0;
            }
        }
        return C;
    }
    // The slots of the subtree of x when it may use at most i of them.
    void expand(int32_t x, int i, int32_t* out, int& n) const {
        while (i > 1 && dec[x].split[i] == 0) --i;
        if (i == 1) {
            out[n++] = x;
            return;
        }
        const int k = dec[x].split[i];
        expand(n2[x].left, k, out, n);
        expand(n2[x].right, i - k, out, n);
    }
    // Children of the wide node at x.
    int children(int32_t x, int32_t* out) const {
        int n = 0;
        expand(n2[x].left, dec[x].wk, out, n);
        expand(n2[x].right, W - dec[x].wk, out, n);
        return n;
    }
};

bool build_bvh8(const float* v1, const float* e1, const float* e2, uint32_t n,
                uint32_t max_levels, Bvh8& out, const char** msg, int max_children) {
    if (max_children != 4 && max_children != 8) { *msg = "BVH width must be 4 or 8"; return false; }
    if (n == 0) { *msg = "scene has no triangles"; return false; }
    // Margin: 2^-15 of the largest coordinate magnitude (at least 2^-15).
    std::mutex scale_mutex;
    double scale = 1.0;
    parallel_for(n, [&](size_t t0, size_t t1) {
        double s = 1.0;
        for (uint64_t i = 3 * t0; i < 3 * t1; ++i) {
            s = std::max(s, (double)std::fabs(v1[i]));
            s = std::max(s, (double)std::fabs(v1[i] + e1[i]));
            s = std::max(s, (double)std::fabs(v1[i] + e2[i]));
        }
        std::lock_guard<std::mutex> lock(scale_mutex);
        scale = std::max(scale, s);
    });
    const float margin = (float)std::ldexp(scale, -15);
    std::vector<Box> tbox(n);
    std::vector<float> cent(3ull * n);
    parallel_for(n, [&](size_t t0, size_t t1) {
        for (size_t t = t0; t < t1; ++t) {
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
    });
    std::vector<uint32_t> idx(n);
    for (uint32_t i = 0; i < n; ++i) idx[i] = i;
    Builder b{tbox.data(), cent.data(), idx.data(), std::max(1u, std::thread::hardware_concurrency())};
    std::unique_ptr<Node2[]> n2_store(new Node2[2ull * n - 1]);   // slots, see Builder::build
    const Node2* n2 = n2_store.get();
    unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    int par_depth = 0;
    while ((1u << par_depth) < hw * 2 && par_depth < 8) ++par_depth;
    b.build(0, n, n2_store.get(), 0, par_depth);
    const int32_t root = 0;
    DpCollapse dp{n2, {}, max_children, kTriCost};
    dp.dec.resize(2ull * n - 1);
    dp.run(root, par_depth);
    // a slot of a wide node is a leaf slot or another wide node
    auto leaf_slot = [&](int32_t x) { return dp.dec[x].leaf != 0; };

    // ---- collapse to max_children-wide nodes, breadth-first layout --------
    // 1. (serial, cheap) each wide node takes the children the SAH-optimal
    //    collapse chose;
    // 2. (parallel) children are assigned to slots by octant;
    // 3. (serial, cheap) breadth-first numbering in slot order gives each
    //    node its child and triangle base;
    // 4. (parallel) nodes are encoded and triangle records written.
    struct Wide {
        int32_t nch;
        int32_t ch[8];       // BVH2 children
        int32_t rec[8];      // wide record of an internal child, else -1
        int32_t slot_of[8];
        uint32_t depth;
    };
    std::vector<Wide> recs;
    recs.reserve(n / 2 + 1);
    auto add_record = [&](int32_t node2, uint32_t depth) {
        Wide w;
        std::memset(&w, 0, sizeof(w));
        w.depth = depth;
        int32_t* ch = w.ch;
        int nch = 0;
        if (leaf_slot(node2)) {
            ch[nch++] = node2;                 // single-leaf root
        } else {
            nch = dp.children(node2, ch);
        }
        w.nch = nch;
        recs.push_back(w);
    };
    add_record(root, 1);
    out.max_depth = 0;
    for (size_t r = 0; r < recs.size(); ++r) {
        const uint32_t depth = recs[r].depth;
        out.max_depth = std::max(out.max_depth, depth);
        if (depth > max_levels) { *msg = "BVH deeper than the traversal stack allows"; return false; }
        for (int c = 0; c < recs[r].nch; ++c) {
            const int32_t x = recs[r].ch[c];
            if (!leaf_slot(x)) {
                recs[r].rec[c] = (int32_t)recs.size();
                add_record(x, depth + 1);
            } else {
                recs[r].rec[c] = -1;
            }
        }
    }
    parallel_for(recs.size(), [&](size_t r0, size_t r1) {
        for (size_t r = r0; r < r1; ++r) {
            Wide& w = recs[r];
            Box nb;
            nb.reset();
            for (int c = 0; c < w.nch; ++c) nb.grow(n2[w.ch[c]].box);
            float pc[3];
            for (int k = 0; k < 3; ++k) pc[k] = 0.5f * (nb.lo[k] + nb.hi[k]);
            bool used_slot[8] = {false}, placed[8] = {false};
            for (int round = 0; round < w.nch; ++round) {
                float best = -FLT_MAX;
                int bc = -1, bs = -1;
                for (int c = 0; c < w.nch; ++c) {
                    if (placed[c]) continue;
                    const Box& cb = n2[w.ch[c]].box;
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
                w.slot_of[bc] = bs;
            }
        }
    });
    // breadth-first numbering in slot order
    std::vector<int32_t> rec_at;                   // record of each wide node
    rec_at.reserve(recs.size());
    std::vector<uint32_t> child_base(recs.size()), tri_base(recs.size());
    rec_at.push_back(0);
    uint32_t tris_so_far = 0;
    for (size_t q = 0; q < rec_at.size(); ++q) {
        const Wide& w = recs[rec_at[q]];
        int child_at[8];
        for (int s = 0; s < 8; ++s) child_at[s] = -1;
        for (int c = 0; c < w.nch; ++c) child_at[w.slot_of[c]] = c;
        child_base[q] = (uint32_t)rec_at.size();
        tri_base[q] = tris_so_far;
        for (int s = 0; s < 8; ++s) {
            const int c = child_at[s];
            if (c < 0) continue;
            if (w.rec[c] >= 0) rec_at.push_back(w.rec[c]);
            else tris_so_far += n2[w.ch[c]].count;
        }
    }
    const size_t nn = rec_at.size();
    out.nodes.assign(nn, Bvh8Node{});
    out.fnodes.assign(nn, Bvh8FloatNode{});
    out.tris.assign(tris_so_far, TriRecord{});
    out.margin = margin;
    out.fnodes_ok = nn == 0 || child_base[nn - 1] < (1u << 24);   // 24-bit child index
    parallel_for(nn, [&](size_t q0, size_t q1) {
        for (size_t q = q0; q < q1; ++q) {
            const Wide& w = recs[rec_at[q]];
            int child_at[8];
            for (int s = 0; s < 8; ++s) child_at[s] = -1;
            for (int c = 0; c < w.nch; ++c) child_at[w.slot_of[c]] = c;
            Box nb;
            nb.reset();
            for (int c = 0; c < w.nch; ++c) nb.grow(n2[w.ch[c]].box);
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
            node.child_base = child_base[q];
            node.tri_base = tri_base[q];
            uint32_t tri_off = 0;
            for (int s = 0; s < 8; ++s) {
                const int c = child_at[s];
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
                const Node2& cn = n2[w.ch[c]];
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
                if (w.rec[c] >= 0) {
                    node.imask |= (uint8_t)(1u << s);
                    node.meta[s] = 0x80;
                } else {
                    node.meta[s] = (uint8_t)((cn.count << 5) | tri_off);
                    for (uint32_t i = 0; i < cn.count; ++i) {
                        uint32_t t = idx[cn.first + i];
                        TriRecord& r = out.tris[node.tri_base + tri_off + i];
                        for (int k = 0; k < 3; ++k) {
                            r.v1[k] = v1[3 * t + k];
                            r.e1[k] = e1[3 * t + k];
                            r.e2[k] = e2[3 * t + k];
                        }
                        r.face = t;
                        r.pad1 = r.pad2 = 0.f;
                    }
                    tri_off += cn.count;
                }
            }
            out.nodes[q] = node;
            fnode.child_base_imask = node.child_base | ((uint32_t)node.imask << 24);
            fnode.tri_base = node.tri_base;
            std::memcpy(fnode.meta, node.meta, 8);
            out.fnodes[q] = fnode;
        }
    });
    *msg = nullptr;
    return true;
}

}  // namespace crt
