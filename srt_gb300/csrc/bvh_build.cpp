// bvh_build.cpp — binned-SAH binary BVH, collapsed to 8-wide quantised nodes.
#include "bvh_build.h"

#include <algorithm>
#include <atomic>
#include <functional>
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>

namespace srt {
namespace {

constexpr int kBins = 32;
#ifndef SRT_BVH_MAX_LEAF
#define SRT_BVH_MAX_LEAF 3
#endif
constexpr int kMaxLeaf = SRT_BVH_MAX_LEAF;  // triangles per leaf child; 8 leaves fill the 32-bit leaf mask at 4
// SAH cost of a triangle test relative to a node visit in the collapse
#ifndef SRT_BVH_COST_PRIM
#define SRT_BVH_COST_PRIM 1.5f
#endif

struct Box {
    float lo[3], hi[3];
    void reset()
    {
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::numeric_limits<float>::infinity();
            hi[k] = -std::numeric_limits<float>::infinity();
        }
    }
    void grow(const Box& b)
    {
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], b.lo[k]);
            hi[k] = std::max(hi[k], b.hi[k]);
        }
    }
    void grow_pt(const float* p)
    {
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], p[k]);
            hi[k] = std::max(hi[k], p[k]);
        }
    }
    float area() const
    {
        float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        if (!(dx >= 0.0f) || !(dy >= 0.0f) || !(dz >= 0.0f)) return 0.0f;
        return 2.0f * (dx * dy + dy * dz + dz * dx);
    }
};

struct BinNode {
    Box box;
    int32_t left, right;    // children (internal)
    int32_t begin, count;   // prims (leaf, count > 0)
    int32_t rbegin, rcount; // the subtree's prims: idx[rbegin, rbegin + rcount)
};

struct Builder {
    const Box* tbox = nullptr;
    const float* cent = nullptr;
    std::vector<int32_t> idx;
    std::vector<BinNode> nodes;
    std::atomic<int32_t> nnodes{0};
    std::atomic<int> max_depth{0};

    void make_leaf(int ni, int begin, int n)
    {
        nodes[ni].left = nodes[ni].right = -1;
        nodes[ni].begin = begin;
        nodes[ni].count = n;
    }

    void build(int ni, int begin, int end, int depth, int spawn)
    {
        int md = max_depth.load();
        while (depth > md && !max_depth.compare_exchange_weak(md, depth)) {
        }
        Box bb, cb;
        bb.reset();
        cb.reset();
        for (int i = begin; i < end; ++i) {
            bb.grow(tbox[idx[i]]);
            cb.grow_pt(cent + 3 * (size_t)idx[i]);
        }
        nodes[ni].box = bb;
        nodes[ni].rbegin = begin;
        nodes[ni].rcount = end - begin;
        const int n = end - begin;
        if (n <= 1) {
            make_leaf(ni, begin, n);
            return;
        }
        // binned SAH over the three axes
        float best = std::numeric_limits<float>::infinity();
        int best_axis = -1, best_bin = -1;
        for (int ax = 0; ax < 3; ++ax) {
            float ext = cb.hi[ax] - cb.lo[ax];
            if (!(ext > 0.0f)) continue;
            float k = (float)kBins / ext;
            Box bin[kBins];
            int cnt[kBins];
            for (int b = 0; b < kBins; ++b) {
                bin[b].reset();
                cnt[b] = 0;
            }
            for (int i = begin; i < end; ++i) {
                int t = idx[i];
                int b = std::min(kBins - 1, (int)((cent[3 * (size_t)t + ax] - cb.lo[ax]) * k));
                cnt[b]++;
                bin[b].grow(tbox[t]);
            }
            float rarea[kBins];
            int rcnt[kBins];
            Box acc;
            acc.reset();
            int c = 0;
            for (int b = kBins - 1; b > 0; --b) {
                acc.grow(bin[b]);
                c += cnt[b];
                rarea[b] = acc.area();
                rcnt[b] = c;
            }
            acc.reset();
            c = 0;
            for (int b = 0; b < kBins - 1; ++b) {
                acc.grow(bin[b]);
                c += cnt[b];
                if (c == 0 || rcnt[b + 1] == 0) continue;
                float cost = acc.area() * (float)c + rarea[b + 1] * (float)rcnt[b + 1];
                if (cost < best) {
                    best = cost;
                    best_axis = ax;
                    best_bin = b;
                }
            }
        }
        float area = bb.area();
        if (n <= kMaxLeaf && (best_axis < 0 || (float)n * area <= area + best)) {
            make_leaf(ni, begin, n);
            return;
        }
        int mid = begin + n / 2;
        if (best_axis >= 0) {
            float ext = cb.hi[best_axis] - cb.lo[best_axis];
            float k = (float)kBins / ext;
            const float* cc = cent;
            int ax = best_axis, bsplit = best_bin;
            float lo = cb.lo[ax];
            auto it = std::partition(idx.begin() + begin, idx.begin() + end, [&](int32_t t) {
                int b = std::min(kBins - 1, (int)((cc[3 * (size_t)t + ax] - lo) * k));
                return b <= bsplit;
            });
            mid = (int)(it - idx.begin());
        }
        if (mid <= begin || mid >= end) {
            // all centroids in one bin: object median along the widest axis
            int ax = 0;
            for (int k2 = 1; k2 < 3; ++k2)
                if (cb.hi[k2] - cb.lo[k2] > cb.hi[ax] - cb.lo[ax]) ax = k2;
            mid = begin + n / 2;
            const float* cc = cent;
            std::nth_element(idx.begin() + begin, idx.begin() + mid, idx.begin() + end,
                             [&](int32_t a, int32_t b) { return cc[3 * (size_t)a + ax] < cc[3 * (size_t)b + ax]; });
        }
        int c = nnodes.fetch_add(2);
        nodes[ni].left = c;
        nodes[ni].right = c + 1;
        nodes[ni].begin = 0;
        nodes[ni].count = 0;
        if (spawn > 0 && n > 65536) {
            std::thread th([&, c, begin, mid, depth, spawn]() { build(c, begin, mid, depth + 1, spawn - 1); });
            build(c + 1, mid, end, depth + 1, spawn - 1);
            th.join();
        } else {
            build(c, begin, mid, depth + 1, 0);
            build(c + 1, mid, end, depth + 1, 0);
        }
    }
};

// Conservative 16-bit quantisation of a child interval on one axis.
void quantize(float origin, float scale, float clo, float chi, uint16_t& qlo, uint16_t& qhi)
{
    double l = std::floor(((double)clo - origin) / scale);
    double h = std::ceil(((double)chi - origin) / scale);
    long ql = (long)std::max(0.0, std::min(65535.0, l));
    long qh = (long)std::max(0.0, std::min(65535.0, h));
    while (ql > 0 && origin + (float)ql * scale > clo) --ql;
    while (qh < 65535 && origin + (float)qh * scale < chi) ++qh;
    qlo = (uint16_t)ql;
    qhi = (uint16_t)qh;
}

}  // namespace

void build_wide_bvh(int64_t num_tris, const float* tri9, int threads, WideBvh& out)
{
    out.nodes.clear();
    out.tri_order.clear();
    const int64_t n = num_tris;
    std::vector<Box> tbox((size_t)n);
    std::vector<float> cent((size_t)n * 3);
    for (int64_t i = 0; i < n; ++i) {
        Box& b = tbox[i];
        b.reset();
        b.grow_pt(tri9 + 9 * i);
        b.grow_pt(tri9 + 9 * i + 3);
        b.grow_pt(tri9 + 9 * i + 6);
        for (int k = 0; k < 3; ++k) cent[3 * i + k] = 0.5f * (b.lo[k] + b.hi[k]);
    }
    Builder B;
    B.tbox = tbox.data();
    B.cent = cent.data();
    B.idx.resize((size_t)n);
    for (int64_t i = 0; i < n; ++i) B.idx[i] = (int32_t)i;
    B.nodes.resize((size_t)std::max<int64_t>(1, 2 * n));
    B.nnodes = 1;
    int spawn = 0;
    while ((1 << spawn) < std::max(1, threads)) ++spawn;
    if (n > 0) {
        B.build(0, 0, (int)n, 1, spawn);
    } else {
        B.nodes[0].box.reset();
        B.make_leaf(0, 0, 0);
    }
    out.binary_depth = B.max_depth.load();

    // SAH-optimal collapse of the binary tree into 8-wide nodes (Ylitie,
    // Karras, Laine, HPG 2017, section 3.1): cost[n][i] is the least SAH cost
    // of the subtree at n given as at most i children of a wide node, with a
    // child either a leaf (at most kMaxLeaf triangles), or a wide node of its
    // own, or its subtree distributed over several slots.
    const int nn = B.nnodes.load();
    constexpr float kCostNode = 1.0f, kCostPrim = SRT_BVH_COST_PRIM;
    const float kInf = std::numeric_limits<float>::infinity();
    std::vector<float> cost((size_t)nn * 8, kInf);
    std::vector<uint8_t> dec((size_t)nn * 8, 0);  // [0]: 0 leaf / 1 wide node; [i]: 0 = as i, k = k slots left
    std::vector<uint8_t> split8((size_t)nn, 1);   // left slots when the node's own wide node splits 8 ways
    for (int ni = nn - 1; ni >= 0; --ni) {
        const BinNode& bn = B.nodes[ni];
        float* c = &cost[(size_t)ni * 8];
        uint8_t* d = &dec[(size_t)ni * 8];
        const float A = bn.box.area();
        if (bn.count > 0 || bn.left < 0) {
            for (int i = 0; i < 8; ++i) c[i] = A * (float)bn.count * kCostPrim;
            continue;
        }
        const float* cl = &cost[(size_t)bn.left * 8];
        const float* cr = &cost[(size_t)bn.right * 8];
        float dist[9];
        uint8_t kbest[9];
        for (int j = 2; j <= 8; ++j) {
            dist[j] = kInf;
            kbest[j] = 1;
            for (int k = 1; k < j; ++k) {
                const float v = cl[k - 1] + cr[j - k - 1];
                if (v < dist[j]) {
                    dist[j] = v;
                    kbest[j] = (uint8_t)k;
                }
            }
        }
        const float c_int = A * kCostNode + dist[8];
        const float c_leaf = bn.rcount <= kMaxLeaf ? A * (float)bn.rcount * kCostPrim : kInf;
        c[0] = std::min(c_leaf, c_int);
        d[0] = c_leaf <= c_int ? 0 : 1;
        split8[ni] = kbest[8];
        for (int i = 2; i <= 8; ++i) {
            if (dist[i] < c[i - 2]) {
                c[i - 1] = dist[i];
                d[i - 1] = kbest[i];
            } else {
                c[i - 1] = c[i - 2];
                d[i - 1] = 0;
            }
        }
    }
    // children of the wide node made at binary node m given j slots
    std::vector<std::pair<int, bool>> kids;  // (binary node, as a leaf)
    std::function<void(int, int)> resolve = [&](int m, int j) {
        const BinNode& bm = B.nodes[m];
        if (bm.count > 0 || bm.left < 0) {
            kids.push_back({m, true});
            return;
        }
        while (j > 1 && dec[(size_t)m * 8 + j - 1] == 0) --j;
        if (j == 1) {
            kids.push_back({m, dec[(size_t)m * 8] == 0});
            return;
        }
        const int k = dec[(size_t)m * 8 + j - 1];
        resolve(bm.left, k);
        resolve(bm.right, j - k);
    };

    static const float dirs[8][3] = {{1, 1, 1},  {-1, 1, 1},  {1, -1, 1},  {-1, -1, 1},
                                     {1, 1, -1}, {-1, 1, -1}, {1, -1, -1}, {-1, -1, -1}};
    struct Pending {
        int32_t wide, bin, depth;
    };
    std::vector<Pending> queue;
    queue.push_back({0, 0, 1});
    out.nodes.resize(1);
    out.tri_order.reserve((size_t)n);
    size_t qi = 0;
    int depth = 1;
    while (qi < queue.size()) {
        Pending p = queue[qi++];
        depth = std::max(depth, p.depth);
        const BinNode& b = B.nodes[p.bin];
        int ch[8];
        bool as_leaf[8] = {false, false, false, false, false, false, false, false};
        int nc = 0;
        kids.clear();
        if (b.count > 0 || b.left < 0) {
            if (b.count > 0) kids.push_back({p.bin, true});
        } else if (p.bin == 0 && dec[0] == 0) {
            kids.push_back({0, true});  // the whole scene is one leaf
        } else {
            const int k = split8[p.bin];
            resolve(b.left, k);
            resolve(b.right, 8 - k);
        }
        for (const auto& kd : kids) {
            ch[nc] = kd.first;
            as_leaf[nc] = kd.second;
            ++nc;
        }
        // octant slot assignment: slot s holds the child nearest along dirs[s]
        int slot_child[8];
        bool slot_leaf[8] = {false, false, false, false, false, false, false, false};
        for (int s = 0; s < 8; ++s) slot_child[s] = -1;
        {
            float pc[3];
            for (int k = 0; k < 3; ++k) pc[k] = 0.5f * (b.box.lo[k] + b.box.hi[k]);
            struct Cand {
                float cost;
                int c, s;
            };
            Cand cand[64];
            int ncand = 0;
            for (int i = 0; i < nc; ++i) {
                const Box& cb = B.nodes[ch[i]].box;
                float cc[3];
                for (int k = 0; k < 3; ++k) cc[k] = 0.5f * (cb.lo[k] + cb.hi[k]) - pc[k];
                for (int s = 0; s < 8; ++s)
                    cand[ncand++] = {cc[0] * dirs[s][0] + cc[1] * dirs[s][1] + cc[2] * dirs[s][2], i, s};
            }
            std::sort(cand, cand + ncand, [](const Cand& a, const Cand& c) {
                if (a.cost != c.cost) return a.cost < c.cost;
                if (a.c != c.c) return a.c < c.c;
                return a.s < c.s;
            });
            bool used[8] = {false};
            for (int k = 0; k < ncand; ++k) {
                if (used[cand[k].c] || slot_child[cand[k].s] >= 0) continue;
                used[cand[k].c] = true;
                slot_child[cand[k].s] = ch[cand[k].c];
                slot_leaf[cand[k].s] = as_leaf[cand[k].c];
            }
        }
        WideNode wn;
        std::memset(&wn, 0, sizeof(wn));
        // internal children first (ranks follow slot order)
        uint32_t child_base = (uint32_t)out.nodes.size();
        int rank = 0;
        for (int s = 0; s < 8; ++s) {
            int c = slot_child[s];
            if (c < 0) continue;
            if (!slot_leaf[s]) {
                wn.imask |= (uint8_t)(1u << s);
                wn.meta[s] = (uint8_t)(kMetaInternal | s);
                queue.push_back({(int32_t)(child_base + rank), c, p.depth + 1});
                ++rank;
            }
        }
        out.nodes.resize(out.nodes.size() + rank);
        uint32_t tri_base = (uint32_t)out.tri_order.size();
        for (int s = 0; s < 8; ++s) {
            int c = slot_child[s];
            if (c < 0) continue;
            const BinNode& cn = B.nodes[c];
            if (slot_leaf[s] && cn.rcount > 0) {
                // a leaf: the triangles of the binary subtree (at most kMaxLeaf)
                uint32_t off = (uint32_t)out.tri_order.size() - tri_base;
                for (int i = 0; i < cn.rcount; ++i) out.tri_order.push_back(B.idx[cn.rbegin + i]);
                wn.meta[s] = (uint8_t)((((1u << cn.rcount) - 1u) << 5) | off);
            }
        }
        wn.child_base = child_base;
        wn.tri_base = tri_base;
        // quantisation
        Box nb;
        nb.reset();
        for (int s = 0; s < 8; ++s)
            if (slot_child[s] >= 0) nb.grow(B.nodes[slot_child[s]].box);
        for (int k = 0; k < 3; ++k) {
            if (!(nb.lo[k] <= nb.hi[k])) {
                wn.origin[k] = 0.0f;
                wn.exp[k] = 0;
                continue;
            }
            float ext = nb.hi[k] - nb.lo[k];
            int e = -126;
            if (ext > 0.0f) e = (int)std::ceil(std::log2((double)ext / 65534.0));
            e = std::max(-126, std::min(127, e));
            while (e < 127 && (double)ext / std::ldexp(1.0, e) > 65534.0) ++e;
            wn.exp[k] = (int8_t)e;
            wn.origin[k] = nb.lo[k];
            float scale = (float)std::ldexp(1.0, e);
            for (int s = 0; s < 8; ++s) {
                if (slot_child[s] < 0) continue;
                const Box& cb = B.nodes[slot_child[s]].box;
                quantize(nb.lo[k], scale, cb.lo[k], cb.hi[k], wn.qlo[k][s], wn.qhi[k][s]);
            }
        }
        out.nodes[p.wide] = wn;
    }
    out.depth = depth;
}

}  // namespace srt
