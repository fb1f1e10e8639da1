// Host-side acceleration-structure builder.  Replaces the driver-built
// BLAS/TLAS of the reference (WaveFrontPathTracer.cpp:202-457): a binned-SAH
// binary BVH (the plain form's traversal format) and a collapse of it (SAH
// dynamic programme, or greedy) into the 8-wide compressed format with 8-bit
// child boxes rounded outward (the chosen form).
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstring>
#include <future>
#include <limits>
#include <stdexcept>

#include "scene.h"

namespace wfpt {

namespace {

struct Box {
    float lo[3] = {std::numeric_limits<float>::infinity(), std::numeric_limits<float>::infinity(),
                   std::numeric_limits<float>::infinity()};
    float hi[3] = {-std::numeric_limits<float>::infinity(), -std::numeric_limits<float>::infinity(),
                   -std::numeric_limits<float>::infinity()};
    void grow(const float* p) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], p[k]);
            hi[k] = std::max(hi[k], p[k]);
        }
    }
    void grow(const Box& b) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], b.lo[k]);
            hi[k] = std::max(hi[k], b.hi[k]);
        }
    }
    // Empty boxes are stored as lo = hi = +inf, which every slab test rejects.
    bool empty() const {
        return !(lo[0] <= hi[0]) || !(lo[1] <= hi[1]) || !(lo[2] <= hi[2]) || std::isinf(lo[0]);
    }
    float area() const {
        if (empty()) return 0.0f;
        float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        return 2.0f * (dx * dy + dy * dz + dz * dx);
    }
};

struct Prim {
    Box box;
    float c[3];
};

struct BNode {
    Box box;
    int32_t left = -1, right = -1;
    uint32_t first = 0, count = 0;  // leaf when count > 0
};

constexpr int kBins = 32;
constexpr int kMedianDepth = 32;  // below this depth split at the object median

struct Builder {
    const std::vector<Prim>& prims;
    std::vector<uint32_t>& idx;
    std::vector<BNode> nodes;
    std::atomic<uint32_t> next{0};
    int max_leaf;
    std::atomic<int> max_depth{0};

    Builder(const std::vector<Prim>& p, std::vector<uint32_t>& i, int ml) : prims(p), idx(i), max_leaf(ml) {
        nodes.resize(std::max<size_t>(1, 2 * p.size()));
    }

    uint32_t alloc() {
        uint32_t id = next.fetch_add(1);
        if (id >= nodes.size()) throw std::runtime_error("bvh arena exhausted");
        return id;
    }

    uint32_t make_leaf(uint32_t begin, uint32_t end, const Box& b) {
        uint32_t id = alloc();
        nodes[id].box = b;
        nodes[id].first = begin;
        nodes[id].count = end - begin;
        return id;
    }

    uint32_t build(uint32_t begin, uint32_t end, int depth) {
        int md = max_depth.load();
        while (depth > md && !max_depth.compare_exchange_weak(md, depth)) {
        }
        Box b, cb;
        for (uint32_t i = begin; i < end; ++i) {
            b.grow(prims[idx[i]].box);
            cb.grow(prims[idx[i]].c);
        }
        uint32_t n = end - begin;
        if (n <= 1) return make_leaf(begin, end, b);
        int axis = 0;
        float ext[3];
        for (int k = 0; k < 3; ++k) ext[k] = cb.hi[k] - cb.lo[k];
        if (ext[1] > ext[axis]) axis = 1;
        if (ext[2] > ext[axis]) axis = 2;
        uint32_t mid = begin;
        bool split_found = false;
        if (ext[axis] > 0.0f && depth < kMedianDepth) {
            // Binned SAH over all three axes.
            float best_cost = std::numeric_limits<float>::infinity();
            int best_axis = -1, best_bin = -1;
            for (int k = 0; k < 3; ++k) {
                if (!(ext[k] > 0.0f)) continue;
                Box bb[kBins];
                uint32_t bc[kBins] = {0};
                float scale = kBins / ext[k];
                for (uint32_t i = begin; i < end; ++i) {
                    const Prim& p = prims[idx[i]];
                    int bi = std::min(kBins - 1, std::max(0, (int)((p.c[k] - cb.lo[k]) * scale)));
                    bb[bi].grow(p.box);
                    bc[bi]++;
                }
                float right_area[kBins];
                uint32_t right_cnt[kBins];
                Box acc;
                uint32_t cnt = 0;
                for (int i = kBins - 1; i > 0; --i) {
                    acc.grow(bb[i]);
                    cnt += bc[i];
                    right_area[i] = acc.area();
                    right_cnt[i] = cnt;
                }
                Box lacc;
                uint32_t lcnt = 0;
                for (int i = 0; i < kBins - 1; ++i) {
                    lacc.grow(bb[i]);
                    lcnt += bc[i];
                    if (lcnt == 0 || right_cnt[i + 1] == 0) continue;
                    float cost = lacc.area() * lcnt + right_area[i + 1] * right_cnt[i + 1];
                    if (cost < best_cost) {
                        best_cost = cost;
                        best_axis = k;
                        best_bin = i;
                    }
                }
            }
            float parent_area = b.area();
            float leaf_cost = (float)n;
            float split_cost = parent_area > 0.0f ? 1.0f + best_cost / parent_area : 1.0f + (float)n;
            if (best_axis < 0) {
                // fall through to median split
            } else if ((int)n <= max_leaf && leaf_cost <= split_cost) {
                return make_leaf(begin, end, b);
            } else {
                float scale = kBins / ext[best_axis];
                float lo = cb.lo[best_axis];
                auto it = std::partition(idx.begin() + begin, idx.begin() + end, [&](uint32_t t) {
                    int bi = std::min(kBins - 1, std::max(0, (int)((prims[t].c[best_axis] - lo) * scale)));
                    return bi <= best_bin;
                });
                mid = (uint32_t)(it - idx.begin());
                split_found = mid > begin && mid < end;
            }
        }
        if (!split_found) {
            if ((int)n <= max_leaf) return make_leaf(begin, end, b);
            mid = begin + n / 2;
            std::nth_element(idx.begin() + begin, idx.begin() + mid, idx.begin() + end,
                             [&](uint32_t a, uint32_t c) { return prims[a].c[axis] < prims[c].c[axis]; });
        }
        uint32_t id = alloc();
        nodes[id].box = b;
        uint32_t l, r;
        if (n > 65536 && depth < 8) {
            auto fut = std::async(std::launch::async, [&] { return build(begin, mid, depth + 1); });
            r = build(mid, end, depth + 1);
            l = fut.get();
        } else {
            l = build(begin, mid, depth + 1);
            r = build(mid, end, depth + 1);
        }
        nodes[id].left = (int32_t)l;
        nodes[id].right = (int32_t)r;
        return id;
    }
};

TriRec make_tri(const BuildInput& in, uint32_t g) {
    TriRec t;
    const float* P = in.positions;
    uint32_t a = in.indices[3 * g + 0], b = in.indices[3 * g + 1], c = in.indices[3 * g + 2];
    for (int k = 0; k < 3; ++k) {
        t.v0[k] = P[3 * a + k];
        t.v1[k] = P[3 * b + k];
        t.v2[k] = P[3 * c + k];
    }
    uint32_t geom = 0;
    if (in.geom_first && in.num_geoms > 1) {
        const uint32_t* it = std::upper_bound(in.geom_first, in.geom_first + in.num_geoms, g);
        geom = (uint32_t)(it - in.geom_first) - 1;
    }
    uint32_t first = in.geom_first ? in.geom_first[geom] : 0;
    t.prim = (int32_t)(g - first);
    t.geom = (int32_t)geom;
    t.global = g;
    return t;
}

void set_child(Bvh2Node& n, int c, const Box& b, int32_t link) {
    if (c == 0) {
        n.f[0] = b.lo[0]; n.f[1] = b.hi[0]; n.f[2] = b.lo[1]; n.f[3] = b.hi[1];
        n.f[8] = b.lo[2]; n.f[9] = b.hi[2];
    } else {
        n.f[4] = b.lo[0]; n.f[5] = b.hi[0]; n.f[6] = b.lo[1]; n.f[7] = b.hi[1];
        n.f[10] = b.lo[2]; n.f[11] = b.hi[2];
    }
    n.link[c] = link;
}

Box child_box(const Bvh2Node& n, int c) {
    Box b;
    if (c == 0) {
        b.lo[0] = n.f[0]; b.hi[0] = n.f[1]; b.lo[1] = n.f[2]; b.hi[1] = n.f[3]; b.lo[2] = n.f[8]; b.hi[2] = n.f[9];
    } else {
        b.lo[0] = n.f[4]; b.hi[0] = n.f[5]; b.lo[1] = n.f[6]; b.hi[1] = n.f[7]; b.lo[2] = n.f[10]; b.hi[2] = n.f[11];
    }
    return b;
}

}  // namespace

void build_bvh2(const BuildInput& in, int max_leaf, HostBvh2& out) {
    max_leaf = std::max(1, std::min(8, max_leaf));
    uint32_t N = in.num_triangles;
    out.nodes.clear();
    out.tris.clear();
    std::vector<Prim> prims(N);
    for (uint32_t g = 0; g < N; ++g) {
        Prim& p = prims[g];
        for (int v = 0; v < 3; ++v) p.box.grow(in.positions + 3 * (size_t)in.indices[3 * g + v]);
        for (int k = 0; k < 3; ++k) p.c[k] = 0.5f * (p.box.lo[k] + p.box.hi[k]);
    }
    Bvh2Node empty_node;
    std::memset(&empty_node, 0, sizeof(empty_node));
    Box none;
    for (int k = 0; k < 3; ++k) none.lo[k] = none.hi[k] = std::numeric_limits<float>::infinity();
    if (N == 0) {
        Bvh2Node root = empty_node;
        set_child(root, 0, none, ~0);
        set_child(root, 1, none, ~0);
        out.nodes.push_back(root);
        TriRec dummy;
        std::memset(&dummy, 0, sizeof(dummy));
        out.tris.push_back(dummy);
        out.depth = 1;
        return;
    }
    // Stored boxes are the triangle bounds grown by delta = 2^-22 * P on
    // every side, P = the largest absolute vertex coordinate.  With
    // u = 2^-24, the traversal's slab distances fma(p, inv, -o*inv) are off
    // by at most about u * (|o| + P) * |inv|, which delta * |inv| = 4 u * P *
    // |inv| covers while |o| <= 3 P; from |o| >= 2 P on that error is within
    // 2 u of t itself and inside the relative slack on exit distances.  The
    // rounding of a triangle's own t near the ray origin (a few u times the
    // triangle's size) is covered as well for triangles up to about P / 2
    // across.  So culling does not drop a triangle that ties the current
    // closest hit, including hits at t = 0 of rays that start on a surface:
    // checked against a brute-force oracle on such rays.  (Each doubling of
    // delta costs about 1% of frame throughput: shadow rays start 1e-5
    // before their surface and enter its grown box.)
    float P = 0.0f;
    for (const Prim& p : prims)
        for (int k = 0; k < 3; ++k) P = std::max(P, std::max(std::fabs(p.box.lo[k]), std::fabs(p.box.hi[k])));
    const float delta = P * 0x1p-22f;
    auto grown = [delta](Box b) {
        for (int k = 0; k < 3; ++k) {
            b.lo[k] -= delta;
            b.hi[k] += delta;
        }
        return b;
    };
    std::vector<uint32_t> idx(N);
    for (uint32_t i = 0; i < N; ++i) idx[i] = i;
    Builder B(prims, idx, max_leaf);
    uint32_t root = B.build(0, N, 0);
    out.depth = B.max_depth.load() + 1;
    // Flatten depth-first; node 0 is the root (wrapped when the root is a leaf).
    out.nodes.reserve(B.next.load());
    out.tris.reserve(N);
    auto emit_leaf = [&](const BNode& bn) -> int32_t {
        uint32_t first = (uint32_t)out.tris.size();
        for (uint32_t i = 0; i < bn.count; ++i) out.tris.push_back(make_tri(in, idx[bn.first + i]));
        return (int32_t)~((first << 3) | (bn.count - 1));
    };
    struct Item {
        uint32_t bnode;
        uint32_t slot;  // out node index to fill
    };
    std::vector<Item> stack;
    if (B.nodes[root].count > 0) {
        Bvh2Node r = empty_node;
        set_child(r, 0, grown(B.nodes[root].box), emit_leaf(B.nodes[root]));
        set_child(r, 1, none, r.link[0]);
        out.nodes.push_back(r);
        return;
    }
    out.nodes.push_back(empty_node);
    stack.push_back({root, 0});
    while (!stack.empty()) {
        Item it = stack.back();
        stack.pop_back();
        const BNode& bn = B.nodes[it.bnode];
        int32_t ch[2] = {bn.left, bn.right};
        for (int c = 0; c < 2; ++c) {
            const BNode& cn = B.nodes[ch[c]];
            int32_t link;
            if (cn.count > 0) {
                link = emit_leaf(cn);
            } else {
                link = (int32_t)out.nodes.size();
                out.nodes.push_back(empty_node);
                stack.push_back({(uint32_t)ch[c], (uint32_t)link});
            }
            set_child(out.nodes[it.slot], c, grown(cn.box), link);
        }
    }
}

// ------------------------------------------------------------------ BVH8
// Collapse policy, read when a scene is built: 1 = SAH-optimal collapse
// (default), 0 = greedy fill by surface area.  The triangle cost is the
// cost of one triangle test relative to one node step, in percent.  The
// cooperative traversal tests a warp's triangles 32 at a time, so a
// triangle costs far less than a node step: on the courtyard's bounce-1
// rays 20 % gave 1-3 % faster traversal than the greedy collapse (22.3
// instead of 23.2 node steps per closest-hit ray, 9.0 instead of 7.3
// triangle tests), while 100 % cut triangle tests to 4.7 but added node
// steps and was slower.
static std::atomic<int> g_collapse{1};
static std::atomic<int> g_tri_cost_pct{20};
void set_bvh8_collapse(int mode) { g_collapse = mode != 0 ? 1 : 0; }
int get_bvh8_collapse() { return g_collapse; }
void set_bvh8_tri_cost_pct(int pct) { g_tri_cost_pct = std::max(1, std::min(10000, pct)); }
int get_bvh8_tri_cost_pct() { return g_tri_cost_pct; }

namespace {

struct Collapser {
    const HostBvh2& b2;
    HostBvh8& out;
    std::vector<uint32_t> subtree_tris;  // per BVH2 node
    bool sah = true;
    float tri_cost = 1.0f;
    // SAH collapse tables per BVH2 node n, for i = 1..8 slots:
    //   cost[n][i-1]  the least SAH cost of representing n's subtree with at
    //                 most i BVH8 children;
    //   how[n][0]     -1: as one leaf child, 0: as one inner child;
    //   how[n][i-1]   (i > 1) 0: same as with i-1 slots, a > 0: a slots to
    //                 the first BVH2 child, i-a to the second.
    //   split8[n]     slots of the first child when n is a BVH8 inner node.
    std::vector<std::array<float, 8>> cost;
    std::vector<std::array<int8_t, 8>> how;
    std::vector<int8_t> split8;

    Collapser(const HostBvh2& b, HostBvh8& o) : b2(b), out(o) {}

    uint32_t count_link(int32_t link) const {
        if (link < 0) return ((~(uint32_t)link) & 7u) + 1u;
        return subtree_tris[link];
    }

    void count_all() {
        subtree_tris.assign(b2.nodes.size(), 0);
        // Children have larger indices than parents (depth-first flatten).
        for (size_t i = b2.nodes.size(); i-- > 0;) {
            const Bvh2Node& n = b2.nodes[i];
            uint32_t c = 0;
            for (int k = 0; k < 2; ++k) {
                if (child_box(n, k).empty()) continue;
                c += count_link(n.link[k]);
            }
            subtree_tris[i] = c;
        }
    }

    void gather_tris(int32_t link, std::vector<uint32_t>& tris) {
        if (link < 0) {
            uint32_t code = ~(uint32_t)link;
            uint32_t first = code >> 3, cnt = (code & 7u) + 1u;
            for (uint32_t k = 0; k < cnt; ++k) tris.push_back(first + k);
            return;
        }
        const Bvh2Node& n = b2.nodes[link];
        for (int k = 0; k < 2; ++k)
            if (!child_box(n, k).empty()) gather_tris(n.link[k], tris);
    }

    struct Child {
        Box box;
        int32_t link;  // BVH2 link
        bool leaf;     // becomes a triangle child
    };

    // Cost of BVH2 child k of node p with at most i slots (i = 1..8).
    float link_cost(const Bvh2Node& p, int k, int i) const {
        const int32_t link = p.link[k];
        if (link < 0) return child_box(p, k).area() * (float)count_link(link) * tri_cost;
        return cost[link][i - 1];
    }

    // The SAH collapse of Ylitie, Karras and Laine ("Efficient Incoherent
    // Ray Traversal on GPUs Through Compressed Wide BVHs", 2017, sec. 3.1):
    // bottom-up over the BVH2, each subtree's least cost as a leaf child
    // (at most three triangles: area x triangles x tri_cost), as an inner
    // child (area x 1 + its two children sharing 8 slots), or spread over
    // several slots of the parent.  Areas are unnormalised (a common factor).
    void plan_sah() {
        const size_t N = b2.nodes.size();
        const float inf = std::numeric_limits<float>::infinity();
        cost.assign(N, {});
        how.assign(N, {});
        split8.assign(N, 0);
        for (size_t idx = N; idx-- > 0;) {  // children after parents
            const Bvh2Node& n = b2.nodes[idx];
            const bool e0 = child_box(n, 0).empty(), e1 = child_box(n, 1).empty();
            if (e0 || e1) {
                // One child (a wrapped leaf root) or none: this node passes
                // its single child through.
                const int k = e0 ? 1 : 0;
                for (int i = 1; i <= 8; ++i) {
                    cost[idx][i - 1] = (e0 && e1) ? 0.0f : link_cost(n, k, i);
                    how[idx][i - 1] = 0;
                }
                continue;
            }
            Box ub = child_box(n, 0);
            ub.grow(child_box(n, 1));
            const float A = ub.area();
            float dist[9];
            int8_t arg[9];
            for (int j = 2; j <= 8; ++j) {
                dist[j] = inf;
                arg[j] = 1;
                for (int a = 1; a < j; ++a) {
                    float c = link_cost(n, 0, a) + link_cost(n, 1, j - a);
                    if (c < dist[j]) {
                        dist[j] = c;
                        arg[j] = (int8_t)a;
                    }
                }
            }
            split8[idx] = arg[8];
            const float c_inner = A + dist[8];
            const uint32_t t = subtree_tris[idx];
            const float c_leaf = t <= 3 ? A * (float)t * tri_cost : inf;
            cost[idx][0] = std::min(c_leaf, c_inner);
            how[idx][0] = c_leaf <= c_inner ? -1 : 0;
            for (int i = 2; i <= 8; ++i) {
                if (dist[i] < cost[idx][i - 2]) {
                    cost[idx][i - 1] = dist[i];
                    how[idx][i - 1] = arg[i];
                } else {
                    cost[idx][i - 1] = cost[idx][i - 2];
                    how[idx][i - 1] = 0;
                }
            }
        }
    }

    // BVH8 children of BVH2 child k of node p given at most i slots.
    void collect(const Bvh2Node& p, int k, int i, std::vector<Child>& ch) {
        const Box b = child_box(p, k);
        if (b.empty()) return;
        const int32_t link = p.link[k];
        if (link < 0) {
            ch.push_back({b, link, true});
            return;
        }
        const Bvh2Node& m = b2.nodes[link];
        const bool e0 = child_box(m, 0).empty(), e1 = child_box(m, 1).empty();
        if (e0 || e1) {
            if (!(e0 && e1)) collect(m, e0 ? 1 : 0, i, ch);
            return;
        }
        while (i > 1 && how[link][i - 1] == 0) --i;
        if (i == 1) {
            ch.push_back({b, link, how[link][0] == -1});
            return;
        }
        const int a = how[link][i - 1];
        collect(m, 0, a, ch);
        collect(m, 1, i - a, ch);
    }

    // Fills out.nodes[slot] from BVH2 node `n2` whose box is `box`.
    void emit(uint32_t slot, uint32_t n2) {
        std::vector<Child> ch;
        const Bvh2Node& n = b2.nodes[n2];
        if (sah) {
            const bool e0 = child_box(n, 0).empty(), e1 = child_box(n, 1).empty();
            if (e0 || e1) {
                if (!(e0 && e1)) collect(n, e0 ? 1 : 0, 8, ch);
            } else {
                collect(n, 0, split8[n2], ch);
                collect(n, 1, 8 - split8[n2], ch);
            }
            emit_children(slot, ch);
            return;
        }
        for (int k = 0; k < 2; ++k) {
            Box b = child_box(n, k);
            if (b.empty()) continue;
            ch.push_back({b, n.link[k], false});
        }
        // Greedy fill: split the child of largest surface area while slots
        // remain, small subtrees included (a split gives tighter boxes).  Only
        // when the node is full (or nothing can be split) do subtrees of at
        // most three triangles become leaf children; larger ones become inner
        // children.  BVH2 leaves (link < 0) cannot be split.
        while (ch.size() < 8) {
            int best = -1;
            float best_area = -1.0f;
            for (int i = 0; i < (int)ch.size(); ++i) {
                if (ch[i].link < 0) continue;
                float a = ch[i].box.area();
                if (a > best_area) {
                    best_area = a;
                    best = i;
                }
            }
            if (best < 0) break;
            const Bvh2Node& m = b2.nodes[ch[best].link];
            std::vector<Child> repl;
            for (int k = 0; k < 2; ++k) {
                Box b = child_box(m, k);
                if (b.empty()) continue;
                repl.push_back(Child{b, m.link[k], false});
            }
            ch.erase(ch.begin() + best);  // at most 6 left, so the two children fit
            ch.insert(ch.end(), repl.begin(), repl.end());
        }
        for (auto& c : ch) c.leaf = c.link < 0 || count_link(c.link) <= 3;
        emit_children(slot, ch);
    }

    // Quantises the children into out.nodes[slot] and emits inner children.
    void emit_children(uint32_t slot, std::vector<Child>& ch) {
        Bvh8Node node;
        std::memset(&node, 0, sizeof(node));
        if (ch.empty()) {  // empty scene: a root without children
            out.nodes[slot] = node;
            return;
        }
        // Node box and quantisation grid.
        Box nb;
        for (auto& c : ch) nb.grow(c.box);
        float scale[3];
        for (int k = 0; k < 3; ++k) {
            node.p[k] = nb.lo[k];
            float ext = nb.hi[k] - nb.lo[k];
            int ex = -126;
            if (ext > 0.0f) {
                int e2;
                std::frexp(ext / 255.0f, &e2);
                ex = e2;
            }
            for (;;) {
                ex = std::max(-126, std::min(127, ex));
                scale[k] = std::ldexp(1.0f, ex);
                float top = node.p[k] + 255.0f * scale[k];
                if (top >= nb.hi[k] || ex == 127) break;
                ++ex;
            }
            node.e[k] = (uint8_t)(ex + 127);
        }
        // Slot assignment: child with centroid offset sign pattern s goes to
        // slot s (bit k set = negative side along axis k), greedily by score.
        float pc[3];
        for (int k = 0; k < 3; ++k) pc[k] = 0.5f * (nb.lo[k] + nb.hi[k]);
        struct Cand {
            float score;
            int child, slot;
        };
        std::vector<Cand> cands;
        for (int i = 0; i < (int)ch.size(); ++i) {
            float off[3];
            for (int k = 0; k < 3; ++k) off[k] = 0.5f * (ch[i].box.lo[k] + ch[i].box.hi[k]) - pc[k];
            for (int s = 0; s < 8; ++s) {
                float sc = 0.0f;
                for (int k = 0; k < 3; ++k) sc += ((s >> k) & 1) ? -off[k] : off[k];
                cands.push_back({sc, i, s});
            }
        }
        std::stable_sort(cands.begin(), cands.end(), [](const Cand& a, const Cand& b) { return a.score > b.score; });
        int slot_of[8];
        int child_at[8];
        for (int i = 0; i < 8; ++i) slot_of[i] = child_at[i] = -1;
        for (const Cand& c : cands) {
            if (slot_of[c.child] >= 0 || child_at[c.slot] >= 0) continue;
            slot_of[c.child] = c.slot;
            child_at[c.slot] = c.child;
        }
        // Quantised boxes, meta, children and triangles in slot order.
        uint32_t num_inner = 0;
        for (auto& c : ch)
            if (!c.leaf) ++num_inner;
        node.child_base = (uint32_t)out.nodes.size();
        node.tri_base = (uint32_t)out.tris.size();
        out.nodes.resize(out.nodes.size() + num_inner);
        std::vector<std::pair<uint32_t, uint32_t>> pending;  // (bvh8 slot, bvh2 node)
        uint32_t inner_i = 0, tri_off = 0;
        for (int s = 0; s < 8; ++s) {
            int ci = child_at[s];
            if (ci < 0) continue;
            const Child& c = ch[ci];
            for (int k = 0; k < 3; ++k) {
                float sc = scale[k];
                float lo = std::floor((c.box.lo[k] - node.p[k]) / sc);
                float hi = std::ceil((c.box.hi[k] - node.p[k]) / sc);
                int ql = (int)std::max(0.0f, std::min(255.0f, lo));
                int qh = (int)std::max(0.0f, std::min(255.0f, hi));
                while (ql > 0 && node.p[k] + (float)ql * sc > c.box.lo[k]) --ql;
                while (qh < 255 && node.p[k] + (float)qh * sc < c.box.hi[k]) ++qh;
                uint8_t* qlo = k == 0 ? node.qlo_x : (k == 1 ? node.qlo_y : node.qlo_z);
                uint8_t* qhi = k == 0 ? node.qhi_x : (k == 1 ? node.qhi_y : node.qhi_z);
                qlo[s] = (uint8_t)ql;
                qhi[s] = (uint8_t)qh;
            }
            if (c.leaf) {
                std::vector<uint32_t> t;
                gather_tris(c.link, t);
                uint32_t cnt = (uint32_t)t.size();
                uint32_t unary = cnt == 1 ? 1u : (cnt == 2 ? 3u : 7u);
                node.meta[s] = (uint8_t)((unary << 5) | tri_off);
                for (uint32_t x : t) out.tris.push_back(b2.tris[x]);
                tri_off += cnt;
            } else {
                node.imask |= (uint8_t)(1u << s);
                node.meta[s] = (uint8_t)((1u << 5) | (24u + (uint32_t)s));
                pending.push_back({node.child_base + inner_i, (uint32_t)c.link});
                ++inner_i;
            }
        }
        out.nodes[slot] = node;
        for (auto& pr : pending) emit(pr.first, pr.second);
    }
};

}  // namespace

void build_bvh8(const HostBvh2& bvh2, HostBvh8& out) {
    out.nodes.clear();
    out.tris.clear();
    Collapser C(bvh2, out);
    C.count_all();
    C.sah = g_collapse != 0;
    C.tri_cost = (float)g_tri_cost_pct * 0.01f;
    if (C.sah) C.plan_sah();
    out.nodes.resize(1);
    C.emit(0, 0);
    if (out.tris.empty()) {
        TriRec dummy;
        std::memset(&dummy, 0, sizeof(dummy));
        out.tris.push_back(dummy);
    }
}

}  // namespace wfpt
