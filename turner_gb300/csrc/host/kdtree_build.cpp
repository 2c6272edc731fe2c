// Host SAH kd-tree builder whose output is the reference's flattened kd-tree,
// word for word (tests/test_builder.py checks it against the reference's own
// builder via tests/golden/).
//
// Algorithm: [WH06] Wald & Havran, "On building fast kd-Trees for Ray Tracing,
// and on doing that in O(N log N)", Algorithm 4 (per-node event sort), with
// the reference's choices, which determine the node words and therefore have
// to be the same here:
//   - leaf if <= 3 triangles or zero box area; automatic termination when
//     20 * n * lambda < best cost                      lib/kdtree.cpp:128-174
//   - cost = lambda * (15 + 20 * (SA_l/SA * n_l + SA_r/SA * n_r)),
//     lambda = 0.8 if a side is empty; planar triangles go to the cheaper
//     side                                              lib/kdtree.cpp:178-243
//   - events from triangles clipped to the node box by Sutherland-Hodgman
//     against thick planes (EPS = 1e-5), sorted by (position, END < PLANAR <
//     START) with std::sort, swept per axis; the first strict minimum wins;
//     classification walks the winning axis' sorted events
//                                                       lib/kdtree.cpp:245-408,
//                                                       lib/clipping.h:125-235
//   - DFS flattening, left child adjacent, leaves packed two ids per 64-bit
//     word and closed by a sentinel                    lib/kdtree.cpp:420-467
//   - triangle precomputation (u, v, normal via a double cross product, uv,
//     vv, uu, denom)                                    lib/triangle.h:22-39
// Differences from the reference, none of which change the output: clipping
// reuses per-thread buffers instead of allocating per triangle, subtrees above
// a size threshold are built on separate threads, and the tree is built
// directly into an index-linked node pool.
#include "turner_gpu.h"
#include "tree.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <future>
#include <limits>
#include <memory>
#include <new>
#include <thread>
#include <vector>


namespace {

constexpr float kEps = 0.00001f;
constexpr float kFltMax = std::numeric_limits<float>::max();
constexpr float kFltLowest = std::numeric_limits<float>::lowest();
constexpr int kCostTraversal = 15;
constexpr int kCostIntersection = 20;

struct P3 {
    float c[3];
    float& operator[](int i) { return c[i]; }
    float operator[](int i) const { return c[i]; }
};

struct Box {
    P3 lo, hi;
};

// Bbox3(p1, p2) stores the component-wise std::min / std::max of its corners.
inline Box make_box(const P3& a, const P3& b) {
    Box r;
    for (int i = 0; i < 3; ++i) {
        r.lo[i] = std::min(a[i], b[i]);
        r.hi[i] = std::max(a[i], b[i]);
    }
    return r;
}

inline float surface_area(const Box& b) {
    const float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    return 2 * (dx * dy + dx * dz + dy * dz);
}

inline void split_box(const Box& b, int ax, float pos, Box& l, Box& r) {
    P3 lmax = b.hi;
    lmax[ax] = pos;
    P3 rmin = b.lo;
    rmin[ax] = pos;
    l = make_box(b.lo, lmax);
    r = make_box(rmin, b.hi);
}

// dot(Normal3f, Vector3f), left to right
inline float dot3(const float n[3], const P3& p) { return n[0] * p[0] + n[1] * p[1] + n[2] * p[2]; }

enum Side { ON_PLANE, BEHIND, IN_FRONT };

inline Side classify(const P3& p, const float n[3], float d) {
    const float dist = dot3(n, p) - d;
    if (dist > kEps) return IN_FRONT;
    if (dist < -kEps) return BEHIND;
    return ON_PLANE;
}

// point where segment a-b meets the plane n.x = d: a + t (b - a)
inline P3 cut(const P3& a, const P3& b, const float n[3], float d) {
    const P3 ab{{b[0] - a[0], b[1] - a[1], b[2] - a[2]}};
    const float t = (d - dot3(n, a)) / dot3(n, ab);
    const P3 ba{{b[0] - a[0], b[1] - a[1], b[2] - a[2]}};
    return P3{{a[0] + t * ba[0], a[1] + t * ba[1], a[2] + t * ba[2]}};
}

// Sutherland-Hodgman against one thick plane; returns the kept polygon.
void clip_plane(const std::vector<P3>& poly, const float n[3], float d, std::vector<P3>& out) {
    out.clear();
    P3 a = poly.back();
    Side as = classify(a, n, d);
    for (const P3& b : poly) {
        const Side bs = classify(b, n, d);
        if (bs == IN_FRONT) {
            if (as == BEHIND) out.push_back(cut(a, b, n, d));
            out.push_back(b);
        } else if (bs == BEHIND) {
            if (as == IN_FRONT) out.push_back(cut(a, b, n, d));
        } else {
            out.push_back(b);
        }
        a = b;
        as = bs;
    }
}

struct ClipScratch {
    std::vector<P3> a, b;
};

// Bounding box of the triangle clipped to `box`. A triangle clipped to fewer
// than two points yields Bbox3f's default value (lowest .. max), as in the
// reference, which is not "empty" and keeps the triangle in both children.
Box clip_triangle(const turner_triangle& tri, const Box& box, ClipScratch& s) {
    s.a.assign({P3{{tri.vertices[0][0], tri.vertices[0][1], tri.vertices[0][2]}},
                P3{{tri.vertices[1][0], tri.vertices[1][1], tri.vertices[1][2]}},
                P3{{tri.vertices[2][0], tri.vertices[2][1], tri.vertices[2][2]}}});
    for (int ax = 0; ax < 3; ++ax) {
        for (int side = 0; side < 2; ++side) {
            float n[3] = {0, 0, 0};
            n[ax] = side == 0 ? 1.f : -1.f;
            const float dist = side == 0 ? box.lo[ax] : -box.hi[ax];
            clip_plane(s.a, n, dist, s.b);
            std::swap(s.a, s.b);
            if (s.a.size() < 2) {
                return Box{P3{{kFltLowest, kFltLowest, kFltLowest}}, P3{{kFltMax, kFltMax, kFltMax}}};
            }
        }
    }
    P3 lo{{kFltMax, kFltMax, kFltMax}}, hi{{kFltLowest, kFltLowest, kFltLowest}};
    for (int ax = 0; ax < 3; ++ax) {
        for (const P3& p : s.a) {
            if (p[ax] < lo[ax]) lo[ax] = p[ax];
            if (hi[ax] < p[ax]) hi[ax] = p[ax];
        }
    }
    return make_box(lo, hi);
}

constexpr int kEnding = 0, kPlanar = 1, kStarting = 2;

struct Event {
    float point;
    float aux;
    uint32_t id;
    int type;
};

struct Node {
    bool leaf;
    int axis;
    float pos;
    Node* left;
    Node* right;
    std::vector<uint32_t> ids;
};

inline float lambda(size_t nl, size_t nr) { return (nl == 0 || nr == 0) ? 0.8f : 1.f; }

inline float split_cost(float lr, float rr, size_t nl, size_t nr) {
    return lambda(nl, nr) *
           (kCostTraversal + kCostIntersection * (lr * static_cast<float>(nl) + rr * static_cast<float>(nr)));
}

class Builder {
public:
    Builder(const std::vector<turner_triangle>& tris, int threads) : tris_(tris), threads_(threads) {}

    Node* build(std::vector<uint32_t> ids, const Box& box, int par_depth) {
        if (ids.empty()) return nullptr;
        if (ids.size() <= 3 || surface_area(box) == 0) return leaf(std::move(ids));

        float min_cost;
        int ax;
        float pos;
        std::vector<uint32_t> lt, rt;
        find_plane(ids, box, min_cost, ax, pos, lt, rt);

        // the bias is dropped again here so that an empty-space split cannot
        // repeat forever (lib/kdtree.cpp:151-159)
        if (static_cast<float>(kCostIntersection * ids.size()) * lambda(lt.size(), rt.size()) < min_cost) {
            return leaf(std::move(ids));
        }
        ids.clear();
        ids.shrink_to_fit();

        Box lbox, rbox;
        split_box(box, ax, pos, lbox, rbox);

        Node* left;
        Node* right;
        if (par_depth > 0 && lt.size() + rt.size() > 4096) {
            auto fut = std::async(std::launch::async, [this, &lt, &lbox, par_depth]() {
                return build(std::move(lt), lbox, par_depth - 1);
            });
            right = build(std::move(rt), rbox, par_depth - 1);
            left = fut.get();
        } else {
            left = build(std::move(lt), lbox, 0);
            right = build(std::move(rt), rbox, 0);
        }
        if (!left) return right;
        if (!right) return left;
        return new Node{false, ax, pos, left, right, {}};
    }

private:
    static Node* leaf(std::vector<uint32_t> ids) { return new Node{true, 0, 0.f, nullptr, nullptr, std::move(ids)}; }

    void find_plane(const std::vector<uint32_t>& ids, const Box& box, float& min_cost, int& min_ax, float& min_pos,
                    std::vector<uint32_t>& lt, std::vector<uint32_t>& rt) const {
        thread_local ClipScratch scratch;
        std::vector<Event> ev[3];
        for (auto& e : ev) e.reserve(2 * ids.size());
        size_t num = 0;
        for (uint32_t id : ids) {
            const Box cb = clip_triangle(tris_[id], box, scratch);
            if (cb.hi[0] <= cb.lo[0] && cb.hi[1] <= cb.lo[1] && cb.hi[2] <= cb.lo[2]) continue;   // empty()
            ++num;
            for (int ax = 0; ax < 3; ++ax) {
                if (std::abs(cb.hi[ax] - cb.lo[ax]) < kEps) {   // planar(ax)
                    ev[ax].push_back(Event{cb.lo[ax], cb.lo[ax], id, kPlanar});
                } else {
                    ev[ax].push_back(Event{cb.lo[ax], cb.hi[ax], id, kStarting});
                    ev[ax].push_back(Event{cb.hi[ax], cb.lo[ax], id, kEnding});
                }
            }
        }
        if (num == 0) {
            min_cost = kFltMax;
            min_ax = 0;
            min_pos = 0;
            return;
        }

        min_cost = kFltMax;
        min_ax = 0;
        min_pos = 0;
        bool min_left = true;
        const float area = surface_area(box);
        for (int ax = 0; ax < 3; ++ax) {
            auto& events = ev[ax];
            std::sort(events.begin(), events.end(), [](const Event& a, const Event& b) {
                return a.point < b.point || (a.point == b.point && a.type < b.type);
            });
            size_t nl = 0, nr = num;
            for (size_t i = 0; i < events.size();) {
                const float p = events[i].point;
                size_t ending = 0, planar = 0, starting = 0;
                while (i < events.size() && events[i].point == p && events[i].type == kEnding) { ++ending; ++i; }
                while (i < events.size() && events[i].point == p && events[i].type == kPlanar) { ++planar; ++i; }
                while (i < events.size() && events[i].point == p && events[i].type == kStarting) { ++starting; ++i; }
                const size_t np = planar;
                nr -= planar + ending;

                Box lbox, rbox;
                split_box(box, ax, p, lbox, rbox);
                const float lr = surface_area(lbox) / area;
                const float rr = surface_area(rbox) / area;
                const float lcost = split_cost(lr, rr, nl + np, nr);
                const float rcost = split_cost(lr, rr, nl, np + nr);
                const bool left = lcost < rcost;
                const float cost = left ? lcost : rcost;
                if (cost < min_cost) {
                    min_cost = cost;
                    min_ax = ax;
                    min_pos = p;
                    min_left = left;
                }
                nl += starting + planar;
            }
        }

        const auto& events = ev[min_ax];
        lt.reserve(events.size() / 2);
        rt.reserve(events.size() / 2);
        for (const Event& e : events) {
            if (e.point < min_pos) {
                if (e.type == kEnding || e.type == kPlanar) {
                    lt.push_back(e.id);
                } else if (min_pos < e.aux) {
                    lt.push_back(e.id);
                    rt.push_back(e.id);
                }
            } else if (e.point == min_pos) {
                if (e.type == kEnding) {
                    lt.push_back(e.id);
                } else if (e.type == kPlanar) {
                    (min_left ? lt : rt).push_back(e.id);
                } else {
                    rt.push_back(e.id);
                }
            } else if (e.type == kStarting || e.type == kPlanar) {
                rt.push_back(e.id);
            }
        }
    }

    const std::vector<turner_triangle>& tris_;
    int threads_;
};

void free_tree(Node* n) {
    if (!n) return;
    std::vector<Node*> st{n};
    while (!st.empty()) {
        Node* x = st.back();
        st.pop_back();
        if (!x->leaf) {
            st.push_back(x->left);
            st.push_back(x->right);
        }
        delete x;
    }
}

inline uint32_t float_bits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

// FlatNode encodings (lib/kdtree.h:62-154)
inline uint64_t inner_word(int axis, float pos, uint32_t right) {
    return static_cast<uint64_t>(float_bits(pos)) << 32 | static_cast<uint32_t>(right << 2 | static_cast<uint32_t>(axis));
}
inline uint64_t leaf_word(uint32_t a, uint32_t b) {
    return static_cast<uint64_t>(a) << 32 | static_cast<uint64_t>(b << 2 | 3u);
}
constexpr uint32_t kInvalidIndex = 0xFFFFFFFFu >> 2;

std::vector<uint64_t> flatten(Node* root, uint32_t& height) {
    std::vector<uint64_t> nodes;
    struct Item {
        Node* n;
        uint32_t parent;
        uint32_t level;
    };
    std::vector<Item> st{{root, kInvalidIndex, 0}};
    height = 0;
    while (!st.empty()) {
        const Item it = st.back();
        st.pop_back();
        const uint32_t idx = static_cast<uint32_t>(nodes.size());
        if (it.parent != kInvalidIndex) {
            const uint64_t w = nodes[it.parent];
            nodes[it.parent] = (w & 0xFFFFFFFF00000000ull) | static_cast<uint32_t>(idx << 2 | static_cast<uint32_t>(w & 3u));
        }
        height = std::max(height, it.level);
        if (!it.n->leaf) {
            nodes.push_back(inner_word(it.n->axis, it.n->pos, kInvalidIndex));
            st.push_back({it.n->right, idx, it.level + 1});
            st.push_back({it.n->left, kInvalidIndex, it.level + 1});
        } else {
            const auto& ids = it.n->ids;
            size_t i = 1;
            for (; i < ids.size(); i += 2) nodes.push_back(leaf_word(ids[i - 1], ids[i]));
            if (i - 1 < ids.size()) {
                nodes.push_back(leaf_word(ids[i - 1], kInvalidIndex));   // half-empty leaf closes the run
            } else {
                nodes.push_back(inner_word(0, 0.f, 0));                    // sentinel
            }
        }
    }
    return nodes;
}

// Triangle constructor (lib/triangle.h:22-39)
void precompute(turner_triangle& t) {
    for (int i = 0; i < 3; ++i) {
        t.u[i] = t.vertices[1][i] - t.vertices[0][i];
        t.v[i] = t.vertices[2][i] - t.vertices[0][i];
    }
    // cross in double to avoid cancellation (src/geometry.h:288-300)
    const double ux = t.u[0], uy = t.u[1], uz = t.u[2], vx = t.v[0], vy = t.v[1], vz = t.v[2];
    const float cx = static_cast<float>((uy * vz) - (uz * vy));
    const float cy = static_cast<float>((uz * vx) - (ux * vz));
    const float cz = static_cast<float>((ux * vy) - (uy * vx));
    const float len = std::sqrt(cx * cx + cy * cy + cz * cz);
    const float inv = 1 / len;
    t.normal[0] = inv * cx;
    t.normal[1] = inv * cy;
    t.normal[2] = inv * cz;
    t.uv = t.u[0] * t.v[0] + t.u[1] * t.v[1] + t.u[2] * t.v[2];
    t.vv = t.v[0] * t.v[0] + t.v[1] * t.v[1] + t.v[2] * t.v[2];
    t.uu = t.u[0] * t.u[0] + t.u[1] * t.u[1] + t.u[2] * t.u[2];
    t.denom = t.uv * t.uv - t.uu * t.vv;
}

// Triangle::bbox (lib/triangle.h:61-71) with fmin(x, min(y, z))
Box triangle_box(const turner_triangle& t) {
    P3 lo, hi;
    for (int i = 0; i < 3; ++i) {
        lo[i] = std::fmin(t.vertices[0][i], std::min(t.vertices[1][i], t.vertices[2][i]));
        hi[i] = std::fmax(t.vertices[0][i], std::max(t.vertices[1][i], t.vertices[2][i]));
    }
    return make_box(lo, hi);
}

} // namespace

namespace turner {
namespace host {

Box records_and_box(const float* vertices, const float* normals, const float* diffuse, uint32_t n_tris,
                    std::vector<turner_triangle>& tris) {
    tris.resize(n_tris);
    for (uint32_t i = 0; i < n_tris; ++i) {
        turner_triangle& t = tris[i];
        std::memset(&t, 0, sizeof(t));
        std::memcpy(t.vertices, vertices + 9 * size_t(i), 9 * sizeof(float));
        if (normals) std::memcpy(t.normals, normals + 9 * size_t(i), 9 * sizeof(float));
        if (diffuse) {
            std::memcpy(t.diffuse, diffuse + 4 * size_t(i), 4 * sizeof(float));
            // main.cpp:43 reads the emissive colour from the diffuse key
            std::memcpy(t.emissive, diffuse + 4 * size_t(i), 4 * sizeof(float));
        }
        precompute(t);
    }
    // KDTree::KDTree (lib/kdtree.cpp:474-490): box = union of triangle boxes
    Box box = triangle_box(tris[0]);
    for (uint32_t i = 1; i < n_tris; ++i) {
        const Box b = triangle_box(tris[i]);
        P3 lo, hi;
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(box.lo[k], b.lo[k]);
            hi[k] = std::max(box.hi[k], b.hi[k]);
        }
        box = make_box(lo, hi);
    }
    return box;
}

void make_records(const float* vertices, const float* normals, const float* diffuse, uint32_t n_tris,
                  std::vector<turner_triangle>& tris, float box[6]) {
    const Box b = records_and_box(vertices, normals, diffuse, n_tris, tris);
    for (int k = 0; k < 3; ++k) {
        box[k] = b.lo[k];
        box[3 + k] = b.hi[k];
    }
}

} // namespace host
} // namespace turner

extern "C" {

int turner_kdtree_set_reflective(turner_kdtree* tree, const float* reflective) {
    if (!tree || !reflective) return TURNER_ERR_INVALID_ARG;
    for (size_t i = 0; i < tree->tris.size(); ++i) {
        std::memcpy(tree->tris[i].reflective, reflective + 5 * i, 4 * sizeof(float));
        tree->tris[i].reflectivity = reflective[5 * i + 4];
    }
    return TURNER_OK;
}

int turner_kdtree_build(const float* vertices, const float* normals, const float* diffuse, uint32_t n_tris,
                        int threads, turner_kdtree** out) {
    if (!vertices || !out || n_tris == 0) return TURNER_ERR_INVALID_ARG;
    if (n_tris >= TURNER_MISS) return TURNER_ERR_TOO_LARGE;
    auto tree = std::unique_ptr<turner_kdtree>(new (std::nothrow) turner_kdtree);
    if (!tree) return TURNER_ERR_OUT_OF_MEMORY;
    try {
        const Box box = turner::host::records_and_box(vertices, normals, diffuse, n_tris, tree->tris);
        std::vector<uint32_t> ids(n_tris);
        for (uint32_t i = 0; i < n_tris; ++i) ids[i] = i;
        if (threads <= 0) threads = static_cast<int>(std::max(1u, std::thread::hardware_concurrency()));
        int par_depth = 0;
        while ((1 << par_depth) < 2 * threads && par_depth < 12) ++par_depth;
        if (threads == 1) par_depth = 0;
        Builder builder(tree->tris, threads);
        Node* root = builder.build(std::move(ids), box, par_depth);
        tree->nodes = flatten(root, tree->height);
        free_tree(root);
        for (int k = 0; k < 3; ++k) {
            tree->box[k] = box.lo[k];
            tree->box[3 + k] = box.hi[k];
        }
        if (tree->nodes.size() >= TURNER_MISS) return TURNER_ERR_TOO_LARGE;
    } catch (const std::bad_alloc&) {
        return TURNER_ERR_OUT_OF_MEMORY;
    }
    *out = tree.release();
    return TURNER_OK;
}

uint32_t turner_kdtree_num_nodes(const turner_kdtree* t) { return t ? static_cast<uint32_t>(t->nodes.size()) : 0; }
uint32_t turner_kdtree_num_triangles(const turner_kdtree* t) { return t ? static_cast<uint32_t>(t->tris.size()) : 0; }
uint32_t turner_kdtree_height(const turner_kdtree* t) { return t ? t->height : 0; }

int turner_kdtree_export(const turner_kdtree* t, uint64_t* nodes, turner_triangle* tris, float box[6]) {
    if (!t) return TURNER_ERR_INVALID_ARG;
    if (nodes) std::memcpy(nodes, t->nodes.data(), t->nodes.size() * sizeof(uint64_t));
    if (tris) std::memcpy(tris, t->tris.data(), t->tris.size() * sizeof(turner_triangle));
    if (box) std::memcpy(box, t->box, sizeof(t->box));
    return TURNER_OK;
}

void turner_kdtree_free(turner_kdtree* t) { delete t; }

} // extern "C"
