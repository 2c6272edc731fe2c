// Device-side scene layout, geometry and kd-tree traversal.
//
// The translation units that include this header are compiled with
// -fmad=false (and IEEE division / square root, the nvcc defaults), so every
// expression below rounds exactly like the reference's C++ built with
// -ffp-contract=off: hit indices are bit-identical to the reference's
// KDTreeIntersection::intersect, not merely close.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace turner {

constexpr uint32_t kMiss = 0x40000000u;     // FlatNode::MAX_TRIANGLE_ID (lib/kdtree.h:66)
constexpr float kEps = 0.00001f;            // lib/types.h:14
constexpr float kFltMax = 3.40282346638528859812e+38f;
constexpr int kStackCap = 128;              // entries; scenes deeper than this are rejected

// HBM layout of one uploaded scene.
//   nodes : FlatNode words verbatim, read as uint2 {lo = type/axis/right or
//           second id, hi = split bits or first id}; DFS order keeps the near
//           child adjacent to its parent.
//   tri   : 64-byte intersection record per triangle, 4 x float4:
//           {v0, uv} {normal, vv} {u, uu} {v, denom}; the first two (one
//           32-byte sector) decide the plane test, the rest is read only for
//           the barycentric test.
//   shade : 64-byte shading record per triangle, read once per hit:
//           {n0, diffuse.r} {n1, diffuse.g} {n2, diffuse.b} {diffuse.a, 0, 0, 0}
struct SceneView {
    const uint2* nodes;
    const float4* tri;
    const float4* shade;   // {n0, d.r} {n1, d.g} {n2, d.b} {d.a, reflectivity, 0, 0}
    const float4* refl;    // reflective colour per triangle; null when no triangle reflects
    float lo[3], hi[3];
    uint32_t n_nodes, n_tris, height;
};

struct Hit {
    uint32_t id;
    float r, s, t;
};

// intersect_ray_plane + intersect_ray_triangle (lib/intersection.h:40-89)
__device__ __forceinline__ bool triangle_test(const float4* __restrict__ tri, uint32_t id, float3 o, float3 d, float& r,
                                              float& s, float& t) {
    const float4 a = __ldg(tri + 4 * size_t(id) + 0);   // v0, uv
    const float4 n = __ldg(tri + 4 * size_t(id) + 1);   // normal, vv
    const float denom = n.x * d.x + n.y * d.y + n.z * d.z;
    if (denom == 0.f) return false;                      // r = lowest < 0
    const float nom = n.x * (a.x - o.x) + n.y * (a.y - o.y) + n.z * (a.z - o.z);
    r = nom / denom;
    if (r < 0) return false;                             // NaN continues, as in the reference
    const float4 u = __ldg(tri + 4 * size_t(id) + 2);   // u, uu
    const float4 v = __ldg(tri + 4 * size_t(id) + 3);   // v, denom
    const float wx = (o.x + r * d.x) - a.x;
    const float wy = (o.y + r * d.y) - a.y;
    const float wz = (o.z + r * d.z) - a.z;
    const float wv = wx * v.x + wy * v.y + wz * v.z;
    const float wu = wx * u.x + wy * u.y + wz * u.z;
    s = (a.w * wv - n.w * wu) / v.w;
    if (s < 0) return false;
    t = (a.w * wu - u.w * wv) / v.w;
    if (t < 0 || 1 < s + t) return false;
    return true;
}

// true only if the IEEE quotient x / y is < 0: the signs differ and |x / y|
// > 2^-100, so the rounded quotient is a negative normal number, never -0.
// NaN operands and tiny quotients answer false (the caller divides).
__device__ __forceinline__ bool quotient_negative(float x, float y) {
    return ((__float_as_uint(x) ^ __float_as_uint(y)) & 0x80000000u) && fabsf(x) > fabsf(y) * 7.8886090522101181e-31f;
}

// triangle_test restricted to candidates that can change a traversal's
// answer: a valid intersection with r < bound (closest hit, bound = best r
// so far) or r <= bound (any hit, bound = distance to the light). Skipping
// the others is exact: the reference records a hit only if r < min_r
// (strict, lib/kdtree.cpp:568-574) and the shadow test only asks whether some
// valid r <= dist exists. NaN r never satisfies either comparison.
//   - r < 0 is decided from the signs of nom and denom when nom/denom cannot
//     underflow to -0 (|nom| > |denom| * 2^-100), without dividing;
//   - s and t (the second 32-byte half of the record) are only computed for
//     r inside the bound, and their two divides only when neither numerator
//     has the opposite sign of the common denominator.
// One 32-byte read-only load (sm_100 and later); p must be 32-byte aligned.
// Intersection records are 64 bytes and the array is 256-byte aligned, so
// each half of a record is one such load: one L1 request instead of two.
__device__ __forceinline__ void ldg_pair(const float4* p, float4& x, float4& y) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(x.x), "=f"(x.y), "=f"(x.z), "=f"(x.w), "=f"(y.x), "=f"(y.y), "=f"(y.z), "=f"(y.w)
        : "l"(p));
}

template <bool INCLUSIVE>
__device__ __forceinline__ bool triangle_test_bounded(const float4* __restrict__ tri, uint32_t id, float3 o, float3 d,
                                                      float bound, float& r, float& s, float& t) {
    float4 a, n;   // {v0, uv}, {normal, vv}
    ldg_pair(tri + 4 * size_t(id), a, n);
    const float denom = n.x * d.x + n.y * d.y + n.z * d.z;
    if (denom == 0.f) return false;
    const float nom = n.x * (a.x - o.x) + n.y * (a.y - o.y) + n.z * (a.z - o.z);
    if (quotient_negative(nom, denom)) return false;    // r < 0
    r = nom / denom;
    if (INCLUSIVE ? !(r <= bound) : !(r < bound)) return false;
    if (r < 0) return false;
    float4 u, v;   // {u, uu}, {v, denom}
    ldg_pair(tri + 4 * size_t(id) + 2, u, v);
    const float wx = (o.x + r * d.x) - a.x;
    const float wy = (o.y + r * d.y) - a.y;
    const float wz = (o.z + r * d.z) - a.z;
    const float wv = wx * v.x + wy * v.y + wz * v.z;
    const float wu = wx * u.x + wy * u.y + wz * u.z;
    const float s_num = a.w * wv - n.w * wu;
    const float t_num = a.w * wu - u.w * wv;
    // s < 0 or t < 0 from the signs, as for r above; both divides only for
    // points that can lie inside the triangle
    if (quotient_negative(s_num, v.w) || quotient_negative(t_num, v.w)) return false;
    s = s_num / v.w;
    if (s < 0) return false;
    t = t_num / v.w;
    if (t < 0 || 1 < s + t) return false;
    return true;
}

__device__ __forceinline__ float pick(float3 v, uint32_t ax) { return ax == 0 ? v.x : (ax == 1 ? v.y : v.z); }

// Traversal stacks. An entry is {far child, exit distance of the cell it was
// split from}; its entry distance is not stored. Between a push and the
// matching pop the current exit distance is exactly the pushed split
// distance t (a push sets texit = t, descents without a push leave it, and a
// pop restores the exit that the entry below it recorded), so a pop takes
// tenter = texit and texit = the stored exit: the same floats the reference's
// three-field stack (lib/kdtree.cpp:530-560) holds, in 8 bytes instead of 12.
template <int N>
struct LocalStack {
    uint2 e[N];
    __device__ __forceinline__ void reset() {}
    __device__ __forceinline__ void put(int k, uint2 v) { e[k] = v; }
    __device__ __forceinline__ uint2 get(int k) const { return e[k]; }
};

// A stack whose newest R entries live in shared memory, the older ones in
// local memory. Shared memory holds two words per entry, [slot][thread] for
// the far child and the exit distance, so lanes at different depths of their
// own stacks never conflict on a bank (word = slot * BLOCK + thread): a
// divergent push or pop is one shared-memory wavefront per word, where the
// same access to local memory touches up to 32 cache lines. A push onto a
// full ring first moves the oldest ring entry to local memory; a pop from an
// empty ring takes the entry from local memory. Entries stay in push order,
// so pops return exactly what LocalStack would.
template <int R, int BLOCK, int N>
struct RingStack {
    static_assert((R & (R - 1)) == 0, "ring size is a power of two");
    uint2 spill[N];    // entries below `base`
    int base;          // entries [base, sp) are in the ring
    // the block's dynamic shared memory: [R][BLOCK] far-child words, then
    // [R][BLOCK] exit-distance words (addresses recomputed per access, so no
    // register holds a pointer)
    __device__ __forceinline__ static uint32_t* words() {
        extern __shared__ uint32_t ring_smem[];
        return ring_smem;
    }
    __device__ __forceinline__ void init() { base = 0; }
    __device__ __forceinline__ void reset() { base = 0; }
    __device__ __forceinline__ void put(int k, uint2 v) {
        uint32_t* w = words();
        if (k - base >= R) {   // the ring is full: its oldest entry (slot of base) goes to local memory
            const int o = (base & (R - 1)) * BLOCK + static_cast<int>(threadIdx.x);
            spill[base] = make_uint2(w[o], w[R * BLOCK + o]);
            ++base;
        }
        const int s = (k & (R - 1)) * BLOCK + static_cast<int>(threadIdx.x);
        w[s] = v.x;
        w[R * BLOCK + s] = v.y;
    }
    __device__ __forceinline__ uint2 get(int k) {
        if (k < base) {   // the ring is empty: the entry is in local memory
            base = k;
            return spill[k];
        }
        const uint32_t* w = words();
        const int s = (k & (R - 1)) * BLOCK + static_cast<int>(threadIdx.x);
        return make_uint2(w[s], w[R * BLOCK + s]);
    }
};

// KDTreeIntersection::intersect (lib/kdtree.cpp:516-607).
//   CLOSEST: every leaf overlapped by [tenter, texit] is visited in the
//   reference's order (near child first, far child pushed, LIFO), and the
//   first strict minimum of r is kept. Keeping one running minimum with a
//   strict "<" picks the same triangle as the reference's per-run minimum
//   followed by a strict comparison with the best so far.
//   ANY (shadow rays): returns a hit as soon as one valid intersection has
//   r <= tmax. The reference tests `!hit || r_closest > dist`; "lit" is the
//   same predicate as "no valid intersection with r <= dist", so this is exact.
//   FAST_EXIT (closest only): after a leaf run, stop when the best r is below
//   every pending cell's entry distance minus a margin.
template <bool ANY, bool FAST_EXIT>
__device__ __forceinline__ Hit traverse(const SceneView& sc, float3 o, float3 d, float tmax) {
    Hit best{kMiss, kFltMax, 0.f, 0.f};
    // fix_direction (kdtree.cpp:503-511)
    const float3 fd = make_float3(d.x == 0.f ? kEps : d.x, d.y == 0.f ? kEps : d.y, d.z == 0.f ? kEps : d.z);
    const float3 inv = make_float3(1.0f / fd.x, 1.0f / fd.y, 1.0f / fd.z);
    // intersect_ray_box (intersection.h:105-128) on the fixed ray
    float tenter, texit;
    {
        const float tx1 = (sc.lo[0] - o.x) * inv.x, tx2 = (sc.hi[0] - o.x) * inv.x;
        tenter = fminf(tx1, tx2);
        texit = fmaxf(tx1, tx2);
        const float ty1 = (sc.lo[1] - o.y) * inv.y, ty2 = (sc.hi[1] - o.y) * inv.y;
        tenter = fmaxf(tenter, fminf(ty1, ty2));
        texit = fminf(texit, fmaxf(ty1, ty2));
        const float tz1 = (sc.lo[2] - o.z) * inv.z, tz2 = (sc.hi[2] - o.z) * inv.z;
        tenter = fmaxf(tenter, fminf(tz1, tz2));
        texit = fminf(texit, fmaxf(tz1, tz2));
        if (texit < tenter) return best;
    }

    LocalStack<kStackCap> st;
    int sp = 0;
    uint32_t node = 0;
    const uint2* __restrict__ nodes = sc.nodes;
    for (;;) {
        uint2 w = __ldg(nodes + node);
        while ((w.x & 3u) != 3u) {
            const uint32_t ax = w.x & 3u;
            const float t = (__uint_as_float(w.y) - pick(o, ax)) * pick(inv, ax);
            uint32_t near_c = node + 1, far_c = w.x >> 2;
            if (pick(fd, ax) <= 0.f) {
                const uint32_t tmp = near_c;
                near_c = far_c;
                far_c = tmp;
            }
            if (texit < t) {
                node = near_c;
            } else if (t < tenter) {
                node = far_c;
            } else {
                st.put(sp, make_uint2(far_c, __float_as_uint(texit)));
                ++sp;
                node = near_c;
                texit = t;
            }
            w = __ldg(nodes + node);
        }
        // leaf run: two ids per word until a half-empty leaf or an inner node
        for (;;) {
            float r, s, t;
            if (triangle_test(sc.tri, w.y, o, d, r, s, t)) {
                if (ANY) {
                    if (r <= tmax) return Hit{w.y, r, s, t};
                } else if (r < best.r) {
                    best = Hit{w.y, r, s, t};
                }
            }
            if (w.x == 0xFFFFFFFFu) break;
            const uint32_t id2 = w.x >> 2;
            if (triangle_test(sc.tri, id2, o, d, r, s, t)) {
                if (ANY) {
                    if (r <= tmax) return Hit{id2, r, s, t};
                } else if (r < best.r) {
                    best = Hit{id2, r, s, t};
                }
            }
            ++node;
            w = __ldg(nodes + node);
            if ((w.x & 3u) != 3u) break;
        }
        if (sp == 0) break;
        --sp;
        if (FAST_EXIT && !ANY) {
            // cells are popped in increasing entry distance along the ray;
            // a hit closer than the next cell's entry (with margin for the
            // thick-plane classification of the builder) cannot be beaten
            if (best.r < texit - (1e-3f + 1e-3f * fabsf(texit))) break;
        }
        const uint2 e = st.get(sp);
        node = e.x;
        tenter = texit;   // the popped cell starts at the split plane, the current exit
        texit = __uint_as_float(e.y);
    }
    return best;
}

// Resumable form of traverse() for persistent kernels: the same visit order
// and arithmetic, split into rounds so that a lane can take a new ray as soon
// as its current one is finished (ray replacement, Aila & Laine 2009).
struct TravState {
    const uint2* nodes;
    const float4* tri;
    float3 o, d, inv;
    uint32_t neg;    // bit ax: fixed direction component <= 0 (near child is the right one)
    uint32_t node;
    float tenter, texit;
    int sp;
    Hit best;
    // the last four triangles tested by this ray. A triangle referenced by
    // several leaves is tested again by the reference; the repeat gives the
    // same r, which can no longer pass `r < best` (or newly satisfy r <= dist),
    // so skipping it leaves the answer unchanged.
    uint32_t mb[4];
    uint32_t mb_next;
};

template <bool MAILBOX>
__device__ __forceinline__ bool mailbox_seen(TravState& s, uint32_t id) {
    if (!MAILBOX) return false;
    if (id == s.mb[0] || id == s.mb[1] || id == s.mb[2] || id == s.mb[3]) return true;
    const uint32_t k = s.mb_next & 3u;
    s.mb[0] = k == 0 ? id : s.mb[0];
    s.mb[1] = k == 1 ? id : s.mb[1];
    s.mb[2] = k == 2 ? id : s.mb[2];
    s.mb[3] = k == 3 ? id : s.mb[3];
    s.mb_next = k + 1;
    return false;
}

// fix_direction + root box test. false: the ray misses the scene box.
__device__ __forceinline__ bool trav_begin(const SceneView& sc, float3 o, float3 d, TravState& s) {
    s.nodes = sc.nodes;
    s.tri = sc.tri;
    s.best = Hit{kMiss, kFltMax, 0.f, 0.f};
    s.mb[0] = s.mb[1] = s.mb[2] = s.mb[3] = kMiss;
    s.mb_next = 0;
    const float3 fd = make_float3(d.x == 0.f ? kEps : d.x, d.y == 0.f ? kEps : d.y, d.z == 0.f ? kEps : d.z);
    s.o = o;
    s.d = d;
    s.inv = make_float3(1.0f / fd.x, 1.0f / fd.y, 1.0f / fd.z);
    s.neg = (fd.x <= 0.f ? 1u : 0u) | (fd.y <= 0.f ? 2u : 0u) | (fd.z <= 0.f ? 4u : 0u);
    const float tx1 = (sc.lo[0] - o.x) * s.inv.x, tx2 = (sc.hi[0] - o.x) * s.inv.x;
    float tenter = fminf(tx1, tx2);
    float texit = fmaxf(tx1, tx2);
    const float ty1 = (sc.lo[1] - o.y) * s.inv.y, ty2 = (sc.hi[1] - o.y) * s.inv.y;
    tenter = fmaxf(tenter, fminf(ty1, ty2));
    texit = fminf(texit, fmaxf(ty1, ty2));
    const float tz1 = (sc.lo[2] - o.z) * s.inv.z, tz2 = (sc.hi[2] - o.z) * s.inv.z;
    tenter = fmaxf(tenter, fminf(tz1, tz2));
    texit = fminf(texit, fmaxf(tz1, tz2));
    s.tenter = tenter;
    s.texit = texit;
    s.node = 0;
    s.sp = 0;
    return !(texit < tenter);
}

// One round: descend from s.node to a leaf, test its run, pop the next cell.
// Returns true when the ray is finished (s.best holds the answer).
template <bool ANY, bool FAST_EXIT, bool MAILBOX = false, class Stack>
__device__ __forceinline__ bool trav_round(TravState& s, float tmax, Stack& st) {
    const uint2* __restrict__ nodes = s.nodes;
    uint32_t node = s.node;
    float tenter = s.tenter, texit = s.texit;
    int sp = s.sp;
    uint2 w = __ldg(nodes + node);
    while ((w.x & 3u) != 3u) {
        const uint32_t ax = w.x & 3u;
        const float t = (__uint_as_float(w.y) - pick(s.o, ax)) * pick(s.inv, ax);
        uint32_t near_c = node + 1, far_c = w.x >> 2;
        if (s.neg & (1u << ax)) {
            const uint32_t tmp = near_c;
            near_c = far_c;
            far_c = tmp;
        }
        if (texit < t) {
            node = near_c;
        } else if (t < tenter) {
            node = far_c;
        } else {
            st.put(sp, make_uint2(far_c, __float_as_uint(texit)));
            ++sp;
            node = near_c;
            texit = t;
        }
        w = __ldg(nodes + node);
    }
    for (;;) {
        // a full pair is always followed by another word (a leaf or the
        // run's sentinel): fetch it while the pair is tested
        const bool pair = w.x != 0xFFFFFFFFu;
        uint2 next = w;
        if (pair) next = __ldg(nodes + node + 1);
        float r, u, v;
        if (!mailbox_seen<MAILBOX>(s, w.y) &&
            triangle_test_bounded<ANY>(s.tri, w.y, s.o, s.d, ANY ? tmax : s.best.r, r, u, v)) {
            s.best = Hit{w.y, r, u, v};
            if (ANY) return true;
        }
        if (!pair) break;
        const uint32_t id2 = w.x >> 2;
        if (!mailbox_seen<MAILBOX>(s, id2) &&
            triangle_test_bounded<ANY>(s.tri, id2, s.o, s.d, ANY ? tmax : s.best.r, r, u, v)) {
            s.best = Hit{id2, r, u, v};
            if (ANY) return true;
        }
        ++node;
        w = next;
        if ((w.x & 3u) != 3u) break;
    }
    if (sp == 0) return true;
    --sp;
    if (FAST_EXIT && !ANY) {
        if (s.best.r < texit - (1e-3f + 1e-3f * fabsf(texit))) return true;
    }
    const uint2 e = st.get(sp);
    s.node = e.x;
    s.tenter = texit;
    s.texit = __uint_as_float(e.y);
    s.sp = sp;
    return false;
}

// Speculative form of trav_round (Aila & Laine 2009), called by all 32 lanes
// of a warp together (`live`: the lane holds a ray). A lane that reaches a
// leaf keeps its run aside, pops the next cell and descends on toward the
// next leaf while some lane of its warp has not found a leaf yet; it stops at
// that second leaf, which starts its next round. Then every lane tests the
// run it kept. Each ray still tests its leaf runs in the reference's order
// (the run kept aside before the one found after it), with the same bounds,
// so the answers are those of trav_round; only FAST_EXIT's early stop is not
// available here. s.node == kNoNode: the ray has no cell left. Returns true
// when the lane's ray is finished.
constexpr uint32_t kNoNode = 0xFFFFFFFFu;

template <bool ANY, bool MAILBOX, class Stack>
__device__ __forceinline__ bool trav_round_spec(TravState& s, bool live, float tmax, Stack& st) {
    const uint2* __restrict__ nodes = s.nodes;
    uint32_t node = s.node;
    float tenter = s.tenter, texit = s.texit;
    int sp = s.sp;
    uint32_t kept = kNoNode;   // first word of the leaf run set aside
    bool stepping = live && node != kNoNode;
    uint2 w = make_uint2(0u, 0u);
    if (stepping) w = __ldg(nodes + node);
    // descend while some lane of the warp has no leaf yet
    while (__any_sync(0xFFFFFFFFu, live && kept == kNoNode && node != kNoNode)) {
        if (stepping) {
            if ((w.x & 3u) != 3u) {
                const uint32_t ax = w.x & 3u;
                const float t = (__uint_as_float(w.y) - pick(s.o, ax)) * pick(s.inv, ax);
                uint32_t near_c = node + 1, far_c = w.x >> 2;
                if (s.neg & (1u << ax)) {
                    const uint32_t tmp = near_c;
                    near_c = far_c;
                    far_c = tmp;
                }
                if (texit < t) {
                    node = near_c;
                } else if (t < tenter) {
                    node = far_c;
                } else {
                    st.put(sp, make_uint2(far_c, __float_as_uint(texit)));
                    ++sp;
                    node = near_c;
                    texit = t;
                }
                w = __ldg(nodes + node);
            } else if (kept == kNoNode) {
                // set this leaf's run aside and go on to the next cell
                kept = node;
                if (sp == 0) {
                    node = kNoNode;
                    stepping = false;
                } else {
                    --sp;
                    const uint2 e = st.get(sp);
                    node = e.x;
                    tenter = texit;
                    texit = __uint_as_float(e.y);
                    w = __ldg(nodes + node);
                }
            } else {
                stepping = false;   // a second leaf: it starts the next round
            }
        }
    }
    s.node = node;
    s.tenter = tenter;
    s.texit = texit;
    s.sp = sp;
    // test the runs set aside: two ids per word until a half-empty leaf or an inner node
    bool hit_any = false;
    bool testing = live && kept != kNoNode;
    uint32_t wi = kept;
    uint2 lw = make_uint2(0u, 0u);
    if (testing) lw = __ldg(nodes + wi);
    while (__any_sync(0xFFFFFFFFu, testing)) {
        if (testing) {
            const bool pair = lw.x != 0xFFFFFFFFu;
            uint2 next = lw;
            if (pair) next = __ldg(nodes + wi + 1);
            float r, u, v;
            if (!mailbox_seen<MAILBOX>(s, lw.y) &&
                triangle_test_bounded<ANY>(s.tri, lw.y, s.o, s.d, ANY ? tmax : s.best.r, r, u, v)) {
                s.best = Hit{lw.y, r, u, v};
                if (ANY) {
                    hit_any = true;
                    testing = false;
                }
            }
            if (testing) {
                if (!pair) {
                    testing = false;
                } else {
                    const uint32_t id2 = lw.x >> 2;
                    if (!mailbox_seen<MAILBOX>(s, id2) &&
                        triangle_test_bounded<ANY>(s.tri, id2, s.o, s.d, ANY ? tmax : s.best.r, r, u, v)) {
                        s.best = Hit{id2, r, u, v};
                        if (ANY) {
                            hit_any = true;
                            testing = false;
                        }
                    }
                    if (testing) {
                        ++wi;
                        lw = next;
                        if ((lw.x & 3u) != 3u) testing = false;
                    }
                }
            }
        }
    }
    return hit_any || s.node == kNoNode;
}

// Packet traversal of a warp whose live rays share their direction signs
// (`neg`) and scene (`nodes`, `tri`): camera rays of neighbouring pixels and
// their shadow rays. Called by all 32 lanes; it runs until every live ray is
// finished. The warp walks the tree as one: a child is entered when some
// lane's interval overlaps it, the near child first, so every lane visits the
// cells its own traversal (trav_round) would visit, in the same order, with
// the same [tenter, texit], and tests the same leaf runs with the same
// bounds: the answers are bit-identical. Lanes whose interval misses a cell
// only wait while the warp is inside it. Node words and triangle records are
// then the same address in every lane, one load for the warp.
// A stack entry holds the far child (with the lane's "continues there" bit)
// and the lane's entry and exit distances for it.
template <bool ANY>
__device__ __forceinline__ void trav_packet(TravState& s, bool live, float tmax, uint32_t neg,
                                            const uint2* __restrict__ nodes, const float4* __restrict__ tri) {
    uint4 pk[kStackCap];
    bool alive = live, done = false;
    float tenter = s.tenter, texit = s.texit;
    uint32_t node = 0;
    int sp = 0;
    for (;;) {
        uint2 w = __ldg(nodes + node);
        if ((w.x & 3u) != 3u) {
            const uint32_t ax = w.x & 3u;
            const float t = (__uint_as_float(w.y) - pick(s.o, ax)) * pick(s.inv, ax);
            uint32_t near_c = node + 1, far_c = w.x >> 2;
            if (neg & (1u << ax)) {
                const uint32_t tmp = near_c;
                near_c = far_c;
                far_c = tmp;
            }
            // the cases of trav_round: near only, far only, or both (far pushed)
            const bool both = alive && !(texit < t) && !(t < tenter);
            const bool want_near = alive && (texit < t || both);
            const bool want_far = alive && !(texit < t) && (t < tenter || both);
            const bool any_near = __any_sync(0xFFFFFFFFu, want_near);
            const bool any_far = __any_sync(0xFFFFFFFFu, want_far);
            if (any_near || any_far) {
                if (any_near && any_far) {
                    pk[sp] = make_uint4(far_c | (want_far ? 0x80000000u : 0u), __float_as_uint(both ? t : tenter),
                                        __float_as_uint(texit), 0u);
                    ++sp;
                }
                if (any_near) {
                    node = near_c;
                    alive = want_near;
                    if (both) texit = t;
                } else {
                    node = far_c;
                    alive = want_far;
                }
                continue;
            }
        } else if (__any_sync(0xFFFFFFFFu, alive)) {
            // the leaf run: the same words for every lane, tested by the lanes inside the cell
            uint32_t wi = node;
            for (;;) {
                const bool pair = w.x != 0xFFFFFFFFu;
                uint2 next = w;
                if (pair) next = __ldg(nodes + wi + 1);
                float r, u, v;
                if (alive && triangle_test_bounded<ANY>(tri, w.y, s.o, s.d, ANY ? tmax : s.best.r, r, u, v)) {
                    s.best = Hit{w.y, r, u, v};
                    if (ANY) {
                        alive = false;
                        done = true;
                    }
                }
                if (!pair) break;
                const uint32_t id2 = w.x >> 2;
                if (alive && triangle_test_bounded<ANY>(tri, id2, s.o, s.d, ANY ? tmax : s.best.r, r, u, v)) {
                    s.best = Hit{id2, r, u, v};
                    if (ANY) {
                        alive = false;
                        done = true;
                    }
                }
                ++wi;
                w = next;
                if ((w.x & 3u) != 3u) break;
            }
        }
        if (sp == 0) break;
        --sp;
        const uint4 e = pk[sp];
        node = e.x & 0x7FFFFFFFu;
        alive = (e.x >> 31) != 0u && !done;
        tenter = __uint_as_float(e.y);
        texit = __uint_as_float(e.z);
    }
}

// xorshift64* (lib/xorshift.h:27-70): float = (x & (2^24 - 1)) * 2^-24
__device__ __forceinline__ float xorshift_float(uint64_t& s) {
    s ^= s >> 12;
    s ^= s << 25;
    s ^= s >> 27;
    const uint64_t x = s * 2685821657736338717ULL;
    return static_cast<float>(static_cast<uint32_t>(x & 0xFFFFFFull)) * 5.9604644775390625e-8f;
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

// Per-(pixel, sample) streams: key = pixel_index * spp + sample.
// Stream of child k of a hit under the branching estimator (-m > 1), derived
// from the stream state of the ray that made the hit (same as the oracle's).
__device__ __forceinline__ uint64_t branch_seed(uint64_t parent_state, uint32_t k) {
    const uint64_t s = splitmix64(parent_state ^ (0xA0761D6478BD642FULL * (uint64_t(k) + 1)));
    return s ? s : 1;
}

__device__ __forceinline__ void path_seeds(uint64_t seed, uint64_t key, uint64_t& jitter, uint64_t& bounce) {
    const uint64_t a = splitmix64(seed ^ key);
    const uint64_t b = splitmix64(a ^ 0xD1B54A32D192ED03ULL);
    jitter = a ? a : 1;
    bounce = b ? b : 1;
}

// Moeller-Hughes from-to rotation (JGT 1999) taking (0, 0, 1) onto n, row-major.
__device__ __forceinline__ void from_to_z(float3 n, float m[9]) {
    const float fx = 0.f, fy = 0.f, fz = 1.f;
    const float vx = fy * n.z - fz * n.y;
    const float vy = fz * n.x - fx * n.z;
    const float vz = fx * n.y - fy * n.x;
    const float e = fx * n.x + fy * n.y + fz * n.z;
    const float f = e < 0 ? -e : e;
    if (f > 1.0f - 0.000001f) {
        // `from` = +z is least aligned with the y axis (|0| < |1|, ties -> y)
        const float x0 = 0.f, x1 = 1.f, x2 = 0.f;
        const float u[3] = {x0 - fx, x1 - fy, x2 - fz};
        const float w[3] = {x0 - n.x, x1 - n.y, x2 - n.z};
        const float c1 = 2.0f / (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        const float c2 = 2.0f / (w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        const float c3 = c1 * c2 * (u[0] * w[0] + u[1] * w[1] + u[2] * w[2]);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
#pragma unroll
            for (int j = 0; j < 3; ++j) m[3 * i + j] = -c1 * u[i] * u[j] - c2 * w[i] * w[j] + c3 * w[i] * u[j];
            m[3 * i + i] += 1.0f;
        }
    } else {
        const float h = 1.0f / (1.0f + e);
        const float hvx = h * vx, hvz = h * vz;
        const float hvxy = hvx * vy, hvxz = hvx * vz, hvyz = hvz * vy;
        m[0] = e + hvx * vx;
        m[1] = hvxy - vz;
        m[2] = hvxz + vy;
        m[3] = hvxy + vz;
        m[4] = e + h * vy * vy;
        m[5] = hvyz - vx;
        m[6] = hvxz - vy;
        m[7] = hvyz + vx;
        m[8] = e + hvz * vz;
    }
}

} // namespace turner
