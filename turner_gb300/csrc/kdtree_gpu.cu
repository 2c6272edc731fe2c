// GPU kd-tree build: a binned-SAH kd-tree built level by level on the GPU and
// flattened into the reference's FlatNode format (lib/kdtree.h:62-154), so
// that turner_upload_scene and every traversal kernel take it unchanged.
//
// It is not the reference's builder (lib/kdtree.cpp:124-412): the reference
// sweeps exact event lists sorted with std::sort, whose order among equal
// keys is that library's and decides the triangle order inside leaves. This
// build chooses planes among 32 bins per axis for cells of more than kMidMax
// references and among all clipped-box bounds for smaller cells, so its tree
// differs. Every leaf lists every triangle whose clipped box reaches into the
// leaf's cell, so closest hits are the same triangles at the same r (checked
// against a brute-force leaf and the reference's tree in the tests).
//
// Splits leave triangles on both sides. The flattening drops an empty child
// (so does the reference's, lib/kdtree.cpp:164-172), and with it the cut: an
// empty-space split never narrows a cell that the traversal sees, although
// the SAH credits it with the space it cuts off (and with the 0.8 empty-side
// factor of lib/kdtree.cpp:182-187). Allowing such splits built thin slab
// cells around curved surfaces (twice the node visits and triangle tests of
// the reference's tree on the 327,692-triangle sphere room); without them the
// same build needs about two thirds of the reference tree's visits and a
// quarter of its tests. (The reference's own builder seldom cuts empty space:
// a triangle whose clipped polygon has fewer than two points gets an
// unbounded box there and sits on both sides of every later plane.)
//
// Per level (one CUDA block per node):
//   k_level     bounding box of each triangle reference clipped to the node's
//               cell, 32-bin start/end histograms per axis in shared memory
//               (or, in small cells, the boxes themselves), SAH of the
//               3 x 31 bin boundaries (or of every box bound) with the reference's
//               constants (traversal 15, intersection 20, lib/kdtree.cpp:178-203)
//               and its termination test, then
//               per reference: left / right / leaf flags
//   scans       exclusive scans of the flags (per reference) and of the
//               children, next-level references and leaf references (per node)
//   k_children  child cells and reference ranges; one BFS record per node
//   k_scatter   references to the next level or to the leaf pool
// The host flattens the BFS records into DFS FlatNode words (left child
// adjacent, leaves two ids per word, half-empty leaf or sentinel at the end of
// a run), dropping empty children as KDTree's builder does.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <memory>
#include <new>
#include <system_error>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "host/tree.h"
#include "turner_gpu.h"

namespace {

constexpr int kBins = 32;
constexpr int kLevelThreads = 256;
constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;                         // elements per thread of a scan block
constexpr int kScanBlock = kScanThreads * kScanItems;
constexpr uint32_t kMaxBuildDepth = 60;               // flattened depth, < the traversal stack (128 entries)
constexpr uint32_t kMaxLevels = 512;                  // breadth-first levels, counting empty-space cuts
constexpr uint32_t kExactMax = 1024;                  // cells this small sweep every box bound
constexpr uint32_t kSmallMax = 32;                    // cells this small take one warp instead of a block
constexpr int kSmallWarps = 8;                        // warps (cells) per block of k_level_small
constexpr uint32_t kMidMax = 8192;                     // cells up to this size (above kExactMax) sort their bounds
constexpr int kMidThreads = 512;
constexpr float kCostTraversal = 15.f, kCostIntersection = 20.f;

struct Cell {
    float lo[3], hi[3];
    uint32_t begin, count;   // references [begin, begin + count) of the level
    uint32_t depth;          // splits above with two non-empty children (the flattened depth)
};

struct Decision {
    int32_t split;         // 0 leaf, 1 split
    int32_t axis;
    float pos;
    uint32_t kept;         // references whose box meets the cell
    int32_t planar_left;   // boxes lying in the plane go left (else right)
};

// One node of the breadth-first tree; children are global ids or -1.
struct BfsNode {
    int32_t split;
    int32_t axis;
    float pos;
    int32_t left, right;
    uint32_t leaf_begin, leaf_count;
};

__device__ __forceinline__ float surface(const float lo[3], const float hi[3]) {
    const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    return 2.f * (dx * dy + dx * dz + dy * dz);
}

// Bounding box of the part of triangle t inside cell c (slightly widened, so
// rounding never loses a triangle that touches the cell); false if none. A
// triangle whose box lies inside the cell keeps its box; one that crosses the
// cell's faces is clipped (Sutherland-Hodgman against the six faces), which
// for steep or long triangles is far tighter than its box cut to the cell.
__device__ __forceinline__ bool clip_to(const float* __restrict__ verts, const float* __restrict__ tri_box, uint32_t t,
                                        const Cell& c, float lo[3], float hi[3]) {
    const float* tb = tri_box + 6 * size_t(t);
    bool inside = true, overlap = true;
    float e[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        e[a] = 1e-5f * fmaxf(1.f, fmaxf(fabsf(c.lo[a]), fabsf(c.hi[a])));
        lo[a] = tb[a];
        hi[a] = tb[3 + a];
        inside = inside && lo[a] >= c.lo[a] && hi[a] <= c.hi[a];
        overlap = overlap && lo[a] <= c.hi[a] + e[a] && hi[a] >= c.lo[a] - e[a];
    }
    if (!overlap) return false;
    if (inside) return true;
    float p[9][3], q[9][3];
    const float* v = verts + 9 * size_t(t);
#pragma unroll
    for (int k = 0; k < 9; ++k) p[k / 3][k % 3] = v[k];
    int n = 3;
    for (int f = 0; f < 6; ++f) {
        const int a = f >> 1;
        const bool low = (f & 1) == 0;
        const float bound = low ? c.lo[a] - e[a] : c.hi[a] + e[a];
        int m = 0;
        for (int i = 0; i < n; ++i) {
            const float* pa = p[i];
            const float* pb = p[i + 1 < n ? i + 1 : 0];
            const float da = low ? pa[a] - bound : bound - pa[a];
            const float db = low ? pb[a] - bound : bound - pb[a];
            if (da >= 0.f && m < 9) {   // (rounding can add crossings: never past 9 points)
                q[m][0] = pa[0];
                q[m][1] = pa[1];
                q[m][2] = pa[2];
                ++m;
            }
            if ((da >= 0.f) != (db >= 0.f) && m < 9) {
                const float s = da / (da - db);
#pragma unroll
                for (int k = 0; k < 3; ++k) q[m][k] = pa[k] + s * (pb[k] - pa[k]);
                q[m][a] = bound;
                ++m;
            }
        }
        n = m;
        if (n == 0) return false;
        for (int i = 0; i < n; ++i) {
            p[i][0] = q[i][0];
            p[i][1] = q[i][1];
            p[i][2] = q[i][2];
        }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float mn = p[0][a], mx = p[0][a];
        for (int i = 1; i < n; ++i) {
            mn = fminf(mn, p[i][a]);
            mx = fmaxf(mx, p[i][a]);
        }
        // widen by the clipping slack and keep within the triangle's box
        lo[a] = fmaxf(mn - e[a], tb[a]);
        hi[a] = fminf(mx + e[a], tb[3 + a]);
        lo[a] = fmaxf(lo[a], c.lo[a]);
        hi[a] = fminf(hi[a], c.hi[a]);
        if (lo[a] > hi[a]) {   // the slack reached past the cell: the triangle touches a face
            lo[a] = hi[a] = lo[a] > c.hi[a] ? c.hi[a] : c.lo[a];
        }
    }
    return true;
}

__device__ __forceinline__ int bin_of(float x, float lo, float scale) {
    const int b = static_cast<int>(floorf((x - lo) * scale));
    return min(max(b, 0), kBins - 1);
}

// Triangle bounding boxes, min xyz then max xyz.
__global__ void k_tri_boxes(const float* __restrict__ v, uint32_t n, float* __restrict__ box) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* t = v + 9 * size_t(i);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        box[6 * size_t(i) + a] = fminf(t[a], fminf(t[3 + a], t[6 + a]));
        box[6 * size_t(i) + 3 + a] = fmaxf(t[a], fmaxf(t[3 + a], t[6 + a]));
    }
}

// The better of two SAH candidates: lower cost, then lower axis, then lower
// position, then planar boxes left (independent of the order threads found
// them in).
__device__ __forceinline__ bool better(float c, int a, float p, int pl, float bc, int ba, float bp, int bpl) {
    if (c != bc) return c < bc;
    if (a != ba) return a < ba;
    if (p != bp) return p < bp;
    return pl > bpl;
}

__device__ __forceinline__ float split_cost(const Cell& c, float sa, int a, float pos, uint32_t nl, uint32_t nr) {
    float llo[3], lhi[3], rlo[3], rhi[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        llo[q] = rlo[q] = c.lo[q];
        lhi[q] = rhi[q] = c.hi[q];
    }
    lhi[a] = pos;
    rlo[a] = pos;
    return kCostTraversal + kCostIntersection * (surface(llo, lhi) / sa * static_cast<float>(nl) +
                                                 surface(rlo, rhi) / sa * static_cast<float>(nr));
}

// Which side of the plane a clipped box goes to: left if it starts before the
// plane, right if it ends after it; a box lying in the plane goes to the
// side the split chose (the cheaper one, as the reference places planar
// triangles, lib/kdtree.cpp:178-203). A box that only touches the plane does
// not go to that side: traversal visits both cells wherever a ray crosses the
// plane, and keeping touching boxes on both sides would never separate the
// triangles that share a vertex.
__device__ __forceinline__ bool goes_left(float lo, float hi, float pos, bool planar_left) {
    return lo < pos || (planar_left && lo == pos && hi == pos);
}
__device__ __forceinline__ bool goes_right(float lo, float hi, float pos, bool planar_left) {
    return hi > pos || (!planar_left && lo == pos && hi == pos);
}

// Best of the two placements of the boxes lying in the plane; nl, nr count
// the boxes strictly on each side, np those in the plane.
__device__ __forceinline__ void consider(const Cell& c, float sa, uint32_t n, int a, float pos, uint32_t nl,
                                         uint32_t nr, uint32_t np, float& bc, int& ba, float& bp, int& bpl,
                                         uint32_t& bnl, uint32_t& bnr) {
#pragma unroll
    for (int pl = 1; pl >= 0; --pl) {
        const uint32_t l = nl + (pl ? np : 0u), r = nr + (pl ? 0u : np);
        if (l == n && r == n) continue;   // separates nothing
        if (l == 0 || r == 0) continue;   // empty space: the flattening would drop the cut
        // a plane in a face is useful only to move the boxes lying in it
        // into a flat cell, not to keep the cell whole
        if (pos == c.lo[a] && r == n) continue;
        if (pos == c.hi[a] && l == n) continue;
        const float cost = split_cost(c, sa, a, pos, l, r);
        if (better(cost, a, pos, pl, bc, ba, bp, bpl)) {
            bc = cost;
            ba = a;
            bp = pos;
            bpl = pl;
            bnl = l;
            bnr = r;
        }
    }
}

// One block per listed cell (the cells of more than kSmallMax references):
// the best split, the decision and the per-reference flags (low 32 bits: goes
// left / stays in the leaf; high 32 bits: goes right). Cells with at most kExactMax references sweep every clipped-box
// bound as a candidate plane, as the reference's event sweep does; larger
// cells evaluate 31 bin boundaries per axis from start / end histograms and
// the two faces of the cell (where boxes lying in a face can be split off
// into a flat cell, as the reference's planar events allow).
__global__ void __launch_bounds__(kLevelThreads) k_level(const Cell* __restrict__ cells, const uint32_t* __restrict__ list,
                                                         const uint32_t* __restrict__ refs,
                                                         const float* __restrict__ verts,
                                                         const float* __restrict__ tri_box, bool last_level,
                                                         Decision* __restrict__ dec, uint64_t* __restrict__ flags) {
    __shared__ uint32_t starts[3][kBins], ends[3][kBins];
    __shared__ uint32_t face_lo[3], face_hi[3];   // boxes lying in a face of the cell
    __shared__ float box_lo[kExactMax][3], box_hi[kExactMax][3];
    __shared__ uint32_t kept;
    __shared__ float r_cost[kLevelThreads], r_pos[kLevelThreads];
    __shared__ int r_axis[kLevelThreads], r_pl[kLevelThreads];
    __shared__ uint32_t r_nl[kLevelThreads], r_nr[kLevelThreads];
    __shared__ Decision d;
    const uint32_t ci = list[blockIdx.x];
    const Cell c = cells[ci];
    const int tid = threadIdx.x;
    const bool exact = c.count <= kExactMax;
    for (int k = tid; k < 3 * kBins; k += kLevelThreads) {
        starts[k / kBins][k % kBins] = 0;
        ends[k / kBins][k % kBins] = 0;
    }
    if (tid < 3) {
        face_lo[tid] = 0;
        face_hi[tid] = 0;
    }
    if (tid == 0) kept = 0;
    __syncthreads();
    float scale[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float ext = c.hi[a] - c.lo[a];
        scale[a] = ext > 0.f ? static_cast<float>(kBins) / ext : 0.f;
    }
    for (uint32_t i = tid; i < c.count; i += kLevelThreads) {
        float lo[3], hi[3];
        if (!clip_to(verts, tri_box, refs[c.begin + i], c, lo, hi)) continue;
        const uint32_t slot = atomicAdd(&kept, 1u);
        if (exact) {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                box_lo[slot][a] = lo[a];
                box_hi[slot][a] = hi[a];
            }
            continue;
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            if (scale[a] == 0.f) continue;
            atomicAdd(&starts[a][bin_of(lo[a], c.lo[a], scale[a])], 1u);
            atomicAdd(&ends[a][bin_of(hi[a], c.lo[a], scale[a])], 1u);
            if (lo[a] == hi[a] && lo[a] == c.lo[a]) atomicAdd(&face_lo[a], 1u);
            if (lo[a] == hi[a] && hi[a] == c.hi[a]) atomicAdd(&face_hi[a], 1u);
        }
    }
    __syncthreads();
    const uint32_t n = kept;
    const float sa = surface(c.lo, c.hi);
    float bc = 3.4e38f, bp = 0.f;
    int ba = 3, bpl = 0;
    uint32_t bnl = 0, bnr = 0;
    if (n > 3 && sa > 0.f) {
        if (exact) {
            // candidate t: axis t / (2n), bound (t % (2n)) / 2, lower or upper
            for (uint32_t t = tid; t < 6 * n; t += kLevelThreads) {
                const int a = static_cast<int>(t / (2 * n));
                const uint32_t j = (t % (2 * n)) >> 1;
                const float pos = (t & 1u) ? box_hi[j][a] : box_lo[j][a];
                if (!(pos >= c.lo[a] && pos <= c.hi[a])) continue;
                uint32_t nl = 0, nr = 0, np = 0;
                for (uint32_t q = 0; q < n; ++q) {
                    const float lo = box_lo[q][a], hi = box_hi[q][a];
                    nl += lo < pos ? 1u : 0u;
                    nr += hi > pos ? 1u : 0u;
                    np += (lo == pos && hi == pos) ? 1u : 0u;
                }
                consider(c, sa, n, a, pos, nl, nr, np, bc, ba, bp, bpl, bnl, bnr);
            }
        } else if (tid < 3 * (kBins - 1)) {
            // the boundary between bins k - 1 and k
            const int a = tid / (kBins - 1), k = tid % (kBins - 1) + 1;
            if (scale[a] > 0.f) {
                uint32_t nl = 0, nr = 0;
                for (int b = 0; b < k; ++b) nl += starts[a][b];
                for (int b = k; b < kBins; ++b) nr += ends[a][b];
                const float pos = c.lo[a] + (c.hi[a] - c.lo[a]) * (static_cast<float>(k) / kBins);
                if (pos > c.lo[a] && pos < c.hi[a]) consider(c, sa, n, a, pos, nl, nr, 0, bc, ba, bp, bpl, bnl, bnr);
            }
        } else if (tid < 3 * (kBins - 1) + 6) {
            // a face: the boxes lying in it against everything else
            const int f = tid - 3 * (kBins - 1), a = f >> 1;
            const bool low = (f & 1) == 0;
            const uint32_t np = low ? face_lo[a] : face_hi[a];
            if (scale[a] > 0.f && np > 0) {
                if (low) consider(c, sa, n, a, c.lo[a], 0, n - np, np, bc, ba, bp, bpl, bnl, bnr);
                else consider(c, sa, n, a, c.hi[a], n - np, 0, np, bc, ba, bp, bpl, bnl, bnr);
            }
        }
    }
    r_cost[tid] = bc;
    r_axis[tid] = ba;
    r_pos[tid] = bp;
    r_pl[tid] = bpl;
    r_nl[tid] = bnl;
    r_nr[tid] = bnr;
    __syncthreads();
    for (int s = kLevelThreads / 2; s > 0; s >>= 1) {
        if (tid < s && better(r_cost[tid + s], r_axis[tid + s], r_pos[tid + s], r_pl[tid + s], r_cost[tid], r_axis[tid],
                              r_pos[tid], r_pl[tid])) {
            r_cost[tid] = r_cost[tid + s];
            r_axis[tid] = r_axis[tid + s];
            r_pos[tid] = r_pos[tid + s];
            r_pl[tid] = r_pl[tid + s];
            r_nl[tid] = r_nl[tid + s];
            r_nr[tid] = r_nr[tid + s];
        }
        __syncthreads();
    }
    if (tid == 0) {
        Decision r{0, 0, 0.f, n, 1};
        if (n > 3 && c.depth < kMaxBuildDepth && !last_level && r_axis[0] < 3) {
            // the termination test of lib/kdtree.cpp:151-159: a leaf when
            // intersecting everything costs less than the best split (both
            // sides are non-empty, so its empty-side factor is 1)
            if (!(kCostIntersection * static_cast<float>(n) < r_cost[0])) {
                r.split = 1;
                r.axis = r_axis[0];
                r.pos = r_pos[0];
                r.planar_left = r_pl[0];
            }
        }
        d = r;
        dec[ci] = r;
    }
    __syncthreads();
    for (uint32_t i = tid; i < c.count; i += kLevelThreads) {
        float lo[3], hi[3];
        uint64_t f = 0;
        if (clip_to(verts, tri_box, refs[c.begin + i], c, lo, hi)) {
            if (!d.split) {
                f = 1;
            } else {
                const bool pl = d.planar_left != 0;
                const bool l = goes_left(lo[d.axis], hi[d.axis], d.pos, pl);
                const bool r = goes_right(lo[d.axis], hi[d.axis], d.pos, pl);
                f = (l ? 1ull : 0ull) | (r ? (1ull << 32) : 0ull);
            }
        }
        flags[c.begin + i] = f;
    }
}

// Number of a[0..n) below x (lower bound) and not above x (upper bound) in
// an ascending array.
__device__ __forceinline__ uint32_t count_below(const float* a, uint32_t n, float x) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t m = (lo + hi) >> 1;
        if (a[m] < x) lo = m + 1;
        else hi = m;
    }
    return lo;
}
__device__ __forceinline__ uint32_t count_not_above(const float* a, uint32_t n, float x) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t m = (lo + hi) >> 1;
        if (a[m] <= x) lo = m + 1;
        else hi = m;
    }
    return lo;
}

// Ascending bitonic sort of three shared arrays of length len (a power of
// two) at once, by all threads of the block.
__device__ void bitonic_sort3(float* a, float* b, float* c, uint32_t len) {
    for (uint32_t k = 2; k <= len; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < len; i += blockDim.x) {
                const uint32_t ixj = i ^ j;
                if (ixj > i) {
                    const bool up = (i & k) == 0;
                    float x = a[i], y = a[ixj];
                    if ((x > y) == up) { a[i] = y; a[ixj] = x; }
                    x = b[i]; y = b[ixj];
                    if ((x > y) == up) { b[i] = y; b[ixj] = x; }
                    x = c[i]; y = c[ixj];
                    if ((x > y) == up) { c[i] = y; c[ixj] = x; }
                }
            }
            __syncthreads();
        }
    }
}

// One block per listed cell of kExactMax + 1 .. kMidMax references: the exact
// sweep of k_level (every clipped-box bound is a candidate, with the same
// counts, choice and termination test), but each axis sorts its kept boxes'
// lower bounds, upper bounds and flat positions in shared memory and counts by
// binary search, O(n log^2 n) instead of O(n^2). The clipped boxes go through
// `boxes` (6 floats per reference, an empty box for one that misses the cell).
__global__ void __launch_bounds__(kMidThreads) k_level_mid(const Cell* __restrict__ cells,
                                                           const uint32_t* __restrict__ list,
                                                           const uint32_t* __restrict__ refs,
                                                           const float* __restrict__ verts,
                                                           const float* __restrict__ tri_box, bool last_level,
                                                           Decision* __restrict__ dec, uint64_t* __restrict__ flags,
                                                           float* __restrict__ boxes) {
    extern __shared__ float mid_smem[];
    float* s_lo = mid_smem;
    float* s_hi = s_lo + kMidMax;
    float* s_pl = s_hi + kMidMax;
    float* r_cost = s_pl + kMidMax;
    float* r_pos = r_cost + kMidThreads;
    int* r_axis = reinterpret_cast<int*>(r_pos + kMidThreads);
    int* r_pl = r_axis + kMidThreads;
    uint32_t* r_nl = reinterpret_cast<uint32_t*>(r_pl + kMidThreads);
    uint32_t* r_nr = r_nl + kMidThreads;
    __shared__ uint32_t kept, n_axis, n_pl;
    __shared__ Decision d;
    const uint32_t ci = list[blockIdx.x];
    const Cell c = cells[ci];
    const int tid = threadIdx.x;
    if (tid == 0) kept = 0;
    __syncthreads();
    for (uint32_t i = tid; i < c.count; i += kMidThreads) {
        float lo[3], hi[3];
        float* bx = boxes + 6 * size_t(c.begin + i);
        if (clip_to(verts, tri_box, refs[c.begin + i], c, lo, hi)) {
            atomicAdd(&kept, 1u);
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                bx[a] = lo[a];
                bx[3 + a] = hi[a];
            }
        } else {
            bx[0] = INFINITY;   // lower above upper: misses the cell
            bx[3] = -INFINITY;
        }
    }
    __syncthreads();
    const uint32_t n = kept;
    const float sa = surface(c.lo, c.hi);
    float bc = 3.4e38f, bp = 0.f;
    int ba = 3, bpl = 0;
    uint32_t bnl = 0, bnr = 0;
    if (n > 3 && sa > 0.f) {
        uint32_t len = 1;
        while (len < n) len <<= 1;   // n <= c.count <= kMidMax
        for (int a = 0; a < 3; ++a) {
            if (tid == 0) {
                n_axis = 0;
                n_pl = 0;
            }
            __syncthreads();
            for (uint32_t i = tid; i < c.count; i += kMidThreads) {
                const float* bx = boxes + 6 * size_t(c.begin + i);
                if (!(bx[0] <= bx[3])) continue;
                const float lo = bx[a], hi = bx[3 + a];
                const uint32_t j = atomicAdd(&n_axis, 1u);
                s_lo[j] = lo;
                s_hi[j] = hi;
                if (lo == hi) s_pl[atomicAdd(&n_pl, 1u)] = lo;
            }
            __syncthreads();
            // the boxes that were written: the same as the kept ones whenever
            // clipping gives lo <= hi on axis 0 (na <= n <= len in any case)
            const uint32_t na = n_axis;
            const uint32_t npl = n_pl;
            for (uint32_t i = na + tid; i < len; i += kMidThreads) {
                s_lo[i] = INFINITY;
                s_hi[i] = INFINITY;
            }
            for (uint32_t i = npl + tid; i < len; i += kMidThreads) s_pl[i] = INFINITY;
            __syncthreads();
            bitonic_sort3(s_lo, s_hi, s_pl, len);
            for (uint32_t t = tid; t < 2 * na; t += kMidThreads) {
                const float pos = t < na ? s_lo[t] : s_hi[t - na];
                if (!(pos >= c.lo[a] && pos <= c.hi[a])) continue;
                const uint32_t nl = count_below(s_lo, na, pos);
                const uint32_t nr = na - count_not_above(s_hi, na, pos);
                const uint32_t np = count_not_above(s_pl, npl, pos) - count_below(s_pl, npl, pos);
                consider(c, sa, na, a, pos, nl, nr, np, bc, ba, bp, bpl, bnl, bnr);
            }
            __syncthreads();   // the next axis refills the arrays
        }
    }
    r_cost[tid] = bc;
    r_axis[tid] = ba;
    r_pos[tid] = bp;
    r_pl[tid] = bpl;
    r_nl[tid] = bnl;
    r_nr[tid] = bnr;
    __syncthreads();
    for (int h = kMidThreads / 2; h > 0; h >>= 1) {
        if (tid < h && better(r_cost[tid + h], r_axis[tid + h], r_pos[tid + h], r_pl[tid + h], r_cost[tid], r_axis[tid],
                              r_pos[tid], r_pl[tid])) {
            r_cost[tid] = r_cost[tid + h];
            r_axis[tid] = r_axis[tid + h];
            r_pos[tid] = r_pos[tid + h];
            r_pl[tid] = r_pl[tid + h];
            r_nl[tid] = r_nl[tid + h];
            r_nr[tid] = r_nr[tid + h];
        }
        __syncthreads();
    }
    if (tid == 0) {
        Decision r{0, 0, 0.f, n, 1};
        if (n > 3 && c.depth < kMaxBuildDepth && !last_level && r_axis[0] < 3) {
            if (!(kCostIntersection * static_cast<float>(n) < r_cost[0])) {   // the termination test of k_level
                r.split = 1;
                r.axis = r_axis[0];
                r.pos = r_pos[0];
                r.planar_left = r_pl[0];
            }
        }
        d = r;
        dec[ci] = r;
    }
    __syncthreads();
    for (uint32_t i = tid; i < c.count; i += kMidThreads) {
        const float* bx = boxes + 6 * size_t(c.begin + i);
        uint64_t f = 0;
        if (bx[0] <= bx[3]) {
            if (!d.split) {
                f = 1;
            } else {
                const bool pl = d.planar_left != 0;
                const bool gl = goes_left(bx[d.axis], bx[3 + d.axis], d.pos, pl);
                const bool gr = goes_right(bx[d.axis], bx[3 + d.axis], d.pos, pl);
                f = (gl ? 1ull : 0ull) | (gr ? (1ull << 32) : 0ull);
            }
        }
        flags[c.begin + i] = f;
    }
}
constexpr size_t kMidSmem = sizeof(float) * 3 * kMidMax + sizeof(float) * 6 * kMidThreads;

// One warp per listed cell of at most kSmallMax references (one reference per
// lane): the same clipping, exact candidate sweep, choice and termination test
// as k_level, without its block-wide histograms and reductions. Deep levels
// hold hundreds of thousands of such cells.
__global__ void __launch_bounds__(32 * kSmallWarps) k_level_small(const Cell* __restrict__ cells,
                                                                  const uint32_t* __restrict__ list, uint32_t n_list,
                                                                  const uint32_t* __restrict__ refs,
                                                                  const float* __restrict__ verts,
                                                                  const float* __restrict__ tri_box, bool last_level,
                                                                  Decision* __restrict__ dec,
                                                                  uint64_t* __restrict__ flags) {
    __shared__ float box_lo[kSmallWarps][kSmallMax][3], box_hi[kSmallWarps][kSmallMax][3];
    const int warp = threadIdx.x >> 5;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t k = blockIdx.x * kSmallWarps + static_cast<uint32_t>(warp);
    if (k >= n_list) return;   // the whole warp
    const uint32_t ci = list[k];
    const Cell c = cells[ci];
    float lo[3] = {0.f, 0.f, 0.f}, hi[3] = {0.f, 0.f, 0.f};
    const bool mine = lane < c.count;
    const bool kept = mine && clip_to(verts, tri_box, refs[c.begin + lane], c, lo, hi);
    const unsigned km = __ballot_sync(0xFFFFFFFFu, kept);
    const uint32_t n = static_cast<uint32_t>(__popc(km));
    if (kept) {
        const uint32_t slot = static_cast<uint32_t>(__popc(km & ((1u << lane) - 1u)));
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            box_lo[warp][slot][a] = lo[a];
            box_hi[warp][slot][a] = hi[a];
        }
    }
    __syncwarp();
    const float sa = surface(c.lo, c.hi);
    float bc = 3.4e38f, bp = 0.f;
    int ba = 3, bpl = 0;
    uint32_t bnl = 0, bnr = 0;
    if (n > 3 && sa > 0.f) {
        for (uint32_t t = lane; t < 6 * n; t += 32) {
            const int a = static_cast<int>(t / (2 * n));
            const uint32_t j = (t % (2 * n)) >> 1;
            const float pos = (t & 1u) ? box_hi[warp][j][a] : box_lo[warp][j][a];
            if (!(pos >= c.lo[a] && pos <= c.hi[a])) continue;
            uint32_t nl = 0, nr = 0, np = 0;
            for (uint32_t q = 0; q < n; ++q) {
                const float blo = box_lo[warp][q][a], bhi = box_hi[warp][q][a];
                nl += blo < pos ? 1u : 0u;
                nr += bhi > pos ? 1u : 0u;
                np += (blo == pos && bhi == pos) ? 1u : 0u;
            }
            consider(c, sa, n, a, pos, nl, nr, np, bc, ba, bp, bpl, bnl, bnr);
        }
    }
    // better() is a total order, so the warp's best does not depend on which
    // lane found which candidate
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const float oc = __shfl_down_sync(0xFFFFFFFFu, bc, off);
        const int oa = __shfl_down_sync(0xFFFFFFFFu, ba, off);
        const float op = __shfl_down_sync(0xFFFFFFFFu, bp, off);
        const int opl = __shfl_down_sync(0xFFFFFFFFu, bpl, off);
        const uint32_t onl = __shfl_down_sync(0xFFFFFFFFu, bnl, off);
        const uint32_t onr = __shfl_down_sync(0xFFFFFFFFu, bnr, off);
        if (better(oc, oa, op, opl, bc, ba, bp, bpl)) {
            bc = oc;
            ba = oa;
            bp = op;
            bpl = opl;
            bnl = onl;
            bnr = onr;
        }
    }
    Decision r{0, 0, 0.f, n, 1};
    if (lane == 0 && n > 3 && c.depth < kMaxBuildDepth && !last_level && ba < 3) {
        if (!(kCostIntersection * static_cast<float>(n) < bc)) {   // the termination test of k_level
            r.split = 1;
            r.axis = ba;
            r.pos = bp;
            r.planar_left = bpl;
        }
    }
    r.split = __shfl_sync(0xFFFFFFFFu, r.split, 0);
    r.axis = __shfl_sync(0xFFFFFFFFu, r.axis, 0);
    r.pos = __shfl_sync(0xFFFFFFFFu, r.pos, 0);
    r.planar_left = __shfl_sync(0xFFFFFFFFu, r.planar_left, 0);
    if (lane == 0) dec[ci] = r;
    if (mine) {
        uint64_t f = 0;
        if (kept) {
            if (!r.split) {
                f = 1;
            } else {
                const bool pl = r.planar_left != 0;
                const bool gl = goes_left(lo[r.axis], hi[r.axis], r.pos, pl);
                const bool gr = goes_right(lo[r.axis], hi[r.axis], r.pos, pl);
                f = (gl ? 1ull : 0ull) | (gr ? (1ull << 32) : 0ull);
            }
        }
        flags[c.begin + lane] = f;
    }
}

// ------------------------------------------------------------- scans
// Exclusive scan of n values into out[0..n] (out[n] = total), in place safe.
template <class T>
__global__ void __launch_bounds__(kScanThreads) k_scan_block(const T* __restrict__ in, uint32_t n, T* __restrict__ out,
                                                             T* __restrict__ block_sums) {
    __shared__ T s[kScanThreads];
    const uint32_t base = blockIdx.x * kScanBlock + threadIdx.x * kScanItems;
    T v[kScanItems];
    T local = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < n ? in[base + k] : T(0);
        local += v[k];
    }
    s[threadIdx.x] = local;
    __syncthreads();
    for (int off = 1; off < kScanThreads; off <<= 1) {
        const T add = threadIdx.x >= static_cast<unsigned>(off) ? s[threadIdx.x - off] : T(0);
        __syncthreads();
        s[threadIdx.x] += add;
        __syncthreads();
    }
    T run = s[threadIdx.x] - local;   // exclusive prefix of this thread
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == kScanThreads - 1) block_sums[blockIdx.x] = s[threadIdx.x];
}

template <class T>
__global__ void k_scan_add(T* __restrict__ out, uint32_t n, const T* __restrict__ block_offsets) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += block_offsets[i / kScanBlock];
}

template <class T>
__global__ void k_scan_total(T* __restrict__ out, uint32_t n, const T* __restrict__ in) {
    // out[n] = out[n - 1] + in[n - 1]
    out[n] = n ? out[n - 1] + in[n - 1] : T(0);
}

// Device buffers of the build, by slot, kept for the whole build and grown
// (by at least half) only when a level needs more: levels reuse them instead
// of allocating and freeing their own. Growing frees the old buffer, which
// waits for the work queued on it.
struct Arena {
    struct Slot {
        void* p = nullptr;
        size_t bytes = 0;
    };
    std::vector<Slot> slots;
    ~Arena() {
        for (Slot& s : slots)
            if (s.p) cudaFree(s.p);
    }
    template <class T> cudaError_t get(size_t id, T** out, size_t count) {
        *out = nullptr;
        if (slots.size() <= id) slots.resize(id + 1);
        Slot& s = slots[id];
        const size_t need = std::max<size_t>(count, 1) * sizeof(T);
        if (s.bytes < need) {
            const size_t cap = std::max(need, s.bytes + s.bytes / 2);
            if (s.p) cudaFree(s.p);
            s.p = nullptr;
            s.bytes = 0;
            const cudaError_t e = cudaMalloc(&s.p, cap);
            if (e != cudaSuccess) {
                s.p = nullptr;
                return e;
            }
            s.bytes = cap;
        }
        *out = static_cast<T*>(s.p);
        return cudaSuccess;
    }
};

// Arena slots. A scan at recursion depth k uses kSlotScan + 2k and + 2k + 1.
enum : size_t {
    kSlotVerts, kSlotBoxes, kSlotCells0, kSlotCells1, kSlotRefs0, kSlotRefs1, kSlotRefCell0, kSlotRefCell1,
    kSlotSmall0, kSlotSmall1, kSlotLarge0, kSlotLarge1, kSlotMid0, kSlotMid1, kSlotBoxes6, kSlotDec, kSlotFlags, kSlotFscan, kSlotNChild, kSlotNNext,
    kSlotNLeaf, kSlotChildBase, kSlotNextBase, kSlotLeafBase, kSlotLeafPool, kSlotLevelNodes, kSlotLists, kSlotScan
};

// out has n + 1 elements; in and out may not alias.
template <class T>
cudaError_t scan_exclusive(const T* in, uint32_t n, T* out, cudaStream_t st, Arena& arena, size_t slot = kSlotScan) {
    if (n == 0) {
        k_scan_total<T><<<1, 1, 0, st>>>(out, 0, in);
        return cudaGetLastError();
    }
    const uint32_t blocks = (n + kScanBlock - 1) / kScanBlock;
    T *sums = nullptr, *offs = nullptr;
    cudaError_t e = arena.get(slot, &sums, blocks);
    if (e == cudaSuccess) e = arena.get(slot + 1, &offs, size_t(blocks) + 1);
    if (e != cudaSuccess) return e;
    k_scan_block<T><<<blocks, kScanThreads, 0, st>>>(in, n, out, sums);
    if (blocks > 1) {
        e = scan_exclusive<T>(sums, blocks, offs, st, arena, slot + 2);
        if (e != cudaSuccess) return e;
        k_scan_add<T><<<(n + 255) / 256, 256, 0, st>>>(out, n, offs);
    }
    k_scan_total<T><<<1, 1, 0, st>>>(out, n, in);
    return cudaGetLastError();
}

// ------------------------------------------------------------- per level
// Per cell: how many children, next-level references and leaf references.
__global__ void k_counts(const Cell* __restrict__ cells, const Decision* __restrict__ dec,
                         const uint64_t* __restrict__ fscan, uint32_t n, uint32_t* __restrict__ n_child,
                         uint32_t* __restrict__ n_next, uint32_t* __restrict__ n_leaf) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Cell c = cells[i];
    const uint64_t a = fscan[c.begin], b = fscan[c.begin + c.count];
    const uint32_t nl = static_cast<uint32_t>(b) - static_cast<uint32_t>(a);
    const uint32_t nr = static_cast<uint32_t>(b >> 32) - static_cast<uint32_t>(a >> 32);
    if (dec[i].split) {
        n_child[i] = (nl ? 1u : 0u) + (nr ? 1u : 0u);
        n_next[i] = nl + nr;
        n_leaf[i] = 0;
    } else {
        n_child[i] = 0;
        n_next[i] = 0;
        n_leaf[i] = nl;
    }
}

// Reserves n slots of *counter for this lane: one atomicAdd per warp.
__device__ __forceinline__ uint32_t warp_reserve(uint32_t* counter, uint32_t n) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t incl = n;
#pragma unroll
    for (int k = 1; k < 32; k <<= 1) {
        const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, k);
        if (lane >= static_cast<uint32_t>(k)) incl += v;
    }
    uint32_t base = 0;
    if (lane == 31 && incl) base = atomicAdd(counter, incl);
    base = __shfl_sync(0xFFFFFFFFu, base, 31);
    return base + incl - n;
}

// The next level's cells and BFS records of this level's nodes; the children
// are also listed by size for the next level's three kernels: lists[0] counts
// and small_list holds cells of at most kSmallMax references, lists[2] and
// mid_list those of kExactMax + 1 .. kMidMax, lists[1] and large_list the
// others.
__global__ void k_children(const Cell* __restrict__ cells, const Decision* __restrict__ dec,
                           const uint64_t* __restrict__ fscan, uint32_t n, const uint32_t* __restrict__ child_base,
                           const uint32_t* __restrict__ next_base, const uint32_t* __restrict__ leaf_base,
                           uint32_t leaf_offset, int32_t next_level_offset, Cell* __restrict__ next_cells,
                           BfsNode* __restrict__ out, uint32_t* __restrict__ lists, uint32_t* __restrict__ small_list,
                           uint32_t* __restrict__ large_list, uint32_t* __restrict__ mid_list) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    // every lane takes part in the list appends; lanes past n add nothing
    uint32_t child[2] = {0, 0}, count[2] = {0, 0};
    uint32_t n_children = 0;
    if (i < n) {
    const Cell c = cells[i];
    const Decision d = dec[i];
    const uint64_t a = fscan[c.begin], b = fscan[c.begin + c.count];
    const uint32_t nl = static_cast<uint32_t>(b) - static_cast<uint32_t>(a);
    const uint32_t nr = static_cast<uint32_t>(b >> 32) - static_cast<uint32_t>(a >> 32);
    BfsNode r{d.split, d.axis, d.pos, -1, -1, 0, 0};
    if (d.split) {
        uint32_t slot = child_base[i];
        const uint32_t child_depth = c.depth + ((nl && nr) ? 1u : 0u);
        if (nl) {
            Cell l = c;
            l.hi[d.axis] = d.pos;
            l.begin = next_base[i];
            l.count = nl;
            l.depth = child_depth;
            next_cells[slot] = l;
            r.left = next_level_offset + static_cast<int32_t>(slot);
            child[n_children] = slot;
            count[n_children++] = nl;
            ++slot;
        }
        if (nr) {
            Cell rr = c;
            rr.lo[d.axis] = d.pos;
            rr.begin = next_base[i] + nl;
            rr.count = nr;
            rr.depth = child_depth;
            next_cells[slot] = rr;
            r.right = next_level_offset + static_cast<int32_t>(slot);
            child[n_children] = slot;
            count[n_children++] = nr;
        }
    } else {
        r.leaf_begin = leaf_offset + leaf_base[i];
        r.leaf_count = nl;
    }
    out[i] = r;
    }
    uint32_t n_small = 0, n_mid = 0;
    for (uint32_t k = 0; k < n_children; ++k) {
        n_small += count[k] <= kSmallMax ? 1u : 0u;
        n_mid += (count[k] > kExactMax && count[k] <= kMidMax) ? 1u : 0u;
    }
    uint32_t small_at = warp_reserve(lists, n_small);
    uint32_t large_at = warp_reserve(lists + 1, n_children - n_small - n_mid);
    uint32_t mid_at = warp_reserve(lists + 2, n_mid);
    for (uint32_t k = 0; k < n_children; ++k) {
        if (count[k] <= kSmallMax) small_list[small_at++] = child[k];
        else if (count[k] > kExactMax && count[k] <= kMidMax) mid_list[mid_at++] = child[k];
        else large_list[large_at++] = child[k];
    }
}

__global__ void k_scatter(const Cell* __restrict__ cells, const Decision* __restrict__ dec,
                          const uint32_t* __restrict__ refs, const uint32_t* __restrict__ ref_cell,
                          const uint64_t* __restrict__ flags, const uint64_t* __restrict__ fscan, uint32_t n_refs,
                          const uint32_t* __restrict__ child_base, const uint32_t* __restrict__ next_base,
                          const uint32_t* __restrict__ leaf_base, uint32_t* __restrict__ next_refs,
                          uint32_t* __restrict__ next_ref_cell, uint32_t* __restrict__ leaf_pool,
                          uint32_t leaf_offset) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_refs) return;
    const uint64_t f = flags[i];
    if (!f) return;
    const uint32_t ci = ref_cell[i];
    const Cell c = cells[ci];
    const uint64_t a = fscan[c.begin], s = fscan[i];
    const uint32_t t = refs[i];
    const uint32_t rank_l = static_cast<uint32_t>(s) - static_cast<uint32_t>(a);
    if (!dec[ci].split) {
        leaf_pool[leaf_offset + leaf_base[ci] + rank_l] = t;
        return;
    }
    const uint64_t b = fscan[c.begin + c.count];
    const uint32_t nl = static_cast<uint32_t>(b) - static_cast<uint32_t>(a);
    if (static_cast<uint32_t>(f)) {
        const uint32_t p = next_base[ci] + rank_l;
        next_refs[p] = t;
        next_ref_cell[p] = child_base[ci];
    }
    if (f >> 32) {
        const uint32_t rank_r = static_cast<uint32_t>(s >> 32) - static_cast<uint32_t>(a >> 32);
        const uint32_t p = next_base[ci] + nl + rank_r;
        next_refs[p] = t;
        next_ref_cell[p] = child_base[ci] + (nl ? 1u : 0u);
    }
}

__global__ void k_iota(uint32_t* __restrict__ a, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = i;
}

inline uint32_t float_bits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

// FlatNode words (lib/kdtree.h:62-154) of the breadth-first tree, depth
// first with the left child adjacent; empty children are dropped and a node
// left with one child is replaced by it, as KDTree's builder does.
//
// Every kept node's subtree occupies a known number of words (one per inner
// node, count / 2 + 1 per leaf), so its position follows from its parent's:
// the left child right after the parent, the right child after the whole
// left subtree. Subtrees are therefore written independently, on all host
// threads, into a vector sized once.
int flatten(const std::vector<BfsNode>& bfs, const std::vector<uint32_t>& pool, std::vector<uint64_t>& words,
            uint32_t& height) {
    const size_t n = bfs.size();
    if (n == 0) return TURNER_ERR_INVALID_ARG;
    std::vector<int32_t> eff(n, -1);   // the node that stands for i (-1: empty)
    std::vector<uint64_t> size(n, 0);  // words of the subtree of a kept node
    // children come after their parents in breadth-first order
    for (size_t k = n; k-- > 0;) {
        const BfsNode& b = bfs[k];
        if (!b.split) {
            if (b.leaf_count) {
                eff[k] = static_cast<int32_t>(k);
                size[k] = b.leaf_count / 2 + 1;
            }
            continue;
        }
        const int32_t l = b.left >= 0 ? eff[b.left] : -1, r = b.right >= 0 ? eff[b.right] : -1;
        if (l >= 0 && r >= 0) {
            eff[k] = static_cast<int32_t>(k);
            size[k] = 1 + size[l] + size[r];
        } else {
            eff[k] = l >= 0 ? l : r;
        }
    }
    if (eff[0] < 0) return TURNER_ERR_INVALID_ARG;
    const uint64_t total = size[eff[0]];
    if (total >= TURNER_MISS) return TURNER_ERR_TOO_LARGE;
    words.assign(total, 0);
    constexpr uint32_t kNone = 0xFFFFFFFFu >> 2;
    struct Task {
        int32_t node;
        uint32_t pos;     // index of the subtree's first word
        uint32_t level;   // depth of the subtree's root
    };
    auto inner_word = [&](const BfsNode& b, uint32_t right) {
        return static_cast<uint64_t>(float_bits(b.pos)) << 32 | static_cast<uint32_t>(right << 2 | static_cast<uint32_t>(b.axis));
    };
    // writes a subtree depth first; returns its height
    auto emit = [&](Task root) {
        uint32_t h = 0;
        std::vector<Task> st{root};
        while (!st.empty()) {
            const Task t = st.back();
            st.pop_back();
            h = std::max(h, t.level);
            const BfsNode& b = bfs[t.node];
            if (b.split) {
                const int32_t l = eff[b.left], r = eff[b.right];
                const uint32_t rpos = t.pos + 1 + static_cast<uint32_t>(size[l]);
                words[t.pos] = inner_word(b, rpos);
                st.push_back({r, rpos, t.level + 1});
                st.push_back({l, t.pos + 1, t.level + 1});
            } else {
                const uint32_t* ids = pool.data() + b.leaf_begin;
                uint32_t w = t.pos, i = 1;
                for (; i < b.leaf_count; i += 2)
                    words[w++] = static_cast<uint64_t>(ids[i - 1]) << 32 | static_cast<uint64_t>(ids[i] << 2 | 3u);
                words[w] = i - 1 < b.leaf_count
                               ? static_cast<uint64_t>(ids[i - 1]) << 32 | static_cast<uint64_t>(kNone << 2 | 3u)
                               : 0;   // sentinel: ends the run
            }
        }
        return h;
    };
    // split the top of the tree into independent subtrees for the threads
    const unsigned threads = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<Task> tasks{{eff[0], 0, 0}};
    height = 0;
    for (;;) {
        size_t big = tasks.size();
        for (size_t k = 0; k < tasks.size(); ++k) {
            if (!bfs[tasks[k].node].split) continue;
            if (big == tasks.size() || size[tasks[k].node] > size[tasks[big].node]) big = k;
        }
        if (big == tasks.size() || tasks.size() >= 8 * threads || size[tasks[big].node] < (1u << 16)) break;
        const Task t = tasks[big];
        const BfsNode& b = bfs[t.node];
        const int32_t l = eff[b.left], r = eff[b.right];
        const uint32_t rpos = t.pos + 1 + static_cast<uint32_t>(size[l]);
        words[t.pos] = inner_word(b, rpos);
        height = std::max(height, t.level);
        tasks[big] = {l, t.pos + 1, t.level + 1};
        tasks.push_back({r, rpos, t.level + 1});
    }
    std::vector<uint32_t> heights(tasks.size(), 0);
    std::atomic<size_t> next{0};
    auto worker = [&]() {
        for (size_t k; (k = next.fetch_add(1)) < tasks.size();) heights[k] = emit(tasks[k]);
    };
    std::vector<std::thread> pool_threads;
    for (unsigned k = 1; k < std::min<size_t>(threads, tasks.size()); ++k) {
        try {
            pool_threads.emplace_back(worker);
        } catch (const std::system_error&) {
            break;   // fewer threads: the remaining tasks run on the ones there are
        }
    }
    worker();
    for (auto& th : pool_threads) th.join();
    for (uint32_t h : heights) height = std::max(height, h);
    return TURNER_OK;
}

} // namespace

namespace turner {
cudaStream_t ctx_stream(turner_ctx* ctx);
int ctx_device(turner_ctx* ctx);
} // namespace turner

extern "C" {

int turner_kdtree_build_gpu(turner_ctx* ctx, const float* vertices, const float* normals, const float* diffuse,
                            uint32_t n_tris, turner_kdtree** out) {
    if (!ctx || !vertices || !out || n_tris == 0) return TURNER_ERR_INVALID_ARG;
    *out = nullptr;
    if (n_tris >= TURNER_MISS) return TURNER_ERR_TOO_LARGE;
    auto tree = std::unique_ptr<turner_kdtree>(new (std::nothrow) turner_kdtree);
    if (!tree) return TURNER_ERR_OUT_OF_MEMORY;
    try {
        turner::host::make_records(vertices, normals, diffuse, n_tris, tree->tris, tree->box);
    } catch (const std::bad_alloc&) {
        return TURNER_ERR_OUT_OF_MEMORY;
    }
    if (cudaSetDevice(turner::ctx_device(ctx)) != cudaSuccess) return TURNER_ERR_CUDA;
    cudaStream_t st = turner::ctx_stream(ctx);
    Arena arena;   // every device buffer of the build
#define GB_CK(call)                                                                              \
    do {                                                                                         \
        const cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) return e_ == cudaErrorMemoryAllocation ? TURNER_ERR_OUT_OF_MEMORY \
                                                                      : TURNER_ERR_CUDA;         \
    } while (0)
    float *d_v = nullptr, *d_box = nullptr;
    GB_CK(arena.get(kSlotVerts, &d_v, 9 * size_t(n_tris)));
    GB_CK(arena.get(kSlotBoxes, &d_box, 6 * size_t(n_tris)));
    GB_CK(cudaMemcpyAsync(d_v, vertices, sizeof(float) * 9 * size_t(n_tris), cudaMemcpyHostToDevice, st));
    k_tri_boxes<<<(n_tris + 255) / 256, 256, 0, st>>>(d_v, n_tris, d_box);
    GB_CK(cudaGetLastError());

    // level 0: the scene box, every triangle
    Cell root{};
    for (int a = 0; a < 3; ++a) {
        root.lo[a] = tree->box[a];
        root.hi[a] = tree->box[3 + a];
    }
    root.begin = 0;
    root.count = n_tris;
    root.depth = 0;
    uint32_t n_cells = 1, n_refs = n_tris;
    // the root is the only cell of level 0, in the small or the large list
    uint32_t n_small = n_tris <= kSmallMax ? 1u : 0u;
    uint32_t n_mid = (n_tris > kExactMax && n_tris <= kMidMax) ? 1u : 0u;
    uint32_t n_large = 1u - n_small - n_mid;
    Cell* cells = nullptr;
    uint32_t *refs = nullptr, *ref_cell = nullptr, *small_list = nullptr, *large_list = nullptr, *mid_list = nullptr;
    GB_CK(arena.get(kSlotCells0, &cells, 1));
    GB_CK(arena.get(kSlotRefs0, &refs, n_refs));
    GB_CK(arena.get(kSlotRefCell0, &ref_cell, n_refs));
    GB_CK(arena.get(kSlotSmall0, &small_list, 1));
    GB_CK(arena.get(kSlotLarge0, &large_list, 1));
    GB_CK(arena.get(kSlotMid0, &mid_list, 1));
    GB_CK(cudaMemsetAsync(mid_list, 0, sizeof(uint32_t), st));
    GB_CK(cudaFuncSetAttribute(k_level_mid, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kMidSmem)));
    GB_CK(cudaMemcpyAsync(cells, &root, sizeof(Cell), cudaMemcpyHostToDevice, st));
    GB_CK(cudaMemsetAsync(small_list, 0, sizeof(uint32_t), st));
    GB_CK(cudaMemsetAsync(large_list, 0, sizeof(uint32_t), st));
    k_iota<<<(n_refs + 255) / 256, 256, 0, st>>>(refs, n_refs);
    GB_CK(cudaMemsetAsync(ref_cell, 0, sizeof(uint32_t) * n_refs, st));

    std::vector<BfsNode> bfs;
    std::vector<uint32_t> pool;   // leaf references of all levels, in level order
    uint32_t leaf_total = 0;
    // the leaf pool grows in pieces, one per level (host copies)
    // an empty-space cut leaves one child and is dropped when the tree is
    // flattened, so cells count only two-sided splits as depth; the number
    // of levels is bounded separately
    for (uint32_t level = 0; n_cells > 0; ++level) {
        // this level's cells, references and lists are in the slots of its
        // parity; the next level's go to the others
        const size_t nxt = (level + 1) & 1u;
        Decision* dec = nullptr;
        uint64_t *flags = nullptr, *fscan = nullptr;
        uint32_t *n_child = nullptr, *n_next = nullptr, *n_leaf = nullptr, *child_base = nullptr,
                 *next_base = nullptr, *leaf_base = nullptr, *lists = nullptr;
        GB_CK(arena.get(kSlotDec, &dec, n_cells));
        GB_CK(arena.get(kSlotFlags, &flags, n_refs));
        GB_CK(arena.get(kSlotFscan, &fscan, size_t(n_refs) + 1));
        GB_CK(arena.get(kSlotNChild, &n_child, n_cells));
        GB_CK(arena.get(kSlotNNext, &n_next, n_cells));
        GB_CK(arena.get(kSlotNLeaf, &n_leaf, n_cells));
        GB_CK(arena.get(kSlotChildBase, &child_base, size_t(n_cells) + 1));
        GB_CK(arena.get(kSlotNextBase, &next_base, size_t(n_cells) + 1));
        GB_CK(arena.get(kSlotLeafBase, &leaf_base, size_t(n_cells) + 1));
        GB_CK(arena.get(kSlotLists, &lists, 3));
        const bool last = level + 1 >= kMaxLevels;
        if (n_large) {
            k_level<<<n_large, kLevelThreads, 0, st>>>(cells, large_list, refs, d_v, d_box, last, dec, flags);
        }
        if (n_small) {
            k_level_small<<<(n_small + kSmallWarps - 1) / kSmallWarps, 32 * kSmallWarps, 0, st>>>(
                cells, small_list, n_small, refs, d_v, d_box, last, dec, flags);
        }
        if (n_mid) {
            float* boxes6 = nullptr;
            GB_CK(arena.get(kSlotBoxes6, &boxes6, 6 * size_t(n_refs)));
            k_level_mid<<<n_mid, kMidThreads, kMidSmem, st>>>(cells, mid_list, refs, d_v, d_box, last, dec, flags,
                                                              boxes6);
        }
        GB_CK(cudaGetLastError());
        GB_CK(scan_exclusive<uint64_t>(flags, n_refs, fscan, st, arena));
        const unsigned gc = (n_cells + 255) / 256;
        k_counts<<<gc, 256, 0, st>>>(cells, dec, fscan, n_cells, n_child, n_next, n_leaf);
        GB_CK(cudaGetLastError());
        GB_CK(scan_exclusive<uint32_t>(n_child, n_cells, child_base, st, arena));
        GB_CK(scan_exclusive<uint32_t>(n_next, n_cells, next_base, st, arena));
        GB_CK(scan_exclusive<uint32_t>(n_leaf, n_cells, leaf_base, st, arena));
        uint32_t totals[3] = {0, 0, 0};
        GB_CK(cudaMemcpyAsync(&totals[0], child_base + n_cells, 4, cudaMemcpyDeviceToHost, st));
        GB_CK(cudaMemcpyAsync(&totals[1], next_base + n_cells, 4, cudaMemcpyDeviceToHost, st));
        GB_CK(cudaMemcpyAsync(&totals[2], leaf_base + n_cells, 4, cudaMemcpyDeviceToHost, st));
        GB_CK(cudaStreamSynchronize(st));
        const uint32_t next_cells_n = totals[0], next_refs_n = totals[1], leaf_n = totals[2];
        if (uint64_t(bfs.size()) + n_cells + next_cells_n >= (1ull << 31)) return TURNER_ERR_TOO_LARGE;

        Cell* next_cells = nullptr;
        uint32_t *next_refs = nullptr, *next_ref_cell = nullptr, *next_small = nullptr, *next_large = nullptr,
                 *next_mid = nullptr, *leaf_pool = nullptr;
        BfsNode* level_nodes = nullptr;
        GB_CK(arena.get(kSlotCells0 + nxt, &next_cells, next_cells_n));
        GB_CK(arena.get(kSlotRefs0 + nxt, &next_refs, next_refs_n));
        GB_CK(arena.get(kSlotRefCell0 + nxt, &next_ref_cell, next_refs_n));
        GB_CK(arena.get(kSlotSmall0 + nxt, &next_small, next_cells_n));
        GB_CK(arena.get(kSlotLarge0 + nxt, &next_large, next_cells_n));
        GB_CK(arena.get(kSlotMid0 + nxt, &next_mid, next_cells_n));
        GB_CK(arena.get(kSlotLeafPool, &leaf_pool, leaf_n));
        GB_CK(arena.get(kSlotLevelNodes, &level_nodes, n_cells));
        GB_CK(cudaMemsetAsync(lists, 0, 3 * sizeof(uint32_t), st));
        const int32_t next_offset = static_cast<int32_t>(bfs.size() + n_cells);
        k_children<<<gc, 256, 0, st>>>(cells, dec, fscan, n_cells, child_base, next_base, leaf_base, leaf_total,
                                       next_offset, next_cells, level_nodes, lists, next_small, next_large, next_mid);
        if (n_refs) {
            k_scatter<<<(n_refs + 255) / 256, 256, 0, st>>>(cells, dec, refs, ref_cell, flags, fscan, n_refs,
                                                            child_base, next_base, leaf_base, next_refs,
                                                            next_ref_cell, leaf_pool, 0);
        }
        GB_CK(cudaGetLastError());
        const size_t base = bfs.size();
        try {
            bfs.resize(base + n_cells);
            pool.resize(size_t(leaf_total) + leaf_n);
        } catch (const std::bad_alloc&) {
            return TURNER_ERR_OUT_OF_MEMORY;
        }
        uint32_t counts[3] = {0, 0, 0};
        GB_CK(cudaMemcpyAsync(bfs.data() + base, level_nodes, sizeof(BfsNode) * n_cells, cudaMemcpyDeviceToHost, st));
        if (leaf_n)
            GB_CK(cudaMemcpyAsync(pool.data() + leaf_total, leaf_pool, sizeof(uint32_t) * leaf_n,
                                  cudaMemcpyDeviceToHost, st));
        GB_CK(cudaMemcpyAsync(counts, lists, sizeof(counts), cudaMemcpyDeviceToHost, st));
        GB_CK(cudaStreamSynchronize(st));
        leaf_total += leaf_n;
        // the next level becomes current
        cells = next_cells;
        refs = next_refs;
        ref_cell = next_ref_cell;
        small_list = next_small;
        large_list = next_large;
        mid_list = next_mid;
        n_cells = next_cells_n;
        n_refs = next_refs_n;
        n_small = counts[0];
        n_large = counts[1];
        n_mid = counts[2];
        if (n_small + n_large + n_mid != n_cells) return TURNER_ERR_CUDA;
    }
#undef GB_CK
    int status;
    try {
        status = flatten(bfs, pool, tree->nodes, tree->height);
    } catch (const std::bad_alloc&) {
        return TURNER_ERR_OUT_OF_MEMORY;
    }
    if (status != TURNER_OK) return status;
    *out = tree.release();
    return TURNER_OK;
}

} // extern "C"
