// ORACLE — test infrastructure only. A CPU restatement of the Turner path
// tracer's hot path, used by tests/ and by bench.py's CPU-baseline leg as the
// checker. The product (turner_gb300/) never links, loads or calls it.
//
// Parity is pinned: tests/test_oracle_pins.py checks this restatement against
// the reference's own known-answer tests (tests/test_kdtree.cpp,
// tests/test_intersection.cpp, tests/test_raster.cpp, tests/test_effects.cpp)
// and against golden outputs of the reference itself (tests/golden/, written by
// tests/golden/make_golden.py from oracle/_ref, which is compiled from the
// reference's sources by oracle/build_ref.sh).
//
// The structure deliberately follows the reference's so that its timing is a
// fair CPU baseline: 192-byte AoS triangles, a heap-backed std::stack per
// intersector, recursion in trace(), one intersector per image row.
//
// Build: g++ -std=c++17 -O2 -ffp-contract=off -fPIC -shared (no -march).

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <sstream>
#include <iomanip>
#include <stack>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

namespace orc {

constexpr float kFltMax = std::numeric_limits<float>::max();
constexpr float kEps = 0.00001f;                 // lib/types.h:14
constexpr uint32_t kMaxTriangleId = 1u << 30;    // lib/kdtree.h:66 (also the miss id)

// ---------------------------------------------------------------- math
// Vector arithmetic in the reference's operation order (src/geometry.h).
struct V3 {
    float x, y, z;
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(float s, V3 v) { return {s * v.x, s * v.y, s * v.z}; }       // geometry.h:262
inline V3 operator*(V3 v, float s) { return {s * v.x, s * v.y, s * v.z}; }       // geometry.h:227 (s*x)
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }       // geometry.h:270
inline float length(V3 v) { return std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }
// normalize = v / |v| = (1/|v|) * v   (geometry.h:240-243, 301-303)
inline V3 normalize(V3 v) { return (1 / length(v)) * v; }

// aiColor4D-style RGBA radiance (alpha carried as a 4th channel).
struct C4 {
    float r = 0, g = 0, b = 0, a = 0;
};
inline C4 operator+(C4 p, C4 q) { return {p.r + q.r, p.g + q.g, p.b + q.b, p.a + q.a}; }
inline C4 operator*(C4 p, C4 q) { return {p.r * q.r, p.g * q.g, p.b * q.b, p.a * q.a}; }
inline C4 operator*(C4 p, float f) { return {p.r * f, p.g * f, p.b * f, p.a * f}; }
inline C4 operator*(float f, C4 p) { return {f * p.r, f * p.g, f * p.b, f * p.a}; }

// Triangle record in Triangle::serialize order (lib/triangle.h:89-114).
struct Tri {
    V3 vertices[3];
    V3 normals[3];
    float ambient[4], diffuse[4], emissive[4], reflective[4];
    float reflectivity;
    V3 u, v, normal;
    float uv, vv, uu, denom;
};
static_assert(sizeof(Tri) == 48 * sizeof(float), "triangle record is 48 floats");

struct Ray {
    V3 o, d;
};

// ---------------------------------------------------------------- RNG
// xorshift64* (lib/xorshift.h:27-70): float = ldexp(x & (2^24-1), -24).
struct Xorshift {
    uint64_t s;
    uint64_t next_u64() {
        s ^= s >> 12;
        s ^= s << 25;
        s ^= s >> 27;
        return s * 2685821657736338717ULL;
    }
    float next_float() { return std::ldexp(static_cast<float>(next_u64() & 0xFFFFFFull), -24); }
};

inline uint64_t splitmix64(uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

// Branching estimator (-m > 1): child k of a hit draws from its own stream,
// derived from the stream state of the ray that made the hit, so that every
// ray of the tree has a stream that does not depend on traversal order (the
// reference draws them depth-first from one thread-local generator,
// lib/sampling.h:12, which a wavefront cannot reproduce). -m 1 keeps one
// stream per path.
inline uint64_t branch_seed(uint64_t parent_state, uint32_t k) {
    const uint64_t s = splitmix64(parent_state ^ (0xA0761D6478BD642FULL * (uint64_t(k) + 1)));
    return s ? s : 1;
}

// Harness seeding per (pixel, sample): key = pixel_index * spp + sample.
inline void path_seeds(uint64_t seed, uint64_t key, uint64_t& jitter, uint64_t& bounce) {
    uint64_t a = splitmix64(seed ^ key);
    uint64_t b = splitmix64(a ^ 0xD1B54A32D192ED03ULL);
    jitter = a ? a : 1;
    bounce = b ? b : 1;
}

// ---------------------------------------------------------------- scene
struct Scene {
    std::vector<uint64_t> nodes;
    std::vector<Tri> tris;
    V3 box_min, box_max;
};

inline bool node_is_leaf(uint64_t n) { return (n & 3u) == 3u; }                 // kdtree.h:91
inline int node_axis(uint64_t n) { return static_cast<int>(n & 3u); }           // kdtree.h:96
inline float node_split(uint64_t n) {                                            // kdtree.h:101
    uint32_t bits = static_cast<uint32_t>(n >> 32);
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
}
inline uint32_t node_right(uint64_t n) { return static_cast<uint32_t>(n) >> 2; }  // kdtree.h:106
inline uint32_t leaf_first(uint64_t n) { return static_cast<uint32_t>(n >> 32); } // kdtree.h:120
inline bool leaf_has_second(uint64_t n) { return static_cast<uint32_t>(n) != 0xFFFFFFFFu; } // :125
inline uint32_t leaf_second(uint64_t n) { return static_cast<uint32_t>(n) >> 2; } // kdtree.h:130

// intersect_ray_plane + intersect_ray_triangle (lib/intersection.h:40-89).
inline bool intersect_ray_triangle(const Ray& ray, const Tri& tri, float& r, float& s, float& t) {
    float denom = dot(tri.normal, ray.d);
    if (denom == 0.f) {
        r = std::numeric_limits<float>::lowest();
    } else {
        float nom = dot(tri.normal, tri.vertices[0] - ray.o);
        r = nom / denom;
    }
    if (r < 0) return false;
    V3 p_int = ray.o + r * ray.d;
    V3 w = p_int - tri.vertices[0];
    float wv = dot(w, tri.v);
    float wu = dot(w, tri.u);
    s = (tri.uv * wv - tri.vv * wu) / tri.denom;
    if (s < 0) return false;
    t = (tri.uv * wu - tri.uu * wv) / tri.denom;
    if (t < 0 || 1 < s + t) return false;
    return true;
}

// intersect_ray_box (lib/intersection.h:105-128), slab test with fmin/fmax.
inline bool intersect_ray_box(const Ray& ray, V3 pmin, V3 pmax, float& tmin, float& tmax) {
    V3 d_inv{1 / ray.d.x, 1 / ray.d.y, 1 / ray.d.z};
    float tx1 = (pmin.x - ray.o.x) * d_inv.x;
    float tx2 = (pmax.x - ray.o.x) * d_inv.x;
    tmin = std::fmin(tx1, tx2);
    tmax = std::fmax(tx1, tx2);
    float ty1 = (pmin.y - ray.o.y) * d_inv.y;
    float ty2 = (pmax.y - ray.o.y) * d_inv.y;
    tmin = std::fmax(tmin, std::fmin(ty1, ty2));
    tmax = std::fmin(tmax, std::fmax(ty1, ty2));
    float tz1 = (pmin.z - ray.o.z) * d_inv.z;
    float tz2 = (pmax.z - ray.o.z) * d_inv.z;
    tmin = std::fmax(tmin, std::fmin(tz1, tz2));
    tmax = std::fmin(tmax, std::fmax(tz1, tz2));
    return !(tmax < tmin);
}

// KDTreeIntersection (lib/kdtree.cpp:503-607): visits every leaf overlapped by
// the ray's [tenter, texit] interval (no early termination) and keeps the
// first strict minimum. Counters are for the traversal roofline.
struct Intersector {
    const Scene* sc;
    std::stack<std::tuple<const uint64_t*, float, float>> stack_;
    uint64_t node_visits = 0, tri_tests = 0;                // all traversals
    uint64_t shadow_visits = 0, shadow_tests = 0;           // shadow-ray share of them

    explicit Intersector(const Scene& s) : sc(&s) {}

    uint32_t leaf_run(const uint64_t* node, const Ray& ray, float& min_r, float& min_s, float& min_t) {
        min_r = kFltMax;
        uint32_t res = kMaxTriangleId;
        auto test = [&](uint32_t id) {
            ++tri_tests;
            float r, s, t;
            if (intersect_ray_triangle(ray, sc->tris[id], r, s, t) && r < min_r) {
                min_r = r;
                min_s = s;
                min_t = t;
                res = id;
            }
        };
        for (; node_is_leaf(*node); ++node) {
            ++node_visits;
            test(leaf_first(*node));
            if (!leaf_has_second(*node)) break;
            test(leaf_second(*node));
        }
        return res;
    }

    uint32_t intersect(const Ray& ray, float& r, float& a, float& b) {
        // fix_direction (kdtree.cpp:503-511): zero components become EPS
        Ray fixed = ray;
        if (fixed.d.x == 0) fixed.d.x = kEps;
        if (fixed.d.y == 0) fixed.d.y = kEps;
        if (fixed.d.z == 0) fixed.d.z = kEps;

        float tenter, texit;
        if (!intersect_ray_box(fixed, sc->box_min, sc->box_max, tenter, texit)) return kMaxTriangleId;

        const uint64_t* root = sc->nodes.data();
        stack_.emplace(root, tenter, texit);
        V3 d_inv{1 / fixed.d.x, 1 / fixed.d.y, 1 / fixed.d.z};
        const uint64_t* node;
        uint32_t res = kMaxTriangleId;
        r = kFltMax;
        while (!stack_.empty()) {
            std::tie(node, tenter, texit) = stack_.top();
            stack_.pop();
            while (!node_is_leaf(*node)) {
                ++node_visits;
                const int ax = node_axis(*node);
                const float t = (node_split(*node) - fixed.o[ax]) * d_inv[ax];
                const uint64_t* near = node + 1;
                const uint64_t* far = root + node_right(*node);
                if (fixed.d[ax] <= 0) std::swap(near, far);
                if (texit < t) {
                    node = near;
                } else if (t < tenter) {
                    node = far;
                } else {
                    stack_.emplace(far, t, texit);
                    node = near;
                    texit = t;
                }
            }
            float nr, na, nb;
            uint32_t next = leaf_run(node, ray, nr, na, nb);
            if (next < kMaxTriangleId && nr < r) {
                res = next;
                r = nr;
                a = na;
                b = nb;
            }
        }
        return res;
    }
};

// ---------------------------------------------------------------- shading
// Moeller-Hughes from-to rotation (JGT 1999), float arithmetic; the product's
// kernels evaluate the same expression sequence.
inline void from_to_matrix(V3 from, V3 to, float m[9]) {
    const float vx = from.y * to.z - from.z * to.y;
    const float vy = from.z * to.x - from.x * to.z;
    const float vz = from.x * to.y - from.y * to.x;
    const float e = from.x * to.x + from.y * to.y + from.z * to.z;
    const float f = e < 0 ? -e : e;
    if (f > 1.0f - 0.000001f) {
        float ax = from.x > 0 ? from.x : -from.x;
        float ay = from.y > 0 ? from.y : -from.y;
        float az = from.z > 0 ? from.z : -from.z;
        float x[3];
        if (ax < ay) {
            if (ax < az) { x[0] = 1; x[1] = 0; x[2] = 0; }
            else         { x[0] = 0; x[1] = 0; x[2] = 1; }
        } else {
            if (ay < az) { x[0] = 0; x[1] = 1; x[2] = 0; }
            else         { x[0] = 0; x[1] = 0; x[2] = 1; }
        }
        const float u[3] = {x[0] - from.x, x[1] - from.y, x[2] - from.z};
        const float w[3] = {x[0] - to.x, x[1] - to.y, x[2] - to.z};
        const float c1 = 2.0f / (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        const float c2 = 2.0f / (w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        const float c3 = c1 * c2 * (u[0] * w[0] + u[1] * w[1] + u[2] * w[2]);
        for (int i = 0; i < 3; ++i) {
            for (int j = 0; j < 3; ++j) {
                m[3 * i + j] = -c1 * u[i] * u[j] - c2 * w[i] * w[j] + c3 * w[i] * u[j];
            }
            m[3 * i + i] += 1.0f;
        }
    } else {
        const float h = 1.0f / (1.0f + e);
        const float hvx = h * vx;
        const float hvz = h * vz;
        const float hvxy = hvx * vy;
        const float hvxz = hvx * vz;
        const float hvyz = hvz * vy;
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

inline V3 mat_vec(const float m[9], V3 v) {
    return {m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z,
            m[6] * v.x + m[7] * v.y + m[8] * v.z};
}

constexpr float kTwoPi = 2.f * static_cast<float>(M_PI);   // float(2 * pi) as 2.f * M_PI rounds

struct Light {
    V3 position;
    C4 color;
};

struct Conf {
    int max_depth = 3;
    int mc_samples = 1;
    int sampling = 0;   // 0 = uniform hemisphere (reference), 1 = cosine-weighted
    C4 bg{0, 0, 0, 1};
    int renderer = 0;   // 0 path tracer, 1 Whitted raytracer, 2 raycaster
    float shadow_intensity = 0.5f;
    float max_visibility = 2.f;
};

struct Counters {
    uint64_t rays = 0, shadow_rays = 0;
};

// trace() (pathtracer.cpp:14-102). The hemisphere stream is per path.
C4 trace(const Ray& ray, Intersector& ti, const std::vector<Light>& lights, int depth, const Conf& conf,
         Xorshift& uniform, Counters& cnt) {
    if (depth > conf.max_depth) return C4{};
    cnt.rays += 1;

    float dist_to_triangle = 0, s = 0, t = 0;
    uint32_t id = ti.intersect(ray, dist_to_triangle, s, t);
    if (id >= kMaxTriangleId) return conf.bg;

    const V3 p = ray.o + dist_to_triangle * ray.d;
    const Tri& tri = ti.sc->tris[id];
    // Triangle::interpolate_normal (lib/triangle.h:54-56) with r = 1 - s - t
    const float w0 = 1.f - s - t;
    const V3 normal = normalize(w0 * tri.normals[0] + s * tri.normals[1] + t * tri.normals[2]);
    const V3 p2 = p + normal * 0.0001f;

    C4 direct;
    for (const Light& light : lights) {
        const V3 light_dir = normalize(light.position - p);
        const float dist_to_light = length(light.position - p2);
        float dist_to_next = 0, s2, t2;
        cnt.shadow_rays += 1;
        const uint64_t v0 = ti.node_visits, t0 = ti.tri_tests;
        uint32_t sh = ti.intersect(Ray{p2, light_dir}, dist_to_next, s2, t2);
        ti.shadow_visits += ti.node_visits - v0;
        ti.shadow_tests += ti.tri_tests - t0;
        if (sh >= kMaxTriangleId || dist_to_next > dist_to_light) {
            direct = std::max(0.f, dot(light_dir, normal)) * light.color;
        }
    }

    C4 indirect;
    float m[9];
    from_to_matrix(V3{0, 0, 1}, normal, m);
    const uint64_t parent_state = uniform.s;
    for (int run = 0; run < conf.mc_samples; ++run) {
        Xorshift branch{conf.mc_samples > 1 ? branch_seed(parent_state, static_cast<uint32_t>(run)) : 0};
        Xorshift& gen = conf.mc_samples > 1 ? branch : uniform;
        const float u1 = gen.next_float();
        const float u2 = gen.next_float();
        float x, y, z, weight;
        if (conf.sampling == 0) {
            // sampling::hemisphere (lib/sampling.h:20-32): uniform, z = u1
            z = u1;
            const float rr = sqrtf(std::fmax(0.f, 1.f - z * z));
            const float phi = kTwoPi * u2;
            x = rr * cosf(phi);
            y = rr * sinf(phi);
            weight = u1;   // cos(theta); the estimator multiplies by 2 (= 1/pdf * 1/pi)
        } else {
            // cosine-weighted (Malley): z = sqrt(u1), pdf = cos/pi; estimator weight 1/2
            const float rr = sqrtf(u1);
            z = sqrtf(std::fmax(0.f, 1.f - u1));
            const float phi = kTwoPi * u2;
            x = rr * cosf(phi);
            y = rr * sinf(phi);
            weight = 0.5f;
        }
        const V3 dir = mat_vec(m, V3{x, y, z});
        const C4 li = trace(Ray{p2, dir}, ti, lights, depth + 1, conf, gen, cnt);
        indirect = indirect + weight * li;
    }
    if (conf.mc_samples > 0) {
        const float inv_m = static_cast<float>(conf.mc_samples);
        indirect = C4{indirect.r / inv_m, indirect.g / inv_m, indirect.b / inv_m, indirect.a / inv_m};
    }

    const C4 diffuse{tri.diffuse[0], tri.diffuse[1], tri.diffuse[2], tri.diffuse[3]};
    return diffuse * (direct * static_cast<float>(M_1_PI) + indirect * 2.f);
}

// trace() of the Whitted raytracer (raytracer.cpp:5-67): Lambertian direct
// light (lib/lambertian.h:15-19), a mirror bounce when the triangle is
// reflective, and a shadow test that darkens the whole colour by
// shadow_intensity. Every call counts as a ray, also the one past max depth.
C4 trace_whitted(const Ray& ray, Intersector& ti, const Light& light, int depth, const Conf& conf, Counters& cnt) {
    cnt.rays += 1;
    if (depth > conf.max_depth) return C4{};

    float dist_to_triangle = 0, s = 0, t = 0;
    const uint32_t id = ti.intersect(ray, dist_to_triangle, s, t);
    if (id >= kMaxTriangleId) return conf.bg;

    const V3 p = ray.o + dist_to_triangle * ray.d;
    V3 light_dir = normalize(light.position - p);
    const Tri& tri = ti.sc->tris[id];
    const float w0 = 1.f - s - t;
    const V3 normal = normalize(w0 * tri.normals[0] + s * tri.normals[1] + t * tri.normals[2]);
    const C4 diffuse{tri.diffuse[0], tri.diffuse[1], tri.diffuse[2], tri.diffuse[3]};
    const float cos_alpha = std::max(0.f, dot(light_dir, normal));
    const C4 direct = cos_alpha * diffuse * light.color;
    const V3 p2 = p + normal * 0.0001f;

    C4 color = direct;
    if (tri.reflectivity > 0) {
        // reflected direction d - 2 (n.d) n
        const V3 refl = ray.d - (2.f * dot(normal, ray.d)) * normal;
        const C4 reflected = trace_whitted(Ray{p2, refl}, ti, light, depth + 1, conf, cnt);
        const C4 rc{tri.reflective[0], tri.reflective[1], tri.reflective[2], tri.reflective[3]};
        color = (1.f - tri.reflectivity) * direct + tri.reflectivity * rc * reflected;
    }

    light_dir = normalize(light.position - p2);
    const float dist_to_light = length(light.position - p2);
    float dist_to_next = 0;
    cnt.shadow_rays += 1;
    const uint32_t sh = ti.intersect(Ray{p2, light_dir}, dist_to_next, s, t);
    if (sh < kMaxTriangleId && dist_to_next < dist_to_light) {
        const C4 dark = color * conf.shadow_intensity;
        color = C4{color.r - dark.r, color.g - dark.g, color.b - dark.b, color.a - dark.a};
    }
    return color;
}

// trace() of the raycaster (raycaster.cpp:6-24): the diffuse colour, its alpha
// replaced by the fall-off 1 - r / max_visibility clamped to [0, 1]; only
// hits count as rays.
C4 trace_cast(const Ray& ray, Intersector& ti, const Conf& conf, Counters& cnt) {
    float dist_to_triangle = 0, s = 0, t = 0;
    const uint32_t id = ti.intersect(ray, dist_to_triangle, s, t);
    if (id >= kMaxTriangleId) return conf.bg;
    cnt.rays += 1;
    const Tri& tri = ti.sc->tris[id];
    C4 res{tri.diffuse[0], tri.diffuse[1], tri.diffuse[2], tri.diffuse[3]};
    const float a = 1.f - (dist_to_triangle / conf.max_visibility);
    res.a = a < 0.f ? 0.f : (a > 1.f ? 1.f : a);
    return res;
}

// lib/effects.h:15-49
inline float exposure(float light, float value) { return 1 - expf(-light * value); }
inline float gamma_fn(float light, float inverse_gamma) { return powf(light, inverse_gamma); }

} // namespace orc

using namespace orc;

extern "C" {

struct orc_camera {
    float position[3];
    float trafo[9];    // row-major rotation of the camera node
    float delta_x;     // tan(aiCamera::mHorizontalFOV)
    float aspect;      // delta_y = delta_x / aspect (lib/types.h:104)
};

struct orc_params {
    uint32_t width, height, pixel_samples;
    int32_t max_depth;
    int32_t monte_carlo_samples;
    float exposure, inverse_gamma;
    int32_t gamma_correction;
    float background[3];
    uint64_t seed;
    int32_t n_lights;
    float light_position[3];
    float light_color[4];
    int32_t sampling;       // 0 uniform (reference), 1 cosine
    int32_t tone_map;       // 1: divide, exposure, gamma (main.cpp:216-223); 0: mean only
    int32_t renderer;       // 0 path tracer, 1 raytracer, 2 raycaster
    float shadow_intensity; // raytracer --shadow
    float max_visibility;   // raycaster --max-visibility
};

void* orc_scene_create(const uint64_t* nodes, uint64_t n_nodes, const float* tri48, uint64_t n_tris,
                       const float* box6) {
    auto* sc = new Scene;
    sc->nodes.assign(nodes, nodes + n_nodes);
    sc->tris.resize(n_tris);
    std::memcpy(sc->tris.data(), tri48, n_tris * sizeof(Tri));
    sc->box_min = V3{box6[0], box6[1], box6[2]};
    sc->box_max = V3{box6[3], box6[4], box6[5]};
    return sc;
}

void orc_scene_free(void* s) { delete static_cast<Scene*>(s); }

// rays: n * 6 floats (o, d) AoS. counts (optional): [node_visits, tri_tests].
void orc_intersect(void* s, const float* rays, uint64_t n, uint32_t* id, float* r, float* ss, float* tt,
                   uint64_t* counts, int threads) {
    const Scene& sc = *static_cast<Scene*>(s);
    if (threads < 1) threads = 1;
    std::atomic<uint64_t> next{0}, visits{0}, tests{0};
    auto work = [&]() {
        Intersector ti(sc);
        const uint64_t block = 2048;
        for (;;) {
            const uint64_t b = next.fetch_add(block);
            if (b >= n) break;
            const uint64_t e = std::min(n, b + block);
            for (uint64_t i = b; i < e; ++i) {
                const float* q = rays + 6 * i;
                float rr = kFltMax, s2 = 0, t2 = 0;
                const uint32_t h = ti.intersect(Ray{V3{q[0], q[1], q[2]}, V3{q[3], q[4], q[5]}}, rr, s2, t2);
                if (h < kMaxTriangleId) {
                    id[i] = h;
                    r[i] = rr;
                    ss[i] = s2;
                    tt[i] = t2;
                } else {
                    id[i] = kMaxTriangleId;
                    r[i] = kFltMax;
                    ss[i] = 0;
                    tt[i] = 0;
                }
            }
        }
        visits += ti.node_visits;
        tests += ti.tri_tests;
    };
    std::vector<std::thread> pool;
    for (int i = 0; i < threads; ++i) pool.emplace_back(work);
    for (auto& th : pool) th.join();
    if (counts) {
        counts[0] = visits.load();
        counts[1] = tests.load();
    }
}

// Render (main.cpp:181-236 with harness seeding). out_rgba: width*height*4.
// rows row_begin, row_begin + row_step, ... below row_end only (row_end = 0
// means all rows, row_step 0 means 1): bounded CPU samples for the baseline,
// spread over the frame. Threads take one row at a time, as the reference's
// pool takes one task per row (main.cpp:193-226). stats: [rays, primary rays, shadow rays,
// node visits and triangle tests of primary/bounce rays, the same of shadow rays].
void orc_render(void* s, const orc_camera* cam, const orc_params* p, float* out_rgba, uint64_t* stats,
                int threads, uint32_t row_begin, uint32_t row_end, uint32_t row_step) {
    const Scene& sc = *static_cast<Scene*>(s);
    Conf conf;
    conf.max_depth = p->max_depth;
    conf.mc_samples = p->monte_carlo_samples;
    conf.sampling = p->sampling;
    conf.bg = C4{p->background[0], p->background[1], p->background[2], 1};
    conf.renderer = p->renderer;
    conf.shadow_intensity = p->shadow_intensity;
    conf.max_visibility = p->max_visibility;
    std::vector<Light> lights;
    if (p->n_lights > 0) {
        lights.push_back(Light{V3{p->light_position[0], p->light_position[1], p->light_position[2]},
                               C4{p->light_color[0], p->light_color[1], p->light_color[2], p->light_color[3]}});
    }
    const float dx_cam = cam->delta_x;
    const float dy_cam = cam->delta_x / cam->aspect;
    const V3 cam_pos{cam->position[0], cam->position[1], cam->position[2]};
    const int width = static_cast<int>(p->width), height = static_cast<int>(p->height);
    const float w = static_cast<float>(width), h = static_cast<float>(height);
    const int spp = static_cast<int>(p->pixel_samples);
    const uint32_t y_end = row_end ? std::min<uint32_t>(row_end, height) : height;

    const uint32_t step = row_step ? row_step : 1;
    std::atomic<uint32_t> next_row{0};
    std::atomic<uint64_t> n_rays{0}, n_prim{0}, n_shadow{0}, n_visits{0}, n_tests{0}, n_svisits{0}, n_stests{0};
    auto work = [&]() {
        Counters cnt;
        uint64_t prim = 0, visits = 0, tests = 0, svisits = 0, stests = 0;
        for (;;) {
            const uint64_t y64 = row_begin + uint64_t(next_row.fetch_add(1)) * step;
            if (y64 >= y_end) break;
            const uint32_t y = static_cast<uint32_t>(y64);
            Intersector ti(sc);
            for (int x = 0; x < width; ++x) {
                C4 acc;
                for (int i = 0; i < spp; ++i) {
                    uint64_t js, bs;
                    path_seeds(p->seed, (uint64_t(y) * width + x) * spp + i, js, bs);
                    Xorshift jit{js}, bnc{bs};
                    const float jx = jit.next_float();
                    const float jy = jit.next_float();
                    // Camera::raster2cam (lib/types.h:117-123), not normalized
                    const float px = x + jx, py = y + jy;
                    const V3 v{-dx_cam * (1 - 2 * px / w), dy_cam * (1 - 2 * py / h), -1};
                    const V3 d = mat_vec(cam->trafo, v);
                    ++prim;
                    if (conf.renderer == 1) acc = acc + trace_whitted(Ray{cam_pos, d}, ti, lights.front(), 0, conf, cnt);
                    else if (conf.renderer == 2) acc = acc + trace_cast(Ray{cam_pos, d}, ti, conf, cnt);
                    else acc = acc + trace(Ray{cam_pos, d}, ti, lights, 0, conf, bnc, cnt);
                }
                float* o = out_rgba + 4 * (size_t(y) * width + x);
                const float fs = static_cast<float>(spp);
                acc = C4{acc.r / fs, acc.g / fs, acc.b / fs, acc.a / fs};
                if (p->tone_map) {
                    acc = C4{exposure(acc.r, p->exposure), exposure(acc.g, p->exposure),
                             exposure(acc.b, p->exposure), acc.a};
                    if (p->gamma_correction) {
                        acc = C4{gamma_fn(acc.r, p->inverse_gamma), gamma_fn(acc.g, p->inverse_gamma),
                                 gamma_fn(acc.b, p->inverse_gamma), acc.a};
                    }
                }
                o[0] = acc.r;
                o[1] = acc.g;
                o[2] = acc.b;
                o[3] = acc.a;
            }
            visits += ti.node_visits;
            tests += ti.tri_tests;
            svisits += ti.shadow_visits;
            stests += ti.shadow_tests;
        }
        n_rays += cnt.rays;
        n_shadow += cnt.shadow_rays;
        n_prim += prim;
        n_visits += visits - svisits;
        n_tests += tests - stests;
        n_svisits += svisits;
        n_stests += stests;
    };
    if (threads < 1) threads = 1;
    std::vector<std::thread> pool;
    for (int i = 0; i < threads; ++i) pool.emplace_back(work);
    for (auto& th : pool) th.join();
    stats[0] = n_rays.load();
    stats[1] = n_prim.load();
    stats[2] = n_shadow.load();
    stats[3] = n_visits.load();
    stats[4] = n_tests.load();
    stats[5] = n_svisits.load();
    stats[6] = n_stests.load();
}

// P3 writer (lib/raster.h:79-100): "P3\nW H\n255", then per pixel the three
// channels int(clamp(255 * c * alpha)) right-aligned in 3 columns; a newline
// starts each row, a space separates pixels.
uint64_t orc_write_p3(const float* rgba, uint32_t width, uint32_t height, char* out, uint64_t cap) {
    std::ostringstream os;
    os << "P3\n" << width << " " << height << "\n" << 255;
    const uint64_t n = uint64_t(width) * height;
    auto clamp255 = [](float v) { return v < 0.f ? 0.f : (255.f < v ? 255.f : v); };
    for (uint64_t i = 0; i < n; ++i) {
        os << ((i % width == 0) ? "\n" : " ");
        const float* c = rgba + 4 * i;
        os << std::setw(3) << static_cast<int>(clamp255(255 * c[0] * c[3])) << " " << std::setw(3)
           << static_cast<int>(clamp255(255 * c[1] * c[3])) << " " << std::setw(3)
           << static_cast<int>(clamp255(255 * c[2] * c[3]));
    }
    const std::string str = os.str();
    if (out) std::memcpy(out, str.data(), std::min<uint64_t>(cap, str.size()));
    return str.size();
}

// Scalar probes for the pin tests.
void orc_xorshift_floats(uint64_t seed, uint64_t n, float* out) {
    Xorshift g{seed};
    for (uint64_t i = 0; i < n; ++i) out[i] = g.next_float();
}

void orc_from_to(const float* to3, float* m9) { from_to_matrix(V3{0, 0, 1}, V3{to3[0], to3[1], to3[2]}, m9); }

int orc_ray_box(const float* ray6, const float* box6, float* tmin_tmax) {
    Ray r{V3{ray6[0], ray6[1], ray6[2]}, V3{ray6[3], ray6[4], ray6[5]}};
    return intersect_ray_box(r, V3{box6[0], box6[1], box6[2]}, V3{box6[3], box6[4], box6[5]}, tmin_tmax[0],
                             tmin_tmax[1]);
}

void orc_tone(const float* rgba_in, uint64_t n, float exposure_value, float inverse_gamma, int gamma_on,
              float* rgba_out) {
    for (uint64_t i = 0; i < n; ++i) {
        const float* c = rgba_in + 4 * i;
        float* o = rgba_out + 4 * i;
        for (int k = 0; k < 3; ++k) {
            float v = exposure(c[k], exposure_value);
            o[k] = gamma_on ? gamma_fn(v, inverse_gamma) : v;
        }
        o[3] = c[3];
    }
}

} // extern "C"
