// Test infrastructure (checker only): C entry points around the reference
// implementation itself, compiled from the reference's own sources by
// oracle/build_ref.sh into oracle/_ref/libturner_ref.so. It is used to pin the
// oracle restatement (oracle/oracle.cpp) and to generate tests/golden/.
//
// What it wraps, unmodified:
//   KDTree / KDTreeIntersection      lib/kdtree.h:187-308, lib/kdtree.cpp:474-607
//   trace() (path tracer)            pathtracer.cpp:14-102 (included below)
//   trace() (Whitted raytracer)      raytracer.cpp:5-67, compiled as ref_raytracer_trace
//   trace() (raycaster)              raycaster.cpp:6-24, compiled as ref_raycaster_trace
//                                    (oracle/build_ref.sh renames the symbol per
//                                    translation unit: each renderer defines trace())
//   Camera::raster2cam               lib/types.h:92-123
//   exposure / gamma                 lib/effects.h:15-49
// The render driver re-creates main.cpp:181-236 (row tasks, pixel loop,
// division by the sample count, exposure, gamma) with std::thread instead of
// the missing ThreadPool dependency, and with per-(pixel, sample) seeding of
// the jitter stream and of sampling::detail::uniform (lib/sampling.h:12) so
// that the image does not depend on thread scheduling.

#include "pathtracer.cpp"

// The raytracer's and the raycaster's trace() (trace.h:23-25), each from its
// own translation unit with the symbol renamed (oracle/build_ref.sh).
Color ref_raytracer_trace(const Ray& ray, KDTreeIntersection& tree_intersection, const std::vector<Light>& lights,
                          int depth, const TracerConfig& conf);
Color ref_raycaster_trace(const Ray& ray, KDTreeIntersection& tree_intersection, const std::vector<Light>& lights,
                          int depth, const TracerConfig& conf);

#include "lib/effects.h"
#include "lib/raster.h"
#include "lib/xorshift.h"

#include <atomic>
#include <cstdint>
#include <thread>
#include <vector>

namespace {

// splitmix64 (Vigna, public domain): seeds the per-path xorshift streams.
inline uint64_t splitmix64(uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

struct PathSeeds {
    uint64_t jitter, bounce;
};

// The harness-defined per-(pixel, sample) seeding shared with the oracle and
// the GPU path: key = pixel_index * spp + sample.
inline PathSeeds path_seeds(uint64_t seed, uint64_t key) {
    uint64_t a = splitmix64(seed ^ key);
    uint64_t b = splitmix64(a ^ 0xD1B54A32D192ED03ULL);
    return {a ? a : 1, b ? b : 1};
}

// Flattening archive: records every float and uint64 that a serialize()
// template hands it, in order (the reference's cereal field order).
struct Capture {
    std::vector<float> f;
    std::vector<uint64_t> u;

    template <class... Ts> void operator()(Ts&... xs) { (visit(xs), ...); }

    void visit(float& x) { f.push_back(x); }
    void visit(uint64_t& x) { u.push_back(x); }
    template <class T> void visit(std::vector<T>& v) {
        for (auto& x : v) visit(x);
    }
    template <class T, size_t N> void visit(std::array<T, N>& a) {
        for (auto& x : a) visit(x);
    }
    void visit(turner::Vector3f& v) { cereal::serialize(*this, v); }
    void visit(turner::Point3f& v) { cereal::serialize(*this, v); }
    void visit(turner::Normal3f& v) { cereal::serialize(*this, v); }
    void visit(turner::Bbox3f& v) { cereal::serialize(*this, v); }
    void visit(aiColor4D& c) { ::serialize(*this, c); }
    void visit(Triangle& t) { t.serialize(*this); }
    void visit(detail::FlatNode& n) { n.serialize(*this); }
    void visit(KDTree& t) { t.serialize(*this); }
};

Triangles make_triangles(const float* verts, const float* normals, const float* diffuse, uint32_t n,
                         const float* reflect = nullptr) {
    Triangles tris;
    tris.reserve(n);
    for (uint32_t i = 0; i < n; ++i) {
        const float* v = verts + 9 * size_t(i);
        std::array<Point3f, 3> vs = {Point3f{v[0], v[1], v[2]}, Point3f{v[3], v[4], v[5]},
                                     Point3f{v[6], v[7], v[8]}};
        std::array<Normal3f, 3> ns = {Normal3f{}, Normal3f{}, Normal3f{}};
        if (normals) {
            const float* q = normals + 9 * size_t(i);
            ns = {Normal3f{q[0], q[1], q[2]}, Normal3f{q[3], q[4], q[5]}, Normal3f{q[6], q[7], q[8]}};
        }
        aiColor4D dif;
        if (diffuse) {
            const float* c = diffuse + 4 * size_t(i);
            dif = aiColor4D{c[0], c[1], c[2], c[3]};
        }
        aiColor4D rc;
        float rho = 0.f;
        if (reflect) {
            const float* q = reflect + 5 * size_t(i);
            rc = aiColor4D{q[0], q[1], q[2], q[3]};
            rho = q[4];
        }
        tris.emplace_back(vs, ns, aiColor4D{}, dif, dif, rc, rho);
    }
    return tris;
}

} // namespace

extern "C" {

struct ref_camera {
    float position[3];
    float trafo[9];   // row-major rotation of the camera node
    float hfov;       // aiCamera::mHorizontalFOV
    float aspect;     // aiCamera::mAspect
};

struct ref_params {
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
    int32_t threads;
    int32_t renderer;        // 0 pathtracer, 1 raytracer, 2 raycaster
    float shadow_intensity;  // raytracer --shadow
    float max_visibility;    // raycaster --max-visibility
};

// reflect: n * 5 floats (reflective rgba, reflectivity) or NULL.
void* ref_tree_build(const float* verts, const float* normals, const float* diffuse, uint32_t n,
                     const float* reflect) {
    return new KDTree(make_triangles(verts, normals, diffuse, n, reflect));
}

void ref_tree_free(void* t) { delete static_cast<KDTree*>(t); }

uint64_t ref_tree_num_nodes(void* t) { return static_cast<KDTree*>(t)->num_nodes(); }
uint64_t ref_tree_height(void* t) { return static_cast<KDTree*>(t)->height(); }
uint64_t ref_tree_num_triangles(void* t) { return static_cast<KDTree*>(t)->num_triangles(); }

// nodes: num_nodes uint64; tris: num_triangles * 48 floats (Triangle::serialize
// order); box: 6 floats (p_min, p_max).
void ref_tree_export(void* t, uint64_t* nodes, float* tris, float* box) {
    Capture cap;
    static_cast<KDTree*>(t)->serialize(cap);
    const KDTree& tree = *static_cast<KDTree*>(t);
    const size_t nt = tree.num_triangles();
    // layout: tris (nt * 48 floats), then box (6 floats)
    std::memcpy(tris, cap.f.data(), nt * 48 * sizeof(float));
    std::memcpy(box, cap.f.data() + nt * 48, 6 * sizeof(float));
    std::memcpy(nodes, cap.u.data(), cap.u.size() * sizeof(uint64_t));
}

// rays: n * 6 floats (o, d) AoS. Outputs: id (0x40000000 = miss), r, s, t.
void ref_intersect(void* t, const float* rays, uint64_t n, uint32_t* id, float* r, float* s, float* tt,
                   int threads) {
    const KDTree& tree = *static_cast<KDTree*>(t);
    if (threads < 1) threads = 1;
    std::atomic<uint64_t> next{0};
    auto work = [&]() {
        KDTreeIntersection ti(tree);
        const uint64_t block = 4096;
        for (;;) {
            uint64_t b = next.fetch_add(block);
            if (b >= n) break;
            uint64_t e = std::min(n, b + block);
            for (uint64_t i = b; i < e; ++i) {
                const float* q = rays + 6 * i;
                float rr = std::numeric_limits<float>::max(), ss = 0, t2 = 0;
                auto hit = ti.intersect(Ray{Point3f{q[0], q[1], q[2]}, Vector3f{q[3], q[4], q[5]}}, rr, ss, t2);
                if (hit) {
                    id[i] = static_cast<uint32_t>(static_cast<detail::TriangleId>(hit));
                    r[i] = rr;
                    s[i] = ss;
                    tt[i] = t2;
                } else {
                    id[i] = detail::FlatNode::MAX_TRIANGLE_ID;
                    r[i] = std::numeric_limits<float>::max();
                    s[i] = 0;
                    tt[i] = 0;
                }
            }
        }
    };
    std::vector<std::thread> pool;
    for (int i = 0; i < threads; ++i) pool.emplace_back(work);
    for (auto& th : pool) th.join();
}

// Camera::delta_x_ as the reference computes it, recovered through
// raster2cam with an identity transform: raster2cam({0, h/2}) = (-dx, 0, -1).
float ref_camera_delta_x(float hfov, float aspect) {
    aiCamera ac;
    ac.mHorizontalFOV = hfov;
    ac.mAspect = aspect;
    Camera cam(aiMatrix4x4{}, ac);
    return -cam.raster2cam({0.f, 1.f}, 2.f, 2.f).x;
}

// Renders into out_rgba (width*height*4 floats, row-major, after exposure and
// gamma). stats: [rays, primary rays].
void ref_render(void* t, const ref_camera* c, const ref_params* p, float* out_rgba, uint64_t* stats) {
    const KDTree& tree = *static_cast<KDTree*>(t);

    aiMatrix4x4 m;
    m.a1 = c->trafo[0]; m.a2 = c->trafo[1]; m.a3 = c->trafo[2]; m.a4 = c->position[0];
    m.b1 = c->trafo[3]; m.b2 = c->trafo[4]; m.b3 = c->trafo[5]; m.b4 = c->position[1];
    m.c1 = c->trafo[6]; m.c2 = c->trafo[7]; m.c3 = c->trafo[8]; m.c4 = c->position[2];
    aiCamera ac;
    ac.mHorizontalFOV = c->hfov;
    ac.mAspect = c->aspect;
    const Camera cam(m, ac);
    const Point3f cam_pos(cam.mPosition.x, cam.mPosition.y, cam.mPosition.z);

    TracerConfig conf{Config{}};
    conf.max_recursion_depth = p->max_depth;
    conf.num_pixel_samples = static_cast<int>(p->pixel_samples);
    conf.num_monte_carlo_samples = p->monte_carlo_samples;
    conf.exposure = p->exposure;
    conf.inverse_gamma = p->inverse_gamma;
    conf.gamma_correction_enabled = p->gamma_correction != 0;
    conf.bg_color = Color{p->background[0], p->background[1], p->background[2], 1};
    conf.shadow_intensity = p->shadow_intensity;
    conf.max_visibility = p->max_visibility;

    std::vector<Light> lights;
    if (p->n_lights > 0) {
        lights.push_back({{p->light_position[0], p->light_position[1], p->light_position[2]},
                          aiColor4D{p->light_color[0], p->light_color[1], p->light_color[2], p->light_color[3]}});
    }

    const int width = static_cast<int>(p->width);
    const int height = static_cast<int>(p->height);
    Image image(width, height);
    Stats::instance().num_rays = 0;
    Stats::instance().num_prim_rays = 0;

    std::atomic<int> next_row{0};
    auto work = [&]() {
        for (;;) {
            const int y = next_row.fetch_add(1);
            if (y >= height) break;
            KDTreeIntersection tree_intersection(tree);
            for (int x = 0; x < width; ++x) {
                for (int i = 0; i < conf.num_pixel_samples; ++i) {
                    const uint64_t key = (uint64_t(y) * width + x) * conf.num_pixel_samples + i;
                    const PathSeeds ps = path_seeds(p->seed, key);
                    xorshift64star<float> gen(ps.jitter);
                    sampling::detail::uniform = xorshift64star<float>(ps.bounce);
                    const float dx = gen();
                    const float dy = gen();
                    auto cam_dir = cam.raster2cam({x + dx, y + dy}, width, height);
                    Stats::instance().num_prim_rays += 1;
                    if (p->renderer == 1) {
                        image(x, y) += ref_raytracer_trace({cam_pos, cam_dir}, tree_intersection, lights, 0, conf);
                    } else if (p->renderer == 2) {
                        image(x, y) += ref_raycaster_trace({cam_pos, cam_dir}, tree_intersection, lights, 0, conf);
                    } else {
                        image(x, y) += trace({cam_pos, cam_dir}, tree_intersection, lights, 0, conf);
                    }
                }
                image(x, y) /= static_cast<float>(conf.num_pixel_samples);
                image(x, y) = exposure(image(x, y), conf.exposure);
                if (conf.gamma_correction_enabled) {
                    image(x, y) = gamma(image(x, y), conf.inverse_gamma);
                }
            }
        }
    };
    const int threads = p->threads > 0 ? p->threads : 1;
    std::vector<std::thread> pool;
    for (int i = 0; i < threads; ++i) pool.emplace_back(work);
    for (auto& th : pool) th.join();

    size_t k = 0;
    for (const auto& col : image) {
        out_rgba[k++] = col.r;
        out_rgba[k++] = col.g;
        out_rgba[k++] = col.b;
        out_rgba[k++] = col.a;
    }
    stats[0] = Stats::instance().num_rays;
    stats[1] = Stats::instance().num_prim_rays;
}

// Reference P3 writer (lib/raster.h:79-100) applied to an RGBA buffer; writes
// at most cap bytes and returns the full length.
uint64_t ref_write_p3(const float* rgba, uint32_t width, uint32_t height, char* out, uint64_t cap) {
    Image image(width, height);
    size_t k = 0;
    for (auto& col : image) {
        col = Color{rgba[k], rgba[k + 1], rgba[k + 2], rgba[k + 3]};
        k += 4;
    }
    std::ostringstream os;
    os << image;
    const std::string s = os.str();
    std::memcpy(out, s.data(), std::min<uint64_t>(cap, s.size()));
    return s.size();
}

} // extern "C"
