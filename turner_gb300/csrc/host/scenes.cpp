// Seeded synthetic scenes. The reference imports .blend files through assimp
// (main.cpp:25-82,98-136), which is not part of this build; these generators
// produce the same kind of input (triangles with vertex normals and diffuse
// colours, one pinhole camera, at most one point light).
//
// Every coordinate is computed with +, -, *, /, sqrt and floor in double and
// rounded once to float, with literal trigonometric constants, so the same
// scene comes out bit-identical on every host (x86-64 and aarch64).
#include "turner_gpu.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <unordered_map>
#include <vector>

struct turner_mesh {
    std::vector<float> verts, normals, diffuse;
    std::vector<float> reflect;   // per triangle: reflective colour (4), reflectivity
    turner_camera cam{};
    float hfov = 0;
    int n_lights = 0;
    turner_light light{};
};

namespace {

struct D3 {
    double x, y, z;
};
inline D3 operator+(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline D3 operator-(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 operator*(double s, D3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline D3 cross(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline D3 unit(D3 a) {
    const double l = std::sqrt(dot(a, a));
    return l > 0 ? (1.0 / l) * a : D3{0, 0, 0};
}

constexpr double kRoom = 5.56;
constexpr double kTan20 = 0.36397023426620236;   // tan(20 deg): 40 deg vertical field of view
constexpr double kCos17 = 0.95630475596303544;   // cos(17 deg)
constexpr double kSin17 = 0.29237170472273677;   // sin(17 deg)

struct Color4 {
    float r, g, b, a;
};
constexpr Color4 kWhite{0.75f, 0.75f, 0.75f, 1.f};
constexpr Color4 kRed{0.63f, 0.065f, 0.05f, 1.f};
constexpr Color4 kGreen{0.14f, 0.45f, 0.09f, 1.f};

struct Builder {
    turner_mesh* m;
    float refl[5] = {0.f, 0.f, 0.f, 0.f, 0.f};   // material of the triangles added next

    void tri(D3 a, D3 b, D3 c, D3 na, D3 nb, D3 nc, Color4 col) {
        const D3 p[3] = {a, b, c};
        const D3 n[3] = {na, nb, nc};
        for (int i = 0; i < 3; ++i) {
            m->verts.push_back(static_cast<float>(p[i].x));
            m->verts.push_back(static_cast<float>(p[i].y));
            m->verts.push_back(static_cast<float>(p[i].z));
            m->normals.push_back(static_cast<float>(n[i].x));
            m->normals.push_back(static_cast<float>(n[i].y));
            m->normals.push_back(static_cast<float>(n[i].z));
        }
        m->diffuse.push_back(col.r);
        m->diffuse.push_back(col.g);
        m->diffuse.push_back(col.b);
        m->diffuse.push_back(col.a);
        for (float r : refl) m->reflect.push_back(r);
    }
    void flat_tri(D3 a, D3 b, D3 c, D3 n, Color4 col) { tri(a, b, c, n, n, n, col); }

    // Quad p0 p1 p2 p3 split into (p0 p1 p2) and (p0 p2 p3), shared normal n,
    // tessellated into k x k sub-quads.
    void quad(D3 p0, D3 p1, D3 p2, D3 p3, D3 n, Color4 col, int k = 1) {
        const double inv = 1.0 / k;
        auto at = [&](int i, int j) {
            const double a = i * inv, b = j * inv;
            // bilinear: (1-a)(1-b) p0 + a(1-b) p1 + ab p2 + (1-a) b p3
            return (1 - a) * (1 - b) * p0 + a * (1 - b) * p1 + a * b * p2 + (1 - a) * b * p3;
        };
        for (int j = 0; j < k; ++j) {
            for (int i = 0; i < k; ++i) {
                const D3 q0 = at(i, j), q1 = at(i + 1, j), q2 = at(i + 1, j + 1), q3 = at(i, j + 1);
                flat_tri(q0, q1, q2, n, col);
                flat_tri(q0, q2, q3, n, col);
            }
        }
    }

    // Axis-aligned box of half extents h, rotated by (c, s) about the
    // vertical axis through its centre; outward normals; 12 triangles.
    void box(D3 center, D3 h, double c, double s, Color4 col) {
        auto rot = [&](D3 l) { return D3{c * l.x + s * l.z, l.y, -s * l.x + c * l.z}; };
        auto corner = [&](int ix, int iy, int iz) {
            return center + rot(D3{ix ? h.x : -h.x, iy ? h.y : -h.y, iz ? h.z : -h.z});
        };
        const D3 ex = rot(D3{1, 0, 0}), ey{0, 1, 0}, ez = rot(D3{0, 0, 1});
        quad(corner(1, 0, 0), corner(1, 1, 0), corner(1, 1, 1), corner(1, 0, 1), ex, col);   // +x
        quad(corner(0, 0, 1), corner(0, 1, 1), corner(0, 1, 0), corner(0, 0, 0), -1.0 * ex, col); // -x
        quad(corner(0, 1, 0), corner(0, 1, 1), corner(1, 1, 1), corner(1, 1, 0), ey, col);   // +y
        quad(corner(0, 0, 0), corner(1, 0, 0), corner(1, 0, 1), corner(0, 0, 1), -1.0 * ey, col); // -y
        quad(corner(0, 0, 1), corner(1, 0, 1), corner(1, 1, 1), corner(0, 1, 1), ez, col);   // +z
        quad(corner(0, 0, 0), corner(0, 1, 0), corner(1, 1, 0), corner(1, 0, 0), -1.0 * ez, col); // -z
    }
};

// Five walls of the open-front room (normals point inside), k x k quads each.
void room_walls(Builder& b, int k) {
    const double S = kRoom;
    b.quad({0, 0, 0}, {S, 0, 0}, {S, 0, -S}, {0, 0, -S}, {0, 1, 0}, kWhite, k);      // floor
    b.quad({0, S, 0}, {0, S, -S}, {S, S, -S}, {S, S, 0}, {0, -1, 0}, kWhite, k);     // ceiling
    b.quad({0, 0, -S}, {S, 0, -S}, {S, S, -S}, {0, S, -S}, {0, 0, 1}, kWhite, k);    // back
    b.quad({0, 0, 0}, {0, 0, -S}, {0, S, -S}, {0, S, 0}, {1, 0, 0}, kRed, k);        // left
    b.quad({S, 0, 0}, {S, S, 0}, {S, S, -S}, {S, 0, -S}, {-1, 0, 0}, kGreen, k);     // right
}

// 1.3 x 1.05 ceiling quad just below the ceiling, facing down.
void ceiling_quad(Builder& b) {
    const double S = kRoom, y = S - 0.01, cx = 0.5 * S, cz = -0.5 * S, hx = 0.65, hz = 0.525;
    b.quad({cx - hx, y, cz - hz}, {cx + hx, y, cz - hz}, {cx + hx, y, cz + hz}, {cx - hx, y, cz + hz}, {0, -1, 0},
           kWhite);
}

void inner_boxes(Builder& b) {
    b.box({3.70, 0.825, -1.90}, {0.825, 0.825, 0.825}, kCos17, -kSin17, kWhite);   // short, -17 deg
    b.box({1.85, 1.650, -3.70}, {0.825, 1.650, 0.825}, kCos17, kSin17, kWhite);     // tall, +17 deg
}

void room_light_camera(turner_mesh* m, double aspect) {
    const double S = kRoom;
    m->n_lights = 1;
    m->light.position[0] = static_cast<float>(0.5 * S);
    m->light.position[1] = static_cast<float>(S - 0.05);
    m->light.position[2] = static_cast<float>(-0.5 * S);
    m->light.color[0] = m->light.color[1] = m->light.color[2] = 50.f;
    m->light.color[3] = 1.f;
    // pinhole at the centre of the open front, looking down -z
    m->cam.position[0] = static_cast<float>(0.5 * S);
    m->cam.position[1] = static_cast<float>(0.5 * S);
    m->cam.position[2] = 0.f;
    const float id[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    std::memcpy(m->cam.trafo, id, sizeof(id));
    m->cam.aspect = static_cast<float>(aspect);
    // delta_y = tan(20 deg); delta_x = delta_y * aspect; the reference derives
    // delta_x = tan(mHorizontalFOV), so mHorizontalFOV = atan(delta_x).
    m->cam.delta_x = static_cast<float>(kTan20 * aspect);
    m->hfov = static_cast<float>(std::atan(static_cast<double>(m->cam.delta_x)));
}

inline uint64_t splitmix64(uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

struct Rng {
    uint64_t s;
    double uniform() {   // [0, 1) with 53 bits
        s += 0x9E3779B97F4A7C15ULL;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        z ^= z >> 31;
        return static_cast<double>(z >> 11) * (1.0 / 9007199254740992.0);
    }
    double range(double a, double b) { return a + (b - a) * uniform(); }
    // uniform on the unit sphere, Marsaglia (1972): only +, *, sqrt
    D3 sphere() {
        for (;;) {
            const double x1 = range(-1, 1), x2 = range(-1, 1);
            const double q = x1 * x1 + x2 * x2;
            if (q >= 1 || q == 0) continue;
            const double r = 2 * std::sqrt(1 - q);
            return {x1 * r, x2 * r, 1 - 2 * q};
        }
    }
};

// Lattice value noise in [-1, 1] with smoothstep-weighted trilinear blend.
double value_noise(D3 p, uint64_t seed) {
    const double fx = std::floor(p.x), fy = std::floor(p.y), fz = std::floor(p.z);
    const int64_t ix = static_cast<int64_t>(fx), iy = static_cast<int64_t>(fy), iz = static_cast<int64_t>(fz);
    const double tx = p.x - fx, ty = p.y - fy, tz = p.z - fz;
    auto smooth = [](double t) { return t * t * (3 - 2 * t); };
    const double wx = smooth(tx), wy = smooth(ty), wz = smooth(tz);
    auto lattice = [&](int64_t i, int64_t j, int64_t k) {
        const uint64_t key = (static_cast<uint64_t>(i) & 0x1FFFFF) << 42 | (static_cast<uint64_t>(j) & 0x1FFFFF) << 21 |
                             (static_cast<uint64_t>(k) & 0x1FFFFF);
        const uint64_t h = splitmix64(key ^ splitmix64(seed));
        return static_cast<double>(h >> 11) * (2.0 / 9007199254740992.0) - 1.0;
    };
    double acc = 0;
    for (int c = 0; c < 8; ++c) {
        const int dx = c & 1, dy = (c >> 1) & 1, dz = (c >> 2) & 1;
        const double w = (dx ? wx : 1 - wx) * (dy ? wy : 1 - wy) * (dz ? wz : 1 - wz);
        acc += w * lattice(ix + dx, iy + dy, iz + dz);
    }
    return acc;
}

double fbm5(D3 p, double base_frequency, uint64_t seed) {
    double sum = 0, amp = 1, freq = base_frequency, norm = 0;
    for (int o = 0; o < 5; ++o) {
        sum += amp * value_noise(freq * p, seed + static_cast<uint64_t>(o));
        norm += amp;
        amp *= 0.5;
        freq *= 2;
    }
    return sum / norm;
}

// Icosphere subdivided `level` times (20 * 4^level faces), radius
// 1.5 + 0.08 * fbm5(direction, base frequency 4), smooth vertex normals.
void displaced_icosphere(Builder& b, D3 center, int level, uint64_t seed) {
    const double phi = 1.6180339887498949;   // golden ratio
    std::vector<D3> vs = {{-1, phi, 0}, {1, phi, 0}, {-1, -phi, 0}, {1, -phi, 0}, {0, -1, phi}, {0, 1, phi},
                          {0, -1, -phi}, {0, 1, -phi}, {phi, 0, -1}, {phi, 0, 1}, {-phi, 0, -1}, {-phi, 0, 1}};
    for (auto& v : vs) v = unit(v);
    std::vector<uint32_t> faces = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4,
                                   11, 10, 2, 10, 7, 6, 7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8,
                                   3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1};
    for (int l = 0; l < level; ++l) {
        std::unordered_map<uint64_t, uint32_t> mid;
        mid.reserve(faces.size());
        auto midpoint = [&](uint32_t a, uint32_t c) {
            const uint64_t key = a < c ? (uint64_t(a) << 32 | c) : (uint64_t(c) << 32 | a);
            auto it = mid.find(key);
            if (it != mid.end()) return it->second;
            const uint32_t idx = static_cast<uint32_t>(vs.size());
            vs.push_back(unit(0.5 * (vs[a] + vs[c])));
            mid.emplace(key, idx);
            return idx;
        };
        std::vector<uint32_t> next;
        next.reserve(faces.size() * 4);
        for (size_t f = 0; f < faces.size(); f += 3) {
            const uint32_t a = faces[f], c = faces[f + 1], e = faces[f + 2];
            const uint32_t ac = midpoint(a, c), ce = midpoint(c, e), ea = midpoint(e, a);
            const uint32_t quads[12] = {a, ac, ea, c, ce, ac, e, ea, ce, ac, ce, ea};
            next.insert(next.end(), quads, quads + 12);
        }
        faces.swap(next);
    }
    // displace, round to float once
    std::vector<D3> pos(vs.size());
    for (size_t i = 0; i < vs.size(); ++i) {
        const double rad = 1.5 + 0.08 * fbm5(vs[i], 4.0, seed);
        const D3 p = center + rad * vs[i];
        pos[i] = {static_cast<float>(p.x), static_cast<float>(p.y), static_cast<float>(p.z)};
    }
    // smooth normals: area-weighted face normals, summed in face order
    std::vector<D3> nrm(vs.size(), D3{0, 0, 0});
    for (size_t f = 0; f < faces.size(); f += 3) {
        const D3 a = pos[faces[f]], c = pos[faces[f + 1]], e = pos[faces[f + 2]];
        const D3 fn = cross(c - a, e - a);
        for (int k = 0; k < 3; ++k) nrm[faces[f + k]] = nrm[faces[f + k]] + fn;
    }
    for (auto& n : nrm) n = unit(n);
    for (size_t f = 0; f < faces.size(); f += 3) {
        const uint32_t a = faces[f], c = faces[f + 1], e = faces[f + 2];
        b.tri(pos[a], pos[c], pos[e], nrm[a], nrm[c], nrm[e], kWhite);
    }
}

// Clustered soup: `count` triangles around 64 cluster centres in a unit cube
// in the middle of the room; edges 0.01-0.2 long, flat normals.
void soup(Builder& b, uint32_t count, uint64_t seed) {
    Rng rng{splitmix64(seed ^ 0x5D1CEULL)};
    const D3 lo{0.5 * kRoom - 0.5, 1.2, -0.5 * kRoom - 0.5};
    std::vector<D3> centers(64);
    for (auto& c : centers) {
        const double cx = rng.uniform();
        const double cy = rng.uniform();
        const double cz = rng.uniform();
        c = lo + D3{cx, cy, cz};
    }
    for (uint32_t i = 0; i < count; ++i) {
        const D3 c = centers[static_cast<size_t>(rng.uniform() * 64) & 63];
        const double ox = rng.range(-0.12, 0.12);
        const double oy = rng.range(-0.12, 0.12);
        const double oz = rng.range(-0.12, 0.12);
        D3 v0 = c + D3{ox, oy, oz};
        v0 = D3{std::min(std::max(v0.x, lo.x), lo.x + 1), std::min(std::max(v0.y, lo.y), lo.y + 1),
                std::min(std::max(v0.z, lo.z), lo.z + 1)};
        // one RNG call per statement: the evaluation order of operands is
        // unspecified and differs between compilers' targets
        const double l1 = rng.range(0.01, 0.2);
        const D3 e1 = rng.sphere();
        const double l2 = rng.range(0.01, 0.2);
        const D3 e2 = rng.sphere();
        const D3 v1 = v0 + l1 * e1;
        const D3 v2 = v0 + l2 * e2;
        const D3 n = unit(cross(v1 - v0, v2 - v0));
        b.flat_tri(v0, v1, v2, n, kWhite);
    }
}

// 1.5 x 1.5 baffle, 0.02 thick, 0.3 below the light.
void baffle(Builder& b) {
    const double y = kRoom - 0.05 - 0.3;
    b.box({0.5 * kRoom, y, -0.5 * kRoom}, {0.75, 0.01, 0.75}, 1.0, 0.0, kWhite);
}

} // namespace

extern "C" {

int turner_scene_make(int kind, uint32_t detail, uint32_t count, uint64_t seed, float aspect, turner_mesh** out) {
    if (!out || !(aspect > 0)) return TURNER_ERR_INVALID_ARG;
    auto* m = new (std::nothrow) turner_mesh;
    if (!m) return TURNER_ERR_OUT_OF_MEMORY;
    Builder b{m};
    const D3 sphere_center{0.5 * kRoom, 1.65, -3.5};
    switch (kind) {
    case TURNER_SCENE_ROOM:
        room_walls(b, 1);
        inner_boxes(b);
        ceiling_quad(b);
        break;
    case TURNER_SCENE_MIRROR_ROOM: {
        // the room with reflective boxes, for the Whitted raytracer
        // (raytracer.cpp reads reflectivity and the reflective colour)
        room_walls(b, 1);
        const float short_box[5] = {1.f, 1.f, 1.f, 1.f, 0.3f}, tall_box[5] = {0.9f, 0.9f, 0.95f, 1.f, 0.85f};
        std::memcpy(b.refl, short_box, sizeof(b.refl));
        b.box({3.70, 0.825, -1.90}, {0.825, 0.825, 0.825}, kCos17, -kSin17, kWhite);
        std::memcpy(b.refl, tall_box, sizeof(b.refl));
        b.box({1.85, 1.650, -3.70}, {0.825, 1.650, 0.825}, kCos17, kSin17, kWhite);
        std::memset(b.refl, 0, sizeof(b.refl));
        ceiling_quad(b);
        break;
    }
    case TURNER_SCENE_SPHERE_ROOM:
        if (detail > 9) { delete m; return TURNER_ERR_TOO_LARGE; }
        room_walls(b, 1);
        ceiling_quad(b);
        displaced_icosphere(b, sphere_center, static_cast<int>(detail), seed);
        break;
    case TURNER_SCENE_SOUP:
        if (count == 0 || count > (1u << 26)) { delete m; return TURNER_ERR_INVALID_ARG; }
        room_walls(b, 1);
        ceiling_quad(b);
        soup(b, count, seed);
        break;
    case TURNER_SCENE_BAFFLE_ROOM:
        if (detail == 0 || detail > 1024) { delete m; return TURNER_ERR_INVALID_ARG; }
        room_walls(b, static_cast<int>(detail));
        inner_boxes(b);
        ceiling_quad(b);
        baffle(b);
        break;
    case TURNER_SCENE_BAFFLE_SPHERE:
        if (detail > 9 || count == 0 || count > 1024) { delete m; return TURNER_ERR_INVALID_ARG; }
        room_walls(b, static_cast<int>(count));
        ceiling_quad(b);
        baffle(b);
        displaced_icosphere(b, sphere_center, static_cast<int>(detail), seed);
        break;
    default:
        delete m;
        return TURNER_ERR_INVALID_ARG;
    }
    room_light_camera(m, aspect);
    *out = m;
    return TURNER_OK;
}

uint32_t turner_mesh_num_triangles(const turner_mesh* m) { return m ? static_cast<uint32_t>(m->diffuse.size() / 4) : 0; }
const float* turner_mesh_vertices(const turner_mesh* m) { return m ? m->verts.data() : nullptr; }
const float* turner_mesh_normals(const turner_mesh* m) { return m ? m->normals.data() : nullptr; }
const float* turner_mesh_diffuse(const turner_mesh* m) { return m ? m->diffuse.data() : nullptr; }
const float* turner_mesh_reflective(const turner_mesh* m) { return m ? m->reflect.data() : nullptr; }

void turner_mesh_camera(const turner_mesh* m, turner_camera* cam, float* hfov) {
    if (!m) return;
    if (cam) *cam = m->cam;
    if (hfov) *hfov = m->hfov;
}

int turner_mesh_light(const turner_mesh* m, turner_light* light) {
    if (!m) return 0;
    if (light && m->n_lights) *light = m->light;
    return m->n_lights;
}

void turner_mesh_free(turner_mesh* m) { delete m; }

int turner_make_rays(uint64_t n, const float box[6], uint64_t seed, float* ox, float* oy, float* oz, float* dx,
                     float* dy, float* dz) {
    if (!box || !ox || !oy || !oz || !dx || !dy || !dz) return TURNER_ERR_INVALID_ARG;
    // one stream per block of 4096 rays so that any range can be regenerated
    const uint64_t block = 4096;
    for (uint64_t b0 = 0; b0 < n; b0 += block) {
        Rng rng{splitmix64(seed ^ (b0 / block + 1) * 0xA24BAED4963EE407ULL)};
        const uint64_t e = std::min(n, b0 + block);
        for (uint64_t i = b0; i < e; ++i) {
            ox[i] = static_cast<float>(box[0] + (double(box[3]) - box[0]) * rng.uniform());
            oy[i] = static_cast<float>(box[1] + (double(box[4]) - box[1]) * rng.uniform());
            oz[i] = static_cast<float>(box[2] + (double(box[5]) - box[2]) * rng.uniform());
            const D3 d = rng.sphere();
            dx[i] = static_cast<float>(d.x);
            dy[i] = static_cast<float>(d.y);
            dz[i] = static_cast<float>(d.z);
        }
    }
    return TURNER_OK;
}

} // extern "C"
