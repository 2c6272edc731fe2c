// Test-infrastructure shim: the subset of the assimp value types that the
// reference's hot-path headers name, written from the component-wise
// arithmetic they denote. It exists only so that the reference's own sources
// compile into the oracle/_ref checker; the product never includes it.
//
// Conventions (assimp 3.x/4.x public API):
//   aiColor4D   RGBA, default (0,0,0,0), component-wise + - * with colours,
//               scaling by a float; "/" and "/=" divide component-wise.
//   aiMatrix3x3 row-major a1..c3; matrix * vector = rows dotted with the
//               vector, summed left to right (a1*x + a2*y + a3*z).
//   aiMatrix4x4 row-major a1..d4; matrix * vector applies the 3x3 part then
//               adds the translation column (a4, b4, c4).
//   FromToMatrix: rotation taking unit vector `from` onto unit vector `to`,
//               Moeller & Hughes, "Efficiently Building a Matrix to Rotate One
//               Vector to Another", JGT 4(4), 1999, evaluated in float.
#pragma once

#include <cmath>
#include <cstring>
#include <string>

struct aiVector3D {
    float x = 0, y = 0, z = 0;
    aiVector3D() = default;
    aiVector3D(float x_, float y_, float z_) : x(x_), y(y_), z(z_) {}
    explicit aiVector3D(float v) : x(v), y(v), z(v) {}
    bool operator==(const aiVector3D& o) const { return x == o.x && y == o.y && z == o.z; }
    bool operator!=(const aiVector3D& o) const { return !(*this == o); }
    aiVector3D operator+(const aiVector3D& o) const { return {x + o.x, y + o.y, z + o.z}; }
    aiVector3D operator-(const aiVector3D& o) const { return {x - o.x, y - o.y, z - o.z}; }
    aiVector3D operator-() const { return {-x, -y, -z}; }
    aiVector3D operator*(float f) const { return {x * f, y * f, z * f}; }
    float Length() const { return std::sqrt(x * x + y * y + z * z); }
};

inline aiVector3D operator*(float f, const aiVector3D& v) { return {f * v.x, f * v.y, f * v.z}; }

struct aiColor3D {
    float r = 0, g = 0, b = 0;
    aiColor3D() = default;
    aiColor3D(float r_, float g_, float b_) : r(r_), g(g_), b(b_) {}
};

struct aiColor4D {
    float r = 0, g = 0, b = 0, a = 0;
    aiColor4D() = default;
    aiColor4D(float r_, float g_, float b_, float a_) : r(r_), g(g_), b(b_), a(a_) {}
    explicit aiColor4D(float v) : r(v), g(v), b(v), a(v) {}

    bool operator==(const aiColor4D& o) const { return r == o.r && g == o.g && b == o.b && a == o.a; }
    bool operator!=(const aiColor4D& o) const { return !(*this == o); }
    // lexicographic order over (r, g, b, a), as used by the reference's tests
    bool operator<(const aiColor4D& o) const {
        if (r != o.r) return r < o.r;
        if (g != o.g) return g < o.g;
        if (b != o.b) return b < o.b;
        return a < o.a;
    }

    aiColor4D& operator+=(const aiColor4D& o) { r += o.r; g += o.g; b += o.b; a += o.a; return *this; }
    aiColor4D& operator-=(const aiColor4D& o) { r -= o.r; g -= o.g; b -= o.b; a -= o.a; return *this; }
    aiColor4D& operator*=(float f) { r *= f; g *= f; b *= f; a *= f; return *this; }
    aiColor4D& operator/=(float f) { r /= f; g /= f; b /= f; a /= f; return *this; }
};

inline aiColor4D operator+(const aiColor4D& p, const aiColor4D& q) { return {p.r + q.r, p.g + q.g, p.b + q.b, p.a + q.a}; }
inline aiColor4D operator-(const aiColor4D& p, const aiColor4D& q) { return {p.r - q.r, p.g - q.g, p.b - q.b, p.a - q.a}; }
inline aiColor4D operator*(const aiColor4D& p, const aiColor4D& q) { return {p.r * q.r, p.g * q.g, p.b * q.b, p.a * q.a}; }
inline aiColor4D operator*(const aiColor4D& p, float f) { return {p.r * f, p.g * f, p.b * f, p.a * f}; }
inline aiColor4D operator*(float f, const aiColor4D& p) { return {f * p.r, f * p.g, f * p.b, f * p.a}; }
inline aiColor4D operator/(const aiColor4D& p, float f) { return {p.r / f, p.g / f, p.b / f, p.a / f}; }

struct aiMatrix4x4;

struct aiMatrix3x3 {
    float a1 = 1, a2 = 0, a3 = 0;
    float b1 = 0, b2 = 1, b3 = 0;
    float c1 = 0, c2 = 0, c3 = 1;

    aiMatrix3x3() = default;
    aiMatrix3x3(float a1_, float a2_, float a3_, float b1_, float b2_, float b3_, float c1_, float c2_,
                float c3_)
        : a1(a1_), a2(a2_), a3(a3_), b1(b1_), b2(b2_), b3(b3_), c1(c1_), c2(c2_), c3(c3_) {}
    explicit aiMatrix3x3(const aiMatrix4x4& m);

    float Determinant() const {
        return a1 * b2 * c3 - a1 * b3 * c2 + a2 * b3 * c1 - a2 * b1 * c3 + a3 * b1 * c2 - a3 * b2 * c1;
    }

    // In-place inverse through the adjugate (cofactor transpose / determinant).
    aiMatrix3x3& Inverse() {
        const float det = Determinant();
        const float inv = 1.0f / det;
        aiMatrix3x3 r;
        r.a1 = inv * (b2 * c3 - b3 * c2);
        r.a2 = -inv * (a2 * c3 - a3 * c2);
        r.a3 = inv * (a2 * b3 - a3 * b2);
        r.b1 = -inv * (b1 * c3 - b3 * c1);
        r.b2 = inv * (a1 * c3 - a3 * c1);
        r.b3 = -inv * (a1 * b3 - a3 * b1);
        r.c1 = inv * (b1 * c2 - b2 * c1);
        r.c2 = -inv * (a1 * c2 - a2 * c1);
        r.c3 = inv * (a1 * b2 - a2 * b1);
        *this = r;
        return *this;
    }

    // Moeller-Hughes from-to rotation (JGT 1999). Float arithmetic throughout;
    // the same operation order is used by the GPU kernels so both sides agree.
    static aiMatrix3x3& FromToMatrix(const aiVector3D& from, const aiVector3D& to, aiMatrix3x3& mtx) {
        // v = from x to, e = cos(angle)
        const float vx = from.y * to.z - from.z * to.y;
        const float vy = from.z * to.x - from.x * to.z;
        const float vz = from.x * to.y - from.y * to.x;
        const float e = from.x * to.x + from.y * to.y + from.z * to.z;
        const float f = e < 0 ? -e : e;
        if (f > 1.0f - 0.000001f) {
            // nearly parallel: reflect through the coordinate axis least
            // aligned with `from` (two Householder reflections)
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
            float m[3][3];
            for (int i = 0; i < 3; ++i) {
                for (int j = 0; j < 3; ++j) {
                    m[i][j] = -c1 * u[i] * u[j] - c2 * w[i] * w[j] + c3 * w[i] * u[j];
                }
                m[i][i] += 1.0f;
            }
            mtx = aiMatrix3x3(m[0][0], m[0][1], m[0][2], m[1][0], m[1][1], m[1][2], m[2][0], m[2][1],
                              m[2][2]);
        } else {
            const float h = 1.0f / (1.0f + e);
            const float hvx = h * vx;
            const float hvz = h * vz;
            const float hvxy = hvx * vy;
            const float hvxz = hvx * vz;
            const float hvyz = hvz * vy;
            mtx.a1 = e + hvx * vx;
            mtx.a2 = hvxy - vz;
            mtx.a3 = hvxz + vy;
            mtx.b1 = hvxy + vz;
            mtx.b2 = e + h * vy * vy;
            mtx.b3 = hvyz - vx;
            mtx.c1 = hvxz - vy;
            mtx.c2 = hvyz + vx;
            mtx.c3 = e + hvz * vz;
        }
        return mtx;
    }
};

inline aiVector3D operator*(const aiMatrix3x3& m, const aiVector3D& v) {
    return {m.a1 * v.x + m.a2 * v.y + m.a3 * v.z, m.b1 * v.x + m.b2 * v.y + m.b3 * v.z,
            m.c1 * v.x + m.c2 * v.y + m.c3 * v.z};
}

struct aiMatrix4x4 {
    float a1 = 1, a2 = 0, a3 = 0, a4 = 0;
    float b1 = 0, b2 = 1, b3 = 0, b4 = 0;
    float c1 = 0, c2 = 0, c3 = 1, c4 = 0;
    float d1 = 0, d2 = 0, d3 = 0, d4 = 1;
};

inline aiMatrix3x3::aiMatrix3x3(const aiMatrix4x4& m)
    : a1(m.a1), a2(m.a2), a3(m.a3), b1(m.b1), b2(m.b2), b3(m.b3), c1(m.c1), c2(m.c2), c3(m.c3) {}

inline aiVector3D operator*(const aiMatrix4x4& m, const aiVector3D& v) {
    return {m.a1 * v.x + m.a2 * v.y + m.a3 * v.z + m.a4, m.b1 * v.x + m.b2 * v.y + m.b3 * v.z + m.b4,
            m.c1 * v.x + m.c2 * v.y + m.c3 * v.z + m.c4};
}

struct aiString {
    std::string data;
    const char* C_Str() const { return data.c_str(); }
};

struct aiRay {
    aiVector3D pos, dir;
};
