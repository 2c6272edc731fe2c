// Test infrastructure (checker only): exports the reference's own test
// fixtures (tests/helper.h) so that tests/golden/make_golden.py can record the
// exact triangles and rays of the reference's kd-tree tests
// (tests/test_kdtree.cpp:188-245). helper.h keeps its generators in function
// statics, so each export replays the whole sequence of one test case and must
// be called once per process.
#include "tests/helper.h"

#include <cstring>

namespace {
void put(const Triangle& t, float* out) {
    for (int i = 0; i < 3; ++i) {
        out[3 * i + 0] = t.vertices[i].x;
        out[3 * i + 1] = t.vertices[i].y;
        out[3 * i + 2] = t.vertices[i].z;
    }
}
} // namespace

extern "C" {

// "All triangles are in the same plane" (test_kdtree.cpp:188-209): per axis,
// 1000 triangles on the unit circle in the plane ax = 0, then the direction of
// the parallel ray. tris: 3 * 1000 * 9 floats; dirs: 3 * 3 floats.
void ref_fixture_coplanar(float* tris, float* dirs) {
    for (int a = 0; a < 3; ++a) {
        const Axis3 ax = AXES3[a];
        for (int i = 0; i < 1000; ++i) put(random_triangle_on_unit_sphere(ax, 0), tris + (a * 1000 + i) * 9);
        const Point3f d = random_vec_on_unit_sphere(ax, 0);
        dirs[3 * a + 0] = d.x;
        dirs[3 * a + 1] = d.y;
        dirs[3 * a + 2] = d.z;
    }
}

// "Intersect coplanar triangles" (test_kdtree.cpp:211-245): per axis, ten
// regular triangles in the planes ax = 0..9. tris: 3 * 10 * 9 floats.
void ref_fixture_stacked(float* tris) {
    for (int a = 0; a < 3; ++a) {
        const Axis3 ax = AXES3[a];
        int i = 0;
        for (float pos = 0.f; pos < 10.f; pos += 1.f, ++i) {
            put(random_regular_triangle_on_unit_sphere(ax, pos), tris + (a * 10 + i) * 9);
        }
    }
}

} // extern "C"
