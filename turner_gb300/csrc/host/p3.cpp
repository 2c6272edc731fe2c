// P3 image writer of lib/raster.h:79-100: header "P3\n<w> <h>\n255", then each
// pixel's channels int(clamp(255 * c * alpha, 0, 255)) right-aligned in three
// columns, pixels separated by a space and rows started with a newline.
#include "turner_gpu.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>

extern "C" uint64_t turner_write_p3(const float* rgba, uint32_t width, uint32_t height, char* out, uint64_t cap) {
    if (!rgba || width == 0) return 0;
    std::string s = "P3\n" + std::to_string(width) + " " + std::to_string(height) + "\n255";
    const uint64_t n = uint64_t(width) * height;
    s.reserve(s.size() + n * 12);
    char buf[48];
    auto channel = [](float c, float a) {
        float v = 255 * c * a;
        v = v < 0.f ? 0.f : (255.f < v ? 255.f : v);
        return static_cast<int>(v);
    };
    for (uint64_t i = 0; i < n; ++i) {
        const float* c = rgba + 4 * i;
        const int len = std::snprintf(buf, sizeof(buf), "%c%3d %3d %3d", (i % width == 0) ? '\n' : ' ',
                                      channel(c[0], c[3]), channel(c[1], c[3]), channel(c[2], c[3]));
        s.append(buf, static_cast<size_t>(len));
    }
    if (out && cap) std::memcpy(out, s.data(), std::min<uint64_t>(cap, s.size()));
    return s.size();
}
