// turner_pathtracer: the `pathtracer` executable's interface (pathtracer.h:4-24,
// config.h:13-165, main.cpp:88-244) on the GB300 core. Same flags and
// defaults; the image goes to stdout as P3, statistics to stderr in the
// reference's format (lib/output.h:101-113).
//
// <scene> names a built-in synthetic scene (no assimp importer here):
//   room | sphere[:DETAIL] | soup:COUNT[:SEED] | baffle[:DETAIL] | baffle-sphere[:DETAIL]
#include "turner_gpu.h"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

namespace {

const char* kUsage = R"(Usage: turner_pathtracer <scene> [options]

Options:
  -w --width=<px>                   Width of the image [default: 640].
  -a --aspect=<num>                 Aspect ratio of the image [default: 1].
  --background=<3x float>           Background color [default: 0 0 0].
  -t --threads=<int>                Accepted for compatibility; the GPU is used [default: 1].
  --inverse-gamma=<float>           Inverse of gamma for gamma correction [default: 0.454545].
  --no-gamma-correction             Disables gamma correction.
  --exposure=<float>                Exposure [default: 1].
  -v --verbose                      Verbose output.

Pathtracer options:
  -d --max-depth=<int>              Maximum recursion depth for raytracing [default: 3].
  -p --pixel-samples=<int>          Number of samples per pixel [default: 1].
  -m --monte-carlo-samples=<int>    Monte Carlo samples per ray [default: 8].

GB300 options:
  --seed=<int>                      Stream seed base [default: 1].
  --renderer=<name>                 trace() plug-in: path (pathtracer), raytrace
                                    (raytracer) or raycast (raycaster) [default: path].
  --shadow=<float>                  Raytracer: intensity of shadow [default: 0.5].
  --max-visibility=<float>          Raycaster: any object farther away is dark [default: 2.0].
  --cosine                          Cosine-weighted bounces instead of uniform.
  --fast                            Early-exit closest-hit traversal for bounce rays.
  --device=<int>                    CUDA device [default: 0].
  --kdtree-cache=<dir>              Directory of content-keyed kd-tree files: load the
                                    scene's tree from it, or build and store it.
  --gpu-kdtree                      Build the kd-tree on the GPU (its own SAH planes,
                                    not the reference's node words; same closest hits).
                                    Not with --kdtree-cache.

Scenes: room | sphere[:DETAIL] | soup:COUNT[:SEED] | baffle[:DETAIL] | baffle-sphere[:DETAIL] | mirror
)";

struct Options {
    std::string scene;
    long width = 640;
    float aspect = 1;
    float bg[3] = {0, 0, 0};
    float inverse_gamma = 0.454545f;
    float exposure = 1;
    bool gamma = true;
    bool verbose = false;
    int depth = 3;
    int pixel_samples = 1;
    int mc = 8;
    uint64_t seed = 1;
    bool cosine = false, fast = false;
    int renderer = TURNER_RENDERER_PATH;
    float shadow = 0.5f, max_visibility = 2.f;
    int device = 0;
    std::string kdtree_cache;
    bool gpu_kdtree = false;
};

bool take(int& i, int argc, char** argv, const char* s, const char* l, std::string& val) {
    const std::string a = argv[i];
    const std::string ls = std::string(l) + "=";
    if ((s && a == s) || a == l) {
        if (i + 1 >= argc) return false;
        val = argv[++i];
        return true;
    }
    if (a.compare(0, ls.size(), ls) == 0) {
        val = a.substr(ls.size());
        return true;
    }
    return false;
}

// Config::parse_color (config.h:43-58): one value or three space-separated values
bool parse_color(const std::string& s, float out[3]) {
    std::stringstream ss(s);
    std::vector<float> v;
    std::string item;
    while (std::getline(ss, item, ' ')) {
        if (!item.empty()) v.push_back(std::stof(item));
    }
    if (v.size() == 1) {
        out[0] = out[1] = out[2] = v[0];
        return true;
    }
    if (v.size() == 3) {
        for (int k = 0; k < 3; ++k) out[k] = v[k];
        return true;
    }
    return false;
}

int parse(int argc, char** argv, Options& o) {
    for (int i = 1; i < argc; ++i) {
        std::string v;
        const std::string a = argv[i];
        if (a == "-h" || a == "--help") return 1;
        if (take(i, argc, argv, "-w", "--width", v)) o.width = std::stol(v);
        else if (take(i, argc, argv, "-a", "--aspect", v)) o.aspect = std::stof(v);
        else if (take(i, argc, argv, nullptr, "--background", v)) { if (!parse_color(v, o.bg)) return 2; }
        else if (take(i, argc, argv, "-t", "--threads", v)) (void)std::stol(v);
        else if (take(i, argc, argv, nullptr, "--inverse-gamma", v)) o.inverse_gamma = std::stof(v);
        else if (a == "--no-gamma-correction") o.gamma = false;
        else if (take(i, argc, argv, nullptr, "--exposure", v)) o.exposure = std::stof(v);
        else if (a == "-v" || a == "--verbose") o.verbose = true;
        else if (take(i, argc, argv, "-d", "--max-depth", v)) o.depth = std::stoi(v);
        else if (take(i, argc, argv, "-p", "--pixel-samples", v)) o.pixel_samples = std::stoi(v);
        else if (take(i, argc, argv, "-m", "--monte-carlo-samples", v)) o.mc = std::stoi(v);
        else if (take(i, argc, argv, nullptr, "--seed", v)) o.seed = std::stoull(v);
        else if (a == "--cosine") o.cosine = true;
        else if (take(i, argc, argv, nullptr, "--shadow", v)) o.shadow = std::stof(v);
        else if (take(i, argc, argv, nullptr, "--max-visibility", v)) o.max_visibility = std::stof(v);
        else if (take(i, argc, argv, nullptr, "--renderer", v)) {
            if (v == "path") o.renderer = TURNER_RENDERER_PATH;
            else if (v == "raytrace") o.renderer = TURNER_RENDERER_RAYTRACE;
            else if (v == "raycast") o.renderer = TURNER_RENDERER_RAYCAST;
            else return 2;
        }
        else if (a == "--fast") o.fast = true;
        else if (take(i, argc, argv, nullptr, "--device", v)) o.device = std::stoi(v);
        else if (take(i, argc, argv, nullptr, "--kdtree-cache", v)) o.kdtree_cache = v;
        else if (a == "--gpu-kdtree") o.gpu_kdtree = true;
        else if (!a.empty() && a[0] != '-' && o.scene.empty()) o.scene = a;
        else return 2;
    }
    // TracerConfig::check (config.h:120-127) and Config::check (config.h:30-34)
    if (o.scene.empty() || !(o.aspect > 0) || o.exposure < 0 || o.depth <= 0 || o.pixel_samples < 1 || o.mc < 0 ||
        o.width < 1 || !(o.shadow >= 0.f && o.shadow <= 1.f) || !(o.max_visibility >= 0.f))
        return 2;
    // a cache file is keyed by the triangles alone, so it cannot tell the two builders' trees apart
    if (o.gpu_kdtree && !o.kdtree_cache.empty()) return 2;
    return 0;
}

std::vector<std::string> split(const std::string& s, char c) {
    std::vector<std::string> out;
    std::stringstream ss(s);
    std::string item;
    while (std::getline(ss, item, c)) out.push_back(item);
    return out;
}

int make_scene(const std::string& spec, float aspect, turner_mesh** mesh) {
    const auto parts = split(spec, ':');
    const std::string& name = parts[0];
    auto num = [&](size_t k, unsigned long dflt) { return parts.size() > k ? std::stoul(parts[k]) : dflt; };
    if (name == "room") return turner_scene_make(TURNER_SCENE_ROOM, 0, 0, 1, aspect, mesh);
    if (name == "sphere") return turner_scene_make(TURNER_SCENE_SPHERE_ROOM, num(1, 7), 0, 1, aspect, mesh);
    if (name == "soup") return turner_scene_make(TURNER_SCENE_SOUP, 0, num(1, 10000), num(2, 1), aspect, mesh);
    if (name == "baffle") return turner_scene_make(TURNER_SCENE_BAFFLE_ROOM, num(1, 64), 0, 1, aspect, mesh);
    if (name == "baffle-sphere") return turner_scene_make(TURNER_SCENE_BAFFLE_SPHERE, num(1, 7), 64, 1, aspect, mesh);
    if (name == "mirror") return turner_scene_make(TURNER_SCENE_MIRROR_ROOM, 0, 0, 1, aspect, mesh);
    return TURNER_ERR_INVALID_ARG;
}

} // namespace

int main(int argc, char** argv) {
    Options o;
    const int pr = parse(argc, argv, o);
    if (pr != 0) {
        std::cerr << kUsage;
        return pr == 1 ? 0 : 1;
    }
    using clock = std::chrono::steady_clock;
    std::cerr << "Loading scene..." << std::endl;
    const auto t_load = clock::now();
    turner_mesh* mesh = nullptr;
    int st = make_scene(o.scene, o.aspect, &mesh);
    if (st != TURNER_OK) {
        std::cerr << "scene: " << turner_strerror(st) << std::endl;
        return 1;
    }
    turner_ctx* ctx = nullptr;
    st = turner_create(&ctx, o.device);
    if (st != TURNER_OK) {
        std::cerr << "device: " << turner_strerror(st) << std::endl;
        return 1;
    }
    std::cerr << "Loading triangles and building kd-tree..." << std::endl;
    turner_kdtree* tree = nullptr;
    const auto t_tree = clock::now();
    int from_cache = 0;
    if (o.gpu_kdtree) {
        st = turner_kdtree_build_gpu(ctx, turner_mesh_vertices(mesh), turner_mesh_normals(mesh),
                                     turner_mesh_diffuse(mesh), turner_mesh_num_triangles(mesh), &tree);
    } else {
        st = turner_kdtree_build_cached(turner_mesh_vertices(mesh), turner_mesh_normals(mesh),
                                        turner_mesh_diffuse(mesh), turner_mesh_num_triangles(mesh), 0,
                                        o.kdtree_cache.empty() ? nullptr : o.kdtree_cache.c_str(), &tree, &from_cache);
    }
    if (st != TURNER_OK) {
        std::cerr << "kd-tree: " << turner_strerror(st) << std::endl;
        return 1;
    }
    if (from_cache) std::cerr << "Loaded kd-tree from " << o.kdtree_cache << std::endl;
    turner_kdtree_set_reflective(tree, turner_mesh_reflective(mesh));   // the raytracer's materials
    const double tree_ms = std::chrono::duration<double, std::milli>(clock::now() - t_tree).count();
    std::cerr << "KDTree runtime: " << static_cast<long>(tree_ms) << std::endl;
    const double load_s = std::chrono::duration<double>(clock::now() - t_load).count();
    uint32_t scene_id = 0;
    st = turner_upload_kdtree(ctx, tree, &scene_id);
    if (st != TURNER_OK) {
        std::cerr << "upload: " << turner_strerror(st) << std::endl;
        return 1;
    }

    turner_job job{};
    job.scene_id = scene_id;
    job.width = static_cast<uint32_t>(o.width);
    turner_camera cam;
    float hfov;
    turner_mesh_camera(mesh, &cam, &hfov);
    job.height = static_cast<uint32_t>(static_cast<int>(o.width / cam.aspect));   // main.cpp:179
    job.pixel_samples = static_cast<uint32_t>(o.pixel_samples);
    job.max_depth = o.depth;
    job.monte_carlo_samples = o.mc;
    job.exposure = o.exposure;
    job.inverse_gamma = o.inverse_gamma;
    job.gamma_correction = o.gamma ? 1 : 0;
    std::memcpy(job.background, o.bg, sizeof(o.bg));
    job.seed = o.seed;
    job.n_lights = turner_mesh_light(mesh, &job.light);
    job.camera = cam;
    job.sampling = o.cosine ? TURNER_SAMPLING_COSINE : TURNER_SAMPLING_UNIFORM;
    job.traversal = o.fast ? TURNER_TRAVERSAL_FAST : TURNER_TRAVERSAL_PARITY;
    job.renderer = o.renderer;
    job.shadow_intensity = o.shadow;
    job.max_visibility = o.max_visibility;
    if (o.verbose) {
        std::cerr << "Scene: " << o.scene << "\nImage: " << job.width << "x" << job.height << "\nSamples: "
                  << job.pixel_samples << "\nMax depth: " << job.max_depth << std::endl;
    }

    std::vector<float> image(size_t(job.width) * job.height * 4);
    float* outs[1] = {image.data()};
    turner_stats stats{};
    std::cerr << "Rendering ";
    const auto t0 = clock::now();
    st = turner_render(ctx, &job, 1, outs, &stats, TURNER_HOST_BUFFERS);
    const double render_s = std::chrono::duration<double>(clock::now() - t0).count();
    std::cerr << std::endl;
    if (st != TURNER_OK) {
        std::cerr << "render: " << turner_strerror(st) << std::endl;
        return 1;
    }
    const uint64_t runtime_ms = static_cast<uint64_t>(render_s * 1000);
    std::cerr << "Triangles      : " << turner_kdtree_num_triangles(tree) << std::endl
              << "Kd-Tree Height : " << turner_kdtree_height(tree) << std::endl
              << "Rays           : " << stats.rays << std::endl
              << "Rays (primary) : " << stats.primary_rays << std::endl
              << "Rays/sec       : " << (runtime_ms ? 1000 * stats.rays / runtime_ms : 0) << std::endl
              << "Loading time   : " << load_s << " sec" << std::endl
              << "Rendering time : " << render_s << " sec" << std::endl;

    std::string p3(turner_write_p3(image.data(), job.width, job.height, nullptr, 0), '\0');
    turner_write_p3(image.data(), job.width, job.height, &p3[0], p3.size());
    std::cout << p3 << std::endl;

    turner_destroy(ctx);
    turner_kdtree_free(tree);
    turner_mesh_free(mesh);
    return 0;
}
