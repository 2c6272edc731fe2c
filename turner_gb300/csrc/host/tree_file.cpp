// Tree files: one kd-tree (node words, triangle records, box) in a binary file
// keyed by the content of the triangles it was built from, memory-mapped
// straight into turner_upload_scene.
//
// The reference caches its tree in a fixed-name cereal archive,
// ./kdtree.cache (main.cpp:142-167). The name is not keyed by the scene, so a
// cache left by another scene is loaded silently. Here the key (a 64-bit
// hash of the input triangles) is stored in the header and checked on load,
// the payload carries a checksum, and a cache directory holds one file per
// key. Files are written under a temporary name and renamed into place, so a
// reader never sees a partial file.
//
// Layout (little-endian, as both supported hosts are):
//   offset 0    char[8]   "TRNKDT01"
//          8    uint32    header bytes (128)
//          12   uint32    flags (0)
//          16   uint64    key (turner_mesh_key of the input triangles)
//          24   uint32    node count
//          28   uint32    triangle count
//          32   float[6]  scene box (min xyz, max xyz)
//          56   uint32    tree height
//          60   uint32    reserved (0)
//          64   uint64    payload checksum (word-wise FNV-1a of nodes, then triangles)
//          72   ...       zero up to 128
//   128                   node words, 8 bytes each
//   128 + 8 n_nodes       triangle records, 192 bytes each (Triangle::serialize order)
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include "tree.h"
#include "turner_gpu.h"

namespace {

constexpr char kMagic[8] = {'T', 'R', 'N', 'K', 'D', 'T', '0', '1'};
constexpr uint32_t kHeaderBytes = 128;

struct Header {
    char magic[8];
    uint32_t header_bytes;
    uint32_t flags;
    uint64_t key;
    uint32_t n_nodes;
    uint32_t n_tris;
    float box[6];
    uint32_t height;
    uint32_t reserved;
    uint64_t checksum;
    uint8_t pad[kHeaderBytes - 72];
};
static_assert(sizeof(Header) == kHeaderBytes, "tree file header is 128 bytes");
static_assert(sizeof(turner_triangle) == 192, "triangle record is 48 floats");

constexpr uint64_t kFnvOffset = 0xCBF29CE484222325ULL;
constexpr uint64_t kFnvPrime = 0x100000001B3ULL;

// FNV-1a over 64-bit words (a trailing partial word is zero-padded).
uint64_t fnv_words(uint64_t h, const void* data, size_t bytes) {
    const auto* p = static_cast<const unsigned char*>(data);
    size_t i = 0;
    for (; i + 8 <= bytes; i += 8) {
        uint64_t w;
        std::memcpy(&w, p + i, 8);
        h = (h ^ w) * kFnvPrime;
    }
    if (i < bytes) {
        uint64_t w = 0;
        std::memcpy(&w, p + i, bytes - i);
        h = (h ^ w) * kFnvPrime;
    }
    return h;
}

uint64_t payload_checksum(const uint64_t* nodes, size_t n_nodes, const turner_triangle* tris, size_t n_tris) {
    uint64_t h = fnv_words(kFnvOffset, nodes, n_nodes * sizeof(uint64_t));
    return fnv_words(h, tris, n_tris * sizeof(turner_triangle));
}

bool write_all(int fd, const void* data, size_t bytes) {
    const auto* p = static_cast<const char*>(data);
    while (bytes > 0) {
        const ssize_t w = ::write(fd, p, bytes);
        if (w < 0) {
            if (errno == EINTR) continue;
            return false;
        }
        p += w;
        bytes -= static_cast<size_t>(w);
    }
    return true;
}

std::string cache_path(const char* dir, uint64_t key) {
    char name[32];
    std::snprintf(name, sizeof(name), "%016llx.tkd", static_cast<unsigned long long>(key));
    std::string p(dir);
    if (!p.empty() && p.back() != '/') p += '/';
    return p + name;
}

} // namespace

struct turner_tree_file {
    void* map = nullptr;
    size_t bytes = 0;
    const Header* header = nullptr;
    const uint64_t* nodes = nullptr;
    const turner_triangle* tris = nullptr;
};

extern "C" {

uint64_t turner_mesh_key(const float* vertices, const float* normals, const float* diffuse, uint32_t n_tris) {
    uint64_t h = fnv_words(kFnvOffset, &n_tris, sizeof(n_tris));
    const uint8_t present = static_cast<uint8_t>((vertices ? 1 : 0) | (normals ? 2 : 0) | (diffuse ? 4 : 0));
    h = fnv_words(h, &present, 1);
    if (vertices) h = fnv_words(h, vertices, size_t(n_tris) * 9 * sizeof(float));
    if (normals) h = fnv_words(h, normals, size_t(n_tris) * 9 * sizeof(float));
    if (diffuse) h = fnv_words(h, diffuse, size_t(n_tris) * 4 * sizeof(float));
    return h;
}

int turner_kdtree_save(const turner_kdtree* tree, uint64_t key, const char* path) {
    if (!tree || !path || tree->nodes.empty() || tree->tris.empty()) return TURNER_ERR_INVALID_ARG;
    Header h{};
    std::memcpy(h.magic, kMagic, sizeof(kMagic));
    h.header_bytes = kHeaderBytes;
    h.key = key;
    h.n_nodes = static_cast<uint32_t>(tree->nodes.size());
    h.n_tris = static_cast<uint32_t>(tree->tris.size());
    std::memcpy(h.box, tree->box, sizeof(h.box));
    h.height = tree->height;
    h.checksum = payload_checksum(tree->nodes.data(), tree->nodes.size(), tree->tris.data(), tree->tris.size());
    const std::string tmp = std::string(path) + ".tmp." + std::to_string(static_cast<long>(::getpid()));
    const int fd = ::open(tmp.c_str(), O_WRONLY | O_CREAT | O_TRUNC, 0644);
    if (fd < 0) return TURNER_ERR_INVALID_ARG;
    const bool ok = write_all(fd, &h, sizeof(h)) &&
                    write_all(fd, tree->nodes.data(), tree->nodes.size() * sizeof(uint64_t)) &&
                    write_all(fd, tree->tris.data(), tree->tris.size() * sizeof(turner_triangle));
    const bool closed = ::close(fd) == 0;
    if (!ok || !closed || std::rename(tmp.c_str(), path) != 0) {
        ::unlink(tmp.c_str());
        return TURNER_ERR_INVALID_ARG;
    }
    return TURNER_OK;
}

int turner_tree_file_map(const char* path, uint64_t key, int verify, turner_tree_file** out) {
    if (!path || !out) return TURNER_ERR_INVALID_ARG;
    *out = nullptr;
    const int fd = ::open(path, O_RDONLY);
    if (fd < 0) return TURNER_ERR_INVALID_ARG;
    struct stat st {};
    if (::fstat(fd, &st) != 0 || st.st_size < static_cast<off_t>(kHeaderBytes)) {
        ::close(fd);
        return TURNER_ERR_BAD_SCENE;
    }
    const size_t bytes = static_cast<size_t>(st.st_size);
    void* map = ::mmap(nullptr, bytes, PROT_READ, MAP_PRIVATE, fd, 0);
    ::close(fd);
    if (map == MAP_FAILED) return TURNER_ERR_OUT_OF_MEMORY;
    const auto* h = static_cast<const Header*>(map);
    const size_t want = size_t(kHeaderBytes) + size_t(h->n_nodes) * sizeof(uint64_t) +
                        size_t(h->n_tris) * sizeof(turner_triangle);
    int status = TURNER_OK;
    if (std::memcmp(h->magic, kMagic, sizeof(kMagic)) != 0 || h->header_bytes != kHeaderBytes || h->flags != 0 ||
        h->n_nodes == 0 || h->n_tris == 0 || bytes != want) {
        status = TURNER_ERR_BAD_SCENE;
    } else if (key != 0 && h->key != key) {
        status = TURNER_ERR_BAD_SCENE;
    }
    auto* f = new (std::nothrow) turner_tree_file;
    if (status == TURNER_OK && !f) status = TURNER_ERR_OUT_OF_MEMORY;
    if (status == TURNER_OK) {
        f->map = map;
        f->bytes = bytes;
        f->header = h;
        f->nodes = reinterpret_cast<const uint64_t*>(static_cast<const char*>(map) + kHeaderBytes);
        f->tris = reinterpret_cast<const turner_triangle*>(static_cast<const char*>(map) + kHeaderBytes +
                                                           size_t(h->n_nodes) * sizeof(uint64_t));
        if (verify && payload_checksum(f->nodes, h->n_nodes, f->tris, h->n_tris) != h->checksum) {
            status = TURNER_ERR_BAD_SCENE;
        }
    }
    if (status != TURNER_OK) {
        delete f;
        ::munmap(map, bytes);
        return status;
    }
    *out = f;
    return TURNER_OK;
}

const uint64_t* turner_tree_file_nodes(const turner_tree_file* f, uint32_t* n) {
    if (n) *n = f ? f->header->n_nodes : 0;
    return f ? f->nodes : nullptr;
}

const turner_triangle* turner_tree_file_triangles(const turner_tree_file* f, uint32_t* n) {
    if (n) *n = f ? f->header->n_tris : 0;
    return f ? f->tris : nullptr;
}

const float* turner_tree_file_box(const turner_tree_file* f) { return f ? f->header->box : nullptr; }

uint64_t turner_tree_file_key(const turner_tree_file* f) { return f ? f->header->key : 0; }

void turner_tree_file_unmap(turner_tree_file* f) {
    if (!f) return;
    ::munmap(f->map, f->bytes);
    delete f;
}

int turner_kdtree_load(const char* path, uint64_t key, turner_kdtree** out) {
    if (!path || !out) return TURNER_ERR_INVALID_ARG;
    *out = nullptr;
    turner_tree_file* f = nullptr;
    int st = turner_tree_file_map(path, key, 1, &f);
    if (st != TURNER_OK) return st;
    auto* t = new (std::nothrow) turner_kdtree;
    if (!t) {
        turner_tree_file_unmap(f);
        return TURNER_ERR_OUT_OF_MEMORY;
    }
    try {
        t->nodes.assign(f->nodes, f->nodes + f->header->n_nodes);
        t->tris.assign(f->tris, f->tris + f->header->n_tris);
    } catch (...) {
        delete t;
        turner_tree_file_unmap(f);
        return TURNER_ERR_OUT_OF_MEMORY;
    }
    std::memcpy(t->box, f->header->box, sizeof(t->box));
    t->height = f->header->height;
    turner_tree_file_unmap(f);
    *out = t;
    return TURNER_OK;
}

int turner_kdtree_build_cached(const float* vertices, const float* normals, const float* diffuse, uint32_t n_tris,
                               int threads, const char* cache_dir, turner_kdtree** out, int* from_cache) {
    if (from_cache) *from_cache = 0;
    if (!vertices || !out || n_tris == 0) return TURNER_ERR_INVALID_ARG;
    if (!cache_dir) return turner_kdtree_build(vertices, normals, diffuse, n_tris, threads, out);
    const uint64_t key = turner_mesh_key(vertices, normals, diffuse, n_tris);
    const std::string path = cache_path(cache_dir, key);
    if (turner_kdtree_load(path.c_str(), key, out) == TURNER_OK) {
        if (from_cache) *from_cache = 1;
        return TURNER_OK;
    }
    const int st = turner_kdtree_build(vertices, normals, diffuse, n_tris, threads, out);
    if (st != TURNER_OK) return st;
    ::mkdir(cache_dir, 0755);              // may exist already
    turner_kdtree_save(*out, key, path.c_str());   // a cache that cannot be written is not an error
    return TURNER_OK;
}

} // extern "C"
