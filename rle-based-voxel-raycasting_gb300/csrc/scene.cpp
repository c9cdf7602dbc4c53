// Scene loading: .rle4 bytes -> validated column tables -> device residency.
//
// The .rle4 format is the reference's (RLE4::save, src/Rle4.cpp:220-242):
// int nummaps, then per level int sx, sy, sz, slabs_size and slabs_size u16
// words.  Each column holds [run_count][colour_count][run headers][colours];
// columns follow each other x fastest, then z.  The column directory is the
// uint2 table RLE4::load builds (src/Rle4.cpp:285-314): {offset of the
// column's first word, run_count | first_header << 16}.
//
// Unlike the reference, every column is validated before upload: run and
// colour counts inside the level's words, the colours the run headers claim
// no more than the column stores, and level m exactly level 0 halved m times.
// A scene that loads can therefore never make the raycast read outside its
// arrays.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "rle_internal.h"

namespace rle {

namespace {
thread_local char g_error[512];

bool pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }

template <typename T>
bool read_at(const uint8_t* p, size_t n, size_t* ofs, T* v) {
    if (*ofs + sizeof(T) > n) return false;
    std::memcpy(v, p + *ofs, sizeof(T));
    *ofs += sizeof(T);
    return true;
}
}  // namespace

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_error, sizeof(g_error), fmt, ap);
    va_end(ap);
}

void clear_error() { g_error[0] = 0; }

rle_status parse_rle4(const void* bytes, size_t nbytes, HostLevel* levels, int* nummaps) {
    const uint8_t* p = static_cast<const uint8_t*>(bytes);
    size_t ofs = 0;
    int32_t n = 0;
    if (!p || !read_at(p, nbytes, &ofs, &n)) {
        set_error(".rle4: missing header");
        return RLE_ERR_FORMAT;
    }
    if (n < 1 || n > RLE_MAX_MIPS) {
        set_error(".rle4: %d levels (1..%d supported)", n, RLE_MAX_MIPS);
        return RLE_ERR_FORMAT;
    }
    for (int m = 0; m < n; m++) {
        int32_t sx, sy, sz;
        uint32_t words;  // the reference's int slabs_size, read unsigned
        if (!read_at(p, nbytes, &ofs, &sx) || !read_at(p, nbytes, &ofs, &sy) ||
            !read_at(p, nbytes, &ofs, &sz) || !read_at(p, nbytes, &ofs, &words)) {
            set_error(".rle4: truncated header of level %d", m);
            return RLE_ERR_FORMAT;
        }
        if (!pow2(sx) || !pow2(sz) || sy < 1 || sy > 65535 || sx > 65536 || sz > 65536) {
            set_error(".rle4: level %d is %dx%dx%d (x, z must be powers of two <= 65536)", m, sx, sy, sz);
            return RLE_ERR_FORMAT;
        }
        if (m > 0 && (sx != (levels[0].sx >> m) || sz != (levels[0].sz >> m))) {
            set_error(".rle4: level %d is %dx%d, expected level 0 halved %d times", m, sx, sz, m);
            return RLE_ERR_FORMAT;
        }
        const size_t bytes_needed = static_cast<size_t>(words) * 2;
        if (ofs + bytes_needed > nbytes || ofs + bytes_needed < ofs) {
            set_error(".rle4: level %d claims %u words, file too short", m, words);
            return RLE_ERR_FORMAT;
        }
        if ((ofs & 1) != 0) {
            set_error(".rle4: misaligned slab words");
            return RLE_ERR_FORMAT;
        }
        levels[m].sx = sx;
        levels[m].sy = sy;
        levels[m].sz = sz;
        levels[m].words = words;
        levels[m].slabs = reinterpret_cast<const uint16_t*>(p + ofs);
        ofs += bytes_needed;
    }
    *nummaps = n;
    return RLE_OK;
}

rle_status build_table(const HostLevel& lv, uint32_t* table, uint64_t* run_headers,
                       uint64_t* surface_voxels, int* top_index) {
    const uint16_t* s = lv.slabs;
    const uint64_t words = lv.words;
    uint64_t ofs = 0, heads = 0, vox = 0;
    uint64_t top = UINT64_MAX;  // smallest index of a stored voxel
    for (int z = 0; z < lv.sz; z++) {
        for (int x = 0; x < lv.sx; x++) {
            if (ofs + 2 > words) {
                set_error(".rle4: column (%d,%d) starts past the level's %llu words", x, z,
                          static_cast<unsigned long long>(words));
                return RLE_ERR_FORMAT;
            }
            const uint32_t runs = s[ofs], colours = s[ofs + 1];
            const uint64_t end = ofs + 2 + runs + static_cast<uint64_t>(colours);
            if (end > words) {
                set_error(".rle4: column (%d,%d) runs past the level's words", x, z);
                return RLE_ERR_FORMAT;
            }
            // Colours the run headers address (solid counts) must exist.
            uint64_t claimed = 0, depth = 0;
            bool found = false;
            for (uint32_t r = 0; r < runs; r++) {
                const uint32_t h = s[ofs + 2 + r];
                claimed += h >> 10;
                if (!found) {
                    depth += h & 1023u;
                    if (h >> 10) {
                        found = true;
                        if (depth < top) top = depth;
                    }
                }
            }
            if (claimed > colours) {
                set_error(".rle4: column (%d,%d) runs need %llu colours, %u stored", x, z,
                          static_cast<unsigned long long>(claimed), colours);
                return RLE_ERR_FORMAT;
            }
            if (ofs > 0xffffffffull) {
                set_error(".rle4: level exceeds 2^32 words");
                return RLE_ERR_CAPACITY;
            }
            // first header: the word after the counts, as RLE4::load reads it
            // even for an empty column (src/Rle4.cpp:301)
            const uint32_t first = (ofs + 2 < words) ? s[ofs + 2] : 0u;
            const size_t c = static_cast<size_t>(z) * lv.sx + x;
            table[2 * c + 0] = static_cast<uint32_t>(ofs);
            table[2 * c + 1] = runs + (first << 16);
            heads += runs;
            vox += colours;
            ofs = end;
        }
    }
    if (run_headers) *run_headers = heads;
    if (surface_voxels) *surface_voxels = vox;
    if (top_index) *top_index = top > 0x7fffffffull ? 0x7fffffff : static_cast<int>(top);
    return RLE_OK;
}

}  // namespace rle

namespace {

rle_status cuda_fail(cudaError_t e, const char* what) {
    rle::set_error("%s: %s", what, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? RLE_ERR_NO_MEMORY : RLE_ERR_CUDA;
}

void release(rle_scene* s) {
    if (!s) return;
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(s->device);
    for (auto& lv : s->lv) {
        if (lv.d_table) cudaFree(lv.d_table);
        if (lv.d_slabs) cudaFree(lv.d_slabs);
        lv.d_table = nullptr;
        lv.d_slabs = nullptr;
    }
    if (prev >= 0) cudaSetDevice(prev);
    delete s;
}

}  // namespace

extern "C" rle_status rle_scene_load_memory(const void* bytes, size_t nbytes, int device, rle_scene** out) {
    if (!bytes || !out) {
        rle::set_error("rle_scene_load_memory: null argument");
        return RLE_ERR_INVALID_ARG;
    }
    *out = nullptr;
    rle::HostLevel levels[RLE_MAX_MIPS];
    int nummaps = 0;
    rle_status st = rle::parse_rle4(bytes, nbytes, levels, &nummaps);
    if (st != RLE_OK) return st;

    // Validate every level and build its table on the host before any
    // device work, so malformed input never reaches the GPU.
    std::vector<std::vector<uint32_t>> tables(nummaps);
    uint64_t heads0 = 0, vox0 = 0;
    long long top_all = 0x7fffffffLL;
    for (int m = 0; m < nummaps; m++) {
        try {
            tables[m].resize(2 * static_cast<size_t>(levels[m].sx) * levels[m].sz);
        } catch (...) {
            rle::set_error("rle_scene_load_memory: out of host memory");
            return RLE_ERR_NO_MEMORY;
        }
        uint64_t heads = 0, vox = 0;
        int top = 0;
        st = rle::build_table(levels[m], tables[m].data(), &heads, &vox, &top);
        if (st != RLE_OK) return st;
        if (m == 0) {
            heads0 = heads;
            vox0 = vox;
        }
        // a voxel of level m at index j spans level-0 indices j << m onwards
        const long long top0 = static_cast<long long>(top) << m;
        if (top0 < top_all) top_all = top0;
    }

    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
    if (device < 0 || device >= ndev) {
        rle::set_error("rle_scene_load_memory: device %d of %d", device, ndev);
        return RLE_ERR_INVALID_ARG;
    }
    rle_scene* s = new (std::nothrow) rle_scene();
    if (!s) return RLE_ERR_NO_MEMORY;
    s->device = device;
    s->nummaps = nummaps;
    int prev = -1;
    cudaGetDevice(&prev);
    e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        delete s;
        return cuda_fail(e, "cudaSetDevice");
    }
    s->run_headers = heads0;
    s->top_index = static_cast<int>(top_all);
    s->height = levels[0].sy;
    s->surface_voxels = vox0;
    for (int m = 0; m < nummaps && st == RLE_OK; m++) {
        const rle::HostLevel& hl = levels[m];
        rle::Level& lv = s->lv[m];
        lv.sx = hl.sx;
        lv.sy = hl.sy;
        lv.sz = hl.sz;
        lv.words = hl.words;
        const size_t cols = static_cast<size_t>(hl.sx) * hl.sz;
        const std::vector<uint32_t>& table = tables[m];
        const size_t tbytes = cols * 8;
        // 16 bytes of zero padding after the words keep 16-byte vector loads
        // of a column's last header group inside the allocation.
        const size_t sbytes = static_cast<size_t>(hl.words) * 2 + rle::kSlabPadBytes;
        if ((e = cudaMalloc(&lv.d_table, tbytes)) != cudaSuccess) { st = cuda_fail(e, "cudaMalloc(table)"); break; }
        if ((e = cudaMalloc(&lv.d_slabs, sbytes)) != cudaSuccess) { st = cuda_fail(e, "cudaMalloc(slabs)"); break; }
        if ((e = cudaMemcpy(lv.d_table, table.data(), tbytes, cudaMemcpyHostToDevice)) != cudaSuccess) { st = cuda_fail(e, "cudaMemcpy(table)"); break; }
        if ((e = cudaMemset(lv.d_slabs, 0, sbytes)) != cudaSuccess) { st = cuda_fail(e, "cudaMemset(slabs)"); break; }
        if (hl.words && (e = cudaMemcpy(lv.d_slabs, hl.slabs, static_cast<size_t>(hl.words) * 2, cudaMemcpyHostToDevice)) != cudaSuccess) { st = cuda_fail(e, "cudaMemcpy(slabs)"); break; }
        s->device_bytes += tbytes + sbytes;
    }
    if (prev >= 0) cudaSetDevice(prev);
    if (st != RLE_OK) {
        release(s);
        return st;
    }
    *out = s;
    return RLE_OK;
}

extern "C" rle_status rle_scene_load_file(const char* path, int device, rle_scene** out) {
    if (!path || !out) {
        rle::set_error("rle_scene_load_file: null argument");
        return RLE_ERR_INVALID_ARG;
    }
    FILE* f = std::fopen(path, "rb");
    if (!f) {
        rle::set_error("rle_scene_load_file: cannot open %s", path);
        return RLE_ERR_IO;
    }
    std::fseek(f, 0, SEEK_END);
    long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (n < 0) {
        std::fclose(f);
        rle::set_error("rle_scene_load_file: cannot size %s", path);
        return RLE_ERR_IO;
    }
    void* buf = std::malloc(static_cast<size_t>(n) + 1);
    if (!buf) {
        std::fclose(f);
        return RLE_ERR_NO_MEMORY;
    }
    size_t got = std::fread(buf, 1, static_cast<size_t>(n), f);
    std::fclose(f);
    if (got != static_cast<size_t>(n)) {
        std::free(buf);
        rle::set_error("rle_scene_load_file: short read of %s", path);
        return RLE_ERR_IO;
    }
    rle_status st = rle_scene_load_memory(buf, got, device, out);
    std::free(buf);
    return st;
}

extern "C" rle_status rle_scene_free(rle_scene* scene) {
    if (!scene) return RLE_ERR_INVALID_ARG;
    release(scene);
    return RLE_OK;
}

extern "C" rle_status rle_scene_get_info(const rle_scene* s, rle_scene_info* out) {
    if (!s || !out) return RLE_ERR_INVALID_ARG;
    std::memset(out, 0, sizeof(*out));
    out->device = s->device;
    out->nummaps = s->nummaps;
    for (int m = 0; m < s->nummaps; m++) {
        out->sx[m] = s->lv[m].sx;
        out->sy[m] = s->lv[m].sy;
        out->sz[m] = s->lv[m].sz;
        out->slab_words[m] = s->lv[m].words;
    }
    out->device_bytes = s->device_bytes;
    out->run_headers = s->run_headers;
    out->surface_voxels = s->surface_voxels;
    return RLE_OK;
}

extern "C" rle_status rle_scene_copy_level(const rle_scene* s, int mip, uint32_t* table, uint16_t* slabs) {
    if (!s || mip < 0 || mip >= s->nummaps) return RLE_ERR_INVALID_ARG;
    const rle::Level& lv = s->lv[mip];
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(s->device);
    cudaError_t e = cudaSuccess;
    if (table) e = cudaMemcpy(table, lv.d_table, static_cast<size_t>(lv.sx) * lv.sz * 8, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && slabs && lv.words)
        e = cudaMemcpy(slabs, lv.d_slabs, static_cast<size_t>(lv.words) * 2, cudaMemcpyDeviceToHost);
    if (prev >= 0) cudaSetDevice(prev);
    if (e != cudaSuccess) return cuda_fail(e, "rle_scene_copy_level");
    return RLE_OK;
}

extern "C" const char* rle_last_error(void) { return rle::g_error; }

extern "C" const char* rle_status_string(rle_status s) {
    switch (s) {
        case RLE_OK: return "RLE_OK";
        case RLE_ERR_INVALID_ARG: return "RLE_ERR_INVALID_ARG";
        case RLE_ERR_IO: return "RLE_ERR_IO";
        case RLE_ERR_FORMAT: return "RLE_ERR_FORMAT";
        case RLE_ERR_CUDA: return "RLE_ERR_CUDA";
        case RLE_ERR_NO_MEMORY: return "RLE_ERR_NO_MEMORY";
        case RLE_ERR_CAPACITY: return "RLE_ERR_CAPACITY";
        case RLE_ERR_TIMEOUT: return "RLE_ERR_TIMEOUT";
        case RLE_ERR_CANCELLED: return "RLE_ERR_CANCELLED";
        case RLE_ERR_UNSUPPORTED: return "RLE_ERR_UNSUPPORTED";
    }
    return "RLE_ERR_UNKNOWN";
}

extern "C" const char* rle_version(void) { return "rle_gb300 1.0 sm_103a"; }

extern "C" void rle_host_free(void* p) { std::free(p); }
