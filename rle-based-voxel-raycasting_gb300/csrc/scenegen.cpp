// Seeded synthetic scenes in the .rle4 layout.
//
// Ground: a toroidally tiling fBm value-noise heightfield.  Caves and
// overhangs: two octaves of 3D simplex noise (Gustavson's formulation of
// Perlin's simplex noise) thresholded inside a height band.  Colour: RGB565
// from a height palette plus a 2D value-noise tint and a per-voxel jitter,
// all integer arithmetic.  Everything is float/integer arithmetic without
// libm calls, compiled with -ffp-contract=off, so every host produces the
// same bytes for the same parameters.
//
// Encoding follows RLE4::compress (src/Rle4.cpp:52-198): a voxel is stored
// only if it is solid and fewer than 27 of the in-bounds voxels of its 3x3x3
// neighbourhood are solid; surface runs are written as u16 headers
// (solid << 10 | skip), skip > 1023 split into 1023-skip headers, solid > 63
// split into 63-solid headers; per column [run count][colour count][headers]
// [colours].  Mip levels follow Tree::get_mipmap (src/tree.h:23-85): a voxel
// of level m+1 is solid when at least 3 of its 8 children are.  The
// implementation is column-bitset based (64 voxels per word) rather than the
// reference's per-voxel loops.
#include <cstdlib>
#include <cstring>
#include <vector>

#include "rle_internal.h"
#include "scenegen_math.h"

namespace {

inline uint64_t splitmix64(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

}  // namespace

namespace rle {

// The generator's permutation table: 0..255 shuffled by a splitmix64
// Fisher-Yates pass, repeated twice.
void scenegen_perm(uint64_t seed, uint8_t* perm) {
    uint8_t p[256];
    for (int i = 0; i < 256; i++) p[i] = static_cast<uint8_t>(i);
    uint64_t s = seed ^ 0x5DEECE66Dull;
    for (int i = 255; i > 0; i--) {
        const int j = static_cast<int>(splitmix64(s) % static_cast<uint64_t>(i + 1));
        const uint8_t t = p[i];
        p[i] = p[j];
        p[j] = t;
    }
    for (int i = 0; i < 512; i++) perm[i] = p[i & 255];
}

gen::Consts scenegen_consts(const rle_scenegen_params& q) {
    gen::Consts c;
    c.sx = q.sx;
    c.sy = q.sy;
    c.sz = q.sz;
    c.octaves = q.octaves;
    c.base_period = q.base_period;
    c.caves = q.caves;
    c.height_min = q.height_min;
    c.height_max = q.height_max;
    c.cave_y0 = q.cave_y0;
    c.cave_y1 = q.cave_y1;
    c.cave_threshold = q.cave_threshold;
    c.cave_period = q.cave_period;
    c.seed32 = static_cast<uint32_t>(q.seed ^ (q.seed >> 32));
    return c;
}

rle_status scenegen_check(const rle_scenegen_params* p) {
    if (!p) return RLE_ERR_INVALID_ARG;
    auto pow2 = [](int v) { return v >= 8 && (v & (v - 1)) == 0; };
    if (!pow2(p->sx) || !pow2(p->sz) || p->sx > 65536 || p->sz > 65536 || p->sy < 64 || p->sy > 1024 ||
        (p->sy & 63) != 0 || p->nummaps < 1 || p->nummaps > RLE_MAX_MIPS || p->octaves < 1 ||
        p->base_period < 1 || (p->base_period & (p->base_period - 1)) != 0 || p->base_period > p->sx ||
        p->base_period > p->sz || !(p->height_max >= p->height_min) || !(p->cave_period > 0.0f)) {
        rle::set_error("rle_scenegen: invalid parameters (sx/sz powers of two >= 8, sy multiple of 64 <= 1024, "
                       "base_period a power of two <= sx, sz)");
        return RLE_ERR_INVALID_ARG;
    }
    if ((p->sx >> (p->nummaps - 1)) < 1 || (p->sz >> (p->nummaps - 1)) < 1 || (p->sy >> (p->nummaps - 1)) < 1) {
        rle::set_error("rle_scenegen: too many mip levels for the grid");
        return RLE_ERR_INVALID_ARG;
    }
    return RLE_OK;
}

}  // namespace rle

namespace {

rle_status check_params(const rle_scenegen_params* p) { return rle::scenegen_check(p); }

struct Gen {
    rle::gen::Consts c;
    uint8_t perm[512];
    int words;  // u64 words per column at level 0

    explicit Gen(const rle_scenegen_params& q) : c(rle::scenegen_consts(q)), words(q.sy / 64) {
        rle::scenegen_perm(q.seed, perm);
    }

    // Level-0 solid bits of column (x, z): u64 words, bit j of word j/64.
    // The renderer's column axis points down (a run's height index grows
    // towards the ground, src/Cuda_Render.h:534,556 pick the near/far cell
    // edge by that sign), so storage index j is sy-1 minus the height y.
    void column(int x, int z, uint64_t* out) const {
        std::memset(out, 0, sizeof(uint64_t) * words);
        const int h = rle::gen::ground_height(c, x, z);
        for (int y = 0; y < h; y++) {
            const int j = c.sy - 1 - y;
            out[j >> 6] |= 1ull << (j & 63);
        }
        if (c.caves) {
            int y0 = static_cast<int>(c.cave_y0), y1 = static_cast<int>(c.cave_y1);
            if (y0 < 1) y0 = 1;
            if (y1 > h) y1 = h;
            for (int y = y0; y < y1; y++) {
                const int j = c.sy - 1 - y;
                if (rle::gen::carved(c, perm, x, y, z)) out[j >> 6] &= ~(1ull << (j & 63));
            }
        }
    }

    // RGB565 colour of level-0 voxel (x, j, z), j counted down from the top.
    uint16_t colour(int x, int j, int z) const { return rle::gen::colour(c, rle::gen::tint(c, x, z), x, j, z); }
};

// One level as column bitsets: cols[(z*sx + x) * words + w].
struct BitLevel {
    int sx = 0, sy = 0, sz = 0, words = 0;
    std::vector<uint64_t> cols;
    const uint64_t* col(int x, int z) const { return &cols[(static_cast<size_t>(z) * sx + x) * words]; }
    bool solid(int x, int y, int z) const { return (col(x, z)[y >> 6] >> (y & 63)) & 1; }
};

// Compact the bits at positions 4k (k = 0..15) into 16 consecutive bits.
inline uint32_t compact_nibble_lsbs(uint64_t v) {
    v &= 0x1111111111111111ull;
    v = (v | (v >> 3)) & 0x0303030303030303ull;
    v = (v | (v >> 6)) & 0x000F000F000F000Full;
    v = (v | (v >> 12)) & 0x000000FF000000FFull;
    v = (v | (v >> 24)) & 0x000000000000FFFFull;
    return static_cast<uint32_t>(v);
}

inline uint32_t spread16(uint32_t v) {
    v &= 0xFFFF;
    v = (v | (v << 8)) & 0x00FF00FFu;
    v = (v | (v << 4)) & 0x0F0F0F0Fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

// Level m+1 from level m: child solid iff >= 3 of its 8 children are solid.
void halve(const BitLevel& a, BitLevel& b) {
    b.sx = a.sx / 2;
    b.sy = a.sy / 2;
    b.sz = a.sz / 2;
    b.words = (b.sy + 63) / 64;
    b.cols.assign(static_cast<size_t>(b.sx) * b.sz * b.words, 0);
    const uint64_t m55 = 0x5555555555555555ull, m33 = 0x3333333333333333ull;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < b.sz; k++) {
        for (int i = 0; i < b.sx; i++) {
            uint64_t* dst = &b.cols[(static_cast<size_t>(k) * b.sx + i) * b.words];
            const uint64_t* c[4] = {a.col(2 * i, 2 * k), a.col(2 * i + 1, 2 * k), a.col(2 * i, 2 * k + 1),
                                    a.col(2 * i + 1, 2 * k + 1)};
            for (int w = 0; w < a.words; w++) {
                uint64_t sa = 0, sb = 0;
                for (int q = 0; q < 4; q++) {
                    const uint64_t v = c[q][w];
                    const uint64_t pc = (v & m55) + ((v >> 1) & m55);  // 2-bit pair counts
                    sa += pc & m33;                                      // even pairs, 4-bit fields
                    sb += (pc >> 2) & m33;                               // odd pairs
                }
                const uint64_t ga = (sa + 0x5555555555555555ull) >> 3;  // nibble >= 3 -> bit 0 of nibble
                const uint64_t gb = (sb + 0x5555555555555555ull) >> 3;
                const uint32_t bits = spread16(compact_nibble_lsbs(ga)) | (spread16(compact_nibble_lsbs(gb)) << 1);
                // child j = 32*w + p for pair p of this word
                const int j0 = 32 * w;
                if (j0 >= b.sy) break;
                dst[j0 >> 6] |= static_cast<uint64_t>(bits) << (j0 & 63);
            }
            if (b.sy & 63) dst[b.words - 1] &= (1ull << (b.sy & 63)) - 1;
        }
    }
}

// Surface bits of column (x, z): solid with fewer than 27 solid in-bounds
// neighbours (out-of-bounds neighbours count as missing).
void surface_bits(const BitLevel& L, int x, int z, uint64_t* out) {
    const int W = L.words;
    const uint64_t* self = L.col(x, z);
    const bool edge = x == 0 || z == 0 || x == L.sx - 1 || z == L.sz - 1;
    if (edge) {
        for (int w = 0; w < W; w++) out[w] = self[w];
        return;
    }
    uint64_t inner[16];
    for (int w = 0; w < W; w++) inner[w] = ~0ull;
    for (int dz = -1; dz <= 1; dz++)
        for (int dx = -1; dx <= 1; dx++) {
            const uint64_t* n = L.col(x + dx, z + dz);
            for (int w = 0; w < W; w++) {
                const uint64_t below = (n[w] << 1) | (w > 0 ? n[w - 1] >> 63 : 0);      // bit y = n[y-1]
                const uint64_t above = (n[w] >> 1) | (w + 1 < W ? n[w + 1] << 63 : 0);  // bit y = n[y+1]
                inner[w] &= n[w] & below & above;
            }
        }
    // y = 0 and y = sy-1 have an out-of-bounds neighbour: never interior.
    inner[0] &= ~1ull;
    const int top = L.sy - 1;
    inner[top >> 6] &= ~(1ull << (top & 63));
    for (int w = 0; w < W; w++) out[w] = self[w] & ~inner[w];
}

// Emit one column: returns words written (or counts them when dst == null).
int encode_column(const uint64_t* surf, int sy, const Gen& g, int x, int z, int mip, uint16_t* dst) {
    int n_head = 0, n_col = 0;
    uint16_t heads[1100];
    uint16_t cols[1024];
    int skip = 0, solid = 0;
    const int scale_shift = mip;
    for (int j = 0; j < sy + 1; j++) {
        const bool store = j < sy && ((surf[j >> 6] >> (j & 63)) & 1);
        if (store && dst) cols[n_col] = g.colour(x << scale_shift, j << scale_shift, z << scale_shift);
        if (store) n_col++;
        if (solid > 0 && !store) {
            while (skip > 1023) {
                heads[n_head++] = 1023;
                skip -= 1023;
            }
            while (solid > 63) {
                heads[n_head++] = static_cast<uint16_t>(63 * 1024 + (skip & 1023));
                solid -= 63;
                skip = 0;
            }
            heads[n_head++] = static_cast<uint16_t>((solid & 63) * 1024 + (skip & 1023));
            solid = 0;
            skip = 0;
        }
        if (store) solid++;
        else skip++;
    }
    if (dst) {
        dst[0] = static_cast<uint16_t>(n_head);
        dst[1] = static_cast<uint16_t>(n_col);
        std::memcpy(dst + 2, heads, sizeof(uint16_t) * n_head);
        std::memcpy(dst + 2 + n_head, cols, sizeof(uint16_t) * n_col);
    }
    return 2 + n_head + n_col;
}

void build_levels(const rle_scenegen_params& p, const Gen& g, std::vector<BitLevel>& lv) {
    lv.resize(p.nummaps);
    BitLevel& L0 = lv[0];
    L0.sx = p.sx;
    L0.sy = p.sy;
    L0.sz = p.sz;
    L0.words = p.sy / 64;
    L0.cols.assign(static_cast<size_t>(p.sx) * p.sz * L0.words, 0);
#pragma omp parallel for schedule(dynamic, 4)
    for (int z = 0; z < p.sz; z++)
        for (int x = 0; x < p.sx; x++) g.column(x, z, &L0.cols[(static_cast<size_t>(z) * p.sx + x) * L0.words]);
    for (int m = 1; m < p.nummaps; m++) halve(lv[m - 1], lv[m]);
}

}  // namespace

extern "C" rle_status rle_scenegen_default(int sx, int sy, int sz, uint64_t seed, int caves,
                                           rle_scenegen_params* out) {
    if (!out) return RLE_ERR_INVALID_ARG;
    std::memset(out, 0, sizeof(*out));
    out->sx = sx;
    out->sy = sy;
    out->sz = sz;
    out->seed = seed;
    out->nummaps = 4;
    const float k = static_cast<float>(sy) / 256.0f;
    out->height_min = 32.0f * k;
    out->height_max = 224.0f * k;
    out->octaves = 6;
    int period = 256;  // at least 4 lattice cells across the map
    while (period > 1 && (period * 4 > sx || period * 4 > sz)) period >>= 1;
    out->base_period = period;
    out->caves = caves;
    out->cave_y0 = 64.0f * k;
    out->cave_y1 = 200.0f * k;
    out->cave_threshold = 0.20f;  // ~8 runs per column at 2048^2 x 256
    out->cave_period = 48.0f * k;
    return check_params(out);
}

extern "C" rle_status rle_scenegen_rle4(const rle_scenegen_params* p, void** bytes, size_t* nbytes) {
    if (!bytes || !nbytes) return RLE_ERR_INVALID_ARG;
    *bytes = nullptr;
    *nbytes = 0;
    rle_status st = check_params(p);
    if (st != RLE_OK) return st;
    try {
        const Gen g(*p);
        std::vector<BitLevel> lv;
        build_levels(*p, g, lv);
        // pass 1: words per column; pass 2: fill
        std::vector<std::vector<uint64_t>> starts(p->nummaps);
        size_t total = 4;
        for (int m = 0; m < p->nummaps; m++) {
            const BitLevel& L = lv[m];
            std::vector<uint64_t>& st_m = starts[m];
            st_m.assign(static_cast<size_t>(L.sx) * L.sz + 1, 0);
#pragma omp parallel for schedule(dynamic, 4)
            for (int z = 0; z < L.sz; z++) {
                uint64_t surf[16];
                for (int x = 0; x < L.sx; x++) {
                    surface_bits(L, x, z, surf);
                    st_m[static_cast<size_t>(z) * L.sx + x + 1] = encode_column(surf, L.sy, g, x, z, m, nullptr);
                }
            }
            for (size_t c = 1; c < st_m.size(); c++) st_m[c] += st_m[c - 1];
            if (st_m.back() > 0x7fffffffull) {
                rle::set_error("rle_scenegen: level %d needs %llu words (> 2^31-1, the .rle4 int limit)", m,
                               static_cast<unsigned long long>(st_m.back()));
                return RLE_ERR_CAPACITY;
            }
            total += 16 + st_m.back() * 2;
        }
        uint8_t* buf = static_cast<uint8_t*>(std::malloc(total));
        if (!buf) return RLE_ERR_NO_MEMORY;
        size_t ofs = 0;
        auto put32 = [&](int32_t v) {
            std::memcpy(buf + ofs, &v, 4);
            ofs += 4;
        };
        put32(p->nummaps);
        for (int m = 0; m < p->nummaps; m++) {
            const BitLevel& L = lv[m];
            put32(L.sx);
            put32(L.sy);
            put32(L.sz);
            put32(static_cast<int32_t>(starts[m].back()));
            uint16_t* words = reinterpret_cast<uint16_t*>(buf + ofs);
            const std::vector<uint64_t>& st_m = starts[m];
#pragma omp parallel for schedule(dynamic, 4)
            for (int z = 0; z < L.sz; z++) {
                uint64_t surf[16];
                for (int x = 0; x < L.sx; x++) {
                    surface_bits(L, x, z, surf);
                    encode_column(surf, L.sy, g, x, z, m, words + st_m[static_cast<size_t>(z) * L.sx + x]);
                }
            }
            ofs += st_m.back() * 2;
        }
        *bytes = buf;
        *nbytes = ofs;
        return RLE_OK;
    } catch (const std::bad_alloc&) {
        rle::set_error("rle_scenegen: out of host memory");
        return RLE_ERR_NO_MEMORY;
    }
}

extern "C" rle_status rle_scenegen_dense(const rle_scenegen_params* p, int mip, uint8_t* bits, uint16_t* colours) {
    rle_status st = check_params(p);
    if (st != RLE_OK) return st;
    if (mip < 0 || mip >= p->nummaps) return RLE_ERR_INVALID_ARG;
    try {
        const Gen g(*p);
        std::vector<BitLevel> lv;
        build_levels(*p, g, lv);
        const BitLevel& L = lv[mip];
        const size_t sxy = static_cast<size_t>(L.sx) * L.sy;
        if (bits) std::memset(bits, 0, (static_cast<size_t>(L.sx) * L.sy * L.sz + 7) / 8);
        for (int k = 0; k < L.sz; k++)
            for (int j = 0; j < L.sy; j++)
                for (int i = 0; i < L.sx; i++) {
                    const size_t idx = i + j * static_cast<size_t>(L.sx) + k * sxy;
                    if (bits && L.solid(i, j, k)) bits[idx >> 3] |= static_cast<uint8_t>(1u << (i & 7));
                    if (colours) colours[idx] = g.colour(i << mip, j << mip, k << mip);
                }
        return RLE_OK;
    } catch (const std::bad_alloc&) {
        return RLE_ERR_NO_MEMORY;
    }
}
