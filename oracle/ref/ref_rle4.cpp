/* Host harness around the reference's RLE4 encoder, mip builder and loader.
 *
 * Links src/Rle4.cpp and src/Tree.cpp unmodified and calls
 *   RLE4::compress    (src/Rle4.cpp:52-198)  bit volume -> surface RLE columns,
 *   Tree::get_mipmap  (src/tree.h:23-85)     2x2x2 -> 1 with the >=3-of-8 rule,
 *   RLE4::load        (src/Rle4.cpp:244-384) .rle4 file -> uint2 column table.
 * Test infrastructure only. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include "Core.h"
#include "Rle4.h"
#include "tree.h"

void* bmalloc(int) { return 0; }
void add_pool(void*, int) {}
int cpu_to_gpu_delta = 0;
void gpu_memcpy(void*, void*, int) {}
void cpu_memcpy(void*, void*, int) {}
void* gpu_malloc(int) { return 0; }
extern "C" void create_cuda_1d_texture(char*, int) {}
extern "C" void create_cuda_2d_texture(uint*, int, int) {}

/* bits: voxel bit volume in the reference's layout, bit (i&7) of byte
   (i + j*sx + k*sx*sy) >> 3.  Returns the slab words through *slabs_out
   (malloc'd; free with ref_free) and the per-column offsets in table_out. */
extern "C" int ref_compress(const uint8_t* bits, int sx, int sy, int sz, int mip,
                            uint32_t* table_out, uint16_t** slabs_out, long long* nslabs)
{
    Tree t;
    t.vx = sx; t.vy = sy; t.vz = sz;
    t.voxel = (char*)bits;
    t.voxel_col1 = 0;
    t.voxel_col2 = 0;
    RLE4 r;
    r.init();
    Map4 m = r.compress(t, mip);
    memcpy(table_out, m.map, (size_t)sx * sz * 4);
    *slabs_out = (uint16_t*)m.slabs;
    *nslabs = m.slabs_size;
    free(m.map);
    return 0;
}

extern "C" void ref_free(void* p) { free(p); }

/* Tree::get_mipmap on a bit volume; out must hold (sx/2)*(sy/2)*(sz/2)/8 bytes. */
extern "C" int ref_mipmap(const uint8_t* bits, int sx, int sy, int sz, uint8_t* out)
{
    Tree src;
    src.vx = sx; src.vy = sy; src.vz = sz;
    src.voxel = (char*)bits;
    src.voxel_col1 = 0;
    src.voxel_col2 = 0;
    Tree dst;
    dst.get_mipmap(src);
    memcpy(out, dst.voxel, (size_t)(sx / 2 / 8) * (sy / 2) * (sz / 2));
    free(dst.voxel);
    return 0;
}

/* RLE4::load on a file; copies mip m's uint2 table (2*sx*sz words). */
extern "C" int ref_load_table(const char* path, int m, uint32_t* table_out, int* dims_out)
{
    RLE4 r;
    r.init();
    if (!r.load((char*)path)) return -1;
    if (m >= r.nummaps) return -2;
    dims_out[0] = r.map[m].sx; dims_out[1] = r.map[m].sy; dims_out[2] = r.map[m].sz;
    dims_out[3] = r.map[m].slabs_size; dims_out[4] = r.nummaps;
    memcpy(table_out, r.map[m].map, (size_t)r.map[m].sx * r.map[m].sz * 8);
    r.clear();
    return 0;
}
