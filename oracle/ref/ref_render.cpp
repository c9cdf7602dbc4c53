/* Host harness around the reference's own per-ray raycast.
 *
 * Compiles src/Cuda_Render.h (Render::render_line, src/Cuda_Render.h:96-737)
 * for the host, unmodified, the way src/Cuda_Main.cu:150-181 calls it: one
 * call per column ray x with viewpos/viewrot taken from the ray map.  The
 * differences from the GPU launch are only the ones that make the call
 * well defined:
 *   - each ray gets a private, zeroed occupancy bitmask of res_y/32 words
 *     (the reference slices 31 words per thread out of shared memory,
 *     src/Cuda_Main.cu:172, which aliases the neighbour's word at y>=992);
 *   - the skip map is sized for the (unused) write at src/Cuda_Render.h:112;
 *   - the slab arrays are placed so no array crosses a 4 GiB boundary, which
 *     keeps the 32-bit pointer compare at src/Cuda_Render.h:509,517 exact.
 * Rays run in parallel with OpenMP; each ray writes only its own row.
 *
 * Test infrastructure only: pins the oracle and times the reference. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <stdint.h>
#include <sys/mman.h>
#define IN_CUDA_ENV
#include <cuda_runtime.h>
#include "cutil_math.h"
#include "Core.h"
#include "RayMap.h"
#include "Cuda_Render.h"
#ifdef _OPENMP
#include <omp.h>
#endif

extern int ref_rays_casted_res;
extern int ref_rays_distance;
extern int ref_mip_distance;

/* Copy n bytes into an anonymous mapping that does not straddle a 2^32
   address boundary. */
static void* place_below_4g_boundary(const void* src, size_t n, void** map_base, size_t* map_len)
{
    const size_t four_g = (size_t)1 << 32;
    if (n >= four_g) return NULL;
    size_t len = n + four_g;
    void* base = mmap(NULL, len, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS | MAP_NORESERVE, -1, 0);
    if (base == MAP_FAILED) return NULL;
    uintptr_t p = ((uintptr_t)base + four_g - 1) & ~(uintptr_t)(four_g - 1);
    memcpy((void*)p, src, n);
    *map_base = base;
    *map_len = len;
    return (void*)p;
}

extern "C" int ref_render_size(void) { return (int)sizeof(Render); }

/* raymap: RayMap_GPU bytes from ref_get_ray_map (its map4_gpu/nummaps are
   replaced here).  maps[m]: uint2 column table of mip m (sx*sz entries),
   slabs[m]: u16 slab words.  out: nrays*S words, caller-initialised. */
extern "C" int ref_render_rays(const void* raymap, int nummaps, const int* sx, const int* sy,
                               const int* sz, const uint32_t* const* maps,
                               const uint16_t* const* slabs, const long long* slabs_words,
                               int S, int nrays, int mip_distance, int rays_distance,
                               uint32_t* out, int nthreads)
{
    ref_mip_distance = mip_distance;
    ref_rays_distance = rays_distance;
    Render* r = (Render*)calloc(1, sizeof(Render));
    if (!r) return -1;
    memcpy(&r->ray_map, raymap, sizeof(RayMap_GPU));
    void* bases[16] = {0};
    size_t lens[16] = {0};
    r->ray_map.nummaps = nummaps;
    for (int m = 0; m < nummaps; m++) {
        void* p = place_below_4g_boundary(slabs[m], (size_t)slabs_words[m] * 2 + 64, &bases[m], &lens[m]);
        if (!p) return -2;
        r->ray_map.map4_gpu[m].sx = sx[m];
        r->ray_map.map4_gpu[m].sy = sy[m];
        r->ray_map.map4_gpu[m].sz = sz[m];
        r->ray_map.map4_gpu[m].slabs_size = (int)slabs_words[m];
        r->ray_map.map4_gpu[m].map = (uint*)maps[m];
        r->ray_map.map4_gpu[m].slabs = (ushort*)p;
    }
    r->set_target(S, S, (int*)out);
    size_t skip_bytes = (size_t)6 * (size_t)(nrays + 1) * (size_t)S + 64;
    ushort* skipmap = (ushort*)calloc(1, skip_bytes);
    /* render_line always clears 31 words (src/Cuda_Render.h:263) */
    const int words = S / 32 + 2 > 32 ? S / 32 + 2 : 32;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel
    {
        uint* ycache = (uint*)malloc(sizeof(uint) * words);
#pragma omp for schedule(dynamic, 16)
        for (int x = 0; x < nrays; x++) {
            memset(ycache, 0, sizeof(uint) * words);
            r->render_line(x, ycache, r->ray_map.position, r->ray_map.rotation, S, S,
                           skipmap + (size_t)x * S);
        }
        free(ycache);
    }
    free(skipmap);
    for (int m = 0; m < nummaps; m++) munmap(bases[m], lens[m]);
    free(r);
    return 0;
}
