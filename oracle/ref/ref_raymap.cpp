/* Host harness around the reference's own ray-map builder.
 *
 * Compiles src/RayMap.h (RayMap::get_ray_map, src/RayMap.h:98-402) with
 * src/VecMath.h and inc/mathlib unmodified.  The only inputs it sets are the
 * ones src/main.cpp:769-779 (compute_ray_map) sets: border, ray limit,
 * position and rotation.  The result is copied out as the RayMap_GPU POD
 * (src/RayMap.h:16-54) that src/Cuda_Main.cu:183 receives.
 *
 * Test infrastructure only: used to pin the oracle's restatement. */
#include <stdio.h>
#include <string.h>
#include <math.h>
#include "Core.h"
#include "RayMap.h"

int ref_rays_casted_res = RAYS_CASTED;
int ref_rays_distance = 80000;
int ref_mip_distance = SCREEN_SIZE_X;

extern "C" int ref_raymap_gpu_size(void) { return (int)sizeof(RayMap_GPU); }

extern "C" void ref_get_ray_map(float px, float py, float pz, float rx, float ry,
                                float rz, float border, int maxres, void* out)
{
    ref_rays_casted_res = 4 * maxres;
    RayMap* rm = new RayMap();
    /* The reference keeps ray_map as a zero-initialised global
       (src/RayMap.cpp:4); start every call from that state. */
    memset((void*)static_cast<RayMap_GPU*>(rm), 0, sizeof(RayMap_GPU));
    rm->set_border(border);
    rm->set_ray_limit(RAYS_CASTED_RES);
    rm->get_ray_map(vec3f(px, py, pz), vec3f(rx, ry, rz));
    memcpy(out, static_cast<RayMap_GPU*>(rm), sizeof(RayMap_GPU));
    delete rm;
}
