/* Build shim for compiling the reference raycaster on a case-sensitive host.
 *
 * The reference includes "Core.h" while the file on disk is src/core.h.
 * This shim includes the real header unchanged and then turns the
 * compile-time geometry macros of src/core.h:3-10 into runtime variables
 * so one host build of the reference can be driven at any resolution.
 * The feature switches (FLOATING_HORIZON, XFLOATING_HORIZON, SHAREMEMCLIP)
 * stay exactly as src/core.h:24-32 sets them. */
#pragma once
#include "core.h"
#undef RAYS_CASTED_RES
#undef RAYS_DISTANCE
#undef MIP_DISTANCE
extern int ref_rays_casted_res;   /* RAYS_CASTED_RES: 4 x maxres */
extern int ref_rays_distance;     /* RAYS_DISTANCE: z_far in DDA units */
extern int ref_mip_distance;      /* MIP_DISTANCE: first LOD switch */
#define RAYS_CASTED_RES (ref_rays_casted_res)
#define RAYS_DISTANCE (ref_rays_distance)
#define MIP_DISTANCE (ref_mip_distance)
/* src/core.h:60-78 defines byte/ushort/uint/uchar as macros; functional
   casts such as uint(slabs) (src/Cuda_Render.h:517, src/tree.h:736) are
   ill-formed for g++ with a two-word macro.  Typedefs name the same types. */
#undef byte
#undef ushort
#undef uint
#undef uchar
typedef unsigned char byte;
typedef unsigned short ushort;
typedef unsigned int uint;
typedef unsigned char uchar;
