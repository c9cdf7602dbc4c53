/* CPU oracle for the RLE column raycaster (test infrastructure only).
 *
 * Restates, operation for operation, the reference's host and device code for
 * the render path so that results can be compared bit for bit.  Built with
 * -ffp-contract=off: every float operation below is one IEEE single-precision
 * operation in the order the reference's C++ evaluates it.  Function calls
 * follow the overloads the reference's C++ resolves to (sinf/cosf/acosf/sqrtf
 * for float arguments).  Conversions from float to int saturate and send NaN
 * to 0, which is what sm_103a and aarch64 do; x86 returns INT_MIN instead, so
 * values outside the int range (degenerate poses only) are the one place the
 * reference built on x86 and this restatement may differ.
 *
 * Parity is pinned against the reference compiled for the host (oracle/ref). */
#include "rle_oracle.h"

#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static inline int f2i(float f)
{
    if (f != f) return 0;
    if (f >= 2147483648.0f) return INT_MAX;
    if (f < -2147483648.0f) return INT_MIN;
    return (int)f;
}

/* ======================================================================= */
/* Scene format                                                            */
/* ======================================================================= */

static inline int bit_at(const uint8_t* bits, long long idx, int i)
{
    return (bits[idx >> 3] >> (i & 7)) & 1;
}

/* Reference colour word for a surface voxel: src/Rle4.cpp:134-161 with no
 * material bits (col1 == NULL).  The normal is the negated centroid of the
 * solid 3x3x3 neighbours, normalised as vec3f::normalize (src/VecMath.h:166-177). */
static uint16_t reference_colour(int mx, int my, int mz, int i, int k, int scale)
{
    float cx = (float)(-mx), cy = (float)my, cz = (float)(-mz);
    float square = cx * cx + cy * cy + cz * cz;
    if (square <= 0.00001f) {
        cx = 1; cy = 0; cz = 0;
    } else {
        float len = 1.0f / sqrtf(square);
        cx *= len; cy *= len; cz *= len;
    }
    (void)cx; (void)cz;
    int ny = f2i(127.0f * cy + 128.0f);
    if (ny > 255) ny = 255;
    if (ny < 0) ny = 0;
    /* mat == 0 branch of src/Rle4.cpp:155 */
    ny = (ny * (((((i * scale) ^ (k * scale)) >> 4) & 15) + 15)) >> 5;
    if (ny > 255) ny = 255;
    if (ny < 0) ny = 0;
    return (uint16_t)ny;
}

typedef struct { uint16_t* p; long long n, cap; } u16vec;

static int u16_push(u16vec* v, uint16_t w)
{
    if (v->n == v->cap) {
        long long cap = v->cap ? v->cap * 2 : 4096;
        uint16_t* p = (uint16_t*)realloc(v->p, (size_t)cap * 2);
        if (!p) return -1;
        v->p = p;
        v->cap = cap;
    }
    v->p[v->n++] = w;
    return 0;
}

int orc_encode_mip(const uint8_t* bits, const uint16_t* colours, int sx, int sy, int sz, int mip,
                   uint32_t* column_start, uint16_t** slabs_out, long long* nwords)
{
    const int scale = 1 << mip;
    const long long sxy = (long long)sx * sy;
    u16vec slab = {0, 0, 0};
    uint16_t* texture = (uint16_t*)malloc(sizeof(uint16_t) * (size_t)(sy + 1));
    if (!texture) return -1;
    /* columns x fastest, then z (src/Rle4.cpp:78-79) */
    for (int k = 0; k < sz; k++)
        for (int i = 0; i < sx; i++) {
            column_start[i + k * sx] = (uint32_t)slab.n;
            long long slab_len = slab.n;
            u16_push(&slab, 0);
            long long tex_len = slab.n;
            u16_push(&slab, 0);
            int skip = 0, solid = 0, ntex = 0;
            for (int j = 0; j < sy + 1; j++) {
                int f = 0;
                long long idx = i + j * (long long)sx + k * sxy;
                if (j < sy) f = bit_at(bits, idx, i);
                int store = 0;
                if (f) {
                    /* surface test: fewer than 27 solid voxels in the
                       in-bounds 3x3x3 neighbourhood (src/Rle4.cpp:100-132) */
                    int cnt = 0, mx = 0, my = 0, mz = 0;
                    for (int a = -1; a < 2; a++)
                        for (int b = -1; b < 2; b++)
                            for (int c = -1; c < 2; c++) {
                                int x = i + a, y = j + b, z = k + c;
                                if (x < 0 || y < 0 || z < 0 || x >= sx || y >= sy || z >= sz) continue;
                                if (bit_at(bits, x + y * (long long)sx + z * sxy, x)) {
                                    mx += a; my += b; mz += c; cnt++;
                                }
                            }
                    if (cnt < 27) {
                        texture[ntex++] = colours ? colours[idx] : reference_colour(mx, my, mz, i, k, scale);
                        store = 1;
                    }
                }
                /* flush a finished surface run (src/Rle4.cpp:166-182) */
                if (solid > 0 && !store) {
                    while (skip > 1023) { u16_push(&slab, 1023); skip -= 1023; }
                    while (solid > 63) {
                        u16_push(&slab, (uint16_t)(63 * 1024 + (skip & 1023)));
                        solid -= 63;
                        skip = 0;
                    }
                    u16_push(&slab, (uint16_t)((solid & 63) * 1024 + (skip & 1023)));
                    solid = 0;
                    skip = 0;
                }
                if (store) solid++; else skip++;
            }
            slab.p[slab_len] = (uint16_t)(slab.n - (slab_len + 2));
            slab.p[tex_len] = (uint16_t)ntex;
            for (int t = 0; t < ntex; t++) u16_push(&slab, texture[t]);
        }
    free(texture);
    *slabs_out = slab.p;
    *nwords = slab.n;
    return 0;
}

int orc_mipmap(const uint8_t* bits, int sx, int sy, int sz, uint8_t* out)
{
    const int hx = sx / 2, hy = sy / 2, hz = sz / 2;
    const long long hxy = (long long)hx * hy;
    const long long sxy = (long long)sx * sy;
    memset(out, 0, (size_t)(hx / 8) * hy * hz);
    for (int i = 0; i < hx; i++)
        for (int j = 0; j < hy; j++)
            for (int k = 0; k < hz; k++) {
                int cnt = 0;
                for (int a = 0; a < 2; a++)
                    for (int b = 0; b < 2; b++)
                        for (int c = 0; c < 2; c++) {
                            int ii = i * 2 + a, jj = j * 2 + b, kk = k * 2 + c;
                            cnt += bit_at(bits, ii + jj * (long long)sx + kk * sxy, ii);
                        }
                if (cnt >= 3) {
                    long long idx = i + j * (long long)hx + k * hxy;
                    out[idx >> 3] |= (uint8_t)(1 << (i & 7));
                }
            }
    return 0;
}

int orc_build_table(const uint16_t* slabs, long long nwords, int sx, int sz, uint32_t* table)
{
    long long ofs = 0;
    for (int z = 0; z < sz; z++)
        for (int x = 0; x < sx; x++) {
            if (ofs + 1 >= nwords) return -1;
            uint32_t count = slabs[ofs];
            uint32_t first = 0;
            /* the reference reads one word past an empty column here
               (src/Rle4.cpp:301); the value is never used for count == 0 */
            if (ofs + 2 < nwords) first = slabs[ofs + 2];
            table[(x + (long long)z * sx) * 2 + 0] = (uint32_t)ofs;
            table[(x + (long long)z * sx) * 2 + 1] = count + (first << 16);
            ofs += (long long)slabs[ofs] + slabs[ofs + 1] + 2;
            if (ofs > nwords) return -1;
        }
    return 0;
}

/* ======================================================================= */
/* Ray map: src/RayMap.h:98-402                                            */
/* ======================================================================= */

static inline orc_v3 v3(float x, float y, float z) { orc_v3 r = {x, y, z}; return r; }
static inline orc_v3 vadd(orc_v3 a, orc_v3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline orc_v3 vsub(orc_v3 a, orc_v3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline orc_v3 vmul(orc_v3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline orc_v3 vdiv(orc_v3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
/* vec3f::dot: a.x*x + a.y*y + a.z*z with `this` on the right (src/VecMath.h:62) */
static inline float vdot(orc_v3 self, orc_v3 a) { return a.x * self.x + a.y * self.y + a.z * self.z; }
static inline float vlen(orc_v3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }

typedef float mat44[4][4];

static void m_ident(mat44 m)
{
    memset(m, 0, sizeof(mat44));
    m[0][0] = m[1][1] = m[2][2] = m[3][3] = 1.0f;
}

/* _matrix44::rotate_x / rotate_y (inc/mathlib/_matrix44.h:529-561) */
static void m_rotate_x(mat44 m, float a)
{
    float c = cosf(a), s = sinf(a);
    for (int i = 0; i < 4; i++) {
        float mi1 = m[i][1], mi2 = m[i][2];
        m[i][1] = mi1 * c + mi2 * -s;
        m[i][2] = mi1 * s + mi2 * c;
    }
}

static void m_rotate_y(mat44 m, float a)
{
    float c = cosf(a), s = sinf(a);
    for (int i = 0; i < 4; i++) {
        float mi0 = m[i][0], mi2 = m[i][2];
        m[i][0] = mi0 * c + mi2 * s;
        m[i][2] = mi0 * -s + mi2 * c;
    }
}

/* operator*(matrix44, vector3) (inc/mathlib/_matrix44.h:863-869) */
static orc_v3 m_mul(mat44 m, orc_v3 v)
{
    return v3(m[0][0] * v.x + m[1][0] * v.y + m[2][0] * v.z + m[3][0],
              m[0][1] * v.x + m[1][1] * v.y + m[2][1] * v.z + m[3][1],
              m[0][2] * v.x + m[1][2] * v.y + m[2][2] * v.z + m[3][2]);
}

/* _matrix44::invert_simpler (inc/mathlib/_matrix44.h:431-442) */
static void m_invert_simpler(mat44 m)
{
    float t;
    t = m[0][1]; m[0][1] = m[1][0]; m[1][0] = t;
    t = m[0][2]; m[0][2] = m[2][0]; m[2][0] = t;
    t = m[1][2]; m[1][2] = m[2][1]; m[2][1] = t;
    float m30 = -(m[0][0] * m[3][0] + m[1][0] * m[3][1] + m[2][0] * m[3][2]);
    float m31 = -(m[0][1] * m[3][0] + m[1][1] * m[3][1] + m[2][1] * m[3][2]);
    m[3][2] = -(m[0][2] * m[3][0] + m[1][2] * m[3][1] + m[2][2] * m[3][2]);
    m[3][1] = m31;
    m[3][0] = m30;
}

static void m_set_rows(mat44 m, orc_v3 r0, orc_v3 r1, orc_v3 r2, orc_v3 r3)
{
    /* _matrix44::set(_vector4 x4) with _vector4(const _vector3&) (w = 1) */
    m[0][0] = r0.x; m[0][1] = r0.y; m[0][2] = r0.z; m[0][3] = 1.0f;
    m[1][0] = r1.x; m[1][1] = r1.y; m[1][2] = r1.z; m[1][3] = 1.0f;
    m[2][0] = r2.x; m[2][1] = r2.y; m[2][2] = r2.z; m[2][3] = 1.0f;
    m[3][0] = r3.x; m[3][1] = r3.y; m[3][2] = r3.z; m[3][3] = 1.0f;
}

/* int(maxres*v) -/+ safety, back to float / maxres (src/RayMap.h:231-232) */
static inline float snap(float v, int maxres, int add)
{
    return (float)(f2i((float)maxres * v) + add) / (float)maxres;
}

static inline int clamp_res(int maxres, float a, float b)
{
    int r = f2i((float)maxres * fabsf(a - b));
    if (a - b > 0) r = 0;
    if (r > maxres * 3) r = maxres * 3;
    return r;
}

void orc_raymap_build(orc_raymap* rm, float px, float py, float pz, float rx, float ry, float rz,
                      float border, int maxres, float fov_scale, int samples, int mip_distance,
                      int z_far)
{
    memset(rm, 0, sizeof(*rm));
    rm->border = border;
    rm->clip_min = border;
    rm->clip_max = 1 - border;
    rm->rotation = v3(rx, ry, rz);
    rm->position = v3(px, py, pz);
    rm->samples = samples;
    rm->mip_distance = mip_distance;
    rm->z_far = z_far;
    rm->fov_scale = fov_scale;

    const float t = fov_scale;
    orc_v3 p[6] = {v3(t, t, 1), v3(-t, t, 1), v3(-t, -t, 1), v3(t, -t, 1), v3(0, 0, 0), v3(0, 0, 0)};

    mat44 m;
    m_ident(m);
    m_rotate_x(m, rx);
    m_rotate_y(m, ry);
    m[3][0] += 3.0f; /* translate(vector3(3,2,0)) */
    m[3][1] += 2.0f;
    m[3][2] += 0.0f;
    for (int i = 0; i < 5; i++) p[i] = m_mul(m, p[i]);

    /* vanishing point of the down vector (src/RayMap.h:135-141) */
    orc_v3 down = v3(0, -1, 0);
    orc_v3 view = vsub(vdiv(vadd(p[0], p[2]), 2.0f), p[4]);
    float angle;
    {
        float dot = view.x * down.x + view.y * down.y + view.z * down.z;
        float len = vlen(view) * vlen(down);
        if (len == 0) len = 0.00001f;
        float input = dot / len;
        if (input < -1) input = -1;
        if (input > 1) input = 1;
        angle = acosf(input);
    }
    float alpha = (float)M_PI / 2 - angle;
    float scale = 1 / sinf(alpha);
    p[5] = vadd(p[4], vmul(down, scale));

    /* frustum plane basis (src/RayMap.h:145-161) */
    orc_v3 a = vsub(p[1], p[0]), b = vsub(p[3], p[0]);
    orc_v3 nrm = v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
    orc_v3 d1 = vsub(p[1], p[0]), d2 = vsub(p[3], p[0]), d3 = nrm, d4 = p[0];
    d1 = vmul(d1, 1 / (d1.x * d1.x + d1.y * d1.y + d1.z * d1.z));
    d2 = vmul(d2, 1 / (d2.x * d2.x + d2.y * d2.y + d2.z * d2.z));
    d3 = vmul(d3, 1 / (d3.x * d3.x + d3.y * d3.y + d3.z * d3.z));
    mat44 to2d;
    m_set_rows(to2d, d1, d2, d3, d4);
    memcpy(rm->to3d, to2d, sizeof(mat44));
    m_invert_simpler(to2d);
    for (int i = 0; i < 6; i++) rm->p_2d[i] = m_mul(to2d, p[i]);
    rm->vanishing_point_2d = rm->p_2d[5];

    rm->maxres = maxres;
    const float ys_min = border, ys_max = 1 - border;
    const orc_v3 plist[4] = {v3(-1, -1, 0), v3(1, -1, 0), v3(1, 1, 0), v3(-1, 1, 0)};
    const orc_v3 plist2[4] = {v3(0, ys_min, 0), v3(1, ys_min, 0), v3(1, ys_max, 0), v3(0, ys_max, 0)};
    rm->p_2d[5].z = 0;
    const orc_v3 c = rm->p_2d[5];
    orc_v3* pn = rm->p_no;

    /* upper fan (src/RayMap.h:209-240) */
    if (c.y > border) {
        float s = fabsf(c.y - border);
        pn[0] = vadd(c, vmul(plist[0], s));
        pn[1] = vadd(c, vmul(plist[1], s));
        orc_v3 in = pn[1];
        if (c.x > 1) { if (pn[1].x > 1) pn[1].x = 1; }
        else if (vdot(vsub(pn[0], c), vsub(plist2[2], c)) > 0)
            pn[1] = vadd(c, vmul(vsub(plist2[2], c), fabsf((plist2[0].y - c.y) / (plist2[2].y - c.y))));
        if (c.x < 0) { if (pn[0].x < 0) pn[0].x = 0; }
        else if (vdot(vsub(in, c), vsub(plist2[3], c)) > 0)
            pn[0] = vadd(c, vmul(vsub(plist2[3], c), fabsf((plist2[1].y - c.y) / (plist2[3].y - c.y))));
        pn[0].y = pn[1].y = plist2[0].y;
        pn[0].x = snap(pn[0].x, maxres, -2);
        pn[1].x = snap(pn[1].x, maxres, +2);
        rm->res[0] = clamp_res(maxres, pn[0].x, pn[1].x);
        rm->p_ofs_min[0] = pn[0].x;
        rm->p_ofs_max[0] = pn[1].x;
    }
    /* lower fan (src/RayMap.h:243-277) */
    if (c.y < 1 - border) {
        float s = fabsf(c.y - 1 + border);
        pn[2] = vadd(c, vmul(plist[3], s));
        pn[3] = vadd(c, vmul(plist[2], s));
        orc_v3 in = pn[2];
        if (c.x < 0) { if (pn[2].x < 0) pn[2].x = 0; }
        else if (vdot(vsub(pn[3], c), vsub(plist2[0], c)) > 0)
            pn[2] = vadd(c, vmul(vsub(plist2[0], c), fabsf((plist2[2].y - c.y) / (plist2[0].y - c.y))));
        if (c.x > 1) { if (pn[3].x > 1) pn[3].x = 1; }
        else {
            orc_v3 delta = vsub(plist2[1], c);
            if (vdot(vsub(in, c), delta) > 0)
                pn[3] = vadd(c, vmul(delta, fabsf((plist2[3].y - c.y) / delta.y)));
        }
        pn[2].y = pn[3].y = plist2[2].y;
        pn[2].x = snap(pn[2].x, maxres, -2);
        pn[3].x = snap(pn[3].x, maxres, +2);
        rm->res[1] = clamp_res(maxres, pn[2].x, pn[3].x);
        rm->p_ofs_min[1] = pn[2].x;
        rm->p_ofs_max[1] = pn[3].x;
    }
    /* left fan (src/RayMap.h:280-313) */
    if (c.x > 0) {
        float s = fabsf(c.x);
        pn[4] = vadd(c, vmul(plist[0], s));
        pn[5] = vadd(c, vmul(plist[3], s));
        orc_v3 in = pn[5];
        if (c.y > 1 - border) { if (pn[5].y > 1 - border) pn[5].y = 1 - border; }
        else if (vdot(vsub(pn[4], c), vsub(plist2[2], c)) > 0)
            pn[5] = vadd(c, vmul(vsub(plist2[2], c), fabsf((plist2[3].x - c.x) / (plist2[2].x - c.x))));
        if (c.y < border) { if (pn[4].y < border) pn[4].y = border; }
        else if (vdot(vsub(in, c), vsub(plist2[1], c)) > 0)
            pn[4] = vadd(c, vmul(vsub(plist2[1], c), fabsf((plist2[0].x - c.x) / (plist2[1].x - c.x))));
        pn[4].x = pn[5].x = 0;
        pn[4].y = snap(pn[4].y, maxres, -2);
        pn[5].y = snap(pn[5].y, maxres, +2);
        rm->res[2] = clamp_res(maxres, pn[4].y, pn[5].y);
        rm->p_ofs_min[2] = pn[4].y;
        rm->p_ofs_max[2] = pn[5].y;
    }
    /* right fan (src/RayMap.h:316-352) */
    if (c.x < 1) {
        float s = fabsf(1 - c.x);
        pn[6] = vadd(c, vmul(plist[1], s));
        pn[7] = vadd(c, vmul(plist[2], s));
        orc_v3 in = pn[7];
        if (c.y > 1 - border) { if (pn[7].y > 1 - border) pn[7].y = 1 - border; }
        else if (vdot(vsub(pn[6], c), vsub(plist2[3], c)) > 0)
            pn[7] = vadd(c, vmul(vsub(plist2[3], c), fabsf((plist2[2].x - c.x) / (plist2[3].x - c.x))));
        if (c.y < border) { if (pn[6].y < border) pn[6].y = border; }
        else if (vdot(vsub(in, c), vsub(plist2[0], c)) > 0)
            pn[6] = vadd(c, vmul(vsub(plist2[0], c), fabsf((plist2[1].x - c.x) / (plist2[0].x - c.x))));
        pn[6].x = pn[7].x = 1;
        pn[6].y = snap(pn[6].y, maxres, -2);
        pn[7].y = snap(pn[7].y, maxres, +2);
        rm->res[3] = clamp_res(maxres, pn[6].y, pn[7].y);
        rm->p_ofs_min[3] = pn[6].y;
        rm->p_ofs_max[3] = pn[7].y;
    }
    rm->p4 = p[4];
    rm->map_line_count = rm->res[0] + rm->res[1] + rm->res[2] + rm->res[3];
}

int orc_raybuf_rows(const orc_raymap* rm) { return 4 * rm->maxres; }

int orc_rays_to_render(const orc_raymap* rm)
{
    int n = rm->map_line_count, rows = orc_raybuf_rows(rm);
    return n < rows ? n : rows;
}

/* ======================================================================= */
/* Raycast: Render::render_line, src/Cuda_Render.h:96-737                   */
/* ======================================================================= */

/* Render::LineScale / ClipLine (src/Cuda_Render.h:39-65) */
static float line_scale(orc_v3 input, orc_v3 center, float clip_max, float clip_min)
{
    float scale_x = 1, scale_y = 1;
    if (center.x > 1) scale_x = (1 - input.x) / (center.x - input.x);
    if (center.x < 0) scale_x = input.x / (input.x - center.x);
    if (center.y > clip_max) scale_y = (clip_max - input.y) / (center.y - input.y);
    if (center.y < clip_min) scale_y = (-clip_min + input.y) / (input.y - center.y);
    return (scale_x < scale_y) ? scale_x : scale_y;
}

static void clip_line(orc_v3* p1, orc_v3* p2, float clip_max, float clip_min)
{
    float s;
    orc_v3 c1, c2;
    s = line_scale(*p1, *p2, clip_max, clip_min);
    c2 = vadd(*p1, vmul(vsub(*p2, *p1), s));
    s = line_scale(*p2, *p1, clip_max, clip_min);
    c1 = vadd(*p2, vmul(vsub(*p1, *p2), s));
    *p1 = c1;
    *p2 = c2;
}

/* MatMul with the to3d rows (src/Cuda_Render.h:67-73) */
static orc_v3 mat_mul(const float m[4][4], orc_v3 v)
{
    return v3(m[0][0] * v.x + m[1][0] * v.y + m[2][0] * v.z + m[3][0],
              m[0][1] * v.x + m[1][1] * v.y + m[2][1] * v.z + m[3][1],
              m[0][2] * v.x + m[1][2] * v.y + m[2][2] * v.z + m[3][2]);
}

static inline int mask_get(const uint32_t* m, int y) { return (m[y >> 5] >> (y & 31)) & 1u; }
static inline void mask_set(uint32_t* m, int y) { m[y >> 5] |= 1u << (y & 31); }

static void render_line(const orc_raymap* rm, const orc_mip* mips, int nummaps, int x,
                        uint32_t* row, float* drow, orc_hit* hrow, orc_counters* cnt,
                        uint32_t* mask)
{
    const int res_x = rm->samples, res_y = rm->samples;
    const float res_x2 = (float)(res_x / 2);
    const float res_y2 = (float)(res_y / 2);
    const orc_v3 viewpos = rm->position, viewrot = rm->rotation;

    /* ---- per-ray setup: quadrant, 2D line, 3D direction (:129-172) ---- */
    int rays[4];
    rays[0] = rm->res[0];
    rays[1] = rm->res[1] + rays[0];
    rays[2] = rm->res[2] + rays[1];
    rays[3] = rm->res[3] + rays[2];
    int quadrant = 0;
    if (x >= rays[2]) quadrant = 3;
    else if (x >= rays[1]) quadrant = 2;
    else if (x >= rays[0]) quadrant = 1;
    float quadrant_ofs = (float)x;
    if (quadrant >= 1) quadrant_ofs -= (float)rays[quadrant - 1];
    float quadrant_num = (float)rm->res[quadrant];
    float a = quadrant_ofs / quadrant_num;
    const int j = quadrant;
    orc_v3 p1 = rm->p_2d[5];
    orc_v3 p2 = vadd(rm->p_no[j * 2], vmul(vsub(rm->p_no[j * 2 + 1], rm->p_no[j * 2]), a));
    clip_line(&p1, &p2, rm->clip_max, rm->clip_min);
    orc_v3 p1_3d = mat_mul(rm->to3d, vmul(p1, 4.0f));
    orc_v3 p2_3d = mat_mul(rm->to3d, vmul(p2, 4.0f));
    orc_v3 delta = vsub(vmul(vadd(p1_3d, p2_3d), 0.5f), rm->p4);
    delta.y = 0;
    {
        /* cutil normalize with the host rsqrtf = 1.0f/sqrtf (inc/cutil_math.h:58-60, 1184-1188) */
        float inv = 1.0f / sqrtf(delta.x * delta.x + delta.y * delta.y + delta.z * delta.z);
        delta = vmul(delta, inv);
    }
    {
        /* vec3f_rot_y (src/Cuda_Render.h:75-80) */
        float cm = cosf(-viewrot.y), sm = sinf(-viewrot.y);
        float xx = cm * delta.x + sm * delta.z;
        float zz = cm * delta.z - sm * delta.x;
        delta.x = xx;
        delta.z = zz;
    }
    const float ray_x = delta.x, ray_z = delta.z;
    const orc_v3 start2d = p1, end2d = p2;
    const int vertical = 1 - (j >> 1);

    /* ---- render state (:177-182) ---- */
    int mip_lvl = 0;
    int y_clip_min = 0, y_clip_max = res_y - 1;
    const int z_far = rm->z_far;
    float dz = (float)(1 << mip_lvl);
    int mapswitch = rm->mip_distance;

    const float sin_x = sinf(rm->rotation.x), cos_x = cosf(rm->rotation.x);
    const float sin_y = sinf(rm->rotation.y), cos_y = cosf(rm->rotation.y);

    /* ---- reverse texturing and screen clipping (:203-250) ---- */
    int reverse = 0;
    if (vertical && ray_z <= 0) reverse = 1;
    if (!vertical && ray_x <= 0 && sin_x > 0) reverse = 1;
    if (!vertical && ray_x > 0 && sin_x < 0) reverse = 1;
    const float focal = res_x2 / rm->fov_scale;
    float res_x2_mul_reverse = reverse ? -focal : focal;
    if (vertical) res_x2_mul_reverse = -res_x2_mul_reverse;

    int q1x, q1y, q2x, q2y;
    int p_add = reverse ? 1 : -2;
    q1x = f2i((float)res_x * start2d.x) + p_add;
    q1y = f2i((float)res_y * start2d.y) + p_add;
    q2x = f2i((float)res_x * end2d.x) - p_add;
    q2y = f2i((float)res_y * end2d.y) - p_add;
    if (q1x < 0) q1x = 0;
    if (q1x >= res_x) q1x = res_x - 1;
    if (q1y < 0) q1y = 0;
    if (q1y >= res_y) q1y = res_y - 1;
    if (q2x < 0) q2x = 0;
    if (q2x >= res_x) q2x = res_x - 1;
    if (q2y < 0) q2y = 0;
    if (q2y >= res_y) q2y = res_y - 1;
    if (q1y == q2y) return;
    y_clip_min = res_x - 1 - q1x;
    y_clip_max = res_x - 1 - q2x;
    if (vertical) {
        y_clip_min = res_y - 1 - q1y;
        y_clip_max = res_y - 1 - q2y;
    }
    if (reverse) {
        y_clip_min = res_y - 1 - y_clip_min;
        y_clip_max = res_y - 1 - y_clip_max;
    }
    if (y_clip_min > y_clip_max) {
        int tmp = y_clip_min;
        y_clip_min = y_clip_max;
        y_clip_max = tmp;
    }
    if (y_clip_min >= y_clip_max) return;

    /* ---- clear the row to sky (:255-264) ---- */
    for (int n = y_clip_min; n <= y_clip_max; n++) {
        row[n] = 0xff8844u;
        if (drow) drow[n] = INFINITY;
        if (hrow) hrow[n].flags = 2;
    }

    /* ---- DDA init (:270-304) ---- */
    float dir_x = ray_x * cos_y + ray_z * sin_y;
    float dir_y = ray_x * sin_y - ray_z * cos_y;
    float fix_x_f = -1, fix_y_f = -1, sign_x = -1, sign_y = -1;
    float frac_x = viewpos.x - (float)f2i(viewpos.x);
    float frac_y = viewpos.z - (float)f2i(viewpos.z);
    if (dir_x >= 0) { fix_x_f = 0; sign_x = 1; frac_x = 1 - frac_x; }
    if (dir_y >= 0) { fix_y_f = 0; sign_y = 1; frac_y = 1 - frac_y; }
    float grad0_y = dir_y / fabsf(dir_x), grad0_x = sign_x;
    float grad1_x = dir_x / fabsf(dir_y), grad1_y = sign_y;
    float isect0_x = grad0_x * frac_x, isect0_y = grad0_y * frac_x;
    float isect1_x = grad1_x * frac_y, isect1_y = grad1_y * frac_y;
    float grad_dist0 = sqrtf(grad0_x * grad0_x + grad0_y * grad0_y);
    float grad_dist1 = sqrtf(grad1_x * grad1_x + grad1_y * grad1_y);
    float dds_dist0 = sqrtf(isect0_x * isect0_x + isect0_y * isect0_y);
    float dds_dist1 = sqrtf(isect1_x * isect1_x + isect1_y * isect1_y);
    float pos_before_x = 0, pos_before_y = 0, dds_dist_before = 0;
    float pos_x = 0, pos_y = 0, dds_dist_now = 0;
    int index = 0, index_before = 0;

    int gridx = mips[0].sx, gridz = mips[0].sz;
    const float pos3d_z_add = sin_x;
    float pos3d_y_add = vertical ? cos_x : 0;
    pos3d_y_add *= res_x2_mul_reverse;
    const uint32_t* map_ptr = mips[0].table;
    const uint16_t* slab_ptr = mips[0].slabs;
    float z = 0;
    float y_map_switch = viewpos.y;
    /* mapswitch * (0.25*(4-abs(viewrot.x))): float subtract, double product (:335) */
    mapswitch = (int)((double)mapswitch * (0.25 * (double)(4.0f - fabsf(viewrot.x))));

    /* ---- main loop (:339-734) ---- */
    for (;;) {
        while (z > (float)mapswitch || (double)y_map_switch > 512.0) {
            y_map_switch = (float)((double)y_map_switch * 0.5);
            if (mip_lvl < nummaps - 1) {
                mip_lvl++;
                gridx >>= 1;
                gridz >>= 1;
                map_ptr = mips[mip_lvl].table;
                slab_ptr = mips[mip_lvl].slabs;
            }
            grad0_x *= 2; grad0_y *= 2;
            grad1_x *= 2; grad1_y *= 2;
            grad_dist0 *= 2; grad_dist1 *= 2;
            mapswitch *= 2;
            dz *= 2;
        }
        z += dz;
        if (z > (float)z_far) return;
        if (y_clip_min >= y_clip_max) return;

        dds_dist_before = dds_dist_now;
        pos_before_x = pos_x;
        pos_before_y = pos_y;
        index_before = index;
        if (dds_dist1 < dds_dist0) {
            dds_dist_now = dds_dist1;
            index = 1;
            dds_dist1 += grad_dist1;
            pos_x = isect1_x; pos_y = isect1_y;
            isect1_x += grad1_x;
            isect1_y += grad1_y;
        } else {
            dds_dist_now = dds_dist0;
            index = 0;
            pos_x = isect0_x; pos_y = isect0_y;
            dds_dist0 += grad_dist0;
            isect0_x += grad0_x;
            isect0_y += grad0_y;
        }
        if (cnt) cnt->cells++;
        int fix_x = f2i((float)(1 - index_before) * fix_x_f);
        int fix_z = f2i((float)index_before * fix_y_f);
        float dds_dist_delta = dds_dist_now - dds_dist_before;
        float vs_x = ray_x * dds_dist_before;
        float vs_z = ray_z * dds_dist_before;
        int voxel_x = f2i(viewpos.x + pos_before_x) + fix_x;
        int voxel_z = f2i(viewpos.z + pos_before_y) + fix_z;
        int vx = (voxel_x >> mip_lvl) & (gridx - 1);
        int vz = (voxel_z >> mip_lvl) & (gridz - 1);
        const float mountain = viewpos.y;
        float correct_x = ray_x * dds_dist_delta;
        float correct_z = ray_z * dds_dist_delta;
        float pos3d_z = cos_x * vs_z + sin_x * mountain;
        float pos3d_y = vertical ? cos_x * mountain - sin_x * vs_z : vs_x;
        pos3d_y *= res_x2_mul_reverse;

        /* clip top (:467) */
        if (pos3d_z * res_y2 + pos3d_y <= pos3d_z * (float)y_clip_min) continue;

        const uint32_t* entry = map_ptr + 2 * ((long long)vx + (long long)vz * gridx);
        uint32_t slab_offset = entry[0];
        uint32_t len_first = entry[1];
        uint16_t slen = (uint16_t)len_first;
        if (cnt) cnt->fetched++;

        float corr_zz = cos_x * correct_z;
        float corr_yy = vertical ? -sin_x * correct_z : correct_x;
        corr_yy *= res_x2_mul_reverse;

        int sti_general = 0, sti_skip = 0;
        uint16_t sti = (uint16_t)(len_first >> 16);
        const uint16_t* slabs = slab_ptr + 2 + slab_offset;
        const uint16_t* send = slabs + slen;
        const uint16_t* first = slabs;
        float tex = 0;

        for (; slabs < send; ++slabs) {
            if (slabs > first) {
                sti = *slabs;
                if (cnt) cnt->headers++;
            }
            sti_skip = sti >> 10;
            sti_general += (sti & 1023) << mip_lvl;
            if (sti_skip == 0) continue;
            int texture = (int)tex;
            tex += (float)sti_skip;
            sti_skip <<= mip_lvl;
            float sgs = (float)sti_general; /* sti_general_sti_skip: run bottom */
            sti_general += sti_skip;
            if (cnt) cnt->runs++;

            float czz1 = pos3d_z, cyy1 = pos3d_y;
            if (mountain + sgs >= 0) { czz1 += corr_zz; cyy1 += corr_yy; }
            float pos3d_z1 = czz1 + pos3d_z_add * sgs;
            if (pos3d_z1 <= 0) continue;
            float pos3d_y1 = cyy1 + pos3d_y_add * sgs;
            int scr_y2 = f2i(res_y2 + pos3d_y1 / pos3d_z1);
            if (scr_y2 <= y_clip_min) break;

            float czz2 = pos3d_z, cyy2 = pos3d_y;
            if (mountain + (float)sti_general < 0) { czz2 += corr_zz; cyy2 += corr_yy; }
            float pos3d_z2 = czz2 + pos3d_z_add * (float)sti_general;
            if (pos3d_z2 <= 0) continue;
            float pos3d_y2 = cyy2 + pos3d_y_add * (float)sti_general;
            int scr_y1 = f2i(res_y2 + pos3d_y2 / pos3d_z2 - 1);
            if (scr_y1 >= y_clip_max) continue;

            /* floating horizon (:563-580) */
            if (scr_y2 >= y_clip_max) {
                scr_y2 = y_clip_max;
                y_clip_max = scr_y1;
            }
            if (scr_y1 <= y_clip_min) {
                scr_y1 = y_clip_min;
                y_clip_min = scr_y2;
                while (y_clip_max > y_clip_min && mask_get(mask, y_clip_min)) ++y_clip_min;
            }
            /* occupancy bitmask (:639-640) */
            int y = scr_y1;
            while (y < scr_y2 && mask_get(mask, y)) ++y;
            if (y >= scr_y2) continue;

            /* perspective-correct interpolation (:645-680) */
            float pos3d_z1r = pos3d_z + pos3d_z_add * sgs;
            float pos3d_y1r = pos3d_y + pos3d_y_add * sgs;
            float pos3d_z2r = pos3d_z + pos3d_z_add * (float)sti_general;
            float pos3d_y2r = pos3d_y + pos3d_y_add * (float)sti_general;
            float scr_y2r = res_y2 + pos3d_y1r / pos3d_z1r;
            float scr_y1r = res_y2 + pos3d_y2r / pos3d_z2r;
            float u1z = tex / pos3d_z2r;
            float u2dz = (float)texture / pos3d_z1r - u1z;
            float onez1 = 1 / pos3d_z2r;
            float onedz2 = 1 / pos3d_z1r - onez1;
            u2dz /= scr_y2r - scr_y1r;
            onedz2 /= scr_y2r - scr_y1r;
            if (cnt) cnt->spans++;
            float mult = (float)(y + 1) - scr_y1r;
            float uz = u1z + u2dz * mult;
            float onez = onez1 + onedz2 * mult;

            for (; y < scr_y2; ++y, uz += u2dz, onez += onedz2) {
                if (mask_get(mask, y)) continue;
                float uf = fminf(fmaxf(uz / onez, (float)texture), (float)((double)tex - 1.0));
                uint32_t u = (uint32_t)uf;
                float depth = 1 / onez;
                uint32_t real_z = (uint32_t)(f2i(depth) & 0xfffe);
                uint32_t colour16 = send[u];
                row[y] = colour16 + (real_z << 16);
                if (drow) drow[y] = depth;
                if (hrow) {
                    hrow[y].x = (uint16_t)vx;
                    hrow[y].z = (uint16_t)vz;
                    hrow[y].y = (uint16_t)(((int)sgs >> mip_lvl) + (int)(u - (uint32_t)texture));
                    hrow[y].mip = (uint8_t)mip_lvl;
                    hrow[y].flags = 1;
                }
                if (cnt) cnt->pixels++;
                mask_set(mask, y);
            }
        }
    }
}

int orc_render_rays(const orc_raymap* rm, const orc_mip* mips, int nummaps, int nrays,
                    uint32_t* out, float* depth, orc_hit* hits, orc_counters* counters,
                    int nthreads)
{
    const int S = rm->samples;
    if (S <= 0 || nummaps <= 0) return -1;
    const int words = S / 32 + 2;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel
    {
        uint32_t* mask = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)words);
#pragma omp for schedule(dynamic, 16)
        for (int x = 0; x < nrays; x++) {
            uint32_t* row = out + (size_t)x * S;
            float* drow = depth ? depth + (size_t)x * S : NULL;
            orc_hit* hrow = hits ? hits + (size_t)x * S : NULL;
            memset(row, 0, sizeof(uint32_t) * (size_t)S);
            if (drow) memset(drow, 0, sizeof(float) * (size_t)S);
            if (hrow) memset(hrow, 0, sizeof(orc_hit) * (size_t)S);
            memset(mask, 0, sizeof(uint32_t) * (size_t)words);
            orc_counters* c = counters ? counters + x : NULL;
            if (c) memset(c, 0, sizeof(*c));
            render_line(rm, mips, nummaps, x, row, drow, hrow, c, mask);
        }
        free(mask);
    }
    return 0;
}

/* ======================================================================= */
/* Resolve: bin/shader/colorize_buddha_soft.frag:12-80, uniforms from      */
/* src/main.cpp:575-603                                                    */
/* ======================================================================= */

static inline float step_f(float edge, float x) { return x < edge ? 0.0f : 1.0f; }

static inline int texel(float t, int size)
{
    int i = f2i(floorf(t * (float)size));
    if (i < 0) i = 0;
    if (i > size - 1) i = size - 1;
    return i;
}

static inline uint32_t rgb565_to_rgba8(uint32_t c)
{
    uint32_t r = (c >> 11) & 31, g = (c >> 5) & 63, b = c & 31;
    r = (r << 3) | (r >> 2);
    g = (g << 2) | (g >> 4);
    b = (b << 3) | (b >> 2);
    return r | (g << 8) | (b << 16) | 0xff000000u;
}

void orc_resolve(const orc_raymap* rm, int width, int height, int rows, const uint32_t* raybuf,
                 const float* raydepth, const orc_hit* rayhit, uint32_t* colour, float* depth,
                 orc_hit* hit, int64_t* sample_index)
{
    const int S = rm->samples;
    const float RESX = (float)width, RESY = (float)height;
    const float rcr = (float)(4 * rm->maxres);           /* RAYS_CASTED_RES */
    const float ratio = rcr / (float)rows;                /* res_x_y_ray_ratio.w */
    const float vanish_x = 1 - rm->vanishing_point_2d.x;
    const float vanish_y = (1 - rm->vanishing_point_2d.y - rm->border) * RESX / RESY;
    const float ofs1 = 4 * (float)rm->res[0] / rcr;
    const float ofs2 = 4 * (float)rm->res[1] / rcr + ofs1;
    const float ofs3 = 4 * (float)rm->res[2] / rcr + ofs2;
    const float ofs_x = -rm->p_ofs_min[0], ofs_y = -rm->p_ofs_min[1] + ofs1;
    const float ofs_z = -rm->p_ofs_min[2] + ofs2, ofs_w = -rm->p_ofs_min[3] + ofs3;
    const float rxg0 = rm->rotation.x > 0 ? 1.0f : 0.0f;
    const int rays = orc_rays_to_render(rm);

    for (int row = 0; row < height; row++)
        for (int col = 0; col < width; col++) {
            const float fx = (float)col + 0.5f;
            const float fy = (float)(height - 1 - row) + 0.5f; /* GL rows count from the bottom */
            float scx = fx / RESX, scy = fy / RESY;
            float border = (RESX - RESY) / (RESX * 2);
            float scx1 = scx - vanish_x, scy1 = scy - vanish_y;
            float upper = step_f(scy1, 0.0f);
            float left = step_f(scx1, 0.0f);
            float ostep = step_f(fabsf(scy1) - fabsf(scx1) * RESX / RESY, 0.0f);
            float seg_up = (1 - upper) * (1 - ostep);
            float seg_dn = upper * (1 - ostep);
            float seg_rt = (1 - left) * ostep;
            float seg_lt = left * ostep;
            float o2 = (ostep * fx + (1 - ostep) * fy) / RESX;
            float ang2 = scx1 * fabsf(1 - step_f(scy1, 0.0f) - vanish_y) / scy1 +
                         step_f(scy1, 0.0f) * (1 - vanish_x) + (1 - step_f(scy1, 0.0f)) * vanish_x;
            float ang3 = scy1 * fabsf(1 - step_f(scx1, 0.0f) - vanish_x) / scx1 +
                         step_f(scx1, 0.0f) * (1 - vanish_y) + (1 - step_f(scx1, 0.0f)) * vanish_y;
            ang3 = ang3 * RESY / RESX + border;
            float x_pre = ostep * ang3 + ang2 * (1 - ostep);
            float ty = seg_dn * (ofs_y + x_pre) + seg_up * (ofs_x + 1.0f - x_pre) +
                       seg_lt * (ofs_w + x_pre) + seg_rt * (ofs_z + 1.0f - x_pre);
            ty = ty * ratio * 0.25f;
            float seg_up_x = rxg0 * seg_up + (1.0f - rxg0) * seg_dn;
            float seg_dn_x = rxg0 * seg_dn + (1.0f - rxg0) * seg_up;
            float seg_rt_x = rxg0 * seg_rt + (1.0f - rxg0) * seg_lt;
            float seg_lt_x = rxg0 * seg_lt + (1.0f - rxg0) * seg_rt;
            float tx = seg_up_x * (o2 + border) + seg_dn_x * (1.0f - (o2 + border)) +
                       seg_rt_x * o2 + seg_lt_x * (1.0f - o2);
            int s = texel(tx, S);
            int r = texel(ty, rows);
            size_t si = (size_t)r * S + s;
            size_t pi = (size_t)row * width + col;
            /* rows past the rays cast hold no data */
            const int cast = r < rays;
            uint32_t w = cast ? raybuf[si] : 0u;
            if (sample_index) sample_index[pi] = cast ? (int64_t)si : -1;
            float d = cast ? raydepth[si] : 0.0f;
            if (((w >> 16) & 0xff) == 0xff) {
                /* sky: the shader's c.z == 1.0 test (byte 2 of 0x00ff8844) */
                colour[pi] = 0xffffccb2u; /* vec4(178,204,255,255)/255 */
                depth[pi] = INFINITY;
            } else if (d == 0.0f) {
                /* outside the ray's clip range: never written by the raycast */
                colour[pi] = 0;
                depth[pi] = 0.0f;
            } else {
                colour[pi] = rgb565_to_rgba8(w & 0xffff);
                depth[pi] = d;
            }
            if (hit) {
                if (rayhit && cast) hit[pi] = rayhit[si];
                else memset(&hit[pi], 0, sizeof(orc_hit));
            }
        }
}

/* ======================================================================= */
/* Soft post-filter: bin/shader/soft.frag over the colorize pass's frame    */
/* buffer (src/main.cpp:627-653; the buffer is RGBA8, GL_LINEAR, clamp to   */
/* edge, src/GL_Main.h:150-165).                                            */
/* ======================================================================= */

/* Frame-buffer texel the colorize pass leaves for one resolved pixel: RGB,
 * and alpha = 0.001/z clamped to [0,1] in 8 bits, z being the sample's
 * depth16 as the shader reads it (low byte/255/256 + high byte/255); sky
 * has alpha 0 (colorize_buddha_soft.frag:86-136). */
static uint32_t soft_texel(const uint32_t* colour, const float* depth, int width, int x, int row)
{
    size_t i = (size_t)row * width + x;
    uint32_t w8;
    float d = depth[i];
    if (isinf(d)) {
        w8 = 0;
    } else {
        uint32_t d16 = (uint32_t)(f2i(d) & 0xfffe);
        float z = ((float)(d16 & 255u) / 255.0f) * (1.0f / 256.0f) + (float)(d16 >> 8) / 255.0f;
        float fragz = 0.001f / z;
        float f = fminf(fmaxf(fragz, 0.0f), 1.0f);
        w8 = (uint32_t)f2i(f * 255.0f + 0.5f);
    }
    return (colour[i] & 0x00ffffffu) | (w8 << 24);
}

typedef struct { float x, y, z, w; } orc_f4;

static orc_f4 soft_unpack(uint32_t t)
{
    orc_f4 r = {(float)(t & 255u) / 255.0f, (float)((t >> 8) & 255u) / 255.0f,
                (float)((t >> 16) & 255u) / 255.0f, (float)(t >> 24) / 255.0f};
    return r;
}

static int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* GL_LINEAR at texture coordinate (u, v) of the 2048^2 buffer (rows from the
 * bottom of the frame), clamped to the frame. */
static orc_f4 soft_sample(const uint32_t* colour, const float* depth, int width, int height, float u, float v)
{
    float uu = u * 2048.0f - 0.5f, vv = v * 2048.0f - 0.5f;
    float fx0 = floorf(uu), fy0 = floorf(vv);
    float a = uu - fx0, b = vv - fy0;
    int i0 = clampi((int)fx0, 0, width - 1), i1 = clampi((int)fx0 + 1, 0, width - 1);
    int j0 = clampi((int)fy0, 0, height - 1), j1 = clampi((int)fy0 + 1, 0, height - 1);
    orc_f4 t00 = soft_unpack(soft_texel(colour, depth, width, i0, height - 1 - j0));
    orc_f4 t10 = soft_unpack(soft_texel(colour, depth, width, i1, height - 1 - j0));
    orc_f4 t01 = soft_unpack(soft_texel(colour, depth, width, i0, height - 1 - j1));
    orc_f4 t11 = soft_unpack(soft_texel(colour, depth, width, i1, height - 1 - j1));
    float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    orc_f4 r;
    r.x = w00 * t00.x + w10 * t10.x + w01 * t01.x + w11 * t11.x;
    r.y = w00 * t00.y + w10 * t10.y + w01 * t01.y + w11 * t11.y;
    r.z = w00 * t00.z + w10 * t10.z + w01 * t01.z + w11 * t11.z;
    r.w = w00 * t00.w + w10 * t10.w + w01 * t01.w + w11 * t11.w;
    return r;
}

static uint32_t soft_byte(float v)
{
    float f = fminf(fmaxf(v, 0.0f), 1.0f);
    return (uint32_t)f2i(f * 255.0f + 0.5f);
}

void orc_soft_filter(const uint32_t* colour, const float* depth, int width, int height, uint32_t* out)
{
    /* soft.frag:12-20 and :33-34: the loops in float */
    float circle[8][2];
    int ncircle = 0;
    const float step = 3.1415f * 1.9f / 6.0f;
    for (float a = 0.0f; a < 3.1415f * 2.0f && ncircle < 8; a += step) {
        circle[ncircle][0] = sinf(a) * 0.005f;
        circle[ncircle][1] = cosf(a) * 0.005f;
        ncircle++;
    }
    float grid[6];
    int ngrid = 0;
    for (float a = -1.0f; a < 1.0f && ngrid < 6; a += 2.0f / 5.0f) grid[ngrid++] = a;
    for (int y = 0; y < height; y++)
        for (int x = 0; x < width; x++) {
            float u = ((float)x + 0.5f) / 2048.0f, v = ((float)y + 0.5f) / 2048.0f;
            orc_f4 col = soft_unpack(soft_texel(colour, depth, width, x, height - 1 - y));
            /* :11-23 largest alpha on the circle */
            float radmax = col.w;
            for (int i = 0; i < ncircle; i++) {
                float w = soft_sample(colour, depth, width, height, circle[i][0] + u, circle[i][1] + v).w;
                radmax = fmaxf(radmax, w);
            }
            /* :27-63 box filter of the samples near the front depth */
            float rad = 0.0023f * radmax;
            if (rad > 0.00008f) {
                orc_f4 avg = col;
                float n = 1.0f;
                float thresh = radmax * 0.7f;
                for (int ia = 0; ia < ngrid; ia++)
                    for (int ib = 0; ib < ngrid; ib++) {
                        orc_f4 c = soft_sample(colour, depth, width, height, u + grid[ia] * rad, v + grid[ib] * rad);
                        if (c.w >= thresh) {
                            avg.x = avg.x + c.x;
                            avg.y = avg.y + c.y;
                            avg.z = avg.z + c.z;
                            avg.w = avg.w + c.w;
                            n = n + 1.0f;
                        }
                    }
                if (n > 6.0f) {
                    float inv = 1.0f / n;
                    col.x = avg.x * inv;
                    col.y = avg.y * inv;
                    col.z = avg.z * inv;
                    col.w = avg.w * inv;
                }
            }
            out[(size_t)(height - 1 - y) * width + x] =
                soft_byte(col.x) | (soft_byte(col.y) << 8) | (soft_byte(col.z) << 16) | (soft_byte(col.w) << 24);
        }
}
