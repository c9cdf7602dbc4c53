// Host ray map: camera -> vanishing point, fans of column rays, 2D<->3D
// transforms.  Restates RayMap::get_ray_map (src/RayMap.h:98-402) and the
// _matrix44 / vec3f helpers it calls (inc/mathlib/_matrix44.h,
// src/VecMath.h) with the same single-precision operations in the same
// order, so the result is bit-identical to the reference on every host
// built with -ffp-contract=off.  The frustum corners may be scaled by
// tan(fov/2) (1 reproduces the reference's fixed 90 degree frustum).
#include <cmath>
#include <cstring>

#include "rle_internal.h"

namespace {

struct F3 {
    float x, y, z;
};
inline F3 mk(float x, float y, float z) { return F3{x, y, z}; }
inline F3 operator+(F3 a, F3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
inline F3 operator-(F3 a, F3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
inline F3 operator*(F3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
inline F3 operator/(F3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
// vec3f::dot evaluates other.x*x + other.y*y + other.z*z (src/VecMath.h:62).
inline float dot_rev(F3 self, F3 other) { return other.x * self.x + other.y * self.y + other.z * self.z; }
inline float length(F3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }

// Row-vector 4x4 matrix as the reference's _matrix44 (m[row][col]).
struct M44 {
    float m[4][4];
    void identity() {
        std::memset(m, 0, sizeof(m));
        m[0][0] = m[1][1] = m[2][2] = m[3][3] = 1.0f;
    }
    void rotate_x(float a) {
        const float c = std::cos(a), s = std::sin(a);
        for (auto& r : m) {
            const float a1 = r[1], a2 = r[2];
            r[1] = a1 * c + a2 * -s;
            r[2] = a1 * s + a2 * c;
        }
    }
    void rotate_y(float a) {
        const float c = std::cos(a), s = std::sin(a);
        for (auto& r : m) {
            const float a0 = r[0], a2 = r[2];
            r[0] = a0 * c + a2 * s;
            r[2] = a0 * -s + a2 * c;
        }
    }
    F3 apply(F3 v) const {
        return mk(m[0][0] * v.x + m[1][0] * v.y + m[2][0] * v.z + m[3][0],
                  m[0][1] * v.x + m[1][1] * v.y + m[2][1] * v.z + m[3][1],
                  m[0][2] * v.x + m[1][2] * v.y + m[2][2] * v.z + m[3][2]);
    }
    // Transpose of the rotation block and -R^T t (invert_simpler).
    void invert_simpler() {
        std::swap(m[0][1], m[1][0]);
        std::swap(m[0][2], m[2][0]);
        std::swap(m[1][2], m[2][1]);
        const float t0 = -(m[0][0] * m[3][0] + m[1][0] * m[3][1] + m[2][0] * m[3][2]);
        const float t1 = -(m[0][1] * m[3][0] + m[1][1] * m[3][1] + m[2][1] * m[3][2]);
        m[3][2] = -(m[0][2] * m[3][0] + m[1][2] * m[3][1] + m[2][2] * m[3][2]);
        m[3][1] = t1;
        m[3][0] = t0;
    }
};

// float -> int with saturation and NaN -> 0 (the device conversion).
inline int to_int(float f) {
    if (!(f == f)) return 0;
    if (f >= 2147483648.0f) return 2147483647;
    if (f < -2147483648.0f) return (-2147483647 - 1);
    return static_cast<int>(f);
}

inline float snap_to_ray(float v, int maxres, int add) {
    return static_cast<float>(to_int(static_cast<float>(maxres) * v) + add) / static_cast<float>(maxres);
}

inline int fan_rays(int maxres, float lo, float hi) {
    int n = to_int(static_cast<float>(maxres) * std::fabs(lo - hi));
    if (lo - hi > 0) n = 0;
    if (n > maxres * 3) n = maxres * 3;
    return n;
}

inline void put(float* dst, F3 v) {
    dst[0] = v.x;
    dst[1] = v.y;
    dst[2] = v.z;
}
inline F3 get(const float* s) { return mk(s[0], s[1], s[2]); }

}  // namespace

extern "C" rle_status rle_raymap_build(const rle_camera* cam, const rle_view_params* view, rle_raymap* out) {
    if (!cam || !view || !out) {
        rle::set_error("rle_raymap_build: null argument");
        return RLE_ERR_INVALID_ARG;
    }
    const int W = view->width, H = view->height;
    if (W < 8 || H < 8 || W > 16384 || H > 16384 || H > W) {
        rle::set_error("rle_raymap_build: screen %dx%d not in 8..16384 with height <= width", W, H);
        return RLE_ERR_INVALID_ARG;
    }
    const int S = view->samples > 0 ? view->samples : W;
    const int maxres = view->maxres > 0 ? view->maxres : W;
    if (S < 8 || S > 16384 || maxres < 8 || maxres > 16384) {
        rle::set_error("rle_raymap_build: samples %d / maxres %d out of range", S, maxres);
        return RLE_ERR_INVALID_ARG;
    }
    for (int i = 0; i < 3; i++) {
        if (!std::isfinite(cam->pos[i]) || std::fabs(cam->pos[i]) > 1.0e6f || !std::isfinite(cam->rot[i])) {
            rle::set_error("rle_raymap_build: camera position/rotation must be finite, |pos| <= 1e6");
            return RLE_ERR_INVALID_ARG;
        }
    }
    const float fov = cam->fov_deg;
    if (!(fov > 1.0f && fov < 179.0f)) {
        rle::set_error("rle_raymap_build: fov %g outside (1, 179) degrees", fov);
        return RLE_ERR_INVALID_ARG;
    }
    std::memset(out, 0, sizeof(*out));
    const float border = view->border <= 0.0f
        ? static_cast<float>(W - H) / static_cast<float>(2 * W) : view->border;
    const float rx = cam->rot[0], ry = cam->rot[1], rz = cam->rot[2];
    out->border = border;
    out->clip_min = border;
    out->clip_max = 1 - border;
    put(out->rotation, mk(rx, ry, rz));
    put(out->position, mk(cam->pos[0], cam->pos[1], cam->pos[2]));
    out->samples = S;
    out->mip_distance = view->mip_distance > 0 ? view->mip_distance : W;
    out->z_far = view->z_far > 0 ? view->z_far : 80000;
    // 90 degrees gives exactly 1 (the reference frustum).
    out->fov_scale = fov == 90.0f ? 1.0f
        : static_cast<float>(std::tan(static_cast<double>(fov) * 0.5 * 3.14159265358979323846 / 180.0));

    // Frustum corners, origin, and (later) the down vanishing point.
    const float t = out->fov_scale;
    F3 p[6] = {mk(t, t, 1), mk(-t, t, 1), mk(-t, -t, 1), mk(t, -t, 1), mk(0, 0, 0), mk(0, 0, 0)};
    M44 m;
    m.identity();
    m.rotate_x(rx);
    m.rotate_y(ry);
    m.m[3][0] += 3.0f;  // translate(vector3(3,2,0))
    m.m[3][1] += 2.0f;
    m.m[3][2] += 0.0f;
    for (int i = 0; i < 5; i++) p[i] = m.apply(p[i]);

    const F3 down = mk(0, -1, 0);
    const F3 view_dir = (p[0] + p[2]) / 2.0f - p[4];
    float cosang = view_dir.x * down.x + view_dir.y * down.y + view_dir.z * down.z;
    float len = length(view_dir) * length(down);
    if (len == 0) len = 0.00001f;
    cosang = cosang / len;
    if (cosang < -1) cosang = -1;
    if (cosang > 1) cosang = 1;
    const float alpha = static_cast<float>(M_PI) / 2 - std::acos(cosang);
    const float scale = 1 / std::sin(alpha);
    p[5] = p[4] + down * scale;

    // Basis of the frustum plane; to3d maps plane coordinates to 3D.
    const F3 e1 = p[1] - p[0], e2 = p[3] - p[0];
    F3 n = mk(e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x);
    F3 b1 = e1 * (1 / (e1.x * e1.x + e1.y * e1.y + e1.z * e1.z));
    F3 b2 = e2 * (1 / (e2.x * e2.x + e2.y * e2.y + e2.z * e2.z));
    F3 b3 = n * (1 / (n.x * n.x + n.y * n.y + n.z * n.z));
    M44 to2d;
    const F3 rows[4] = {b1, b2, b3, p[0]};
    for (int r = 0; r < 4; r++) {
        to2d.m[r][0] = rows[r].x;
        to2d.m[r][1] = rows[r].y;
        to2d.m[r][2] = rows[r].z;
        to2d.m[r][3] = 1.0f;
    }
    std::memcpy(out->to3d, to2d.m, sizeof(to2d.m));
    to2d.invert_simpler();
    F3 p2d[6];
    for (int i = 0; i < 6; i++) {
        p2d[i] = to2d.apply(p[i]);
        put(out->p_2d[i], p2d[i]);
    }
    put(out->vanishing_point_2d, p2d[5]);

    // Four fans of column rays around the vanishing point.
    out->maxres = maxres;
    const float lo = border, hi = 1 - border;
    const F3 dirs[4] = {mk(-1, -1, 0), mk(1, -1, 0), mk(1, 1, 0), mk(-1, 1, 0)};
    const F3 box[4] = {mk(0, lo, 0), mk(1, lo, 0), mk(1, hi, 0), mk(0, hi, 0)};
    out->p_2d[5][2] = 0;
    const F3 c = get(out->p_2d[5]);
    F3 q[8];
    for (int i = 0; i < 8; i++) q[i] = get(out->p_no[i]);

    if (c.y > border) {  // up
        const float s = std::fabs(c.y - border);
        q[0] = c + dirs[0] * s;
        q[1] = c + dirs[1] * s;
        const F3 keep = q[1];
        if (c.x > 1) {
            if (q[1].x > 1) q[1].x = 1;
        } else if (dot_rev(q[0] - c, box[2] - c) > 0) {
            q[1] = c + (box[2] - c) * std::fabs((box[0].y - c.y) / (box[2].y - c.y));
        }
        if (c.x < 0) {
            if (q[0].x < 0) q[0].x = 0;
        } else if (dot_rev(keep - c, box[3] - c) > 0) {
            q[0] = c + (box[3] - c) * std::fabs((box[1].y - c.y) / (box[3].y - c.y));
        }
        q[0].y = q[1].y = box[0].y;
        q[0].x = snap_to_ray(q[0].x, maxres, -2);
        q[1].x = snap_to_ray(q[1].x, maxres, +2);
        out->res[0] = fan_rays(maxres, q[0].x, q[1].x);
        out->p_ofs_min[0] = q[0].x;
        out->p_ofs_max[0] = q[1].x;
    }
    if (c.y < 1 - border) {  // down
        const float s = std::fabs(c.y - 1 + border);
        q[2] = c + dirs[3] * s;
        q[3] = c + dirs[2] * s;
        const F3 keep = q[2];
        if (c.x < 0) {
            if (q[2].x < 0) q[2].x = 0;
        } else if (dot_rev(q[3] - c, box[0] - c) > 0) {
            q[2] = c + (box[0] - c) * std::fabs((box[2].y - c.y) / (box[0].y - c.y));
        }
        if (c.x > 1) {
            if (q[3].x > 1) q[3].x = 1;
        } else {
            const F3 d = box[1] - c;
            if (dot_rev(keep - c, d) > 0) q[3] = c + d * std::fabs((box[3].y - c.y) / d.y);
        }
        q[2].y = q[3].y = box[2].y;
        q[2].x = snap_to_ray(q[2].x, maxres, -2);
        q[3].x = snap_to_ray(q[3].x, maxres, +2);
        out->res[1] = fan_rays(maxres, q[2].x, q[3].x);
        out->p_ofs_min[1] = q[2].x;
        out->p_ofs_max[1] = q[3].x;
    }
    if (c.x > 0) {  // left
        const float s = std::fabs(c.x);
        q[4] = c + dirs[0] * s;
        q[5] = c + dirs[3] * s;
        const F3 keep = q[5];
        if (c.y > 1 - border) {
            if (q[5].y > 1 - border) q[5].y = 1 - border;
        } else if (dot_rev(q[4] - c, box[2] - c) > 0) {
            q[5] = c + (box[2] - c) * std::fabs((box[3].x - c.x) / (box[2].x - c.x));
        }
        if (c.y < border) {
            if (q[4].y < border) q[4].y = border;
        } else if (dot_rev(keep - c, box[1] - c) > 0) {
            q[4] = c + (box[1] - c) * std::fabs((box[0].x - c.x) / (box[1].x - c.x));
        }
        q[4].x = q[5].x = 0;
        q[4].y = snap_to_ray(q[4].y, maxres, -2);
        q[5].y = snap_to_ray(q[5].y, maxres, +2);
        out->res[2] = fan_rays(maxres, q[4].y, q[5].y);
        out->p_ofs_min[2] = q[4].y;
        out->p_ofs_max[2] = q[5].y;
    }
    if (c.x < 1) {  // right
        const float s = std::fabs(1 - c.x);
        q[6] = c + dirs[1] * s;
        q[7] = c + dirs[2] * s;
        const F3 keep = q[7];
        if (c.y > 1 - border) {
            if (q[7].y > 1 - border) q[7].y = 1 - border;
        } else if (dot_rev(q[6] - c, box[3] - c) > 0) {
            q[7] = c + (box[3] - c) * std::fabs((box[2].x - c.x) / (box[3].x - c.x));
        }
        if (c.y < border) {
            if (q[6].y < border) q[6].y = border;
        } else if (dot_rev(keep - c, box[0] - c) > 0) {
            q[6] = c + (box[0] - c) * std::fabs((box[1].x - c.x) / (box[0].x - c.x));
        }
        q[6].x = q[7].x = 1;
        q[6].y = snap_to_ray(q[6].y, maxres, -2);
        q[7].y = snap_to_ray(q[7].y, maxres, +2);
        out->res[3] = fan_rays(maxres, q[6].y, q[7].y);
        out->p_ofs_min[3] = q[6].y;
        out->p_ofs_max[3] = q[7].y;
    }
    for (int i = 0; i < 8; i++) put(out->p_no[i], q[i]);
    put(out->p4, p[4]);
    out->map_line_count = out->res[0] + out->res[1] + out->res[2] + out->res[3];

    // Derived per-frame values.
    out->sin_x = std::sin(rx);
    out->cos_x = std::cos(rx);
    out->sin_y = std::sin(ry);
    out->cos_y = std::cos(ry);
    out->sin_neg_y = std::sin(-ry);
    out->cos_neg_y = std::cos(-ry);
    out->width = W;
    out->height = H;
    out->rows = 4 * maxres;
    out->rays = out->map_line_count < out->rows ? out->map_line_count : out->rows;
    if (!std::isfinite(out->vanishing_point_2d[0]) || !std::isfinite(out->vanishing_point_2d[1]) ||
        out->map_line_count < 0) {
        rle::set_error("rle_raymap_build: degenerate camera (pitch too close to 0?)");
        return RLE_ERR_INVALID_ARG;
    }
    return RLE_OK;
}
