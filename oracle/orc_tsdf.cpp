// Oracle (test infrastructure only): CPU restatement of the reference's TSDF
// volume — reset, voxel-projective integration and the front-face raycast.
// Follows src/tsdf/TSDFVolume.cpp of iphands/azu line by line (cited per function).
#include "orc_api.h"
#include "orc_math.h"

#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

using namespace orc;

namespace {

constexpr float kEmptyTsdf = 1.0f;     // include/tsdf/TSDFVolume.h:26
constexpr float kEmptyWeight = 0.0f;   // include/tsdf/TSDFVolume.h:27
constexpr float kEmptyColor = 128.0f / 255.0f;  // include/tsdf/TSDFVolume.h:37

struct Vol {
    const orc_tsdf_params* p;
    const float* tsdf;
    const float* weight;
    const float* color;
    size_t idx(int x, int y, int z) const {
        const size_t r = static_cast<size_t>(p->res);
        return (static_cast<size_t>(z) * r + static_cast<size_t>(y)) * r + static_cast<size_t>(x);
    }
};

V3 originOf(const orc_tsdf_params* p) { return V3(p->origin[0], p->origin[1], p->origin[2]); }

// TSDFVolume::sampleTSDF (src/tsdf/TSDFVolume.cpp:492-525).
bool sampleTSDF(const Vol& v, V3 wp, float& f_out) {
    const float vs = v.p->voxel_size;
    const int res = v.p->res;
    const V3 q = (wp - originOf(v.p)) / vs;
    const float fx0 = std::floor(q.x), fy0 = std::floor(q.y), fz0 = std::floor(q.z);
    if (!(fx0 >= 0.0f && fy0 >= 0.0f && fz0 >= 0.0f && fx0 < static_cast<float>(res - 1) &&
          fy0 < static_cast<float>(res - 1) && fz0 < static_cast<float>(res - 1)))
        return false;
    const int x0 = static_cast<int>(fx0), y0 = static_cast<int>(fy0), z0 = static_cast<int>(fz0);
    const float tx = q.x - fx0, ty = q.y - fy0, tz = q.z - fz0;
    const size_t sx = 1, sy = static_cast<size_t>(res), sz = static_cast<size_t>(res) * res;
    const size_t b = v.idx(x0, y0, z0);
    const size_t c[8] = {b, b + sx, b + sy, b + sx + sy, b + sz, b + sx + sz, b + sy + sz, b + sx + sy + sz};
    for (size_t ci : c)
        if (!(v.weight[ci] > kEmptyWeight)) return false;
    const float v00 = v.tsdf[c[0]] * (1 - tx) + v.tsdf[c[1]] * tx;
    const float v10 = v.tsdf[c[2]] * (1 - tx) + v.tsdf[c[3]] * tx;
    const float v01 = v.tsdf[c[4]] * (1 - tx) + v.tsdf[c[5]] * tx;
    const float v11 = v.tsdf[c[6]] * (1 - tx) + v.tsdf[c[7]] * tx;
    const float v0 = v00 * (1 - ty) + v10 * ty;
    const float v1 = v01 * (1 - ty) + v11 * ty;
    f_out = v0 * (1 - tz) + v1 * tz;
    return true;
}

// TSDFVolume::computeNormal (src/tsdf/TSDFVolume.cpp:478-490).
bool computeNormal(const Vol& v, V3 p, V3& n_out) {
    const float h = v.p->voxel_size;
    float s[6];
    const V3 off[3] = {V3(h, 0, 0), V3(0, h, 0), V3(0, 0, h)};
    for (int a = 0; a < 3; ++a) {
        if (!sampleTSDF(v, p + off[a], s[2 * a]) || !sampleTSDF(v, p - off[a], s[2 * a + 1])) return false;
    }
    const V3 n(s[0] - s[1], s[2] - s[3], s[4] - s[5]);
    const float len = norm(n);
    if (!(len > 1e-6f) || !std::isfinite(len)) return false;
    n_out = n / len;
    return true;
}

}  // namespace

extern "C" void orc_tsdf_reset(const orc_tsdf_params* p, float* tsdf, float* weight, float* color) {
    const size_t n = static_cast<size_t>(p->res) * p->res * p->res;
    for (size_t i = 0; i < n; ++i) {
        tsdf[i] = kEmptyTsdf;
        weight[i] = kEmptyWeight;
    }
    if (color)
        for (size_t i = 0; i < 3 * n; ++i) color[i] = kEmptyColor;
}

// TSDFVolume::integrateCPU (src/tsdf/TSDFVolume.cpp:214-346).
extern "C" void orc_tsdf_integrate(const orc_tsdf_params* p, float* tsdf, float* weight, float* color,
                                   const float* depth_m, const uint8_t* rgb, const float pose_rm[16],
                                   orc_intrinsics K, int width, int height, float min_depth,
                                   float max_depth, int64_t stats[9]) {
    for (int i = 0; i < 9; ++i) stats[i] = 0;
    for (int i = 3; i < 9; ++i) stats[i] = -1;
    const float trunc = p->truncation;
    const float max_w = p->max_weight;
    const float vs = p->voxel_size;
    const int res = p->res;
    const V3 origin = originOf(p);
    const float fx = K.fx, fy = K.fy, cx = K.cx, cy = K.cy;

    const M4 pose = M4::from(pose_rm);
    const M4 world_to_cam = inverse4(pose);
    const M3 R_wc = world_to_cam.R();
    const V3 t_wc = world_to_cam.t();
    const M3 R_cw = pose.R();
    const V3 t_cw = pose.t();

    // Frustum AABB (:244-264).
    V3 lo = (t_cw - origin) / vs;
    V3 hi = lo;
    const float z_far = max_depth + trunc;
    const float corner_px[4][2] = {{0.0f, 0.0f}, {float(width), 0.0f}, {0.0f, float(height)},
                                   {float(width), float(height)}};
    for (const auto& c : corner_px) {
        const V3 ray((c[0] - cx) / fx * z_far, (c[1] - cy) / fy * z_far, z_far);
        const V3 v = ((R_cw * ray + t_cw) - origin) / vs;
        lo = vmin(lo, v);
        hi = vmax(hi, v);
    }
    if (!finite3(lo) || !finite3(hi)) return;
    auto clampIdx = [res](float f) {
        return static_cast<int>(std::max(0.0f, std::min(static_cast<float>(res - 1), f)));
    };
    const int x0 = clampIdx(std::floor(lo.x)), x1 = clampIdx(std::ceil(hi.x));
    const int y0 = clampIdx(std::floor(lo.y)), y1 = clampIdx(std::ceil(hi.y));
    const int z0 = clampIdx(std::floor(lo.z)), z1 = clampIdx(std::ceil(hi.z));
    stats[3] = x0; stats[4] = x1; stats[5] = y0; stats[6] = y1; stats[7] = z0; stats[8] = z1;

    const V3 step_x = R_wc.col(0) * vs;
    const float color_band = 0.5f * trunc;
    const size_t rr = static_cast<size_t>(res);

    int64_t newly = 0, updated = 0, colored_n = 0;
#pragma omp parallel for collapse(2) schedule(dynamic, 16) reduction(+ : newly, updated, colored_n)
    for (int z = z0; z <= z1; ++z) {
        for (int y = y0; y <= y1; ++y) {
            V3 c = R_wc * (origin + V3(float(x0), float(y), float(z)) * vs) + t_wc;
            for (int x = x0; x <= x1; ++x, c = c + step_x) {
                if (c.z <= 0.0f) continue;
                const float inv_z = 1.0f / c.z;
                const float uf = std::floor(fx * c.x * inv_z + cx + 0.5f);
                const float vf = std::floor(fy * c.y * inv_z + cy + 0.5f);
                if (!(uf >= 0.0f && uf < static_cast<float>(width) && vf >= 0.0f &&
                      vf < static_cast<float>(height)))
                    continue;
                const int pix = static_cast<int>(vf) * width + static_cast<int>(uf);
                const float d = depth_m[pix];
                if (!(d >= min_depth && d <= max_depth)) continue;
                const float sdf = d - c.z;
                if (sdf < -trunc) continue;
                const float tsdf_new = std::min(1.0f, sdf / trunc);
                const size_t vi = (static_cast<size_t>(z) * rr + static_cast<size_t>(y)) * rr + static_cast<size_t>(x);
                const float w_old = weight[vi];
                newly += (w_old == 0.0f) ? 1 : 0;
                ++updated;
                tsdf[vi] = (tsdf[vi] * w_old + tsdf_new) / (w_old + 1.0f);
                weight[vi] = std::min(w_old + 1.0f, max_w);
                if (rgb != nullptr && color != nullptr && std::fabs(sdf) < color_band) {
                    const uint8_t* px = rgb + pix * 3;
                    const float inv = 1.0f / (w_old + 1.0f);
                    float* cv = color + 3 * vi;
                    cv[0] = (cv[0] * w_old + srgbUint8ToFloat(px[0])) * inv;
                    cv[1] = (cv[1] * w_old + srgbUint8ToFloat(px[1])) * inv;
                    cv[2] = (cv[2] * w_old + srgbUint8ToFloat(px[2])) * inv;
                    ++colored_n;
                }
            }
        }
    }
    stats[0] = newly;
    stats[1] = updated;
    stats[2] = colored_n;
}

// TSDFVolume::raycast (src/tsdf/TSDFVolume.cpp:348-476).
extern "C" void orc_tsdf_raycast(const orc_tsdf_params* p, const float* tsdf, const float* weight,
                                 const float* color, const float pose_rm[16], orc_intrinsics K,
                                 int width, int height, float* vertices_out, float* normals_out,
                                 uint8_t* colors_out, int64_t* samples_out) {
    const Vol vol{p, tsdf, weight, color};
    const float vs = p->voxel_size;
    const float trunc = p->truncation;
    const M4 pose = M4::from(pose_rm);
    const V3 cam_origin = pose.t();
    const M3 R_cw = pose.R();
    const V3 box_lo = originOf(p);
    const float span = static_cast<float>(p->res - 1) * vs;
    const V3 box_hi = box_lo + V3(span, span, span);
    const float min_step = 0.5f * vs;
    const float far_step = std::max(min_step, 0.8f * trunc);
    const float fx = K.fx, fy = K.fy, cx = K.cx, cy = K.cy;
    int64_t samples = 0;

#pragma omp parallel for schedule(dynamic, 16) reduction(+ : samples)
    for (int y = 0; y < height; ++y) {
        for (int x = 0; x < width; ++x) {
            const int o = y * width + x;
            for (int k = 0; k < 3; ++k) { vertices_out[3 * o + k] = 0.0f; normals_out[3 * o + k] = 0.0f; }
            if (colors_out) colors_out[3 * o] = colors_out[3 * o + 1] = colors_out[3 * o + 2] = 0;

            const V3 ray_cam((x - cx) / fx, (y - cy) / fy, 1.0f);
            const float ray_norm = norm(ray_cam);
            const V3 dir = (R_cw * ray_cam) / ray_norm;
            float t_near = p->min_depth * ray_norm;
            float t_far = p->max_depth * ray_norm;
            for (int a = 0; a < 3; ++a) {
                const float inv = 1.0f / dir[a];
                float t0 = (box_lo[a] - cam_origin[a]) * inv;
                float t1 = (box_hi[a] - cam_origin[a]) * inv;
                if (t0 > t1) std::swap(t0, t1);
                if (std::isnan(t0) || std::isnan(t1)) {
                    if (cam_origin[a] < box_lo[a] || cam_origin[a] > box_hi[a]) t_far = -1.0f;
                    continue;
                }
                t_near = std::max(t_near, t0);
                t_far = std::min(t_far, t1);
            }
            if (!(t_near < t_far)) continue;

            float t_prev = t_near;
            float f_prev = 1.0f;
            bool prev_valid = sampleTSDF(vol, cam_origin + dir * t_prev, f_prev);
            ++samples;
            if (prev_valid && !std::isfinite(f_prev)) continue;
            if (prev_valid && f_prev < 0.0f) continue;

            bool found = false;
            float t_hit = 0.0f;
            while (t_prev < t_far) {
                const float step = (!prev_valid || f_prev >= 0.999f) ? far_step
                                                                     : std::max(min_step, 0.8f * f_prev * trunc);
                const float t = std::min(t_prev + step, t_far);
                float f = 1.0f;
                const bool valid = sampleTSDF(vol, cam_origin + dir * t, f);
                ++samples;
                if (valid && !std::isfinite(f)) break;
                if (valid && prev_valid) {
                    if (f_prev > 0.0f && f <= 0.0f) {
                        t_hit = t_prev + (t - t_prev) * (f_prev / (f_prev - f));
                        found = true;
                        break;
                    }
                    if (f_prev < 0.0f && f >= 0.0f) break;
                } else if (valid && f < 0.0f) {
                    break;
                }
                t_prev = t;
                f_prev = f;
                prev_valid = valid;
                if (t >= t_far) break;
            }
            if (!found) continue;

            const V3 hit = cam_origin + dir * t_hit;
            V3 nrm;
            if (!computeNormal(vol, hit, nrm)) continue;
            if (!finite3(hit)) continue;

            if (colors_out) {
                // worldToVoxel (:537-553) then the fused-voxel colour.
                const V3 q = (hit - originOf(p)) / vs;
                int vx = 0, vy = 0, vz = 0;
                const bool ok = floorToInt(q.x, &vx) && floorToInt(q.y, &vy) && floorToInt(q.z, &vz);
                if (ok && vx >= 0 && vx < p->res && vy >= 0 && vy < p->res && vz >= 0 && vz < p->res) {
                    const size_t vi = vol.idx(vx, vy, vz);
                    if (weight[vi] > kEmptyWeight) {
                        uint8_t qc[3] = {0, 0, 0};
                        const float r = color ? color[3 * vi] : kEmptyColor;
                        const float g = color ? color[3 * vi + 1] : kEmptyColor;
                        const float b = color ? color[3 * vi + 2] : kEmptyColor;
                        if (!(srgbFloatToUint8(r, qc[0]) && srgbFloatToUint8(g, qc[1]) &&
                              srgbFloatToUint8(b, qc[2])))
                            continue;
                        colors_out[3 * o] = qc[0];
                        colors_out[3 * o + 1] = qc[1];
                        colors_out[3 * o + 2] = qc[2];
                    }
                }
            }
            vertices_out[3 * o] = hit.x; vertices_out[3 * o + 1] = hit.y; vertices_out[3 * o + 2] = hit.z;
            normals_out[3 * o] = nrm.x; normals_out[3 * o + 1] = nrm.y; normals_out[3 * o + 2] = nrm.z;
        }
    }
    if (samples_out) *samples_out = samples;
}

extern "C" void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

extern "C" int orc_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// FP16 tsdf plus a 9-bit residual below half precision (the FP16R volume
// format; no reference counterpart): h = RN_half(t), q = RN((t - h) / s) with
// s = ulp(h) / 512, |q| <= 255; the stored value is h + q s (exact in float).
static float fp16r_roundtrip(float t) {
    const _Float16 hh = static_cast<_Float16>(t);
    const float h = static_cast<float>(hh);
    uint16_t hb;
    std::memcpy(&hb, &hh, sizeof(hb));
    const int e = (hb >> 10) & 0x1f;
    const float s = std::ldexp(1.0f, (e == 0 ? 94 : e + 93) - 127);
    int q = static_cast<int>(std::nearbyint((t - h) / s));
    q = std::max(-255, std::min(255, q));
    return std::fma(static_cast<float>(q), s, h);
}

// Precision form of the same integration: identical projections and decisions
// (float camera stepping), with
//   half_storage == 1: the tsdf stored rounded to IEEE half (round to nearest
//                      even) after every update, i.e. the FP16 + u16 volume;
//   half_storage == 2: the tsdf stored as half plus residual (fp16r_roundtrip);
//   tsdf64 != NULL:    the running average of the same float tsdf_new values
//                      carried in double (the FP64 reference).
extern "C" void orc_tsdf_integrate_prec(const orc_tsdf_params* p, float* tsdf, float* weight, double* tsdf64,
                                        const float* depth_m, const float pose_rm[16], orc_intrinsics K, int width,
                                        int height, float min_depth, float max_depth, int half_storage) {
    const float trunc = p->truncation, max_w = p->max_weight, vs = p->voxel_size;
    const int res = p->res;
    const V3 origin = originOf(p);
    const M4 pose = M4::from(pose_rm);
    const M4 world_to_cam = inverse4(pose);
    const M3 R_wc = world_to_cam.R();
    const V3 t_wc = world_to_cam.t();
    const M3 R_cw = pose.R();
    const V3 t_cw = pose.t();
    V3 lo = (t_cw - origin) / vs, hi = lo;
    const float z_far = max_depth + trunc;
    const float corner_px[4][2] = {{0.0f, 0.0f}, {float(width), 0.0f}, {0.0f, float(height)},
                                   {float(width), float(height)}};
    for (const auto& c : corner_px) {
        const V3 ray((c[0] - K.cx) / K.fx * z_far, (c[1] - K.cy) / K.fy * z_far, z_far);
        const V3 v = ((R_cw * ray + t_cw) - origin) / vs;
        lo = vmin(lo, v);
        hi = vmax(hi, v);
    }
    if (!finite3(lo) || !finite3(hi)) return;
    auto clampIdx = [res](float f) {
        return static_cast<int>(std::max(0.0f, std::min(static_cast<float>(res - 1), f)));
    };
    const int x0 = clampIdx(std::floor(lo.x)), x1 = clampIdx(std::ceil(hi.x));
    const int y0 = clampIdx(std::floor(lo.y)), y1 = clampIdx(std::ceil(hi.y));
    const int z0 = clampIdx(std::floor(lo.z)), z1 = clampIdx(std::ceil(hi.z));
    const V3 step_x = R_wc.col(0) * vs;
    const size_t rr = static_cast<size_t>(res);
#pragma omp parallel for collapse(2) schedule(dynamic, 16)
    for (int z = z0; z <= z1; ++z) {
        for (int y = y0; y <= y1; ++y) {
            V3 c = R_wc * (origin + V3(float(x0), float(y), float(z)) * vs) + t_wc;
            for (int x = x0; x <= x1; ++x, c = c + step_x) {
                if (c.z <= 0.0f) continue;
                const float inv_z = 1.0f / c.z;
                const float uf = std::floor(K.fx * c.x * inv_z + K.cx + 0.5f);
                const float vf = std::floor(K.fy * c.y * inv_z + K.cy + 0.5f);
                if (!(uf >= 0.0f && uf < static_cast<float>(width) && vf >= 0.0f && vf < static_cast<float>(height)))
                    continue;
                const float d = depth_m[static_cast<int>(vf) * width + static_cast<int>(uf)];
                if (!(d >= min_depth && d <= max_depth)) continue;
                const float sdf = d - c.z;
                if (sdf < -trunc) continue;
                const float tsdf_new = std::min(1.0f, sdf / trunc);
                const size_t vi = (static_cast<size_t>(z) * rr + static_cast<size_t>(y)) * rr + static_cast<size_t>(x);
                const float w_old = weight[vi];
                const float t = (tsdf[vi] * w_old + tsdf_new) / (w_old + 1.0f);
                tsdf[vi] = half_storage == 2 ? fp16r_roundtrip(t)
                           : half_storage ? static_cast<float>(static_cast<_Float16>(t)) : t;
                if (tsdf64)
                    tsdf64[vi] = (tsdf64[vi] * static_cast<double>(w_old) + static_cast<double>(tsdf_new)) /
                                 (static_cast<double>(w_old) + 1.0);
                weight[vi] = std::min(w_old + 1.0f, max_w);
            }
        }
    }
}

// TSDFVolume::extractGlobalPointCloud (src/tsdf/TSDFVolume.cpp:571-632) on one
// thread, i.e. in index order z, y, x: voxels with weight > 1 and |tsdf| < 0.2
// whose colour quantises; world position voxelToWorld (:555-561). Returns the
// count; fills pts / cols (3 per point) when non-null.
extern "C" int64_t orc_point_cloud(const orc_tsdf_params* p, const float* tsdf, const float* weight,
                                   const float* color, float* pts, uint8_t* cols) {
    const int res = p->res;
    const V3 origin = originOf(p);
    int64_t n = 0;
    for (int z = 0; z < res; ++z)
        for (int y = 0; y < res; ++y)
            for (int x = 0; x < res; ++x) {
                const size_t i = (static_cast<size_t>(z) * res + y) * res + x;
                if (!(weight[i] > 1.0f && std::fabs(tsdf[i]) < 0.2f)) continue;
                uint8_t qc[3] = {0, 0, 0};
                const float r = color ? color[3 * i] : kEmptyColor;
                const float g = color ? color[3 * i + 1] : kEmptyColor;
                const float b = color ? color[3 * i + 2] : kEmptyColor;
                if (!srgbFloatToUint8(r, qc[0]) || !srgbFloatToUint8(g, qc[1]) || !srgbFloatToUint8(b, qc[2]))
                    continue;
                if (pts) {
                    const V3 w = origin + V3(static_cast<float>(x), static_cast<float>(y), static_cast<float>(z)) *
                                              p->voxel_size;
                    pts[3 * n] = w.x;
                    pts[3 * n + 1] = w.y;
                    pts[3 * n + 2] = w.z;
                }
                if (cols) {
                    cols[3 * n] = qc[0];
                    cols[3 * n + 1] = qc[1];
                    cols[3 * n + 2] = qc[2];
                }
                ++n;
            }
    return n;
}
