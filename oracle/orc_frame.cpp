// Oracle (test infrastructure only): CPU restatement of the reference's frame
// geometry — raw depth to metres and vertices, normals, and the jump-guarded 2x
// pyramid downsample (src/sensor/FrameData.cpp:109-345).
#include "orc_api.h"
#include "orc_math.h"

using namespace orc;

namespace {
// tracking::depthJumpThreshold (include/tracking/ICPShared.h:50-55).
inline float jumpThreshold(float d) { return std::max(0.03f, d * 0.05f); }

inline V3 ld(const float* a, int i) { return V3(a[3 * i], a[3 * i + 1], a[3 * i + 2]); }
inline void st(float* a, int i, V3 v) { a[3 * i] = v.x; a[3 * i + 1] = v.y; a[3 * i + 2] = v.z; }
}  // namespace

// updateVerticesFromDepth (src/sensor/FrameData.cpp:113-133).
extern "C" void orc_vertices_from_depth(const float* depth_m, int W, int H, orc_intrinsics K, float* vertices) {
    const float fx_inv = 1.0f / K.fx;
    const float fy_inv = 1.0f / K.fy;
#pragma omp parallel for schedule(static)
    for (int idx = 0; idx < W * H; ++idx) {
        const float d = depth_m[idx];
        if (d > 0.0f) {
            const int x = idx % W, y = idx / W;
            const float vx = (static_cast<float>(x) - K.cx) * fx_inv * d;
            const float vy = (static_cast<float>(y) - K.cy) * fy_inv * d;
            st(vertices, idx, V3(vx, vy, d));
        } else {
            st(vertices, idx, V3(0, 0, 0));
        }
    }
}

// buildFrameData (src/sensor/FrameData.cpp:137-194), geometry part.
extern "C" void orc_build_frame(const uint16_t* raw, int W, int H, orc_intrinsics K, float min_depth,
                                float max_depth, float* depth_m, float* vertices, float* normals) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < W * H; ++i) {
        depth_m[i] = cpuDepthMeters(raw[i], min_depth, max_depth);
        if (normals) st(normals, i, V3(0, 0, 0));
    }
    orc_vertices_from_depth(depth_m, W, H, K, vertices);
}

// computeNormals (src/sensor/FrameData.cpp:196-251). Border pixels are left as
// the caller initialised them (zero).
extern "C" void orc_compute_normals(const float* dm, const float* V, int W, int H, float* N) {
    for (int x = 0; x < W; ++x) { st(N, x, V3()); st(N, (H - 1) * W + x, V3()); }
    for (int y = 0; y < H; ++y) { st(N, y * W, V3()); st(N, y * W + W - 1, V3()); }
#pragma omp parallel for schedule(static)
    for (int y = 1; y < H - 1; ++y) {
        for (int x = 1; x < W - 1; ++x) {
            const int c = y * W + x, r = y * W + x + 1, l = y * W + x - 1, u = (y - 1) * W + x,
                      d = (y + 1) * W + x;
            if (dm[c] <= 0.0f || dm[r] <= 0.0f || dm[l] <= 0.0f || dm[u] <= 0.0f || dm[d] <= 0.0f) {
                st(N, c, V3());
                continue;
            }
            const float dc = dm[c];
            const float jump = jumpThreshold(dc);
            if (std::fabs(dc - dm[r]) > jump || std::fabs(dc - dm[l]) > jump ||
                std::fabs(dc - dm[u]) > jump || std::fabs(dc - dm[d]) > jump) {
                st(N, c, V3());
                continue;
            }
            const V3 dx = ld(V, r) - ld(V, l);
            const V3 dy = ld(V, d) - ld(V, u);
            const V3 n = cross(dx, dy);
            const float len = norm(n);
            st(N, c, len > 1e-6f ? n / len : V3());
        }
    }
}

// downsample (src/sensor/FrameData.cpp:262-334).
extern "C" void orc_downsample(const float* dm, const float* V, const float* N, int W, int H,
                               float* dmo, float* Vo, float* No) {
    const int DW = W / 2, DH = H / 2;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < DH; ++y) {
        for (int x = 0; x < DW; ++x) {
            const int sx = 2 * x, sy = 2 * y, o = y * DW + x;
            V3 sv(0, 0, 0), sn(0, 0, 0);
            float sd = 0.0f, dmin = 0.0f, dmax = 0.0f;
            int count = 0, mdx = 0, mdy = 0;
            for (int dy = 0; dy < 2; ++dy) {
                for (int dx = 0; dx < 2; ++dx) {
                    const int s = (sy + dy) * W + sx + dx;
                    const float d = dm[s];
                    if (d > 0.0f) {
                        sv = sv + ld(V, s);
                        sn = sn + ld(N, s);
                        sd += d;
                        if (count == 0 || d < dmin) { dmin = d; mdx = dx; mdy = dy; }
                        if (count == 0 || d > dmax) dmax = d;
                        ++count;
                    }
                }
            }
            V3 ov(0, 0, 0), on(0, 0, 0);
            float od = 0.0f;
            if (count > 0) {
                if (dmax - dmin > jumpThreshold(dmin)) {
                    const int m = (sy + mdy) * W + sx + mdx;
                    ov = ld(V, m);
                    od = dm[m];
                    const V3 nm = ld(N, m);
                    const float nl = norm(nm);
                    on = nl > 1e-6f ? nm / nl : V3();
                } else {
                    const float inv = 1.0f / static_cast<float>(count);
                    ov = sv * inv;
                    od = sd * inv;
                    const float nl = norm(sn);
                    on = nl > 1e-6f ? sn / nl : V3();
                }
            }
            st(Vo, o, ov);
            st(No, o, on);
            dmo[o] = od;
        }
    }
}

extern "C" float orc_raw_to_meters(uint16_t raw) { return rawToMeters(raw); }
extern "C" float orc_cpu_depth_meters(uint16_t raw, float lo, float hi) { return cpuDepthMeters(raw, lo, hi); }
extern "C" uint16_t orc_meters_to_raw(float m, float lo, float hi) { return metersToRaw(m, lo, hi); }
