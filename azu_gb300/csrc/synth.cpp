// Seeded synthetic depth sequences for the benchmarks and parity tests: an
// analytic scene (spheres, one box rotated about y, a floor plane) ray-traced to
// Z-depth at 640x480, with depth-dependent Gaussian noise, millimetre
// quantisation and random zero dropout. Host code (OpenMP), deterministic for a
// given seed: every pixel draws from its own counter-based stream.
#include <cmath>
#include <cstdint>
#include <cstring>

extern "C" {

typedef struct {
    double center[3];
    double radius;
} azu_synth_sphere;

typedef struct {
    int n_spheres;
    const azu_synth_sphere* spheres;
    double box_center[3];
    double box_half;      // half extent of the cube
    double box_yaw_deg;   // rotation about +y
    double floor_y;       // plane y = floor_y
    int has_floor;
} azu_synth_scene;

typedef struct {
    double sigma_a;    // noise sigma = sigma_a * z^2 (m)
    double dropout;    // probability of a zero pixel
    uint64_t seed;
    uint64_t frame;
    double max_range;  // Z beyond this -> 0
} azu_synth_noise;

int azu_synth_render(const azu_synth_scene* sc, const double pose_wc[16], double fx, double fy, double cx,
                     double cy, int W, int H, const azu_synth_noise* nz, uint16_t* depth_mm);
}

namespace {

inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline double unit(uint64_t u) { return (static_cast<double>(u >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

double hitSphere(const double* o, const double* d, const azu_synth_sphere& s) {
    const double oc[3] = {o[0] - s.center[0], o[1] - s.center[1], o[2] - s.center[2]};
    const double a = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const double b = oc[0] * d[0] + oc[1] * d[1] + oc[2] * d[2];
    const double c = oc[0] * oc[0] + oc[1] * oc[1] + oc[2] * oc[2] - s.radius * s.radius;
    const double disc = b * b - a * c;
    if (disc < 0) return INFINITY;
    const double sq = std::sqrt(disc);
    double t = (-b - sq) / a;
    if (t > 1e-9) return t;
    t = (-b + sq) / a;
    return t > 1e-9 ? t : INFINITY;
}

double hitBox(const double* o, const double* d, const azu_synth_scene& sc) {
    const double yaw = sc.box_yaw_deg * M_PI / 180.0;
    const double c = std::cos(yaw), s = std::sin(yaw);
    // world -> box: inverse rotation about y.
    const double po[3] = {o[0] - sc.box_center[0], o[1] - sc.box_center[1], o[2] - sc.box_center[2]};
    const double lo[3] = {c * po[0] - s * po[2], po[1], s * po[0] + c * po[2]};
    const double ld[3] = {c * d[0] - s * d[2], d[1], s * d[0] + c * d[2]};
    double tn = -INFINITY, tf = INFINITY;
    for (int a = 0; a < 3; ++a) {
        if (std::fabs(ld[a]) < 1e-15) {
            if (lo[a] < -sc.box_half || lo[a] > sc.box_half) return INFINITY;
            continue;
        }
        double t0 = (-sc.box_half - lo[a]) / ld[a], t1 = (sc.box_half - lo[a]) / ld[a];
        if (t0 > t1) std::swap(t0, t1);
        tn = std::max(tn, t0);
        tf = std::min(tf, t1);
    }
    if (tn > tf || tf <= 1e-9) return INFINITY;
    return tn > 1e-9 ? tn : tf;
}

}  // namespace

extern "C" int azu_synth_render(const azu_synth_scene* sc, const double P[16], double fx, double fy, double cx,
                                double cy, int W, int H, const azu_synth_noise* nz, uint16_t* depth_mm) {
    if (!sc || !P || !nz || !depth_mm || W <= 0 || H <= 0) return -1;
    const double o[3] = {P[3], P[7], P[11]};
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y) {
        for (int x = 0; x < W; ++x) {
            const double dc[3] = {(x - cx) / fx, (y - cy) / fy, 1.0};
            // D = R dc, so the ray parameter t is the camera Z-depth.
            const double d[3] = {P[0] * dc[0] + P[1] * dc[1] + P[2] * dc[2],
                                 P[4] * dc[0] + P[5] * dc[1] + P[6] * dc[2],
                                 P[8] * dc[0] + P[9] * dc[1] + P[10] * dc[2]};
            double t = INFINITY;
            for (int i = 0; i < sc->n_spheres; ++i) t = std::min(t, hitSphere(o, d, sc->spheres[i]));
            if (sc->box_half > 0) t = std::min(t, hitBox(o, d, *sc));
            if (sc->has_floor && std::fabs(d[1]) > 1e-15) {
                const double tp = (sc->floor_y - o[1]) / d[1];
                if (tp > 1e-9) t = std::min(t, tp);
            }
            const uint64_t key = mix64(nz->seed ^ mix64(nz->frame * 0x100000001b3ull + static_cast<uint64_t>(y) * W + x));
            uint16_t out = 0;
            if (std::isfinite(t) && t <= nz->max_range) {
                const double u1 = unit(mix64(key ^ 0x1)), u2 = unit(mix64(key ^ 0x2)), u3 = unit(mix64(key ^ 0x3));
                const double g = std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
                const double z = t + nz->sigma_a * t * t * g;
                const double mm = std::floor(z * 1000.0 + 0.5);
                if (u3 >= nz->dropout && mm > 0 && mm < 65535) out = static_cast<uint16_t>(mm);
            }
            depth_mm[static_cast<size_t>(y) * W + x] = out;
        }
    }
    return 0;
}

// ---------------------------------------------------------------------------
// The reference contract tests' room scene (tests/support/SyntheticScene.h of
// the reference): the inside of a room box (centre (0, -0.05, 1.15), half
// extents (1.2, 0.95, 1.25)), a box (centre (0.35, 0.55, 1.5), half extents
// (0.3, 0.35, 0.25)) and a sphere (centre (-0.5, 0.2, 1.7), radius 0.3), as a
// signed distance, sphere-traced per pixel in float: t from 0.05 m, at most 256
// steps, below 8 m, a hit when the distance drops below 1e-5; Z-depth in metres
// (0 on a miss). Used as a fixture for the parity tests of those contracts.
namespace {

struct F3s {
    float x, y, z;
};

inline float len3(F3s a) { return std::sqrt(a.x * a.x + (a.y * a.y + a.z * a.z)); }

inline float box_sdf(F3s p, F3s c, F3s h) {
    const F3s q{std::fabs(p.x - c.x) - h.x, std::fabs(p.y - c.y) - h.y, std::fabs(p.z - c.z) - h.z};
    const F3s qp{std::fmax(q.x, 0.0f), std::fmax(q.y, 0.0f), std::fmax(q.z, 0.0f)};
    return len3(qp) + std::fmin(std::fmax(q.x, std::fmax(q.y, q.z)), 0.0f);
}

inline float room_sdf(F3s p) {
    const float room = -box_sdf(p, F3s{0.0f, -0.05f, 1.15f}, F3s{1.2f, 0.95f, 1.25f});
    const float box = box_sdf(p, F3s{0.35f, 0.55f, 1.5f}, F3s{0.3f, 0.35f, 0.25f});
    const float sph = len3(F3s{p.x + 0.5f, p.y - 0.2f, p.z - 1.7f}) - 0.3f;
    return std::fmin(room, std::fmin(box, sph));
}

}  // namespace

extern "C" int azu_synth_room_depth(const float pose_wc[16], float fx, float fy, float cx, float cy, int W, int H,
                                    float* depth_m) {
    if (!pose_wc || !depth_m || W <= 0 || H <= 0) return -1;
    const float* P = pose_wc;  // row-major world-from-camera
#pragma omp parallel for schedule(dynamic, 8)
    for (int v = 0; v < H; ++v) {
        for (int u = 0; u < W; ++u) {
            const F3s rc{(static_cast<float>(u) - cx) / fx, (static_cast<float>(v) - cy) / fy, 1.0f};
            const float nrm = len3(rc);
            const F3s d{(P[0] * rc.x + (P[1] * rc.y + P[2] * rc.z)) / nrm, (P[4] * rc.x + (P[5] * rc.y + P[6] * rc.z)) / nrm,
                        (P[8] * rc.x + (P[9] * rc.y + P[10] * rc.z)) / nrm};
            const F3s o{P[3], P[7], P[11]};
            float t = 0.05f, out = 0.0f;
            for (int i = 0; i < 256 && t < 8.0f; ++i) {
                const float s = room_sdf(F3s{o.x + d.x * t, o.y + d.y * t, o.z + d.z * t});
                if (s < 1e-5f) {
                    out = t / nrm;
                    break;
                }
                t += s;
            }
            depth_m[static_cast<size_t>(v) * W + u] = out;
        }
    }
    return 0;
}
