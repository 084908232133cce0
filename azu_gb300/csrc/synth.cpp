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
