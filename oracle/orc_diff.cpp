// Oracle (test infrastructure only): the differentiation form's reference —
// depth rendering by the reference's front-face raycast (TSDFVolume.cpp:372-475,
// sampleTSDF :492-525, computeNormal :478-490), a Huber depth-residual loss, and
// its adjoint with respect to a right se(3) perturbation of the pose
// (pose * Exp(xi), xi = (rho, omega)) and to the tsdf values. No reference
// counterpart: the reference has no differentiable renderer.
//
// Two march precisions:
//   float  — decisions and sample positions exactly as the reference (and the
//            GPU) compute them; the adjoint is then evaluated in double on that
//            march (the "FP64 CPU adjoint" the GPU adjoint is checked against);
//   double — the whole forward in double, so that central finite differences
//            with a 1e-6 step are meaningful; the adjoint of the same march
//            checks the derivative formulas.
//
// The march is piecewise smooth: sample t_{k+1} = t_k + s(f_k) with
// s = far_step (invalid or f >= 0.999), max(min_step, 0.8 f trunc) otherwise;
// the start t_near is the camera-band or box-entry distance; the hit is the
// secant t_a + (t_b - t_a) f_a / (f_a - f_b). The adjoint differentiates all of
// it, holding the discrete branch choices fixed.
#include "orc_api.h"
#include "orc_math.h"

#include <algorithm>
#include <cmath>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <class T>
struct T3 {
    T x, y, z;
    T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

template <class T>
T3<T> mk(T a, T b, T c) { return T3<T>{a, b, c}; }

// One trilinear sample: value, the 8 corner indices and weights, and the
// gradient with respect to the world position.
template <class T>
struct Sample {
    bool valid = false;
    T f = 1;
    size_t corner[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    T w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    T grad[3] = {0, 0, 0};  // dF/dp (world, per metre)
};

template <class T>
struct VolT {
    const orc_tsdf_params* p;
    const T* tsdf;
    const float* weight;
    T vs, ox, oy, oz;
};

// sampleTSDF (TSDFVolume.cpp:492-525) in T, same expression order as the float
// reference; also returns the corners, weights and the position gradient.
template <class T>
bool sample_at(const VolT<T>& v, T px, T py, T pz, Sample<T>& s) {
    const int res = v.p->res;
    const T qx = (px - v.ox) / v.vs, qy = (py - v.oy) / v.vs, qz = (pz - v.oz) / v.vs;
    const T fx0 = std::floor(qx), fy0 = std::floor(qy), fz0 = std::floor(qz);
    const T lim = static_cast<T>(res - 1);
    s.valid = false;
    if (!(fx0 >= 0 && fy0 >= 0 && fz0 >= 0 && fx0 < lim && fy0 < lim && fz0 < lim)) return false;
    const int x0 = static_cast<int>(fx0), y0 = static_cast<int>(fy0), z0 = static_cast<int>(fz0);
    const T tx = qx - fx0, ty = qy - fy0, tz = qz - fz0;
    const size_t r = static_cast<size_t>(res);
    const size_t b = (static_cast<size_t>(z0) * r + static_cast<size_t>(y0)) * r + static_cast<size_t>(x0);
    const size_t c[8] = {b, b + 1, b + r, b + r + 1, b + r * r, b + r * r + 1, b + r * r + r, b + r * r + r + 1};
    for (size_t ci : c)
        if (!(v.weight[ci] > 0.0f)) return false;
    const T V[8] = {v.tsdf[c[0]], v.tsdf[c[1]], v.tsdf[c[2]], v.tsdf[c[3]],
                    v.tsdf[c[4]], v.tsdf[c[5]], v.tsdf[c[6]], v.tsdf[c[7]]};
    const T v00 = V[0] * (1 - tx) + V[1] * tx;
    const T v10 = V[2] * (1 - tx) + V[3] * tx;
    const T v01 = V[4] * (1 - tx) + V[5] * tx;
    const T v11 = V[6] * (1 - tx) + V[7] * tx;
    const T v0 = v00 * (1 - ty) + v10 * ty;
    const T v1 = v01 * (1 - ty) + v11 * ty;
    s.f = v0 * (1 - tz) + v1 * tz;
    s.valid = true;
    for (int i = 0; i < 8; ++i) s.corner[i] = c[i];
    const T ux = 1 - tx, uy = 1 - ty, uz = 1 - tz;
    s.w[0] = ux * uy * uz; s.w[1] = tx * uy * uz; s.w[2] = ux * ty * uz; s.w[3] = tx * ty * uz;
    s.w[4] = ux * uy * tz; s.w[5] = tx * uy * tz; s.w[6] = ux * ty * tz; s.w[7] = tx * ty * tz;
    const T gx = (uy * uz * (V[1] - V[0]) + ty * uz * (V[3] - V[2]) + uy * tz * (V[5] - V[4]) + ty * tz * (V[7] - V[6]));
    const T gy = (ux * uz * (V[2] - V[0]) + tx * uz * (V[3] - V[1]) + ux * tz * (V[6] - V[4]) + tx * tz * (V[7] - V[5]));
    const T gz = (ux * uy * (V[4] - V[0]) + tx * uy * (V[5] - V[1]) + ux * ty * (V[6] - V[2]) + tx * ty * (V[7] - V[3]));
    s.grad[0] = gx / v.vs;
    s.grad[1] = gy / v.vs;
    s.grad[2] = gz / v.vs;
    return true;
}

template <class T>
bool sample_f(const VolT<T>& v, T px, T py, T pz, T& f) {
    Sample<T> s;
    if (!sample_at(v, px, py, pz, s)) return false;
    f = s.f;
    return true;
}

// computeNormal (TSDFVolume.cpp:478-490): only whether a normal exists matters
// for the depth image (the reference drops the pixel otherwise).
template <class T>
bool normal_exists(const VolT<T>& v, T px, T py, T pz) {
    const T h = v.vs;
    T s[6];
    if (!sample_f(v, px + h, py + T(0), pz + T(0), s[0]) || !sample_f(v, px - h, py - T(0), pz - T(0), s[1]))
        return false;
    if (!sample_f(v, px + T(0), py + h, pz + T(0), s[2]) || !sample_f(v, px - T(0), py - h, pz - T(0), s[3]))
        return false;
    if (!sample_f(v, px + T(0), py + T(0), pz + h, s[4]) || !sample_f(v, px - T(0), py - T(0), pz - h, s[5]))
        return false;
    const T nx = s[0] - s[1], ny = s[2] - s[3], nz = s[4] - s[5];
    const T len = std::sqrt(nx * nx + (ny * ny + nz * nz));  // dot3 order of orc_math.h
    return len > T(1e-6) && std::isfinite(len);
}

struct MarchRec {
    std::vector<double> t, f;   // every evaluated sample
    std::vector<char> dep;      // step k -> k+1 depends on f_k
    std::vector<char> clipped;  // t_{k+1} was clipped to t_far
    int near_axis = -1;         // -1: camera band; else the box-entry axis
    double t_near = 0, d_near = 0, t_hit = 0;
    bool hit = false;
};

// The reference's march (TSDFVolume.cpp:372-475) in T for one ray.
template <class T>
void march(const VolT<T>& v, const T o[3], const T d[3], T ray_norm, T min_depth, T max_depth, T trunc,
           const T box_lo[3], const T box_hi[3], MarchRec& rec) {
    rec = MarchRec();
    const T min_step = T(0.5) * v.vs;
    const T far_c = T(0.8) * trunc;
    const T far_step = std::max(min_step, far_c);
    T t_near = min_depth * ray_norm;
    T t_far = max_depth * ray_norm;
    int near_axis = -1;
    for (int a = 0; a < 3; ++a) {
        const T inv = T(1) / d[a];
        T t0 = (box_lo[a] - o[a]) * inv;
        T t1 = (box_hi[a] - o[a]) * inv;
        if (t0 > t1) std::swap(t0, t1);
        if (std::isnan(t0) || std::isnan(t1)) {
            if (o[a] < box_lo[a] || o[a] > box_hi[a]) t_far = T(-1);
            continue;
        }
        if (t0 > t_near) near_axis = a;
        t_near = std::max(t_near, t0);
        t_far = std::min(t_far, t1);
    }
    rec.near_axis = near_axis;
    rec.t_near = t_near;
    if (near_axis >= 0) rec.d_near = d[near_axis];
    if (!(t_near < t_far)) return;
    T t_prev = t_near, f_prev = 1;
    bool prev_valid = sample_f(v, o[0] + d[0] * t_prev, o[1] + d[1] * t_prev, o[2] + d[2] * t_prev, f_prev);
    rec.t.push_back(t_prev);
    rec.f.push_back(f_prev);
    if (prev_valid && !std::isfinite(f_prev)) return;
    if (prev_valid && f_prev < 0) return;
    while (t_prev < t_far) {
        T step;
        bool dep = false;
        if (!prev_valid || f_prev >= T(0.999)) {
            step = far_step;
        } else {
            const T sf = T(0.8) * f_prev * trunc;
            dep = sf > min_step;
            step = std::max(min_step, sf);
        }
        const T tn = t_prev + step;
        const bool clip = !(tn < t_far) && tn != t_far;
        const T t = std::min(tn, t_far);
        rec.dep.push_back(dep);
        rec.clipped.push_back(clip);
        T f = 1;
        const bool valid = sample_f(v, o[0] + d[0] * t, o[1] + d[1] * t, o[2] + d[2] * t, f);
        rec.t.push_back(t);
        rec.f.push_back(f);
        if (valid && !std::isfinite(f)) return;
        if (valid && prev_valid) {
            if (f_prev > 0 && f <= 0) {
                const T th = t_prev + (t - t_prev) * (f_prev / (f_prev - f));
                const T hx = o[0] + d[0] * th, hy = o[1] + d[1] * th, hz = o[2] + d[2] * th;
                if (!normal_exists(v, hx, hy, hz)) return;
                if (!(std::isfinite(hx) && std::isfinite(hy) && std::isfinite(hz))) return;
                rec.t_hit = th;
                rec.hit = true;
                return;
            }
            if (f_prev < 0 && f >= 0) return;
        } else if (valid && f < 0) {
            return;
        }
        t_prev = t;
        f_prev = f;
        prev_valid = valid;
        if (t >= t_far) return;
    }
}

// Adjoint of D = t_hit / ray_norm for one marched ray, in double. Adds
// seed * dD/dxi to jac[6] and seed_v * dD/dV to grad_v (when non-null).
template <class T>
void depth_adjoint(const VolT<T>& v, const double o[3], const double d[3], const double rn[3], const double R0[9],
                   double ray_norm, double trunc, const MarchRec& rec, const T box_face[3], double* jac,
                   double seed_v, double* grad_v) {
    const int b = static_cast<int>(rec.t.size()) - 1, a = b - 1;
    std::vector<double> at(rec.t.size(), 0.0), af(rec.t.size(), 0.0);
    const double ta = rec.t[a], tb = rec.t[b], fa = rec.f[a], fb = rec.f[b];
    const double den = fa - fb;
    const double inv_rn = 1.0 / ray_norm;
    at[a] += (1.0 - fa / den) * inv_rn;
    at[b] += (fa / den) * inv_rn;
    af[a] += (tb - ta) * (-fb) / (den * den) * inv_rn;
    af[b] += (tb - ta) * fa / (den * den) * inv_rn;
    for (int k = b; k >= 0; --k) {
        if (af[k] != 0.0) {
            Sample<T> s;
            const T tk = static_cast<T>(rec.t[k]);
            sample_at(v, static_cast<T>(o[0]) + static_cast<T>(d[0]) * tk, static_cast<T>(o[1]) + static_cast<T>(d[1]) * tk,
                      static_cast<T>(o[2]) + static_cast<T>(d[2]) * tk, s);
            const double g[3] = {double(s.grad[0]), double(s.grad[1]), double(s.grad[2])};
            at[k] += af[k] * (g[0] * d[0] + g[1] * d[1] + g[2] * d[2]);
            // R0^T g
            const double h[3] = {R0[0] * g[0] + R0[3] * g[1] + R0[6] * g[2], R0[1] * g[0] + R0[4] * g[1] + R0[7] * g[2],
                                 R0[2] * g[0] + R0[5] * g[1] + R0[8] * g[2]};
            jac[0] += af[k] * h[0];
            jac[1] += af[k] * h[1];
            jac[2] += af[k] * h[2];
            const double tk_d = rec.t[k];
            jac[3] += af[k] * tk_d * (rn[1] * h[2] - rn[2] * h[1]);
            jac[4] += af[k] * tk_d * (rn[2] * h[0] - rn[0] * h[2]);
            jac[5] += af[k] * tk_d * (rn[0] * h[1] - rn[1] * h[0]);
            if (grad_v)
                for (int i = 0; i < 8; ++i) {
                    const double gv = seed_v * af[k] * double(s.w[i]);
#pragma omp atomic
                    grad_v[s.corner[i]] += gv;
                }
        }
        if (k >= 1) {
            if (!rec.clipped[k - 1]) {
                at[k - 1] += at[k];
                if (rec.dep[k - 1]) af[k - 1] += at[k] * 0.8 * trunc;
            }
        }
    }
    // t_near: box entry (B - o_a) / d_a, or the camera band (no pose dependence)
    if (rec.near_axis >= 0) {
        const int ax = rec.near_axis;
        const double da = d[ax];
        const double t0 = rec.t_near;
        const double Ra[3] = {R0[3 * ax], R0[3 * ax + 1], R0[3 * ax + 2]};
        jac[0] += at[0] * (-Ra[0] / da);
        jac[1] += at[0] * (-Ra[1] / da);
        jac[2] += at[0] * (-Ra[2] / da);
        const double cx = rn[1] * Ra[2] - rn[2] * Ra[1], cy = rn[2] * Ra[0] - rn[0] * Ra[2],
                     cz = rn[0] * Ra[1] - rn[1] * Ra[0];
        jac[3] += at[0] * (-t0 / da) * cx;
        jac[4] += at[0] * (-t0 / da) * cy;
        jac[5] += at[0] * (-t0 / da) * cz;
    }
    (void)box_face;
}

// pose * Exp(xi) in double, xi = (rho, omega).
void perturb(const double P[16], const double xi[6], double out[16]) {
    const double wx = xi[3], wy = xi[4], wz = xi[5];
    const double th2 = wx * wx + wy * wy + wz * wz, th = std::sqrt(th2);
    double A, B, Cc;  // R = I + A W + B W^2, V = I + B W + Cc W^2
    if (th < 1e-4) {
        A = 1.0 - th2 / 6.0;
        B = 0.5 - th2 / 24.0;
        Cc = 1.0 / 6.0 - th2 / 120.0;
    } else {
        A = std::sin(th) / th;
        B = (1.0 - std::cos(th)) / th2;
        Cc = (th - std::sin(th)) / (th2 * th);
    }
    const double W[9] = {0, -wz, wy, wz, 0, -wx, -wy, wx, 0};
    double W2[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0;
            for (int k = 0; k < 3; ++k) s += W[3 * i + k] * W[3 * k + j];
            W2[3 * i + j] = s;
        }
    double R[9], V[9];
    for (int i = 0; i < 9; ++i) {
        const double I = (i % 4 == 0) ? 1.0 : 0.0;
        R[i] = I + A * W[i] + B * W2[i];
        V[i] = I + B * W[i] + Cc * W2[i];
    }
    const double t[3] = {V[0] * xi[0] + V[1] * xi[1] + V[2] * xi[2], V[3] * xi[0] + V[4] * xi[1] + V[5] * xi[2],
                         V[6] * xi[0] + V[7] * xi[1] + V[8] * xi[2]};
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) {
            double s = 0;
            for (int k = 0; k < 3; ++k) s += P[4 * i + k] * R[3 * k + j];
            out[4 * i + j] = s;
        }
        double s = P[4 * i + 3];
        for (int k = 0; k < 3; ++k) s += P[4 * i + k] * t[k];
        out[4 * i + 3] = s;
    }
    out[12] = out[13] = out[14] = 0.0;
    out[15] = 1.0;
}

double huber(double r, double delta, double* dr) {
    const double a = std::fabs(r);
    if (a <= delta) {
        *dr = r;
        return 0.5 * r * r;
    }
    *dr = r > 0 ? delta : -delta;
    return delta * (a - 0.5 * delta);
}

template <class T>
void run(const orc_tsdf_params* p, const T* tsdf, const float* weight, const double pose[16], orc_intrinsics K, int W,
         int H, const float* depth_obs, double delta, double* loss_out, double* grad_xi, double* grad_v,
         double* depth_out, double* jac_out, int* n_valid) {
    VolT<T> v{p, tsdf, weight, static_cast<T>(p->voxel_size), static_cast<T>(p->origin[0]),
              static_cast<T>(p->origin[1]), static_cast<T>(p->origin[2])};
    const T span = static_cast<T>(p->res - 1) * v.vs;
    const T box_lo[3] = {v.ox, v.oy, v.oz};
    const T box_hi[3] = {v.ox + span, v.oy + span, v.oz + span};
    const T Ro[9] = {T(pose[0]), T(pose[1]), T(pose[2]), T(pose[4]), T(pose[5]), T(pose[6]),
                     T(pose[8]), T(pose[9]), T(pose[10])};
    const T o[3] = {T(pose[3]), T(pose[7]), T(pose[11])};
    const double R0[9] = {double(Ro[0]), double(Ro[1]), double(Ro[2]), double(Ro[3]), double(Ro[4]),
                          double(Ro[5]), double(Ro[6]), double(Ro[7]), double(Ro[8])};
    const T fx = T(K.fx), fy = T(K.fy), cx = T(K.cx), cy = T(K.cy);
    const T trunc = T(p->truncation);
    double loss = 0.0, g[6] = {0, 0, 0, 0, 0, 0};
    int nv = 0;
#pragma omp parallel for schedule(dynamic, 8) reduction(+ : loss, nv)
    for (int y = 0; y < H; ++y) {
        double gl[6] = {0, 0, 0, 0, 0, 0};
        MarchRec rec;
        for (int x = 0; x < W; ++x) {
            const int pix = y * W + x;
            if (depth_out) depth_out[pix] = 0.0;
            if (jac_out)
                for (int j = 0; j < 6; ++j) jac_out[6 * pix + j] = 0.0;
            const T rc[3] = {(T(x) - cx) / fx, (T(y) - cy) / fy, T(1)};
            // norm and M3 * v with the dot3 order of orc_math.h: a0 b0 + (a1 b1 + a2 b2)
            const T ray_norm = std::sqrt(rc[0] * rc[0] + (rc[1] * rc[1] + rc[2] * rc[2]));
            const T Rr[3] = {Ro[0] * rc[0] + (Ro[1] * rc[1] + Ro[2] * rc[2]),
                             Ro[3] * rc[0] + (Ro[4] * rc[1] + Ro[5] * rc[2]),
                             Ro[6] * rc[0] + (Ro[7] * rc[1] + Ro[8] * rc[2])};
            const T d[3] = {Rr[0] / ray_norm, Rr[1] / ray_norm, Rr[2] / ray_norm};
            march(v, o, d, ray_norm, T(p->min_depth), T(p->max_depth), trunc, box_lo, box_hi, rec);
            if (!rec.hit) continue;
            const double D = rec.t_hit / double(ray_norm);
            if (depth_out) depth_out[pix] = D;
            const double od[3] = {double(o[0]), double(o[1]), double(o[2])};
            const double dd[3] = {double(d[0]), double(d[1]), double(d[2])};
            const double rn[3] = {double(rc[0]) / double(ray_norm), double(rc[1]) / double(ray_norm),
                                  double(rc[2]) / double(ray_norm)};
            const double obs = depth_obs ? double(depth_obs[pix]) : 0.0;
            const bool use = depth_obs && obs >= p->min_depth && obs <= p->max_depth;
            double dr = 0.0;
            if (use) {
                loss += huber(D - obs, delta, &dr);
                ++nv;
            }
            if (jac_out || (use && (grad_xi || grad_v))) {
                double J[6] = {0, 0, 0, 0, 0, 0};
                depth_adjoint(v, od, dd, rn, R0, double(ray_norm), double(trunc), rec, box_lo, J,
                              use ? dr : 0.0, use ? grad_v : nullptr);
                if (jac_out)
                    for (int j = 0; j < 6; ++j) jac_out[6 * pix + j] = J[j];
                if (use)
                    for (int j = 0; j < 6; ++j) gl[j] += dr * J[j];
            }
        }
#pragma omp critical
        for (int j = 0; j < 6; ++j) g[j] += gl[j];
    }
    if (loss_out) *loss_out = loss;
    if (grad_xi)
        for (int j = 0; j < 6; ++j) grad_xi[j] = g[j];
    if (n_valid) *n_valid = nv;
}

}  // namespace

extern "C" void orc_depth_adjoint_f(const orc_tsdf_params* p, const float* tsdf, const float* weight,
                                    const float pose_rm[16], orc_intrinsics K, int width, int height,
                                    const float* depth_obs, double huber_delta, double* loss, double grad_xi[6],
                                    double* grad_tsdf, double* depth_out, double* jac_out, int* n_valid) {
    double P[16];
    for (int i = 0; i < 16; ++i) P[i] = pose_rm[i];
    run<float>(p, tsdf, weight, P, K, width, height, depth_obs, huber_delta, loss, grad_xi, grad_tsdf, depth_out,
               jac_out, n_valid);
}

extern "C" void orc_depth_loss_d(const orc_tsdf_params* p, const double* tsdf, const float* weight,
                                 const double pose_rm[16], const double xi[6], orc_intrinsics K, int width, int height,
                                 const float* depth_obs, double huber_delta, double* loss, double grad_xi[6],
                                 double* grad_tsdf, double* depth_out, double* jac_out, int* n_valid) {
    double P[16];
    perturb(pose_rm, xi, P);
    run<double>(p, tsdf, weight, P, K, width, height, depth_obs, huber_delta, loss, grad_xi, grad_tsdf, depth_out,
                jac_out, n_valid);
}
