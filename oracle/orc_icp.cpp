// Oracle (test infrastructure only): CPU restatement of the reference's
// coarse-to-fine point-to-plane ICP (src/tracking/ICPTracker.cpp:40-354, numeric
// policy include/tracking/ICPShared.h:34-110) and of the tracking grade
// (include/tracking/TrackingPolicy.h:40-112).
//
// The reference reduces per OpenMP thread under schedule(static) and folds the
// partials in thread order (ICPTracker.cpp:220-229, :334-351); its float sums
// therefore depend on the thread count. Here the partition is explicit
// (orc_icp_params::fold_threads, libgomp's static split of rows 1..H-2), so the
// result is a pure function of that count, whatever OpenMP does.
//
// Eigen's solvers are restated, not reproduced: the damping decision uses
// eigenvalues from a cyclic Jacobi sweep (double), the step solves the damped
// system by LDL^T with diagonal pivoting (float), and the SO(3) projection is
// U V^T of the SVD (double, rounded to float). They agree with Eigen to
// rounding; decisions can differ only at a threshold's exact edge.
#include "orc_api.h"
#include "orc_math.h"
#include "orc_linalg.h"

#include <vector>

using namespace orc;

namespace {

constexpr float kHuberK = 0.02f;
constexpr float kDampingDefault = 0.1f, kDampingLevel0 = 0.01f, kDampingEscalated = 1.0f;
constexpr float kCondEscalate = 1e7f, kMinEigEscalate = 1e-4f;
constexpr float kTranslationCapStep = 0.2f, kRotationCapStep = 0.5f;
constexpr float kModelVertexNormSqMin = 1e-12f, kNormalNormSqMin = 0.9f;
constexpr float kConvergenceStep = 5e-5f, kAcceptableFinalStep = 1e-3f;
constexpr int kMinInliersForIteration = 10, kMinInliersForOk = 100;

inline V3 ld(const float* a, size_t i) { return V3(a[3 * i], a[3 * i + 1], a[3 * i + 2]); }

// ICPTracker::sanitizeParams (src/tracking/ICPTracker.cpp:24-34): a non-finite
// angle threshold falls back to 30 degrees, others are clamped to [0, 85].
inline float sanitizeAngle(float a) {
    if (!std::isfinite(a)) return 30.0f;
    if (a < 0.0f) return 0.0f;
    if (a > 85.0f) return 85.0f;
    return a;
}
inline float huberLoss(float a) { return (a <= kHuberK) ? a * a : 2.0f * kHuberK * a - kHuberK * kHuberK; }
inline bool modelVertexValid(V3 v) { return finite3(v) && sqnorm(v) > kModelVertexNormSqMin; }
inline bool normalValid(V3 n) { return finite3(n) && sqnorm(n) > kNormalNormSqMin; }

// Symmetric eigenvalues by cyclic Jacobi (double), ascending (orc_linalg.h).
inline void jacobiEigen(int n, double* a, double* ev, double* vec) { linalg::jacobi_eigen(n, a, ev, vec); }

// dampingForHessian (include/tracking/ICPShared.h:86-100).
float dampingForHessian(const float A[36], int level) {
    double a[36], ev[6];
    for (int i = 0; i < 36; ++i) a[i] = A[i];
    jacobiEigen(6, a, ev, nullptr);
    const float mn = static_cast<float>(ev[0]), mx = static_cast<float>(ev[5]);
    if (!std::isfinite(mn) || !std::isfinite(mx) || mn < kMinEigEscalate) return kDampingEscalated;
    if (mx > kCondEscalate * mn) return kDampingEscalated;
    return level == 0 ? kDampingLevel0 : kDampingDefault;
}

// A x = b by LDL^T with symmetric diagonal pivoting (float, orc_linalg.h).
inline void ldltSolve(const float A_in[36], const float b[6], float x[6]) { linalg::ldlt_solve6(A_in, b, x); }

// projectToSO3 (include/tracking/ICPShared.h:102-110): U V^T with the sign fix.
M3 projectToSO3(const M3& M) {
    double m[9], mtm[9], ev[3], V[9];
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) m[i * 3 + j] = M.m[i][j];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0;
            for (int k = 0; k < 3; ++k) s += m[k * 3 + i] * m[k * 3 + j];
            mtm[i * 3 + j] = s;
        }
    jacobiEigen(3, mtm, ev, V);
    double U[9];
    for (int j = 0; j < 3; ++j) {
        const double sig = std::sqrt(std::max(ev[j], 1e-300));
        for (int i = 0; i < 3; ++i) {
            double s = 0;
            for (int k = 0; k < 3; ++k) s += m[i * 3 + k] * V[k * 3 + j];
            U[i * 3 + j] = s / sig;
        }
    }
    auto det3 = [](const double* a) {
        return a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) + a[2] * (a[3] * a[7] - a[4] * a[6]);
    };
    double R[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0;
            for (int k = 0; k < 3; ++k) s += U[i * 3 + k] * V[j * 3 + k];
            R[i * 3 + j] = s;
        }
    if (det3(R) < 0.0) {
        // Flip the singular vector of the smallest singular value (ev ascending: column 0).
        for (int i = 0; i < 3; ++i) U[i * 3 + 0] = -U[i * 3 + 0];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double s = 0;
                for (int k = 0; k < 3; ++k) s += U[i * 3 + k] * V[j * 3 + k];
                R[i * 3 + j] = s;
            }
    }
    M3 out;
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) out.m[i][j] = static_cast<float>(R[i * 3 + j]);
    return out;
}

// Eigen::AngleAxisf::toRotationMatrix (Rodrigues).
M3 angleAxis(float angle, V3 axis) {
    const float s = std::sin(angle), c = std::cos(angle);
    const V3 sa = axis * s;
    const V3 ca = axis * (1.0f - c);
    M3 r;
    float tmp = ca.x * axis.y;
    r.m[0][1] = tmp - sa.z; r.m[1][0] = tmp + sa.z;
    tmp = ca.x * axis.z;
    r.m[0][2] = tmp + sa.y; r.m[2][0] = tmp - sa.y;
    tmp = ca.y * axis.z;
    r.m[1][2] = tmp - sa.x; r.m[2][1] = tmp + sa.x;
    r.m[0][0] = ca.x * axis.x + c; r.m[1][1] = ca.y * axis.y + c; r.m[2][2] = ca.z * axis.z + c;
    return r;
}

// S = float: the reference's per-thread float partial sums. S = double: the
// same per-pixel float terms accumulated in double (the FP64 reduction oracle).
template <typename S>
struct Acc {
    S A[21], b[6], residual;
    int count, valid_live, valid_model, projected, dist_f, angle_f;
    Acc() : residual(0), count(0), valid_live(0), valid_model(0), projected(0), dist_f(0), angle_f(0) {
        for (S& v : A) v = 0;
        for (S& v : b) v = 0;
    }
};

template <typename S>
int build_system_impl(const orc_icp_params* prm, orc_intrinsics camK, const float* live_v, const float* live_n,
                      int W, int H, const float* model_v, const float* model_n, int MW, int MH,
                      const float pose_rm[16], const float ref_rm[16], float Aout[36], float bout[6],
                      float* residual, int counts[6], double* A64, double* b64);

}  // namespace

extern "C" int orc_icp_build_system(const orc_icp_params* prm, orc_intrinsics camK, const float* live_v,
                                    const float* live_n, int W, int H, const float* model_v,
                                    const float* model_n, int MW, int MH, const float pose_rm[16],
                                    const float ref_rm[16], float Aout[36], float bout[6], float* residual,
                                    int counts[6]) {
    if (prm->fold_threads <= 0)
        return build_system_impl<double>(prm, camK, live_v, live_n, W, H, model_v, model_n, MW, MH, pose_rm, ref_rm,
                                         Aout, bout, residual, counts, nullptr, nullptr);
    return build_system_impl<float>(prm, camK, live_v, live_n, W, H, model_v, model_n, MW, MH, pose_rm, ref_rm,
                                    Aout, bout, residual, counts, nullptr, nullptr);
}

extern "C" int orc_icp_build_system_f64(const orc_icp_params* prm, orc_intrinsics camK, const float* live_v,
                                        const float* live_n, int W, int H, const float* model_v,
                                        const float* model_n, int MW, int MH, const float pose_rm[16],
                                        const float ref_rm[16], double A64[36], double b64[6], int counts[6]) {
    float A[36], b[6], r;
    return build_system_impl<double>(prm, camK, live_v, live_n, W, H, model_v, model_n, MW, MH, pose_rm, ref_rm, A,
                                     b, &r, counts, A64, b64);
}

namespace {
template <typename S>
int build_system_impl(const orc_icp_params* prm, orc_intrinsics camK, const float* live_v, const float* live_n,
                      int W, int H, const float* model_v, const float* model_n, int MW, int MH,
                      const float pose_rm[16], const float ref_rm[16], float Aout[36], float bout[6],
                      float* residual, int counts[6], double* A64, double* b64) {
    for (int i = 0; i < 36; ++i) Aout[i] = 0;
    for (int i = 0; i < 6; ++i) { bout[i] = 0; counts[i] = 0; }
    *residual = 0;
    if (MW <= 0 || MH <= 0) return 0;
    // scaleIntrinsics (include/sensor/CameraIntrinsics.h:33-40) to the model size.
    orc_intrinsics K = camK;
    if (!(MW == 640 && MH == 480)) {
        const float sx = static_cast<float>(MW) / 640.0f, sy = static_cast<float>(MH) / 480.0f;
        K = orc_intrinsics{camK.fx * sx, camK.fy * sy, (camK.cx + 0.5f) * sx - 0.5f, (camK.cy + 0.5f) * sy - 0.5f};
    }
    const float angle_cos = static_cast<float>(std::cos(sanitizeAngle(prm->angle_threshold) * M_PI / 180.0f));
    const float dist2 = prm->dist_threshold * prm->dist_threshold;
    const M4 pose = M4::from(pose_rm);
    const M3 R_cw = pose.R();
    const V3 t_cw = pose.t();
    const M4 ref_inv = inverse4(M4::from(ref_rm));
    const M3 R_rc = ref_inv.R();
    const V3 t_rc = ref_inv.t();
    const M3 R_rel = R_rc * R_cw;
    const V3 t_rel = R_rc * t_cw + t_rc;
    const M3 R_cwT = R_cw.T();

    const int T = prm->fold_threads > 0 ? prm->fold_threads : 64;
    std::vector<Acc<S>> local(T);
    const int nrows = std::max(0, H - 2);
#pragma omp parallel for schedule(static)
    for (int tid = 0; tid < T; ++tid) {
        // libgomp static split of nrows among T threads.
        int q = nrows / T, t = nrows % T;
        if (tid < t) { t = 0; ++q; }
        const int s0 = q * tid + t, e0 = s0 + q;
        Acc<S>& acc = local[tid];
        for (int yy = s0; yy < e0; ++yy) {
            const int y = 1 + yy;
            for (int x = 1; x < W - 1; ++x) {
                const size_t idx = static_cast<size_t>(y) * W + x;
                const V3 lv = ld(live_v, idx);
                if (lv.z <= 0.001f || !finite3(lv)) continue;
                const V3 vr = R_rel * lv + t_rel;
                if (vr.z <= 0.001f) continue;
                acc.valid_live++;
                const float inv_z = 1.0f / vr.z;
                const float mxf = K.fx * vr.x * inv_z + K.cx;
                const float myf = K.fy * vr.y * inv_z + K.cy;
                int mx = 0, my = 0;
                if (!floorToInt(mxf + 0.5f, &mx) || !floorToInt(myf + 0.5f, &my)) continue;
                if (mx < 0 || mx >= MW || my < 0 || my >= MH) continue;
                acc.projected++;
                const size_t midx = static_cast<size_t>(my) * MW + mx;
                const V3 mv = ld(model_v, midx), mn = ld(model_n, midx);
                if (!modelVertexValid(mv) || !normalValid(mn)) continue;
                acc.valid_model++;
                const V3 vw = R_cw * lv + t_cw;
                const float d2 = sqnorm(vw - mv);
                if (d2 > dist2) { acc.dist_f++; continue; }
                const V3 ln = ld(live_n, idx);
                if (!normalValid(ln)) continue;
                const V3 nw = R_cw * ln;
                const float dot = std::fabs(dot3(nw, mn));
                if (dot < angle_cos) { acc.angle_f++; continue; }
                const float err = dot3(mn, vw - mv);
                if (!std::isfinite(err)) continue;
                const V3 nc = R_cwT * mn;
                const V3 cr = cross(lv, nc);
                const float J[6] = {nc.x, nc.y, nc.z, cr.x, cr.y, cr.z};
                bool ok = true;
                for (float j : J) ok = ok && std::isfinite(j);
                if (!ok) continue;
                const float ae = std::fabs(err);
                const float w = (ae <= kHuberK) ? 1.0f : kHuberK / ae;
                const float we = err * w;
                int k = 0;
                for (int i = 0; i < 6; ++i) {
                    for (int j = i; j < 6; ++j) acc.A[k++] += static_cast<S>(w * J[i] * J[j]);
                    acc.b[i] -= static_cast<S>(J[i] * we);
                }
                acc.residual += static_cast<S>(huberLoss(ae));
                acc.count++;
            }
        }
    }
    S As[36] = {0}, bs[6] = {0}, res = 0;
    for (const Acc<S>& a : local) {
        int k = 0;
        for (int i = 0; i < 6; ++i) {
            for (int j = i; j < 6; ++j) {
                const S v = a.A[k++];
                As[i * 6 + j] += v;
                if (i != j) As[j * 6 + i] += v;
            }
            bs[i] += a.b[i];
        }
        res += a.residual;
        counts[0] += a.count;
        counts[1] += a.valid_live;
        counts[2] += a.valid_model;
        counts[3] += a.projected;
        counts[4] += a.dist_f;
        counts[5] += a.angle_f;
    }
    for (int i = 0; i < 36; ++i) {
        Aout[i] = static_cast<float>(As[i]);
        if (A64) A64[i] = static_cast<double>(As[i]);
    }
    for (int i = 0; i < 6; ++i) {
        bout[i] = static_cast<float>(bs[i]);
        if (b64) b64[i] = static_cast<double>(bs[i]);
    }
    *residual = static_cast<float>(res);
    return counts[0] > 0;
}
}  // namespace

extern "C" void orc_icp_track(const orc_icp_params* prm, orc_intrinsics camK, const float* const live_v[3],
                              const float* const live_n[3], int W, int H, const float* model_v,
                              const float* model_n, int MW, int MH, const float estimate[16],
                              const float ref_pose[16], orc_icp_result* out) {
    orc_icp_result result;
    std::memset(&result, 0, sizeof(result));
    std::memcpy(result.pose, estimate, sizeof(result.pose));
    result.final_step = std::numeric_limits<float>::infinity();
    float last_final_step = std::numeric_limits<float>::infinity();
    int iters_done[3] = {0, 0, 0};

    for (int level = 2; level >= 0; --level) {
        const int max_iter = prm->max_iterations[level];
        if (max_iter <= 0) continue;
        const int LW = W >> level, LH = H >> level;
        // trackLevel (ICPTracker.cpp:68-134)
        orc_icp_result lr;
        std::memset(&lr, 0, sizeof(lr));
        std::memcpy(lr.pose, result.pose, sizeof(lr.pose));
        lr.final_step = std::numeric_limits<float>::infinity();
        for (int iter = 0; iter < max_iter; ++iter) {
            float A[36], b[6], residual;
            int counts[6];
            const int ok = orc_icp_build_system(prm, camK, live_v[level], live_n[level], LW, LH, model_v,
                                                model_n, MW, MH, lr.pose, ref_pose, A, b, &residual, counts);
            lr.valid_live_points = counts[1];
            lr.valid_model_points = counts[2];
            lr.projected_points = counts[3];
            lr.dist_filtered = counts[4];
            lr.angle_filtered = counts[5];
            if (!ok) break;
            const int inl = counts[0];
            if (inl < kMinInliersForIteration) break;
            std::memcpy(lr.information, A, sizeof(A));
            const float damp = dampingForHessian(A, level);
            for (int i = 0; i < 6; ++i) A[i * 6 + i] += damp;
            float x[6];
            ldltSolve(A, b, x);
            bool finite = true;
            for (float v : x) finite = finite && std::isfinite(v);
            const float tn = norm(V3(x[0], x[1], x[2]));
            const float rn = norm(V3(x[3], x[4], x[5]));
            if (!finite || tn > kTranslationCapStep || rn > kRotationCapStep) break;
            const float step_norm = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2] + x[3] * x[3] + x[4] * x[4] + x[5] * x[5]);
            const float rx = x[3], ry = x[4], rz = x[5];
            M3 R = M3::ident();
            const float angle = std::sqrt(rx * rx + ry * ry + rz * rz);
            if (angle > 1e-4f) {
                V3 axis(rx, ry, rz);
                axis = axis / norm(axis);
                R = angleAxis(angle, axis);
            } else {
                R.m[0][1] = -rz; R.m[0][2] = ry;
                R.m[1][0] = rz; R.m[1][2] = -rx;
                R.m[2][0] = -ry; R.m[2][1] = rx;
            }
            M4 delta = M4::ident();
            delta.setR(R);
            delta.m[0][3] = x[0]; delta.m[1][3] = x[1]; delta.m[2][3] = x[2];
            M4 P = M4::from(lr.pose) * delta;
            P.setR(projectToSO3(P.R()));
            P.to(lr.pose);
            lr.final_step = step_norm;
            lr.error = residual / static_cast<float>(std::max(inl, 1));
            lr.inliers = inl;
            iters_done[level]++;
            if (step_norm < kConvergenceStep) { lr.converged = 1; break; }
        }
        if (std::isfinite(lr.final_step)) last_final_step = lr.final_step;
        lr.final_step = last_final_step;
        result = lr;
    }
    result.tracking_ok = M4::from(result.pose).finite() && result.inliers > kMinInliersForOk &&
                         (result.converged || result.final_step <= kAcceptableFinalStep);
    for (int l = 0; l < 3; ++l) result.iterations[l] = iters_done[l];
    *out = result;
}

extern "C" int orc_classify_tracking(const orc_icp_result* r, const float prev_rm[16]) {
    // classifyFit (TrackingPolicy.h:70-80)
    const M4 pose = M4::from(r->pose);
    if (!pose.finite() || !std::isfinite(r->error) || r->inliers < kMinInliersForOk) return 2;
    const float fit = r->valid_model_points > 0 ? float(r->inliers) / float(r->valid_model_points) : 0.0f;
    const float rms = std::sqrt(std::max(0.0f, r->error));
    const int q = (r->inliers >= 2000 && fit >= 0.40f && rms <= 0.015f) ? 0 : 1;
    // withinFrameMotion (:82-89)
    const M4 d = inverse4(M4::from(prev_rm)) * pose;
    const float trans = norm(d.t());
    const float tr = (d.m[0][0] + d.m[1][1]) + d.m[2][2];
    const float c = std::max(-1.0f, std::min(1.0f, (tr - 1.0f) * 0.5f));
    const float ang = std::acos(c);
    if (!(trans <= 0.15f && ang <= 0.52f)) return 2;
    return q;
}

// Constant-velocity motion model (src/app/PipelineController.cpp:1175-1177):
// predicted = current * (last^-1 * current).
extern "C" void orc_predict(const float cur_rm[16], const float last_rm[16], float pred_rm[16]) {
    const M4 cur = M4::from(cur_rm);
    const M4 p = cur * (inverse4(M4::from(last_rm)) * cur);
    p.to(pred_rm);
}
