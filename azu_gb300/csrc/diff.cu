// Differentiable depth rendering of the TSDF volume (the differentiation form;
// no counterpart in the reference): the reference's front-face raycast march
// (src/tsdf/TSDFVolume.cpp:372-475) yields a depth image D = t_hit / |ray|; a
// Huber loss on D - D_obs is differentiated with respect to a right se(3)
// perturbation of the pose (pose * Exp(xi), xi = (rho, omega)) and to the tsdf
// values, by a hand-written adjoint.
//
// The march is piecewise smooth: t_{k+1} = t_k + s(f_k) with the far step for
// invalid samples or f >= 0.999, max(min_step, 0.8 f trunc) otherwise, from
// t_near (camera band or box entry), and the hit is the secant
// t_a + (t_b - t_a) f_a / (f_a - f_b). The adjoint holds the branch choices
// fixed and differentiates every dependence: the secant on both samples, each
// f-dependent step back to the sample that set it, and t_near through the box
// entry. Sample positions are recomputed, not stored: one pass marches and
// keeps only the parameters of the f-dependent steps (a short ring), then the
// reverse sweep re-samples those positions for the trilinear gradients; a
// chain longer than the ring is taken in windows by marching the ray again.
//
// One thread per pixel. Per-block sums of the loss, its pose gradient and the
// Gauss-Newton terms (J^T W J, J^T W r with IRLS Huber weights) are written as
// partials and summed in a fixed order by a second kernel; voxel gradients are
// accumulated with atomics.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "azu_internal.h"
#include "kf_math.cuh"
#include "reduce.cuh"
#include "tsdf_sample.cuh"

namespace azu {

constexpr int kDiffValues = 35;  // loss, dL/dxi[6], JtWJ[21], JtWr[6], count
constexpr int kMaxDep = 24;      // f-dependent steps kept for the reverse sweep

// Trilinear value gradient at p (world, per metre), the base voxel and the
// fractional offsets; false when the sample is invalid.
template <bool kHalf>
__device__ __forceinline__ bool sample_grad(const VolView& v, F3 p, float g[3], size_t& base, float& tx, float& ty,
                                            float& tz) {
    const F3 q = to_voxel(v, p);
    const float fx0 = floorf(q.x), fy0 = floorf(q.y), fz0 = floorf(q.z);
    const float lim = static_cast<float>(v.res - 1);
    if (!(fx0 >= 0.0f && fy0 >= 0.0f && fz0 >= 0.0f && fx0 < lim && fy0 < lim && fz0 < lim)) return false;
    const size_t r = static_cast<size_t>(v.res);
    base = (static_cast<size_t>(fz0) * r + static_cast<size_t>(fy0)) * r + static_cast<size_t>(fx0);
    tx = q.x - fx0;
    ty = q.y - fy0;
    tz = q.z - fz0;
    float V[8];
    const size_t off[8] = {0, 1, r, r + 1, r * r, r * r + 1, r * r + r, r * r + r + 1};
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const float2 c = Vox<kHalf>::load(v.vox, base + off[i]);
        if (!(c.y > 0.0f)) return false;
        V[i] = c.x;
    }
    const float ux = 1.0f - tx, uy = 1.0f - ty, uz = 1.0f - tz;
    const float inv = 1.0f / v.vs;
    g[0] = (uy * uz * (V[1] - V[0]) + ty * uz * (V[3] - V[2]) + uy * tz * (V[5] - V[4]) + ty * tz * (V[7] - V[6])) * inv;
    g[1] = (ux * uz * (V[2] - V[0]) + tx * uz * (V[3] - V[1]) + ux * tz * (V[6] - V[4]) + tx * tz * (V[7] - V[5])) * inv;
    g[2] = (ux * uy * (V[4] - V[0]) + tx * uy * (V[5] - V[1]) + ux * ty * (V[6] - V[2]) + tx * ty * (V[7] - V[3])) * inv;
    return true;
}

struct DiffArgs {
    VolView v;
    const float* pose;  // device, row-major world-from-camera
    float fx, fy, cx, cy;
    int W, H;
    float trunc, min_depth, max_depth;
    const float* obs;   // observed depth (metres) or null
    float delta;        // Huber threshold
    float* depth_out;   // rendered depth or null
    float* jac_out;     // dD/dxi per pixel (6) or null
    float* grad_tsdf;   // dL/dtsdf (res^3, accumulated) or null
    double* partials;   // [blocks][kDiffValues]
    unsigned* overflow; // pixels whose f-dependent chain outgrew the ring (taken by re-marching)
};

// Adjoint contribution of one sample: a_f * dF/d(everything) at t.
template <bool kHalf>
__device__ __forceinline__ void sample_adjoint(const DiffArgs& a, F3 co, F3 dir, F3 rn, const float* R0, float t,
                                               float af, float seed_v, float& at, float J[6]) {
    float g[3], tx, ty, tz;
    size_t base;
    const F3 p = add3(co, mul3(dir, t));
    if (!sample_grad<kHalf>(a.v, p, g, base, tx, ty, tz)) return;
    at += af * (g[0] * dir.x + g[1] * dir.y + g[2] * dir.z);
    // R0^T g
    const float h0 = R0[0] * g[0] + R0[3] * g[1] + R0[6] * g[2];
    const float h1 = R0[1] * g[0] + R0[4] * g[1] + R0[7] * g[2];
    const float h2 = R0[2] * g[0] + R0[5] * g[1] + R0[8] * g[2];
    J[0] += af * h0;
    J[1] += af * h1;
    J[2] += af * h2;
    J[3] += af * t * (rn.y * h2 - rn.z * h1);
    J[4] += af * t * (rn.z * h0 - rn.x * h2);
    J[5] += af * t * (rn.x * h1 - rn.y * h0);
    if (a.grad_tsdf && seed_v != 0.0f) {
        const size_t r = static_cast<size_t>(a.v.res);
        const float ux = 1.0f - tx, uy = 1.0f - ty, uz = 1.0f - tz;
        const float s = seed_v * af;
        atomicAdd(a.grad_tsdf + base, s * ux * uy * uz);
        atomicAdd(a.grad_tsdf + base + 1, s * tx * uy * uz);
        atomicAdd(a.grad_tsdf + base + r, s * ux * ty * uz);
        atomicAdd(a.grad_tsdf + base + r + 1, s * tx * ty * uz);
        atomicAdd(a.grad_tsdf + base + r * r, s * ux * uy * tz);
        atomicAdd(a.grad_tsdf + base + r * r + 1, s * tx * uy * tz);
        atomicAdd(a.grad_tsdf + base + r * r + r, s * ux * ty * tz);
        atomicAdd(a.grad_tsdf + base + r * r + r + 1, s * tx * ty * tz);
    }
}

// Outcome of the forward march of one ray: the bracketing samples of the hit
// (a before, b after the crossing) and the number of f-dependent steps (steps
// whose length 0.8 f trunc exceeded the minimum) taken before it.
struct MarchHit {
    bool hit = false, dep_a = false, clip_b = false;
    float t_a = 0.0f, f_a = 0.0f, t_b = 0.0f, f_b = 0.0f, t_hit = 0.0f;
    int ndep = 0;
};

// The forward march (TSDFVolume.cpp:372-475) from t_near. The start time of
// f-dependent step k is kept in dep_t: with lo < 0 in a ring (dep_t[k %
// kMaxDep], the newest kMaxDep survive), else dep_t[k - lo] for k in [lo, hi),
// hi - lo <= kMaxDep. The march is deterministic, so a second run with a
// window recovers steps the ring overwrote.
template <bool kHalf>
__device__ MarchHit march_ray(const VolView& v, F3 co, F3 dir, float t_near, float t_far, float min_step,
                              float far_step, float trunc, float* dep_t, int lo, int hi) {
    MarchHit m;
    if (!(t_near < t_far)) return m;
    float t_prev = t_near, f_prev = 1.0f;
    bool prev_valid = sample_tsdf<kHalf>(v, add3(co, mul3(dir, t_prev)), f_prev);
    if (prev_valid && !isfinite(f_prev)) return m;
    if (prev_valid && f_prev < 0.0f) return m;
    while (t_prev < t_far) {
        float step;
        bool dep = false;
        if (!prev_valid || f_prev >= 0.999f) {
            step = far_step;
        } else {
            const float s = fm(fm(0.8f, f_prev), trunc);
            dep = min_step < s;
            step = min_step < s ? s : min_step;
        }
        const float tn = fa(t_prev, step);
        const bool clip = !(tn < t_far) && tn != t_far;
        const float t = (t_far < tn) ? t_far : tn;
        if (!(t > t_prev)) break;
        const F3 p = add3(co, mul3(dir, t));
        float f = 1.0f;
        const bool valid = sample_tsdf<kHalf>(v, p, f);
        if (valid && !isfinite(f)) break;
        if (valid && prev_valid) {
            if (f_prev > 0.0f && f <= 0.0f) {
                m.t_hit = fa(t_prev, fm(fs(t, t_prev), fd(f_prev, fs(f_prev, f))));
                const F3 hp = add3(co, mul3(dir, m.t_hit));
                F3 nrm;
                if (compute_normal<kHalf>(v, hp, nrm) && finite3(hp)) {
                    m.hit = true;
                    m.t_a = t_prev; m.f_a = f_prev; m.t_b = t; m.f_b = f;
                    m.dep_a = dep;
                    m.clip_b = clip;
                }
                break;
            }
            if (f_prev < 0.0f && f >= 0.0f) break;
        } else if (valid && f < 0.0f) {
            break;
        }
        if (dep) {
            if (lo < 0) dep_t[m.ndep % kMaxDep] = t_prev;
            else if (m.ndep >= lo && m.ndep < hi) dep_t[m.ndep - lo] = t_prev;
            ++m.ndep;
        }
        t_prev = t;
        f_prev = f;
        prev_valid = valid;
        if (t >= t_far) break;
    }
    return m;
}

template <bool kHalf>
__global__ void __launch_bounds__(256) depth_adjoint_kernel(DiffArgs a) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const bool inside = x < a.W && y < a.H;
    float vals[kDiffValues];
#pragma unroll
    for (int k = 0; k < kDiffValues; ++k) vals[k] = 0.0f;

    if (inside) {
        const int o = y * a.W + x;
        float R0[9];
        R0[0] = __ldg(a.pose + 0); R0[1] = __ldg(a.pose + 1); R0[2] = __ldg(a.pose + 2);
        R0[3] = __ldg(a.pose + 4); R0[4] = __ldg(a.pose + 5); R0[5] = __ldg(a.pose + 6);
        R0[6] = __ldg(a.pose + 8); R0[7] = __ldg(a.pose + 9); R0[8] = __ldg(a.pose + 10);
        const F3 co = mk3(__ldg(a.pose + 3), __ldg(a.pose + 7), __ldg(a.pose + 11));
        const VolView& v = a.v;
        const float vs = v.vs;
        const F3 box_lo = v.origin;
        const float span = fm(static_cast<float>(v.res - 1), vs);
        const F3 box_hi = add3(box_lo, mk3(span, span, span));
        const float min_step = fm(0.5f, vs);
        const float far_c = fm(0.8f, a.trunc);
        const float far_step = min_step < far_c ? far_c : min_step;

        const F3 ray = mk3(fd(fs(static_cast<float>(x), a.cx), a.fx), fd(fs(static_cast<float>(y), a.cy), a.fy), 1.0f);
        const float ray_norm = norm3(ray);
        const F3 dir = div3(mv3(R0, ray), ray_norm);
        float t_near = fm(a.min_depth, ray_norm);
        float t_far = fm(a.max_depth, ray_norm);
        int near_axis = -1;
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const float da = comp(dir, ax), oa = comp(co, ax), la = comp(box_lo, ax), ha = comp(box_hi, ax);
            const float inv = fd(1.0f, da);
            float t0 = fm(fs(la, oa), inv);
            float t1 = fm(fs(ha, oa), inv);
            if (t0 > t1) { const float tmp = t0; t0 = t1; t1 = tmp; }
            if (isnan(t0) || isnan(t1)) {
                if (oa < la || oa > ha) t_far = -1.0f;
                continue;
            }
            if (t_near < t0) near_axis = ax;
            t_near = (t_near < t0) ? t0 : t_near;
            t_far = (t1 < t_far) ? t1 : t_far;
        }

        // forward march, keeping the newest f-dependent steps in a ring
        float dep_t[kMaxDep];
        const MarchHit mh = march_ray<kHalf>(v, co, dir, t_near, t_far, min_step, far_step, a.trunc, dep_t, -1, 0);
        const bool hit = mh.hit;
        const int ndep = mh.ndep;
        const float t_a = mh.t_a, f_a = mh.f_a, t_b = mh.t_b, f_b = mh.f_b, t_hit = mh.t_hit;
        const bool dep_a = mh.dep_a, clip_b = mh.clip_b;

        const float D = hit ? t_hit / ray_norm : 0.0f;
        if (a.depth_out) a.depth_out[o] = D;
        float J[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        const float ob = a.obs ? __ldg(a.obs + o) : 0.0f;
        const bool use = hit && a.obs && ob >= a.min_depth && ob <= a.max_depth;
        float r = 0.0f, dr = 0.0f, wr = 0.0f, loss = 0.0f;
        if (use) {
            r = D - ob;
            const float ar = fabsf(r);
            if (ar <= a.delta) { loss = 0.5f * r * r; dr = r; wr = 1.0f; }
            else { loss = a.delta * (ar - 0.5f * a.delta); dr = r > 0.0f ? a.delta : -a.delta; wr = a.delta / ar; }
        }
        if (hit && (use || a.jac_out)) {
            // reverse sweep: seeds d t_hit / d(t_a, t_b, f_a, f_b), scaled by 1/|ray|
            const F3 rn = mul3(ray, 1.0f / ray_norm);
            const float inv_rn = 1.0f / ray_norm;
            const float den = f_a - f_b;
            float at = (f_a / den) * inv_rn;
            const float af_b = (t_b - t_a) * f_a / (den * den) * inv_rn;
            sample_adjoint<kHalf>(a, co, dir, rn, R0, t_b, af_b, dr, at, J);
            if (clip_b) at = 0.0f;
            float af = (t_b - t_a) * (-f_b) / (den * den) * inv_rn + (dep_a ? at * 0.8f * a.trunc : 0.0f);
            at += (1.0f - f_a / den) * inv_rn;
            sample_adjoint<kHalf>(a, co, dir, rn, R0, t_a, af, dr, at, J);
            const int kept = ndep < kMaxDep ? ndep : kMaxDep;
            for (int i = 0; i < kept; ++i) {
                const float tk = dep_t[(ndep - 1 - i) % kMaxDep];
                sample_adjoint<kHalf>(a, co, dir, rn, R0, tk, at * 0.8f * a.trunc, dr, at, J);
            }
            // older steps the ring overwrote: march again and take them
            // kMaxDep at a time, newest window first
            if (ndep > kMaxDep) atomicAdd(a.overflow, 1u);
            for (int hi = ndep - kMaxDep; hi > 0; hi -= kMaxDep) {
                const int lo = hi > kMaxDep ? hi - kMaxDep : 0;
                march_ray<kHalf>(v, co, dir, t_near, t_far, min_step, far_step, a.trunc, dep_t, lo, hi);
                for (int k = hi - 1; k >= lo; --k)
                    sample_adjoint<kHalf>(a, co, dir, rn, R0, dep_t[k - lo], at * 0.8f * a.trunc, dr, at, J);
            }
            if (near_axis >= 0) {
                const float da = comp(dir, near_axis);
                const float Ra0 = R0[3 * near_axis], Ra1 = R0[3 * near_axis + 1], Ra2 = R0[3 * near_axis + 2];
                J[0] += at * (-Ra0 / da);
                J[1] += at * (-Ra1 / da);
                J[2] += at * (-Ra2 / da);
                const float c = -t_near / da;
                J[3] += at * c * (rn.y * Ra2 - rn.z * Ra1);
                J[4] += at * c * (rn.z * Ra0 - rn.x * Ra2);
                J[5] += at * c * (rn.x * Ra1 - rn.y * Ra0);
            }
        }
        if (a.jac_out)
            for (int j = 0; j < 6; ++j) a.jac_out[6 * o + j] = J[j];
        if (use) {
            vals[0] = loss;
#pragma unroll
            for (int j = 0; j < 6; ++j) vals[1 + j] = dr * J[j];
            int k = 7;
#pragma unroll
            for (int i = 0; i < 6; ++i)
#pragma unroll
                for (int j = i; j < 6; ++j) vals[k++] = wr * J[i] * J[j];
#pragma unroll
            for (int j = 0; j < 6; ++j) vals[28 + j] = wr * J[j] * r;
            vals[34] = 1.0f;
        }
    }
    // block partials: recursive halving for the first 32 values, shuffles for the rest
    __shared__ float s_red[8][kDiffValues];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    float v32[32];
#pragma unroll
    for (int k = 0; k < 32; ++k) v32[k] = vals[k];
    const float e32 = warp_sum(vals[32]), e33 = warp_sum(vals[33]), e34 = warp_sum(vals[34]);
    const float mine = warp_sum_transpose32(v32, lane);
    s_red[warp][lane] = mine;
    if (lane == 0) {
        s_red[warp][32] = e32;
        s_red[warp][33] = e33;
        s_red[warp][34] = e34;
    }
    __syncthreads();
    if (tid < kDiffValues) {
        double sum = 0.0;
        const int nw = (blockDim.x * blockDim.y) >> 5;
        for (int w = 0; w < nw; ++w) sum += static_cast<double>(s_red[w][tid]);
        a.partials[static_cast<size_t>(blockIdx.y * gridDim.x + blockIdx.x) * kDiffValues + tid] = sum;
    }
}

// Sum of the block partials in block order (deterministic).
__global__ void diff_sum_kernel(const double* __restrict__ partials, int nblocks, double* __restrict__ out) {
    const int k = threadIdx.x;
    if (k >= kDiffValues) return;
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) s += partials[static_cast<size_t>(b) * kDiffValues + k];
    out[k] = s;
}

static int ensure_diff_scratch(azu_volume* v, size_t nblocks) {
    if (nblocks <= v->diff_cap) return AZU_OK;
    AZU_TRY_CUDA(cudaStreamSynchronize(v->stream.s));
    if (v->d_diff) cudaFree(v->d_diff);
    v->d_diff = nullptr;
    v->diff_cap = 0;
    // partials, the summed values and the overflow counter
    AZU_TRY_CUDA(cudaMalloc(&v->d_diff, (nblocks + 1) * kDiffValues * sizeof(double) + 16));
    v->diff_cap = nblocks;
    return AZU_OK;
}

static int run_adjoint(azu_volume* v, const float pose[16], float fx, float fy, float cx, float cy, int W, int H,
                       const float* d_obs, float delta, float* d_depth, float* d_jac, float* d_grad, double sums[35],
                       unsigned* overflow) {
    AZU_CHECK_ARG(W > 0 && H > 0 && W <= 16384 && H <= 16384, "image size");
    AZU_TRY_CUDA(cudaSetDevice(v->device));
    cudaStream_t s = v->stream.s;
    const dim3 blk(32, 8), grd((W + 31) / 32, (H + 7) / 8);
    const size_t nblocks = static_cast<size_t>(grd.x) * grd.y;
    if (int rc = ensure_diff_scratch(v, nblocks)) return rc;
    if (int rc = set_pose_async(v->d_pose, pose, s)) return rc;
    double* d_part = v->d_diff;
    double* d_sum = v->d_diff + nblocks * kDiffValues;
    unsigned* d_over = reinterpret_cast<unsigned*>(d_sum + kDiffValues);
    AZU_TRY_CUDA(cudaMemsetAsync(d_over, 0, sizeof(unsigned), s));
    const azu_volume_params& p = v->p;
    DiffArgs a{make_view(v), v->d_pose, fx, fy, cx, cy, W, H, p.truncation, p.min_depth, p.max_depth, d_obs, delta,
               d_depth, d_jac, d_grad, d_part, d_over};
    if (p.format == AZU_TSDF_FP32) depth_adjoint_kernel<false><<<grd, blk, 0, s>>>(a);
    else depth_adjoint_kernel<true><<<grd, blk, 0, s>>>(a);
    AZU_LAUNCH_CHECK();
    diff_sum_kernel<<<1, 64, 0, s>>>(d_part, static_cast<int>(nblocks), d_sum);
    AZU_LAUNCH_CHECK();
    double host[kDiffValues];
    unsigned over = 0;
    AZU_TRY_CUDA(cudaMemcpyAsync(host, d_sum, sizeof(host), cudaMemcpyDeviceToHost, s));
    AZU_TRY_CUDA(cudaMemcpyAsync(&over, d_over, sizeof(over), cudaMemcpyDeviceToHost, s));
    AZU_TRY_CUDA(cudaStreamSynchronize(s));
    if (sums) std::memcpy(sums, host, sizeof(host));
    if (overflow) *overflow = over;
    return AZU_OK;
}

// pose * Exp(xi) in double (xi = rho, omega), re-orthonormalised through the
// exact exponential.
static void compose_exp(const float P[16], const double xi[6], float out[16]) {
    const double wx = xi[3], wy = xi[4], wz = xi[5];
    const double th2 = wx * wx + wy * wy + wz * wz, th = std::sqrt(th2);
    double A, B, Cc;
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
    double W2[9], R[9], V[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0;
            for (int k = 0; k < 3; ++k) s += W[3 * i + k] * W[3 * k + j];
            W2[3 * i + j] = s;
        }
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
            for (int k = 0; k < 3; ++k) s += double(P[4 * i + k]) * R[3 * k + j];
            out[4 * i + j] = static_cast<float>(s);
        }
        double s = P[4 * i + 3];
        for (int k = 0; k < 3; ++k) s += double(P[4 * i + k]) * t[k];
        out[4 * i + 3] = static_cast<float>(s);
    }
    out[12] = out[13] = out[14] = 0.0f;
    out[15] = 1.0f;
}

// Solves (A + lambda diag(A)) x = b for the 6x6 symmetric A (upper, 21 values).
static bool solve6(const double* up, const double* b, double lambda, double* x) {
    double A[36];
    int k = 0;
    for (int i = 0; i < 6; ++i)
        for (int j = i; j < 6; ++j) A[6 * i + j] = A[6 * j + i] = up[k++];
    for (int i = 0; i < 6; ++i) A[7 * i] *= (1.0 + lambda);
    double L[36] = {0};
    for (int j = 0; j < 6; ++j) {
        double s = A[7 * j];
        for (int q = 0; q < j; ++q) s -= L[6 * j + q] * L[6 * j + q];
        if (!(s > 0.0)) return false;
        L[7 * j] = std::sqrt(s);
        for (int i = j + 1; i < 6; ++i) {
            double t = A[6 * i + j];
            for (int q = 0; q < j; ++q) t -= L[6 * i + q] * L[6 * j + q];
            L[6 * i + j] = t / L[7 * j];
        }
    }
    double yv[6];
    for (int i = 0; i < 6; ++i) {
        double s = b[i];
        for (int q = 0; q < i; ++q) s -= L[6 * i + q] * yv[q];
        yv[i] = s / L[7 * i];
    }
    for (int i = 5; i >= 0; --i) {
        double s = yv[i];
        for (int q = i + 1; q < 6; ++q) s -= L[6 * q + i] * x[q];
        x[i] = s / L[7 * i];
    }
    return true;
}

}  // namespace azu

using namespace azu;

extern "C" int azu_volume_render_depth(azu_volume* v, const float pose[16], float fx, float fy, float cx, float cy,
                                       int width, int height, float* d_depth) {
    AZU_CHECK_ARG(v != nullptr && pose != nullptr && d_depth != nullptr, "null argument");
    return run_adjoint(v, pose, fx, fy, cx, cy, width, height, nullptr, 0.01f, d_depth, nullptr, nullptr, nullptr,
                       nullptr);
}

extern "C" int azu_volume_depth_backward(azu_volume* v, const float pose[16], float fx, float fy, float cx, float cy,
                                         int width, int height, const float* d_depth_obs, float huber_delta,
                                         float* d_depth, float* d_jacobian, float* d_grad_tsdf, double sums[35],
                                         unsigned* chain_overflow) {
    AZU_CHECK_ARG(v != nullptr && pose != nullptr && d_depth_obs != nullptr, "null argument");
    AZU_CHECK_ARG(huber_delta > 0.0f && std::isfinite(huber_delta), "huber_delta must be > 0");
    return run_adjoint(v, pose, fx, fy, cx, cy, width, height, d_depth_obs, huber_delta, d_depth, d_jacobian,
                       d_grad_tsdf, sums, chain_overflow);
}

extern "C" int azu_volume_refine_pose(azu_volume* v, const float pose_in[16], float fx, float fy, float cx, float cy,
                                      int width, int height, const float* d_depth_obs, float huber_delta,
                                      int max_iterations, float pose_out[16], double* loss_trace, int* iterations) {
    AZU_CHECK_ARG(v != nullptr && pose_in != nullptr && pose_out != nullptr && d_depth_obs != nullptr,
                  "null argument");
    AZU_CHECK_ARG(max_iterations >= 0 && max_iterations <= 1000, "max_iterations must be in [0, 1000]");
    float pose[16];
    std::memcpy(pose, pose_in, sizeof(pose));
    double sums[kDiffValues];
    if (int rc = run_adjoint(v, pose, fx, fy, cx, cy, width, height, d_depth_obs, huber_delta, nullptr, nullptr,
                             nullptr, sums, nullptr))
        return rc;
    double loss = sums[0];
    if (loss_trace) loss_trace[0] = loss;
    double lambda = 1e-4;
    int it = 0;
    for (; it < max_iterations; ++it) {
        // Levenberg-Marquardt step on the IRLS Gauss-Newton system
        double b[6], x[6];
        for (int j = 0; j < 6; ++j) b[j] = -sums[28 + j];
        bool accepted = false;
        for (int tries = 0; tries < 8 && !accepted; ++tries) {
            if (!solve6(sums + 7, b, lambda, x)) { lambda *= 10.0; continue; }
            float cand[16];
            compose_exp(pose, x, cand);
            double cs[kDiffValues];
            if (int rc = run_adjoint(v, cand, fx, fy, cx, cy, width, height, d_depth_obs, huber_delta, nullptr,
                                     nullptr, nullptr, cs, nullptr))
                return rc;
            // the same pixels must still count: compare mean losses
            const double mean_new = cs[34] > 0 ? cs[0] / cs[34] : INFINITY;
            const double mean_old = sums[34] > 0 ? sums[0] / sums[34] : INFINITY;
            if (mean_new <= mean_old) {
                std::memcpy(pose, cand, sizeof(pose));
                std::memcpy(sums, cs, sizeof(cs));
                lambda = std::max(lambda * 0.3, 1e-7);
                accepted = true;
            } else {
                lambda *= 10.0;
            }
        }
        if (loss_trace) loss_trace[it + 1] = sums[0];
        if (!accepted) break;
        double n2 = 0;
        for (int j = 0; j < 6; ++j) n2 += x[j] * x[j];
        if (std::sqrt(n2) < 1e-7) { ++it; break; }
    }
    std::memcpy(pose_out, pose, sizeof(pose));
    if (iterations) *iterations = it;
    return AZU_OK;
}
