// Live frame geometry on the GPU: vertex and normal maps at 640x480 and the
// 3-level jump-guarded pyramid (src/sensor/FrameData.cpp:113-345 semantics).
//
// Two launches per frame:
//   vn_kernel      — one thread per level-0 pixel: vertex from depth, normal
//                    from the 4 neighbours' vertices (recomputed from depth,
//                    bit-identical to the stored ones).
//   pyramid_kernel — one thread per level-1 pixel (the 2x2 reduction of
//                    level 0), then a quarter of them each level-2 pixel
//                    from four level-1 pixels in shared memory.
// Maps are packed float3 (12 B per pixel), depth float.
#include "azu_internal.h"
#include "kf_math.cuh"

namespace azu {

// depthJumpThreshold (include/tracking/ICPShared.h:53-55).
__device__ __forceinline__ float jump_threshold(float d) {
    const float r = fm(d, 0.05f);
    return 0.03f < r ? r : 0.03f;  // std::max(0.03f, d * 0.05f)
}

__device__ __forceinline__ F3 vertex_at(const float* __restrict__ depth, int x, int y, int W, float fx_inv,
                                        float fy_inv, float cx, float cy) {
    const float d = __ldg(depth + y * W + x);
    if (d > 0.0f)
        return mk3(fm(fm(fs(static_cast<float>(x), cx), fx_inv), d), fm(fm(fs(static_cast<float>(y), cy), fy_inv), d), d);
    return mk3(0.0f, 0.0f, 0.0f);
}
__device__ __forceinline__ void st3(float* a, int i, F3 v) {
    a[3 * i] = v.x;
    a[3 * i + 1] = v.y;
    a[3 * i + 2] = v.z;
}
__device__ __forceinline__ F3 ld3(const float* a, int i) { return mk3(a[3 * i], a[3 * i + 1], a[3 * i + 2]); }

// updateVerticesFromDepth (:113-133) + computeNormals (:196-251).
__global__ void __launch_bounds__(256) vn_kernel(const float* __restrict__ depth, int W, int H, float fx, float fy,
                                                 float cx, float cy, float* __restrict__ V, float* __restrict__ N) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const float fx_inv = fd(1.0f, fx), fy_inv = fd(1.0f, fy);
    const int c = y * W + x;
    const F3 vc = vertex_at(depth, x, y, W, fx_inv, fy_inv, cx, cy);
    st3(V, c, vc);
    F3 n = mk3(0.0f, 0.0f, 0.0f);
    if (x >= 1 && x < W - 1 && y >= 1 && y < H - 1) {
        const float dc = __ldg(depth + c), dr = __ldg(depth + c + 1), dl = __ldg(depth + c - 1),
                    du = __ldg(depth + c - W), dd = __ldg(depth + c + W);
        if (!(dc <= 0.0f || dr <= 0.0f || dl <= 0.0f || du <= 0.0f || dd <= 0.0f)) {
            const float j = jump_threshold(dc);
            if (!(fabsf(fs(dc, dr)) > j || fabsf(fs(dc, dl)) > j || fabsf(fs(dc, du)) > j || fabsf(fs(dc, dd)) > j)) {
                const F3 vr = vertex_at(depth, x + 1, y, W, fx_inv, fy_inv, cx, cy);
                const F3 vl = vertex_at(depth, x - 1, y, W, fx_inv, fy_inv, cx, cy);
                const F3 vu = vertex_at(depth, x, y - 1, W, fx_inv, fy_inv, cx, cy);
                const F3 vd = vertex_at(depth, x, y + 1, W, fx_inv, fy_inv, cx, cy);
                const F3 cr = cross3(sub3(vr, vl), sub3(vd, vu));
                const float len = norm3(cr);
                if (len > 1e-6f) n = div3(cr, len);
            }
        }
    }
    st3(N, c, n);
}

// downsample (:262-334) for one destination pixel (x, y) of a W x H source.
__device__ __forceinline__ void down_px(const float* __restrict__ sd, const float* __restrict__ sv,
                                        const float* __restrict__ sn, int W, int x, int y, float& od, F3& ov, F3& on) {
    const int sx = 2 * x, sy = 2 * y;
    F3 sumv = mk3(0.0f, 0.0f, 0.0f), sumn = mk3(0.0f, 0.0f, 0.0f);
    float sumd = 0.0f, dmin = 0.0f, dmax = 0.0f;
    int count = 0, mdx = 0, mdy = 0;
#pragma unroll
    for (int dy = 0; dy < 2; ++dy)
#pragma unroll
        for (int dx = 0; dx < 2; ++dx) {
            const int s = (sy + dy) * W + sx + dx;
            const float d = sd[s];
            if (d > 0.0f) {
                sumv = add3(sumv, ld3(sv, s));
                sumn = add3(sumn, ld3(sn, s));
                sumd = fa(sumd, d);
                if (count == 0 || d < dmin) { dmin = d; mdx = dx; mdy = dy; }
                if (count == 0 || d > dmax) dmax = d;
                ++count;
            }
        }
    od = 0.0f;
    ov = mk3(0.0f, 0.0f, 0.0f);
    on = mk3(0.0f, 0.0f, 0.0f);
    if (count > 0) {
        if (fs(dmax, dmin) > jump_threshold(dmin)) {
            const int m = (sy + mdy) * W + sx + mdx;
            ov = ld3(sv, m);
            od = sd[m];
            const F3 nm = ld3(sn, m);
            const float nl = norm3(nm);
            if (nl > 1e-6f) on = div3(nm, nl);
        } else {
            const float inv = fd(1.0f, static_cast<float>(count));
            ov = mul3(sumv, inv);
            od = fm(sumd, inv);
            const float nl = norm3(sumn);
            if (nl > 1e-6f) on = div3(sumn, nl);
        }
    }
}

// 16 x 16 level-1 pixels per block (the 2x2 reductions of level 0), staged in
// shared memory, then the block's 8 x 8 level-2 pixels from them.
constexpr int kPyrSide = 16;
__global__ void __launch_bounds__(kPyrSide * kPyrSide) pyramid_kernel(
    const float* __restrict__ d0, const float* __restrict__ v0, const float* __restrict__ n0, int W0, int W1, int H1,
    float* __restrict__ d1, float* __restrict__ v1, float* __restrict__ n1, float* __restrict__ d2,
    float* __restrict__ v2, float* __restrict__ n2, int W2, int H2) {
    __shared__ float s_d[kPyrSide][kPyrSide];
    __shared__ float s_v[kPyrSide][kPyrSide][3];
    __shared__ float s_n[kPyrSide][kPyrSide][3];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x1 = blockIdx.x * kPyrSide + tx, y1 = blockIdx.y * kPyrSide + ty;
    if (x1 < W1 && y1 < H1) {
        float d;
        F3 v, n;
        down_px(d0, v0, n0, W0, x1, y1, d, v, n);
        const int i1 = y1 * W1 + x1;
        d1[i1] = d;
        st3(v1, i1, v);
        st3(n1, i1, n);
        s_d[ty][tx] = d;
        s_v[ty][tx][0] = v.x; s_v[ty][tx][1] = v.y; s_v[ty][tx][2] = v.z;
        s_n[ty][tx][0] = n.x; s_n[ty][tx][1] = n.y; s_n[ty][tx][2] = n.z;
    }
    __syncthreads();
    if (tx >= kPyrSide / 2 || ty >= kPyrSide / 2) return;
    const int x = blockIdx.x * (kPyrSide / 2) + tx, y = blockIdx.y * (kPyrSide / 2) + ty;
    if (x >= W2 || y >= H2) return;
    // Level 2 from the four level-1 pixels, in the order a read-back takes them:
    // (0,0), (1,0), (0,1), (1,1).
    float ld1[4];
    F3 lv1[4], ln1[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int sx = 2 * tx + (k & 1), sy = 2 * ty + (k >> 1);
        ld1[k] = s_d[sy][sx];
        lv1[k] = mk3(s_v[sy][sx][0], s_v[sy][sx][1], s_v[sy][sx][2]);
        ln1[k] = mk3(s_n[sy][sx][0], s_n[sy][sx][1], s_n[sy][sx][2]);
    }
    F3 sumv = mk3(0.0f, 0.0f, 0.0f), sumn = mk3(0.0f, 0.0f, 0.0f);
    float sumd = 0.0f, dmin = 0.0f, dmax = 0.0f;
    int count = 0, mk = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float d = ld1[k];
        if (d > 0.0f) {
            sumv = add3(sumv, lv1[k]);
            sumn = add3(sumn, ln1[k]);
            sumd = fa(sumd, d);
            if (count == 0 || d < dmin) { dmin = d; mk = k; }
            if (count == 0 || d > dmax) dmax = d;
            ++count;
        }
    }
    float od = 0.0f;
    F3 ov = mk3(0.0f, 0.0f, 0.0f), on = mk3(0.0f, 0.0f, 0.0f);
    if (count > 0) {
        if (fs(dmax, dmin) > jump_threshold(dmin)) {
            ov = lv1[mk];
            od = ld1[mk];
            const float nl = norm3(ln1[mk]);
            if (nl > 1e-6f) on = div3(ln1[mk], nl);
        } else {
            const float inv = fd(1.0f, static_cast<float>(count));
            ov = mul3(sumv, inv);
            od = fm(sumd, inv);
            const float nl = norm3(sumn);
            if (nl > 1e-6f) on = div3(sumn, nl);
        }
    }
    const int i2 = y * W2 + x;
    d2[i2] = od;
    st3(v2, i2, ov);
    st3(n2, i2, on);
}

int launch_prepare_live(const float* d_depth, int W, int H, float fx, float fy, float cx, float cy, float* const V[3],
                        float* const N[3], float* const D[3], cudaStream_t s) {
    {
        const dim3 b(32, 8), g((W + 31) / 32, (H + 7) / 8);
        vn_kernel<<<g, b, 0, s>>>(d_depth, W, H, fx, fy, cx, cy, V[0], N[0]);
        AZU_LAUNCH_CHECK();
    }
    if (D[0] != d_depth) AZU_TRY_CUDA(cudaMemcpyAsync(D[0], d_depth, sizeof(float) * W * H, cudaMemcpyDeviceToDevice, s));
    {
        const int W1 = W / 2, H1 = H / 2, W2 = W / 4, H2 = H / 4;
        const dim3 b(kPyrSide, kPyrSide), g((W1 + kPyrSide - 1) / kPyrSide, (H1 + kPyrSide - 1) / kPyrSide);
        pyramid_kernel<<<g, b, 0, s>>>(d_depth, V[0], N[0], W, W1, H1, D[1], V[1], N[1], D[2], V[2], N[2], W2, H2);
        AZU_LAUNCH_CHECK();
    }
    return AZU_OK;
}

}  // namespace azu
