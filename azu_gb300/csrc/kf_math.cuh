// Device-side float math for the KinectFusion kernels.
//
// Every product below is written with explicit round-to-nearest intrinsics
// (__fmul_rn, __fadd_rn, __fsub_rn, __fdiv_rn, __fsqrt_rn), which the compiler
// never contracts into fused multiply-adds. The evaluation order of each
// expression is the one the reference's CPU path yields (Eigen's fixed-size
// products, left-to-right scalar C++), so integer decisions downstream — voxel
// projections, trilinear validity, ICP association — come out bit-identical:
//
//   dot3(a, b) = a0*b0 + (a1*b1 + a2*b2)
//   M3 * v     = dot3(row_i, v);   M3 * M3 = dot3(row_i, col_j)
//   M4 * M4    = ((a0*b0 + a1*b1) + a2*b2) + a3*b3
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace azu {

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fd(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsq(float a) { return __fsqrt_rn(a); }

struct F3 {
    float x, y, z;
};
__host__ __device__ __forceinline__ F3 mk3(float x, float y, float z) { return F3{x, y, z}; }
__device__ __forceinline__ F3 add3(F3 a, F3 b) { return F3{fa(a.x, b.x), fa(a.y, b.y), fa(a.z, b.z)}; }
__device__ __forceinline__ F3 sub3(F3 a, F3 b) { return F3{fs(a.x, b.x), fs(a.y, b.y), fs(a.z, b.z)}; }
__device__ __forceinline__ F3 mul3(F3 a, float s) { return F3{fm(a.x, s), fm(a.y, s), fm(a.z, s)}; }
__device__ __forceinline__ F3 smul3(float s, F3 a) { return F3{fm(s, a.x), fm(s, a.y), fm(s, a.z)}; }
__device__ __forceinline__ F3 div3(F3 a, float s) { return F3{fd(a.x, s), fd(a.y, s), fd(a.z, s)}; }
__device__ __forceinline__ float dot3(F3 a, F3 b) { return fa(fm(a.x, b.x), fa(fm(a.y, b.y), fm(a.z, b.z))); }
__device__ __forceinline__ float sqnorm3(F3 a) { return dot3(a, a); }
__device__ __forceinline__ float norm3(F3 a) { return fsq(sqnorm3(a)); }
__device__ __forceinline__ F3 cross3(F3 a, F3 b) {
    return F3{fs(fm(a.y, b.z), fm(a.z, b.y)), fs(fm(a.z, b.x), fm(a.x, b.z)), fs(fm(a.x, b.y), fm(a.y, b.x))};
}
__device__ __forceinline__ bool finite3(F3 a) { return isfinite(a.x) && isfinite(a.y) && isfinite(a.z); }
__device__ __forceinline__ float comp(F3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

// Row-major 3x3 / 4x4 helpers over plain float arrays.
__device__ __forceinline__ F3 row3(const float* m, int i) { return F3{m[3 * i], m[3 * i + 1], m[3 * i + 2]}; }
__device__ __forceinline__ F3 mv3(const float* m, F3 v) { return F3{dot3(row3(m, 0), v), dot3(row3(m, 1), v), dot3(row3(m, 2), v)}; }
// m^T v (rows of the transpose are the columns of m).
__device__ __forceinline__ F3 mtv3(const float* m, F3 v) {
    return F3{dot3(F3{m[0], m[3], m[6]}, v), dot3(F3{m[1], m[4], m[7]}, v), dot3(F3{m[2], m[5], m[8]}, v)};
}
__device__ __forceinline__ void mm3(const float* a, const float* b, float* r) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r[3 * i + j] = dot3(row3(a, i), F3{b[j], b[3 + j], b[6 + j]});
}
__device__ __forceinline__ void mm4(const float* a, const float* b, float* r) {
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            r[4 * i + j] = fa(fa(fa(fm(a[4 * i], b[j]), fm(a[4 * i + 1], b[4 + j])), fm(a[4 * i + 2], b[8 + j])),
                              fm(a[4 * i + 3], b[12 + j]));
}
// Rotation block and translation of a row-major 4x4.
__device__ __forceinline__ void rot_of(const float* p, float* r) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r[3 * i + j] = p[4 * i + j];
}
__device__ __forceinline__ F3 trans_of(const float* p) { return F3{p[3], p[7], p[11]}; }

// General 4x4 inverse: adjugate from the 2x2 minors of the top and bottom row
// pairs, divided by the determinant (same expression trees as the host side).
__device__ inline void inverse4(const float* A, float* R) {
#define a(i, j) A[4 * (i) + (j)]
    const float s0 = fs(fm(a(0, 0), a(1, 1)), fm(a(1, 0), a(0, 1)));
    const float s1 = fs(fm(a(0, 0), a(1, 2)), fm(a(1, 0), a(0, 2)));
    const float s2 = fs(fm(a(0, 0), a(1, 3)), fm(a(1, 0), a(0, 3)));
    const float s3 = fs(fm(a(0, 1), a(1, 2)), fm(a(1, 1), a(0, 2)));
    const float s4 = fs(fm(a(0, 1), a(1, 3)), fm(a(1, 1), a(0, 3)));
    const float s5 = fs(fm(a(0, 2), a(1, 3)), fm(a(1, 2), a(0, 3)));
    const float c5 = fs(fm(a(2, 2), a(3, 3)), fm(a(3, 2), a(2, 3)));
    const float c4 = fs(fm(a(2, 1), a(3, 3)), fm(a(3, 1), a(2, 3)));
    const float c3 = fs(fm(a(2, 1), a(3, 2)), fm(a(3, 1), a(2, 2)));
    const float c2 = fs(fm(a(2, 0), a(3, 3)), fm(a(3, 0), a(2, 3)));
    const float c1 = fs(fm(a(2, 0), a(3, 2)), fm(a(3, 0), a(2, 2)));
    const float c0 = fs(fm(a(2, 0), a(3, 1)), fm(a(3, 0), a(2, 1)));
    const float det = fa(fs(fa(fa(fs(fm(s0, c5), fm(s1, c4)), fm(s2, c3)), fm(s3, c2)), fm(s4, c1)), fm(s5, c0));
    const float id = fd(1.0f, det);
    R[0] = fm(fa(fs(fm(a(1, 1), c5), fm(a(1, 2), c4)), fm(a(1, 3), c3)), id);
    R[1] = fm(fs(fa(fm(-a(0, 1), c5), fm(a(0, 2), c4)), fm(a(0, 3), c3)), id);
    R[2] = fm(fa(fs(fm(a(3, 1), s5), fm(a(3, 2), s4)), fm(a(3, 3), s3)), id);
    R[3] = fm(fs(fa(fm(-a(2, 1), s5), fm(a(2, 2), s4)), fm(a(2, 3), s3)), id);
    R[4] = fm(fs(fa(fm(-a(1, 0), c5), fm(a(1, 2), c2)), fm(a(1, 3), c1)), id);
    R[5] = fm(fa(fs(fm(a(0, 0), c5), fm(a(0, 2), c2)), fm(a(0, 3), c1)), id);
    R[6] = fm(fs(fa(fm(-a(3, 0), s5), fm(a(3, 2), s2)), fm(a(3, 3), s1)), id);
    R[7] = fm(fa(fs(fm(a(2, 0), s5), fm(a(2, 2), s2)), fm(a(2, 3), s1)), id);
    R[8] = fm(fa(fs(fm(a(1, 0), c4), fm(a(1, 1), c2)), fm(a(1, 3), c0)), id);
    R[9] = fm(fs(fa(fm(-a(0, 0), c4), fm(a(0, 1), c2)), fm(a(0, 3), c0)), id);
    R[10] = fm(fa(fs(fm(a(3, 0), s4), fm(a(3, 1), s2)), fm(a(3, 3), s0)), id);
    R[11] = fm(fs(fa(fm(-a(2, 0), s4), fm(a(2, 1), s2)), fm(a(2, 3), s0)), id);
    R[12] = fm(fs(fa(fm(-a(1, 0), c3), fm(a(1, 1), c1)), fm(a(1, 2), c0)), id);
    R[13] = fm(fa(fs(fm(a(0, 0), c3), fm(a(0, 1), c1)), fm(a(0, 2), c0)), id);
    R[14] = fm(fs(fa(fm(-a(3, 0), s3), fm(a(3, 1), s1)), fm(a(3, 2), s0)), id);
    R[15] = fm(fa(fs(fm(a(2, 0), s3), fm(a(2, 1), s1)), fm(a(2, 2), s0)), id);
#undef a
}

// utils::floorToInt: floor of a finite float that fits an int.
__device__ __forceinline__ bool floor_to_int(float v, int* out) {
    if (!isfinite(v)) return false;
    const float f = floorf(v);
    if (f < -2147483648.0f || f >= 2147483648.0f) return false;
    *out = static_cast<int>(f);
    return true;
}

// utils::srgbFloatToUint8: clamp to [0,1], round half away from zero of v*255.
__device__ __forceinline__ bool srgb_to_byte(float v, uint8_t* out) {
    if (!isfinite(v)) return false;
    const float c = v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v);
    *out = static_cast<uint8_t>(lroundf(fm(c, 255.0f)));
    return true;
}

// Kinect raw disparity code <-> metres (sensor/DepthValidity.h semantics).
constexpr float kCurveA = -0.0030711016f;
constexpr float kCurveB = 3.3309495161f;
__device__ __forceinline__ bool raw_invalid(uint16_t r) { return r == 0 || r >= 2047; }
__device__ __forceinline__ float raw_to_m(uint16_t r) {
    if (raw_invalid(r)) return 0.0f;
    return fd(1.0f, fa(fm(static_cast<float>(r), kCurveA), kCurveB));
}
__device__ __forceinline__ bool in_band(float m, float lo, float hi) { return isfinite(m) && m >= lo && m <= hi; }
__device__ __forceinline__ float depth_m(uint16_t r, float lo, float hi) {
    if (raw_invalid(r)) return 0.0f;
    const float m = raw_to_m(r);
    return in_band(m, lo, hi) ? m : 0.0f;
}
__device__ __forceinline__ uint16_t m_to_raw(float m, float lo, float hi) {
    if (!in_band(m, lo, hi)) return 0;
    const float raw = fd(fs(fd(1.0f, m), kCurveB), kCurveA);
    if (!isfinite(raw)) return 0;
    const float r = roundf(raw);  // half away from zero, as std::lround
    if (r < 1.0f || r > 2046.0f) return 0;
    return static_cast<uint16_t>(r);
}
__device__ __forceinline__ bool usable_raw(uint16_t r, float lo, float hi) {
    return !raw_invalid(r) && in_band(raw_to_m(r), lo, hi);
}
__device__ __forceinline__ int reflect(int c, int n) {
    if (c < 0) return -c - 1;
    if (c >= n) return 2 * n - c - 1;
    return c;
}

}  // namespace azu
