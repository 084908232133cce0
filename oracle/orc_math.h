// Oracle (test infrastructure only): fixed-size float linear algebra used by the
// CPU restatement of Azu's KinectFusion hot path.
//
// The reference builds these operations on Eigen (not vendored, not present
// here). This header restates the handful of operations its hot path uses,
// written from the mathematics, with ONE documented evaluation order per
// operation so that the CUDA path can reproduce the same IEEE-754 float results:
//
//   dot3(a, b)      = a0*b0 + (a1*b1 + a2*b2)        (Eigen's unrolled 3-term sum)
//   M3 * v          = dot3(row_i, v) per row
//   M3 * M3         = dot3(row_i, col_j)
//   M4 * M4         = ((a0*b0 + a1*b1) + a2*b2) + a3*b3
//   squaredNorm(v)  = dot3(v, v);  norm = sqrt(squaredNorm)
//   inverse4        = adjugate / determinant from 2x2 minors (float)
//
// Every file of the oracle is compiled with -ffp-contract=off, so no multiply-add
// is fused behind the code's back (aarch64 GCC fuses by default).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>
#include <limits>

namespace orc {

struct V3 {
    float x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(float a, float b, float c) : x(a), y(b), z(c) {}
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
};

inline V3 operator+(V3 a, V3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator*(V3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
inline V3 operator*(float s, V3 a) { return V3(s * a.x, s * a.y, s * a.z); }
inline V3 operator/(V3 a, float s) { return V3(a.x / s, a.y / s, a.z / s); }
inline V3 operator-(V3 a) { return V3(-a.x, -a.y, -a.z); }

inline float dot3(V3 a, V3 b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }
inline float sqnorm(V3 a) { return dot3(a, a); }
inline float norm(V3 a) { return std::sqrt(sqnorm(a)); }
inline V3 cross(V3 a, V3 b) {
    return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline bool finite3(V3 a) { return std::isfinite(a.x) && std::isfinite(a.y) && std::isfinite(a.z); }
inline V3 vmin(V3 a, V3 b) { return V3(std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z)); }
inline V3 vmax(V3 a, V3 b) { return V3(std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)); }

// Row-major 3x3.
struct M3 {
    float m[3][3];
    static M3 ident() { M3 r; std::memset(r.m, 0, sizeof(r.m)); r.m[0][0] = r.m[1][1] = r.m[2][2] = 1; return r; }
    V3 row(int i) const { return V3(m[i][0], m[i][1], m[i][2]); }
    V3 col(int j) const { return V3(m[0][j], m[1][j], m[2][j]); }
    M3 T() const { M3 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[i][j] = m[j][i]; return r; }
};
inline V3 operator*(const M3& a, V3 v) { return V3(dot3(a.row(0), v), dot3(a.row(1), v), dot3(a.row(2), v)); }
inline M3 operator*(const M3& a, const M3& b) {
    M3 r;
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[i][j] = dot3(a.row(i), b.col(j));
    return r;
}

// Row-major 4x4 (the reference's Eigen::Matrix4f is column-major in memory; the ABI
// passes poses row-major, element (r, c) at [4 r + c]).
struct M4 {
    float m[4][4];
    static M4 ident() { M4 r; std::memset(r.m, 0, sizeof(r.m)); for (int i = 0; i < 4; ++i) r.m[i][i] = 1; return r; }
    static M4 from(const float* p) { M4 r; std::memcpy(r.m, p, sizeof(r.m)); return r; }
    void to(float* p) const { std::memcpy(p, m, sizeof(m)); }
    M3 R() const { M3 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[i][j] = m[i][j]; return r; }
    V3 t() const { return V3(m[0][3], m[1][3], m[2][3]); }
    void setR(const M3& r) { for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) m[i][j] = r.m[i][j]; }
    bool finite() const { for (int i = 0; i < 4; ++i) for (int j = 0; j < 4; ++j) if (!std::isfinite(m[i][j])) return false; return true; }
};
inline M4 operator*(const M4& a, const M4& b) {
    M4 r;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            r.m[i][j] = ((a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j]) + a.m[i][2] * b.m[2][j]) +
                        a.m[i][3] * b.m[3][j];
    return r;
}

// General 4x4 inverse by the adjugate built from 2x2 minors of the top and bottom
// row pairs (Laplace expansion along those pairs).
inline M4 inverse4(const M4& A) {
    const float(*a)[4] = A.m;
    const float s0 = a[0][0] * a[1][1] - a[1][0] * a[0][1];
    const float s1 = a[0][0] * a[1][2] - a[1][0] * a[0][2];
    const float s2 = a[0][0] * a[1][3] - a[1][0] * a[0][3];
    const float s3 = a[0][1] * a[1][2] - a[1][1] * a[0][2];
    const float s4 = a[0][1] * a[1][3] - a[1][1] * a[0][3];
    const float s5 = a[0][2] * a[1][3] - a[1][2] * a[0][3];
    const float c5 = a[2][2] * a[3][3] - a[3][2] * a[2][3];
    const float c4 = a[2][1] * a[3][3] - a[3][1] * a[2][3];
    const float c3 = a[2][1] * a[3][2] - a[3][1] * a[2][2];
    const float c2 = a[2][0] * a[3][3] - a[3][0] * a[2][3];
    const float c1 = a[2][0] * a[3][2] - a[3][0] * a[2][2];
    const float c0 = a[2][0] * a[3][1] - a[3][0] * a[2][1];
    const float det = ((((s0 * c5 - s1 * c4) + s2 * c3) + s3 * c2) - s4 * c1) + s5 * c0;
    const float id = 1.0f / det;
    M4 r;
    r.m[0][0] = ((a[1][1] * c5 - a[1][2] * c4) + a[1][3] * c3) * id;
    r.m[0][1] = ((-a[0][1] * c5 + a[0][2] * c4) - a[0][3] * c3) * id;
    r.m[0][2] = ((a[3][1] * s5 - a[3][2] * s4) + a[3][3] * s3) * id;
    r.m[0][3] = ((-a[2][1] * s5 + a[2][2] * s4) - a[2][3] * s3) * id;
    r.m[1][0] = ((-a[1][0] * c5 + a[1][2] * c2) - a[1][3] * c1) * id;
    r.m[1][1] = ((a[0][0] * c5 - a[0][2] * c2) + a[0][3] * c1) * id;
    r.m[1][2] = ((-a[3][0] * s5 + a[3][2] * s2) - a[3][3] * s1) * id;
    r.m[1][3] = ((a[2][0] * s5 - a[2][2] * s2) + a[2][3] * s1) * id;
    r.m[2][0] = ((a[1][0] * c4 - a[1][1] * c2) + a[1][3] * c0) * id;
    r.m[2][1] = ((-a[0][0] * c4 + a[0][1] * c2) - a[0][3] * c0) * id;
    r.m[2][2] = ((a[3][0] * s4 - a[3][1] * s2) + a[3][3] * s0) * id;
    r.m[2][3] = ((-a[2][0] * s4 + a[2][1] * s2) - a[2][3] * s0) * id;
    r.m[3][0] = ((-a[1][0] * c3 + a[1][1] * c1) - a[1][2] * c0) * id;
    r.m[3][1] = ((a[0][0] * c3 - a[0][1] * c1) + a[0][2] * c0) * id;
    r.m[3][2] = ((-a[3][0] * s3 + a[3][1] * s1) - a[3][2] * s0) * id;
    r.m[3][3] = ((a[2][0] * s3 - a[2][1] * s1) + a[2][2] * s0) * id;
    return r;
}

// utils::floorToInt (include/utils/CoordinateMath.h:27-49): floor of a finite
// float that fits an int, else false.
inline bool floorToInt(float v, int* out) {
    if (!std::isfinite(v)) return false;
    const double f = std::floor(static_cast<double>(v));
    if (f < static_cast<double>(std::numeric_limits<int>::min()) ||
        f > static_cast<double>(std::numeric_limits<int>::max()))
        return false;
    *out = static_cast<int>(f);
    return true;
}

// utils::srgbFloatToUint8 / srgbUint8ToFloat (include/utils/ColorMath.h:50-88).
inline bool srgbFloatToUint8(float v, uint8_t& out) {
    if (!std::isfinite(v)) return false;
    const float c = (v < 0.0f) ? 0.0f : (v > 1.0f ? 1.0f : v);
    const long s = std::lround(c * 255.0f);
    if (s < 0 || s > 255) return false;
    out = static_cast<uint8_t>(s);
    return true;
}
inline float srgbUint8ToFloat(uint8_t v) { return static_cast<float>(v) / 255.0f; }

// Depth validity (include/sensor/DepthValidity.h:48-118).
constexpr uint16_t kRawSentinel = 2047;
constexpr float kCurveA = -0.0030711016f;
constexpr float kCurveB = 3.3309495161f;
inline bool rawInvalid(uint16_t r) { return r == 0 || r >= kRawSentinel; }
inline float rawToMeters(uint16_t r) {
    if (rawInvalid(r)) return 0.0f;
    return 1.0f / (static_cast<float>(r) * kCurveA + kCurveB);
}
inline bool inBand(float m, float lo, float hi) { return std::isfinite(m) && m >= lo && m <= hi; }
inline float cpuDepthMeters(uint16_t r, float lo, float hi) {
    if (rawInvalid(r)) return 0.0f;
    const float m = rawToMeters(r);
    return inBand(m, lo, hi) ? m : 0.0f;
}
inline uint16_t metersToRaw(float m, float lo, float hi) {
    if (!inBand(m, lo, hi)) return 0;
    const float raw = (1.0f / m - kCurveB) / kCurveA;
    if (!std::isfinite(raw)) return 0;
    const long code = std::lround(raw);
    if (code < 1 || code > 2046) return 0;
    return static_cast<uint16_t>(code);
}
inline bool usableRaw(uint16_t r, float lo, float hi) { return !rawInvalid(r) && inBand(rawToMeters(r), lo, hi); }

// sensor::cpuReflectCoord (include/sensor/BorderMode.h:42-46).
inline int reflect(int c, int n) {
    if (c < 0) return -c - 1;
    if (c >= n) return 2 * n - c - 1;
    return c;
}

}  // namespace orc
