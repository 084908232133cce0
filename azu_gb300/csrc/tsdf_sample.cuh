// Voxel records and the trilinear sampling of the TSDF volume, shared by the
// volume kernels (tsdf.cu) and the differentiable renderer (diff.cu).
#pragma once

#include <cuda_fp16.h>

#include <cmath>
#include <cstdint>

#include "azu_internal.h"
#include "kf_math.cuh"

namespace azu {

constexpr float kEmptyTsdf = 1.0f;
constexpr float kEmptyColor = 128.0f / 255.0f;
// A voxel at or above this tsdf counts as free space for the brick map; the
// margin over the march's 0.999 covers the rounding of trilinear interpolation.
constexpr float kFreeTsdf = 0.9995f;
constexpr int kBrickShift = 3;  // 8^3-voxel bricks

// ---- voxel record access -----------------------------------------------
template <bool kHalf>
struct Vox;
template <>
struct Vox<false> {
    using T = float2;
    __device__ static __forceinline__ float2 load(const void* v, size_t i) {
        return __ldg(static_cast<const float2*>(v) + i);
    }
    __device__ static __forceinline__ float2 load_rw(const void* v, size_t i) {
        return static_cast<const float2*>(v)[i];
    }
    __device__ static __forceinline__ void store(void* v, size_t i, float t, float w) {
        static_cast<float2*>(v)[i] = make_float2(t, w);
    }
    __device__ static __forceinline__ float rounded(float t) { return t; }
};
template <>
struct Vox<true> {
    using T = uint32_t;
    __device__ static __forceinline__ float2 unpack(uint32_t u) {
        return make_float2(__half2float(__ushort_as_half(static_cast<unsigned short>(u & 0xFFFFu))),
                           static_cast<float>(u >> 16));
    }
    __device__ static __forceinline__ float2 load(const void* v, size_t i) {
        return unpack(__ldg(static_cast<const uint32_t*>(v) + i));
    }
    __device__ static __forceinline__ float2 load_rw(const void* v, size_t i) {
        return unpack(static_cast<const uint32_t*>(v)[i]);
    }
    __device__ static __forceinline__ void store(void* v, size_t i, float t, float w) {
        const uint32_t h = __half_as_ushort(__float2half_rn(t));
        static_cast<uint32_t*>(v)[i] = h | (static_cast<uint32_t>(w) << 16);
    }
    __device__ static __forceinline__ float rounded(float t) { return __half2float(__float2half_rn(t)); }
};

// FP16 tsdf with a sub-half residual (AZU_TSDF_FP16R). Word: bits 0-15 the
// half h = RN(t); bits 16-31 the weight (7 bits) << 9 | q, q a 9-bit two's
// complement in units s = ulp(h) / 512, |q| <= 255. The fold reads
// t' = h + q s (exact in float: at most 21 significant bits), so repeated
// updates do not stall at half precision; readers use h.
struct VoxR {
    // s = ulp(h) / 512 from the half's exponent field (subnormals: 2^-24 / 512)
    __device__ static __forceinline__ float unit(uint32_t hbits) {
        const int e = static_cast<int>((hbits >> 10) & 0x1fu);
        return __int_as_float((e == 0 ? 94 : e + 93) << 23);
    }
    __device__ static __forceinline__ float2 load_fold(const void* v, size_t i) {
        const uint32_t u = static_cast<const uint32_t*>(v)[i];
        const uint32_t hi = u >> 16;
        const int q = static_cast<int>((hi & 0x1ffu) ^ 0x100u) - 0x100;
        const float h = __half2float(__ushort_as_half(static_cast<unsigned short>(u & 0xFFFFu)));
        return make_float2(fmaf(static_cast<float>(q), unit(u & 0xFFFFu), h), static_cast<float>(hi >> 9));
    }
    __device__ static __forceinline__ void store(void* v, size_t i, float t, float w) {
        const unsigned short hb = __half_as_ushort(__float2half_rn(t));
        const float h = __half2float(__ushort_as_half(hb));
        // t - h is exact; scaling by 1 / s, a power of two, is exact
        const int e = static_cast<int>((hb >> 10) & 0x1fu);
        const float inv_s = __int_as_float((e == 0 ? 160 : 161 - e) << 23);
        int q = __float2int_rn(fs(t, h) * inv_s);
        q = max(-255, min(255, q));
        const uint32_t hi = (static_cast<uint32_t>(w) << 9) | (static_cast<uint32_t>(q) & 0x1ffu);
        static_cast<uint32_t*>(v)[i] = static_cast<uint32_t>(hb) | (hi << 16);
    }
};

// ---- sampling --------------------------------------------------------------
struct VolView {
    const void* vox;
    const float* color;
    int res;
    float vs;
    F3 origin;
    float inv_vs;  // 1 / vs when vs is a power of two (then exact), else 0
};

// (p - origin) / vs. When vs is a power of two the quotient equals the product
// with its exact reciprocal bit for bit, and the multiplication is far cheaper.
__device__ __forceinline__ F3 to_voxel(const VolView& v, F3 p) {
    const F3 d = sub3(p, v.origin);
    if (v.inv_vs != 0.0f) return mul3(d, v.inv_vs);
    return div3(d, v.vs);
}

// sampleTSDF (TSDFVolume.cpp:492-525): trilinear, valid only if all 8 corners
// are observed.
template <bool kHalf>
__device__ __forceinline__ bool sample_tsdf(const VolView& v, F3 p, float& f) {
    const F3 q = to_voxel(v, p);
    const float fx0 = floorf(q.x), fy0 = floorf(q.y), fz0 = floorf(q.z);
    const float lim = static_cast<float>(v.res - 1);
    if (!(fx0 >= 0.0f && fy0 >= 0.0f && fz0 >= 0.0f && fx0 < lim && fy0 < lim && fz0 < lim)) return false;
    const int x0 = static_cast<int>(fx0), y0 = static_cast<int>(fy0), z0 = static_cast<int>(fz0);
    const float tx = fs(q.x, fx0), ty = fs(q.y, fy0), tz = fs(q.z, fz0);
    const size_t r = static_cast<size_t>(v.res);
    const size_t b = (static_cast<size_t>(z0) * r + static_cast<size_t>(y0)) * r + static_cast<size_t>(x0);
    const float2 c0 = Vox<kHalf>::load(v.vox, b), c1 = Vox<kHalf>::load(v.vox, b + 1);
    const float2 c2 = Vox<kHalf>::load(v.vox, b + r), c3 = Vox<kHalf>::load(v.vox, b + r + 1);
    const float2 c4 = Vox<kHalf>::load(v.vox, b + r * r), c5 = Vox<kHalf>::load(v.vox, b + r * r + 1);
    const float2 c6 = Vox<kHalf>::load(v.vox, b + r * r + r), c7 = Vox<kHalf>::load(v.vox, b + r * r + r + 1);
    if (!(c0.y > 0.0f) || !(c1.y > 0.0f) || !(c2.y > 0.0f) || !(c3.y > 0.0f) || !(c4.y > 0.0f) ||
        !(c5.y > 0.0f) || !(c6.y > 0.0f) || !(c7.y > 0.0f))
        return false;
    const float ux = fs(1.0f, tx), uy = fs(1.0f, ty), uz = fs(1.0f, tz);
    const float v00 = fa(fm(c0.x, ux), fm(c1.x, tx));
    const float v10 = fa(fm(c2.x, ux), fm(c3.x, tx));
    const float v01 = fa(fm(c4.x, ux), fm(c5.x, tx));
    const float v11 = fa(fm(c6.x, ux), fm(c7.x, tx));
    const float v0 = fa(fm(v00, uy), fm(v10, ty));
    const float v1 = fa(fm(v01, uy), fm(v11, ty));
    f = fa(fm(v0, uz), fm(v1, tz));
    return true;
}

// computeNormal (TSDFVolume.cpp:478-490).
template <bool kHalf>
__device__ __forceinline__ bool compute_normal(const VolView& v, F3 p, F3& n_out) {
    const float h = v.vs;
    float s[6];
    if (!sample_tsdf<kHalf>(v, mk3(fa(p.x, h), fa(p.y, 0.0f), fa(p.z, 0.0f)), s[0])) return false;
    if (!sample_tsdf<kHalf>(v, mk3(fs(p.x, h), fs(p.y, 0.0f), fs(p.z, 0.0f)), s[1])) return false;
    if (!sample_tsdf<kHalf>(v, mk3(fa(p.x, 0.0f), fa(p.y, h), fa(p.z, 0.0f)), s[2])) return false;
    if (!sample_tsdf<kHalf>(v, mk3(fs(p.x, 0.0f), fs(p.y, h), fs(p.z, 0.0f)), s[3])) return false;
    if (!sample_tsdf<kHalf>(v, mk3(fa(p.x, 0.0f), fa(p.y, 0.0f), fa(p.z, h)), s[4])) return false;
    if (!sample_tsdf<kHalf>(v, mk3(fs(p.x, 0.0f), fs(p.y, 0.0f), fs(p.z, h)), s[5])) return false;
    const F3 n = mk3(fs(s[0], s[1]), fs(s[2], s[3]), fs(s[4], s[5]));
    const float len = norm3(n);
    if (!(len > 1e-6f) || !isfinite(len)) return false;
    n_out = div3(n, len);
    return true;
}

// View of a volume for the samplers. For a power-of-two voxel size the exact
// reciprocal 2^(1-e) is stored so that (p - origin) / vs becomes a product.
inline VolView make_view(const azu_volume* v) {
    const azu_volume_params& p = v->p;
    int e2 = 0;
    const float mant = std::frexp(p.voxel_size, &e2);
    const float inv_vs = (mant == 0.5f && e2 > -120 && e2 < 120) ? std::ldexp(1.0f, 1 - e2) : 0.0f;
    return VolView{v->vox, v->color, p.resolution, p.voxel_size, mk3(p.origin[0], p.origin[1], p.origin[2]), inv_vs};
}

}  // namespace azu
