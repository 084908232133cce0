// Exact closed form of a running float sum.
//
// The reference integrates a voxel row by stepping the camera coordinate,
// c += R_wc.col(0) * vs, one float addition per voxel
// (src/tsdf/TSDFVolume.cpp:282-285), so the coordinate of voxel x is the
// result of x - x0 rounded additions of one constant s. Replaying that chain
// serialises every row. The sums have a closed form, segment by segment:
//
//   Let v lie in the binade [2^e, 2^(e+1)) (in magnitude), u = 2^(e-23) its
//   ulp, and S = s / u (exact: u is a power of two). While the exact sum
//   v + s stays in [2^e + u/2, 2^(e+1) - u/2], it is rounded on the grid of
//   multiples of u, so fl(v + s) = v + Q u with Q = rint(S) unless S is a
//   rounding tie (fraction 1/2); a tie rounds to the even multiple, so from
//   an even v / u every step adds the even neighbour of S. Hence, with
//   d = Q u, the value after j steps is v + j d exactly — one fma, exact
//   because the result is a multiple of u inside the binade — for every j up
//   to the last step that stays in the safe zone [2^e + u, 2^(e+1) - u].
//
// At a binade edge one ordinary addition crosses it and the next segment
// starts. Zero, tiny and huge magnitudes (and a tie from an odd start) have
// no closed form here; they take ordinary additions, which are always exact
// replays. Every function below therefore returns the bits of the sequential
// chain (tests/test_fstep.py checks this against the chain for millions of
// random and edge-case starts, steps and lengths, compiled for the host).
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define FSTEP_HD __host__ __device__ __forceinline__
#else
#define FSTEP_HD inline
#endif

namespace azu {

FSTEP_HD uint32_t fs_bits(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}

FSTEP_HD float fs_float(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}

// One rounded addition (never contracted with a neighbouring multiply).
FSTEP_HD float fs_add(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    volatile float r = a + b;
    return r;
#endif
}

FSTEP_HD float fs_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}

// The segment of the running sum v, v + s, ... that starts at v: after j
// steps, 0 <= j <= m, the value is fs_fma(j, d, v) bit for bit. m = 0 when
// v has no closed form (the next value needs an ordinary addition);
// m = kFsForever when the sum can no longer move (|s| below half an ulp).
constexpr int kFsForever = 0x7fffffff;

struct FSeg {
    float d;
    int m;
};

FSTEP_HD FSeg fs_segment(float v, float s) {
    const uint32_t vb = fs_bits(v);
    FSeg r{fs_float(vb & 0x80000000u), 0};  // a zero of v's sign: fma(0, d, v) is v, also for v = -0
    const int ex = static_cast<int>((vb >> 23) & 0xffu);  // biased exponent of |v|
    // |v| in [2^-100, 2^100): 2^(23-e) and 2^(e-23) are normal floats
    if (ex < 27 || ex >= 227) return r;
    const uint32_t sb = fs_bits(s);
    if (((sb >> 23) & 0xffu) == 0xffu) return r;  // s not finite
    const float inv_u = fs_float(static_cast<uint32_t>(277 - ex) << 23);  // 2^(23-e)
    const float u = fs_float(static_cast<uint32_t>(ex - 23) << 23);       // 2^(e-23)
    const float S = s * inv_u;  // exact (a power-of-two scaling of a finite s, no overflow)
    const int32_t A = static_cast<int32_t>((vb & 0x7fffffu) | 0x800000u);  // |v| / u in [2^23, 2^24)
    float Q = rintf(S);  // round half to even: the non-tie increment
    const float fl = floorf(S);
    if (S - fl == 0.5f) {
        // tie (only possible for |S| < 2^23): the result is the even multiple
        if (A & 1) return r;
        const int32_t fi = static_cast<int32_t>(fl);
        Q = (fi & 1) ? fl + 1.0f : fl;
    }
    r.d = Q * u;  // exact
    if (Q == 0.0f) {
        r.m = kFsForever;
        return r;
    }
    const float aQ = fabsf(Q);
    if (aQ >= 8388608.0f) return r;  // a step jumps a whole binade
    const int32_t D = static_cast<int32_t>(aQ);
    const bool up = (static_cast<int32_t>(vb) < 0) == (Q < 0.0f);  // the magnitude grows
    const int32_t room = up ? (0xffffff - A) : (A - 0x800001);      // units of u to the safe zone's edge
    r.m = room > 0 ? room / D : 0;
    return r;
}

// v after n (>= 0) sequential additions of s, fl(...fl(fl(v + s) + s)...).
FSTEP_HD float fs_walk(float v, float s, int n) {
    while (n > 0) {
        const FSeg g = fs_segment(v, s);
        if (g.m == kFsForever) return v;
        if (g.m == 0) {
            v = fs_add(v, s);
            --n;
            continue;
        }
        const int j = g.m < n ? g.m : n;
        v = fs_fma(static_cast<float>(j), g.d, v);
        n -= j;
    }
    return v;
}

}  // namespace azu
