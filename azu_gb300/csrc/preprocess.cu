// Depth preprocessor on the GPU (SignalConditioner CPU semantics,
// src/sensor/SignalConditioner_omp.cpp:120-715; CAS from
// src/sensor/SuperResolution.cpp:118-166), behind the azu_preprocessor_* ABI.
//
// Per 640x480 frame:
//   RGB guidance   bilateral 5x5 -> median 3x3 (the processed RGB) -> CAS -> luma
//   depth          median 3x3 (metres) -> 5x5 inverse-distance hole fill of raw 0
//                  -> 9x9 luma-guided joint bilateral -> temporal EMA
//   output         processed raw codes and band-gated metres (buildFrameData's
//                  depth_meters) on the device
// One kernel per stage; every stage is a stencil over the previous stage's
// full output, so the stage boundary is the only synchronisation. The RGB
// chain runs on a side stream beside the depth median and hole fill; the
// guided filter, which reads the luma, waits for both.
//
// The exponentials whose arguments take a finite set of values come from
// tables built on the host with the same libm call the CPU path makes, so
// the weights — and everything after them — are bit-identical to it:
//   RGB bilateral: spatial exp(-d^2/8) for d^2 in 0..8 and range
//                  exp(-c/1568) for the integer colour distance c in 0..195075;
//   guided filter: spatial exp(-d^2/32) for d^2 in 0..32 and the depth term
//                  exp(-(m(a)-m(b))^2/0.0132) for every pair of raw codes a, b.
// The luma term exp(-dl^2/0.03) is evaluated with expf; it is exactly 1 when
// the guidance is locally constant (dl = 0).
#include <cmath>
#include <cstring>
#include <vector>

#include "azu_internal.h"
#include "kf_math.cuh"

namespace azu {

constexpr int PW = 640, PH = 480;
constexpr int kRawCodes = 2047;  // codes 0..2046

struct PreTables {
    float rgb_spatial[9];
    float guided_spatial[33];
};
__constant__ PreTables c_tab;

__device__ __forceinline__ uint8_t clamp_byte(float v) {
    const float c = v < 0.0f ? 0.0f : (255.0f < v ? 255.0f : v);
    return static_cast<uint8_t>(c);
}

// bilateralDenoiseRgb (:185-230).
__global__ void __launch_bounds__(256) rgb_bilateral_kernel(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst,
                                                            const float* __restrict__ range_w) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= PW || y >= PH) return;
    const int ci = (y * PW + x) * 3;
    const float c0 = src[ci], c1 = src[ci + 1], c2 = src[ci + 2];
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, ws = 0.0f;
    for (int dy = -2; dy <= 2; ++dy) {
        const int sy = reflect(y + dy, PH);
        for (int dx = -2; dx <= 2; ++dx) {
            const int si = (sy * PW + reflect(x + dx, PW)) * 3;
            const float s0 = src[si], s1 = src[si + 1], s2 = src[si + 2];
            const float d0 = fs(s0, c0), d1 = fs(s1, c1), d2 = fs(s2, c2);
            const float cd2 = fa(fa(fa(0.0f, fm(d0, d0)), fm(d1, d1)), fm(d2, d2));
            const float w = fm(c_tab.rgb_spatial[dx * dx + dy * dy], __ldg(range_w + static_cast<int>(cd2)));
            a0 = fa(a0, fm(w, s0));
            a1 = fa(a1, fm(w, s1));
            a2 = fa(a2, fm(w, s2));
            ws = fa(ws, w);
        }
    }
    if (ws > 1e-6f) {
        dst[ci] = clamp_byte(fd(a0, ws));
        dst[ci + 1] = clamp_byte(fd(a1, ws));
        dst[ci + 2] = clamp_byte(fd(a2, ws));
    } else {
        dst[ci] = src[ci];
        dst[ci + 1] = src[ci + 1];
        dst[ci + 2] = src[ci + 2];
    }
}

template <typename T>
__device__ __forceinline__ void cswap(T& a, T& b) {
    const T lo = a < b ? a : b, hi = a < b ? b : a;
    a = lo;
    b = hi;
}

// medianBlur3x3 (:160-183): per-channel median of the reflect-1 3x3 window.
__global__ void __launch_bounds__(256) rgb_median_kernel(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= PW || y >= PH) return;
    for (int c = 0; c < 3; ++c) {
        int w[9], n = 0;
        for (int dy = -1; dy <= 1; ++dy) {
            const int sy = reflect(y + dy, PH);
            for (int dx = -1; dx <= 1; ++dx) w[n++] = src[(sy * PW + reflect(x + dx, PW)) * 3 + c];
        }
        // full sort of 9 (odd-even transposition), median = w[4]
        for (int i = 0; i < 9; ++i)
            for (int j = (i & 1); j + 1 < 9; j += 2) cswap(w[j], w[j + 1]);
        dst[(y * PW + x) * 3 + c] = static_cast<uint8_t>(w[4]);
    }
}

// applyCAS_CPU at sharpness 0.5 + rgbLuma / 255 (SuperResolution.cpp:118-166,
// SignalConditioner_omp.cpp:381-385).
// The byte / 255 quotients come from a per-block table of the 256 values
// (the same division, once per byte value instead of 15 times per pixel).
__global__ void __launch_bounds__(256) cas_luma_kernel(const uint8_t* __restrict__ src, float* __restrict__ luma) {
    __shared__ float s_unit[256];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    if (tid < 256) s_unit[tid] = fd(static_cast<float>(tid), 255.0f);
    __syncthreads();
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= PW || y >= PH) return;
    const float t = 0.5f;
    const float peak = fd(-1.0f, fa(fm(fs(1.0f, t), 8.0f), fm(t, 5.0f)));
    auto px = [&](int xx, int yy, float* out) {
        xx = reflect(xx, PW);
        yy = reflect(yy, PH);
        const int i = (yy * PW + xx) * 3;
        out[0] = s_unit[src[i]];
        out[1] = s_unit[src[i + 1]];
        out[2] = s_unit[src[i + 2]];
    };
    float a[3], b[3], c[3], d[3], e[3];
    px(x, y - 1, a); px(x - 1, y, b); px(x, y, c); px(x + 1, y, d); px(x, y + 1, e);
    float amp = 1.0f;
    for (int ch = 0; ch < 3; ++ch) {
        const float mn = fminf(fminf(fminf(fminf(a[ch], b[ch]), c[ch]), d[ch]), e[ch]);
        const float mx = fmaxf(fmaxf(fmaxf(fmaxf(a[ch], b[ch]), c[ch]), d[ch]), e[ch]);
        const float mxs = mx < 1e-6f ? 1e-6f : mx;
        const float head = fs(1.0f, mx);
        const float ac = fd(head < mn ? head : mn, mxs);
        amp = ac < amp ? ac : amp;
    }
    const float w = fm(amp, peak);
    const float wsum = fa(1.0f, fm(4.0f, w));
    uint8_t o[3];
    for (int ch = 0; ch < 3; ++ch) {
        const float v = fd(fa(c[ch], fm(w, fa(fa(fa(a[ch], b[ch]), d[ch]), e[ch]))), wsum);
        const float cl = v < 0.0f ? 0.0f : (1.0f < v ? 1.0f : v);
        o[ch] = static_cast<uint8_t>(fm(cl, 255.0f));
    }
    luma[y * PW + x] = fd(fa(fa(fm(0.299f, static_cast<float>(o[0])), fm(0.587f, static_cast<float>(o[1]))),
                             fm(0.114f, static_cast<float>(o[2]))),
                          255.0f);
}

// denoiseDepthSpatial (:442-482). The block's pixels and a 1-pixel apron
// (reflected at the border) are converted to metres once, in shared memory.
constexpr int kMTx = 32, kMTy = 8, kMW = kMTx + 2, kMH = kMTy + 2;
__global__ void __launch_bounds__(kMTx * kMTy) depth_median_kernel(const uint16_t* __restrict__ in,
                                                                  uint16_t* __restrict__ out, float lo, float hi) {
    __shared__ float s_m[kMH][kMW];
    const int x0 = blockIdx.x * kMTx, y0 = blockIdx.y * kMTy;
    for (int i = threadIdx.y * kMTx + threadIdx.x; i < kMW * kMH; i += kMTx * kMTy) {
        const int ty = i / kMW, tx = i - ty * kMW;
        s_m[ty][tx] = depth_m(in[reflect(y0 - 1 + ty, PH) * PW + reflect(x0 - 1 + tx, PW)], lo, hi);
    }
    __syncthreads();
    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
    if (x >= PW || y >= PH) return;
    const int idx = y * PW + x;
    const int cx = threadIdx.x + 1, cy = threadIdx.y + 1;
    uint16_t res = in[idx];
    if (s_m[cy][cx] != 0.0f) {
        float w[9];
        int n = 0;
        for (int dy = -1; dy <= 1; ++dy) {
            for (int dx = -1; dx <= 1; ++dx) {
                const float v = s_m[cy + dy][cx + dx];
                if (v != 0.0f) w[n++] = v;
            }
        }
        if (n >= 3) {
            for (int i = 1; i < n; ++i) {  // insertion sort of <= 9
                const float v = w[i];
                int j = i - 1;
                while (j >= 0 && w[j] > v) { w[j + 1] = w[j]; --j; }
                w[j + 1] = v;
            }
            res = m_to_raw(w[n / 2], lo, hi);
        }
    }
    out[idx] = res;
}

// fillDepthHoles (:578-635): only raw 0 is a hole.
__global__ void __launch_bounds__(256) hole_fill_kernel(const uint16_t* __restrict__ in, uint16_t* __restrict__ out,
                                                        float lo, float hi) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= PW || y >= PH) return;
    const int idx = y * PW + x;
    const uint16_t r0 = in[idx];
    uint16_t res = r0;
    if (r0 == 0) {
        float wsd = 0.0f, wsum = 0.0f;
        int nv = 0;
        for (int dy = -2; dy <= 2; ++dy) {
            const int sy = reflect(y + dy, PH);
            for (int dx = -2; dx <= 2; ++dx) {
                if (dx == 0 && dy == 0) continue;
                const float cm = depth_m(in[sy * PW + reflect(x + dx, PW)], lo, hi);
                if (cm == 0.0f) continue;
                const float w = fd(1.0f, fa(static_cast<float>(dx * dx + dy * dy), 1.0f));
                wsd = fa(wsd, fm(w, cm));
                wsum = fa(wsum, w);
                ++nv;
            }
        }
        if (nv > 0 && wsum > 1e-6f) res = m_to_raw(fd(wsd, wsum), lo, hi);
    }
    out[idx] = res;
}

// guidedDepthFilter (:637-715) with computeDepthGradient (:120-141).
// The block's 32 x 8 pixels and their 4-pixel apron (reflected at the image
// border like every neighbour index) are staged once in shared memory as raw
// code, metres and luma, so each of the 81 taps reads them there instead of
// recomputing the code -> metres division per tap; the taps and their order
// are unchanged.
constexpr int kGTx = 32, kGTy = 8, kGR = 4, kGW = kGTx + 2 * kGR, kGH = kGTy + 2 * kGR;
__global__ void __launch_bounds__(kGTx * kGTy) guided_kernel(const uint16_t* __restrict__ in,
                                                           uint16_t* __restrict__ out,
                                                           const float* __restrict__ luma,
                                                           const float* __restrict__ dw_tab, float lo, float hi) {
    __shared__ uint16_t s_raw[kGH][kGW];
    __shared__ float s_m[kGH][kGW];
    __shared__ float s_l[kGH][kGW];
    const int x0 = blockIdx.x * kGTx, y0 = blockIdx.y * kGTy;
    for (int i = threadIdx.y * kGTx + threadIdx.x; i < kGW * kGH; i += kGTx * kGTy) {
        const int ty = i / kGW, tx = i - ty * kGW;
        const int gi = reflect(y0 - kGR + ty, PH) * PW + reflect(x0 - kGR + tx, PW);
        const uint16_t r = in[gi];
        s_raw[ty][tx] = r;
        s_m[ty][tx] = depth_m(r, lo, hi);
        s_l[ty][tx] = __ldg(luma + gi);
    }
    __syncthreads();
    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
    if (x >= PW || y >= PH) return;
    const int idx = y * PW + x;
    const int cx = threadIdx.x + kGR, cy = threadIdx.y + kGR;
    const uint16_t rc = s_raw[cy][cx];
    const float cd = s_m[cy][cx];
    if (cd == 0.0f) {
        out[idx] = rc;
        return;
    }
    const float cl = s_l[cy][cx];
    float edge = 1.0f;
    if (x > 0 && x < PW - 1 && y > 0 && y < PH - 1) {
        const uint16_t r = s_raw[cy][cx + 1], l = s_raw[cy][cx - 1], d = s_raw[cy + 1][cx], u = s_raw[cy - 1][cx];
        if (usable_raw(rc, lo, hi) && usable_raw(r, lo, hi) && usable_raw(l, lo, hi) && usable_raw(d, lo, hi) &&
            usable_raw(u, lo, hi)) {
            const float gx = fabsf(fs(static_cast<float>(r), static_cast<float>(l)));
            const float gy = fabsf(fs(static_cast<float>(d), static_cast<float>(u)));
            const float g = fsq(fa(fm(gx, gx), fm(gy, gy)));
            const float gn = fd(g, 100.0f);
            edge = gn < 1.0f ? gn : 1.0f;
        }
    }
    const float ef = fs(1.0f, fm(edge, 0.5f));
    const float ldenom = fa(fm(fm(2.0f, 0.10f), 0.10f), 0.01f);
    const float* dwrow = dw_tab + static_cast<size_t>(rc) * kRawCodes;
    float sw = 0.0f, sd = 0.0f;
    for (int dy = -4; dy <= 4; ++dy) {
        for (int dx = -4; dx <= 4; ++dx) {
            const float nd = s_m[cy + dy][cx + dx];
            if (nd == 0.0f) continue;
            const uint16_t rn = s_raw[cy + dy][cx + dx];
            const float gdl = fs(s_l[cy + dy][cx + dx], cl);
            const float lw = (gdl == 0.0f) ? 1.0f : expf(fd(-fm(gdl, gdl), ldenom));
            const float w = fm(fm(fm(c_tab.guided_spatial[dx * dx + dy * dy], lw), __ldg(dwrow + rn)), ef);
            sw = fa(sw, w);
            sd = fa(sd, fm(w, nd));
        }
    }
    out[idx] = (sw > 1e-6f) ? m_to_raw(fd(sd, sw), lo, hi) : rc;
}

// applyDepthEma (:494-576) + band-gated metres of the result (buildFrameData).
__global__ void __launch_bounds__(256) ema_kernel(const uint16_t* __restrict__ src, uint16_t* __restrict__ out,
                                                  float* __restrict__ ema, float* __restrict__ depth_out, float lo,
                                                  float hi, int do_ema) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= PW || y >= PH) return;
    const int i = y * PW + x;
    uint16_t res = src[i];
    if (do_ema) {
        const float dm = depth_m(res, lo, hi);
        if (dm == 0.0f) {
            ema[i] = 0.0f;
        } else {
            const float prev = ema[i];
            const float delta = fabsf(fs(dm, prev));
            bool reset = isnan(prev) || isinf(prev) || prev <= 0.0f || delta > 0.05f;
            if (!reset && delta > fm(0.05f, 0.5f)) {
                float ns = 0.0f;
                int nc = 0;
                for (int dy = -1; dy <= 1; ++dy)
                    for (int dx = -1; dx <= 1; ++dx) {
                        if (dx == 0 && dy == 0) continue;
                        const float nd = depth_m(src[reflect(y + dy, PH) * PW + reflect(x + dx, PW)], lo, hi);
                        if (nd != 0.0f) { ns = fa(ns, nd); ++nc; }
                    }
                if (nc > 0) {
                    const float avg = fd(ns, static_cast<float>(nc));
                    if (fabsf(fs(dm, avg)) > 0.05f) reset = true;
                }
            }
            const float filt = reset ? dm : fa(fm(0.7f, dm), fm(0.3f, prev));
            const uint16_t enc = m_to_raw(filt, lo, hi);
            ema[i] = (enc != 0) ? filt : 0.0f;
            res = enc;
        }
    }
    out[i] = res;
    depth_out[i] = depth_m(res, lo, hi);
}

// mm input: depth_m = float(mm) * 0.001f, band-gated.
__global__ void mm_to_m_kernel(const uint16_t* __restrict__ mm, float* __restrict__ out, int n, float lo, float hi,
                               const int* __restrict__ gate) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float m = fm(static_cast<float>(mm[i]), 0.001f);
    out[i] = in_band(m, lo, hi) ? m : 0.0f;
}

}  // namespace azu

struct azu_preprocessor {
    int device = 0;
    int mode = AZU_PRE_FULL;
    azu::StreamRef stream;
    uint16_t* d_in = nullptr;   // raw input
    uint16_t* d_a = nullptr;    // stage ping
    uint16_t* d_b = nullptr;    // stage pong
    uint16_t* d_out = nullptr;  // processed raw codes
    uint8_t* d_rgb_in = nullptr;
    uint8_t* d_rgb_tmp = nullptr;
    uint8_t* d_rgb_out = nullptr;
    float* d_luma = nullptr;
    float* d_ema = nullptr;
    float* d_depth_m = nullptr;
    float* d_range_w = nullptr;  // 195076
    float* d_dw = nullptr;       // 2047 x 2047
    // The RGB chain runs on a side stream beside the depth median and hole
    // fill (they meet at the guided filter, which reads the luma).
    cudaStream_t s_rgb = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
};

namespace azu {

constexpr int kRangeN = 3 * 255 * 255 + 1;

static int build_tables(azu_preprocessor* p) {
    // Host-side weights: the same float arguments and libm calls as the CPU path.
    PreTables t;
    for (int d2 = 0; d2 < 9; ++d2) t.rgb_spatial[d2] = std::exp(-static_cast<float>(d2) / (2.0f * 2.0f * 2.0f));
    for (int d2 = 0; d2 < 33; ++d2) t.guided_spatial[d2] = std::exp(-static_cast<float>(d2) / (2.0f * 4 * 4));
    AZU_TRY_CUDA(cudaMemcpyToSymbol(c_tab, &t, sizeof(t)));
    std::vector<float> range(kRangeN);
    for (int c = 0; c < kRangeN; ++c) range[c] = std::exp(-static_cast<float>(c) / (2.0f * 28.0f * 28.0f));
    AZU_TRY_CUDA(cudaMemcpy(p->d_range_w, range.data(), range.size() * sizeof(float), cudaMemcpyHostToDevice));
    std::vector<float> m(kRawCodes);
    for (int r = 0; r < kRawCodes; ++r)
        m[r] = (r == 0) ? 0.0f : 1.0f / (static_cast<float>(r) * kCurveA + kCurveB);
    const float denom = 2.0f * 0.04f * 0.04f + 0.01f;
    std::vector<float> dw(static_cast<size_t>(kRawCodes) * kRawCodes);
    for (int a = 0; a < kRawCodes; ++a)
        for (int b = 0; b < kRawCodes; ++b) {
            const float dd = m[b] - m[a];
            dw[static_cast<size_t>(a) * kRawCodes + b] = std::exp(-(dd * dd) / denom);
        }
    AZU_TRY_CUDA(cudaMemcpy(p->d_dw, dw.data(), dw.size() * sizeof(float), cudaMemcpyHostToDevice));
    return AZU_OK;
}

// Enqueues the whole chain from p->d_in / p->d_rgb_in.
int preprocess_enqueue(azu_preprocessor* p, float lo, float hi, cudaStream_t s) {
    const dim3 b(32, 8), g(PW / 32, PH / 8);
    const bool full = p->mode == AZU_PRE_FULL;
    // processCpu runs the RGB chain in both modes (SignalConditioner_omp.cpp:337-341);
    // it runs on the side stream, beside the depth median and hole fill.
    AZU_TRY_CUDA(cudaEventRecord(p->ev_fork, s));
    AZU_TRY_CUDA(cudaStreamWaitEvent(p->s_rgb, p->ev_fork, 0));
    rgb_bilateral_kernel<<<g, b, 0, p->s_rgb>>>(p->d_rgb_in, p->d_rgb_tmp, p->d_range_w);
    rgb_median_kernel<<<g, b, 0, p->s_rgb>>>(p->d_rgb_tmp, p->d_rgb_out);
    cas_luma_kernel<<<g, b, 0, p->s_rgb>>>(p->d_rgb_out, p->d_luma);
    AZU_TRY_CUDA(cudaEventRecord(p->ev_join, p->s_rgb));
    depth_median_kernel<<<dim3(PW / kMTx, PH / kMTy), dim3(kMTx, kMTy), 0, s>>>(p->d_in, p->d_a, lo, hi);
    if (full) hole_fill_kernel<<<g, b, 0, s>>>(p->d_a, p->d_b, lo, hi);
    AZU_TRY_CUDA(cudaStreamWaitEvent(s, p->ev_join, 0));
    if (full) {
        guided_kernel<<<dim3(PW / kGTx, PH / kGTy), dim3(kGTx, kGTy), 0, s>>>(p->d_b, p->d_a, p->d_luma, p->d_dw,
                                                                           lo, hi);
    }
    ema_kernel<<<g, b, 0, s>>>(p->d_a, p->d_out, p->d_ema, p->d_depth_m, lo, hi, full ? 1 : 0);
    AZU_LAUNCH_CHECK();
    return AZU_OK;
}

int mm_to_meters_enqueue(const uint16_t* d_mm, float* d_out, int n, float lo, float hi, cudaStream_t s) {
    mm_to_m_kernel<<<(n + 255) / 256, 256, 0, s>>>(d_mm, d_out, n, lo, hi, nullptr);
    AZU_LAUNCH_CHECK();
    return AZU_OK;
}

uint16_t* preprocess_input(azu_preprocessor* p) { return p->d_in; }
uint8_t* preprocess_rgb_input(azu_preprocessor* p) { return p->d_rgb_in; }
float* preprocess_depth_m(azu_preprocessor* p) { return p->d_depth_m; }

}  // namespace azu

using namespace azu;

extern "C" int azu_preprocessor_create(int device, int mode, void* stream, azu_preprocessor** out) {
    AZU_CHECK_ARG(out != nullptr, "out is null");
    AZU_CHECK_ARG(mode == AZU_PRE_FULL || mode == AZU_PRE_MINIMAL, "mode");
    *out = nullptr;
    if (int rc = bind_device(device)) return rc;
    azu_preprocessor* p = new azu_preprocessor();
    p->device = device;
    p->mode = mode;
    int rc = p->stream.init(stream);
    const size_t n = static_cast<size_t>(PW) * PH;
    cudaError_t e = cudaSuccess;
    if (!rc) {
        e = cudaMalloc(&p->d_in, n * 2);
        if (!e) e = cudaMalloc(&p->d_a, n * 2);
        if (!e) e = cudaMalloc(&p->d_b, n * 2);
        if (!e) e = cudaMalloc(&p->d_out, n * 2);
        if (!e) e = cudaMalloc(&p->d_rgb_in, n * 3);
        if (!e) e = cudaMalloc(&p->d_rgb_tmp, n * 3);
        if (!e) e = cudaMalloc(&p->d_rgb_out, n * 3);
        if (!e) e = cudaMalloc(&p->d_luma, n * 4);
        if (!e) e = cudaMalloc(&p->d_ema, n * 4);
        if (!e) e = cudaMalloc(&p->d_depth_m, n * 4);
        if (!e) e = cudaMalloc(&p->d_range_w, kRangeN * sizeof(float));
        if (!e) e = cudaMalloc(&p->d_dw, sizeof(float) * kRawCodes * kRawCodes);
        if (!e) e = cudaStreamCreateWithFlags(&p->s_rgb, cudaStreamNonBlocking);
        if (!e) e = cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming);
        if (!e) e = cudaEventCreateWithFlags(&p->ev_join, cudaEventDisableTiming);
        if (e) { set_error("preprocessor allocation: %s", cudaGetErrorString(e)); rc = AZU_E_NOMEM; }
    }
    if (!rc) rc = build_tables(p);
    if (!rc) rc = azu_preprocessor_reset(p);
    if (rc) { azu_preprocessor_destroy(p); return rc; }
    *out = p;
    return AZU_OK;
}

extern "C" int azu_preprocessor_destroy(azu_preprocessor* p) {
    if (!p) return AZU_OK;
    cudaSetDevice(p->device);
    if (p->stream.s) cudaStreamSynchronize(p->stream.s);
    if (p->s_rgb) {
        cudaStreamSynchronize(p->s_rgb);
        cudaStreamDestroy(p->s_rgb);
    }
    if (p->ev_fork) cudaEventDestroy(p->ev_fork);
    if (p->ev_join) cudaEventDestroy(p->ev_join);
    for (void* q : {(void*)p->d_in, (void*)p->d_a, (void*)p->d_b, (void*)p->d_out, (void*)p->d_rgb_in,
                    (void*)p->d_rgb_tmp, (void*)p->d_rgb_out, (void*)p->d_luma, (void*)p->d_ema, (void*)p->d_depth_m,
                    (void*)p->d_range_w, (void*)p->d_dw})
        if (q) cudaFree(q);
    p->stream.release();
    delete p;
    return AZU_OK;
}

extern "C" int azu_preprocessor_reset(azu_preprocessor* p) {
    AZU_CHECK_ARG(p != nullptr, "null handle");
    AZU_TRY_CUDA(cudaSetDevice(p->device));
    const size_t n = static_cast<size_t>(PW) * PH;
    AZU_TRY_CUDA(cudaMemsetAsync(p->d_ema, 0, n * 4, p->stream.s));
    AZU_TRY_CUDA(cudaMemsetAsync(p->d_luma, 0, n * 4, p->stream.s));
    AZU_TRY_CUDA(cudaMemsetAsync(p->d_out, 0, n * 2, p->stream.s));
    AZU_TRY_CUDA(cudaMemsetAsync(p->d_depth_m, 0, n * 4, p->stream.s));
    AZU_TRY_CUDA(cudaMemsetAsync(p->d_rgb_out, 0, n * 3, p->stream.s));
    return AZU_OK;
}

extern "C" int azu_preprocessor_reset_temporal(azu_preprocessor* p) {
    AZU_CHECK_ARG(p != nullptr, "null handle");
    AZU_TRY_CUDA(cudaSetDevice(p->device));
    AZU_TRY_CUDA(cudaMemsetAsync(p->d_ema, 0, static_cast<size_t>(PW) * PH * 4, p->stream.s));
    return AZU_OK;
}

extern "C" int azu_preprocessor_process_device(azu_preprocessor* p, const uint16_t* d_depth, const uint8_t* d_rgb,
                                               float min_depth, float max_depth) {
    AZU_CHECK_ARG(p != nullptr && d_depth != nullptr && d_rgb != nullptr, "null argument");
    AZU_TRY_CUDA(cudaSetDevice(p->device));
    const size_t n = static_cast<size_t>(PW) * PH;
    if (d_depth != p->d_in)
        AZU_TRY_CUDA(cudaMemcpyAsync(p->d_in, d_depth, n * 2, cudaMemcpyDeviceToDevice, p->stream.s));
    if (d_rgb != p->d_rgb_in)
        AZU_TRY_CUDA(cudaMemcpyAsync(p->d_rgb_in, d_rgb, n * 3, cudaMemcpyDeviceToDevice, p->stream.s));
    return preprocess_enqueue(p, min_depth, max_depth, p->stream.s);
}

extern "C" int azu_preprocessor_process(azu_preprocessor* p, uint16_t* h_depth, uint8_t* h_rgb, float min_depth,
                                        float max_depth) {
    AZU_CHECK_ARG(p != nullptr && h_depth != nullptr && h_rgb != nullptr, "null argument");
    AZU_TRY_CUDA(cudaSetDevice(p->device));
    const size_t n = static_cast<size_t>(PW) * PH;
    AZU_TRY_CUDA(cudaMemcpyAsync(p->d_in, h_depth, n * 2, cudaMemcpyHostToDevice, p->stream.s));
    AZU_TRY_CUDA(cudaMemcpyAsync(p->d_rgb_in, h_rgb, n * 3, cudaMemcpyHostToDevice, p->stream.s));
    if (int rc = preprocess_enqueue(p, min_depth, max_depth, p->stream.s)) return rc;
    AZU_TRY_CUDA(cudaMemcpyAsync(h_depth, p->d_out, n * 2, cudaMemcpyDeviceToHost, p->stream.s));
    AZU_TRY_CUDA(cudaMemcpyAsync(h_rgb, p->d_rgb_out, n * 3, cudaMemcpyDeviceToHost, p->stream.s));
    AZU_TRY_CUDA(cudaStreamSynchronize(p->stream.s));
    return AZU_OK;
}

extern "C" float* azu_preprocessor_depth_meters(azu_preprocessor* p) { return p ? p->d_depth_m : nullptr; }
extern "C" uint8_t* azu_preprocessor_rgb(azu_preprocessor* p) { return p ? p->d_rgb_out : nullptr; }
extern "C" uint16_t* azu_preprocessor_depth_raw(azu_preprocessor* p) { return p ? p->d_out : nullptr; }
extern "C" float* azu_preprocessor_luma(azu_preprocessor* p) { return p ? p->d_luma : nullptr; }
