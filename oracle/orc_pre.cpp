// Oracle (test infrastructure only): CPU restatement of the reference's depth
// preprocessor on a 640x480 RawFrame (src/sensor/SignalConditioner_omp.cpp:
// 120-715, CAS from src/sensor/SuperResolution.cpp:26-35,118-166).
#include "orc_api.h"
#include "orc_math.h"

#include <vector>

using namespace orc;

namespace {

constexpr int FW = 640, FH = 480;
constexpr int kHoleFillRadius = 2;        // SignalConditioner_omp.cpp:30
constexpr int kGuidedRadius = 4;          // :33
constexpr int kRgbBilateralRadius = 2;    // :34
constexpr int kDepthMedianRadius = 1;     // :35
constexpr float kEmaJumpResetMeters = 0.05f;  // :41
constexpr float kGuidedSigmaLuma = 0.10f;     // :42
constexpr float kGuidedSigmaDepth = 0.04f;    // :43
constexpr float kRgbSigmaSpatial = 2.0f;      // :44
constexpr float kRgbSigmaRange = 28.0f;       // :45

inline uint8_t clampToByte(float v) { return static_cast<uint8_t>(std::min(std::max(v, 0.0f), 255.0f)); }

// computeDepthGradient (:120-141).
float depthGradient(const uint16_t* depth, int x, int y, float lo, float hi) {
    if (x <= 0 || x >= FW - 1 || y <= 0 || y >= FH - 1) return 1.0f;
    const uint16_t c = depth[y * FW + x], r = depth[y * FW + x + 1], l = depth[y * FW + x - 1],
                   d = depth[(y + 1) * FW + x], u = depth[(y - 1) * FW + x];
    if (!usableRaw(c, lo, hi) || !usableRaw(r, lo, hi) || !usableRaw(l, lo, hi) || !usableRaw(d, lo, hi) ||
        !usableRaw(u, lo, hi))
        return 1.0f;
    const float gx = std::fabs(static_cast<float>(r) - static_cast<float>(l));
    const float gy = std::fabs(static_cast<float>(d) - static_cast<float>(u));
    const float g = std::sqrt(gx * gx + gy * gy);
    return std::min(g / 100.0f, 1.0f);
}

inline float rgbLuma(const uint8_t* p) {
    return 0.299f * static_cast<float>(p[0]) + 0.587f * static_cast<float>(p[1]) + 0.114f * static_cast<float>(p[2]);
}

// Median of 9 by sorting (std::nth_element of the reference picks the same value).
template <typename T>
T nth(T* w, int n, int k) {
    std::nth_element(w, w + k, w + n);
    return w[k];
}

// bilateralDenoiseRgb (:185-230).
void bilateralRgb(const uint8_t* src, uint8_t* dst) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < FH; ++y) {
        for (int x = 0; x < FW; ++x) {
            const int ci = (y * FW + x) * 3;
            const float crgb[3] = {float(src[ci]), float(src[ci + 1]), float(src[ci + 2])};
            float acc[3] = {0, 0, 0}, ws = 0.0f;
            for (int dy = -kRgbBilateralRadius; dy <= kRgbBilateralRadius; ++dy) {
                const int sy = reflect(y + dy, FH);
                for (int dx = -kRgbBilateralRadius; dx <= kRgbBilateralRadius; ++dx) {
                    const int sx = reflect(x + dx, FW);
                    const int si = (sy * FW + sx) * 3;
                    const float sd2 = static_cast<float>(dx * dx + dy * dy);
                    float cd2 = 0.0f;
                    for (int c = 0; c < 3; ++c) {
                        const float dl = static_cast<float>(src[si + c]) - crgb[c];
                        cd2 += dl * dl;
                    }
                    const float sw = std::exp(-sd2 / (2.0f * kRgbSigmaSpatial * kRgbSigmaSpatial));
                    const float rw = std::exp(-cd2 / (2.0f * kRgbSigmaRange * kRgbSigmaRange));
                    const float w = sw * rw;
                    for (int c = 0; c < 3; ++c) acc[c] += w * static_cast<float>(src[si + c]);
                    ws += w;
                }
            }
            for (int c = 0; c < 3; ++c) dst[ci + c] = (ws > 1e-6f) ? clampToByte(acc[c] / ws) : src[ci + c];
        }
    }
}

// medianBlur3x3 (:160-183).
void median3Rgb(const uint8_t* src, uint8_t* dst) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < FH; ++y)
        for (int x = 0; x < FW; ++x)
            for (int c = 0; c < 3; ++c) {
                uint8_t w[9];
                int n = 0;
                for (int dy = -1; dy <= 1; ++dy) {
                    const int sy = reflect(y + dy, FH);
                    for (int dx = -1; dx <= 1; ++dx) w[n++] = src[(sy * FW + reflect(x + dx, FW)) * 3 + c];
                }
                dst[(y * FW + x) * 3 + c] = nth(w, 9, 4);
            }
}

// sr::applyCAS_CPU with sharpness 0.5 (SuperResolution.cpp:118-166).
void casRgb(const uint8_t* src, uint8_t* dst) {
    const float t = 0.5f;
    const float peak = -1.0f / ((1.0f - t) * 8.0f + t * 5.0f);
    auto px = [&](int x, int y, float out[3]) {
        x = reflect(x, FW);
        y = reflect(y, FH);
        const int i = (y * FW + x) * 3;
        out[0] = src[i] / 255.0f; out[1] = src[i + 1] / 255.0f; out[2] = src[i + 2] / 255.0f;
    };
#pragma omp parallel for schedule(static)
    for (int y = 0; y < FH; ++y)
        for (int x = 0; x < FW; ++x) {
            float a[3], b[3], c[3], d[3], e[3];
            px(x, y - 1, a); px(x - 1, y, b); px(x, y, c); px(x + 1, y, d); px(x, y + 1, e);
            float amp = 1.0f;
            for (int ch = 0; ch < 3; ++ch) {
                const float mn = std::min({a[ch], b[ch], c[ch], d[ch], e[ch]});
                const float mx = std::max({a[ch], b[ch], c[ch], d[ch], e[ch]});
                const float mxs = std::max(mx, 1e-6f);
                const float ac = std::min(mn, 1.0f - mx) / mxs;
                amp = std::min(amp, ac);
            }
            const float w = amp * peak;
            const float wsum = 1.0f + 4.0f * w;
            for (int ch = 0; ch < 3; ++ch) {
                const float v = (c[ch] + w * (a[ch] + b[ch] + d[ch] + e[ch])) / wsum;
                dst[(y * FW + x) * 3 + ch] = static_cast<uint8_t>(std::min(std::max(v, 0.0f), 1.0f) * 255.0f);
            }
        }
}

}  // namespace

// preprocessRgb + buildSuperResolutionGuidance (:351-386): rgb is replaced by
// bilateral -> median; the guidance luma comes from CAS of that.
extern "C" void orc_pre_rgb(uint8_t* rgb, float* luma_out) {
    std::vector<uint8_t> a(FW * FH * 3), b(FW * FH * 3);
    bilateralRgb(rgb, a.data());
    median3Rgb(a.data(), rgb);
    casRgb(rgb, b.data());
    if (luma_out)
        for (int i = 0; i < FW * FH; ++i) luma_out[i] = rgbLuma(&b[i * 3]) / 255.0f;
}

// denoiseDepthSpatial (:442-482).
extern "C" void orc_pre_depth_median(uint16_t* depth, float lo, float hi) {
    std::vector<uint16_t> out(depth, depth + FW * FH);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < FH; ++y)
        for (int x = 0; x < FW; ++x) {
            const int idx = y * FW + x;
            if (cpuDepthMeters(depth[idx], lo, hi) == 0.0f) continue;
            float w[9];
            int n = 0;
            for (int dy = -kDepthMedianRadius; dy <= kDepthMedianRadius; ++dy) {
                const int sy = reflect(y + dy, FH);
                for (int dx = -kDepthMedianRadius; dx <= kDepthMedianRadius; ++dx) {
                    const float s = cpuDepthMeters(depth[sy * FW + reflect(x + dx, FW)], lo, hi);
                    if (s == 0.0f) continue;
                    w[n++] = s;
                }
            }
            if (n >= 3) out[idx] = metersToRaw(nth(w, n, n / 2), lo, hi);
        }
    std::copy(out.begin(), out.end(), depth);
}

// fillDepthHoles (:578-635).
extern "C" void orc_pre_fill_holes(uint16_t* depth, float lo, float hi) {
    std::vector<uint16_t> out(depth, depth + FW * FH);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < FH; ++y)
        for (int x = 0; x < FW; ++x) {
            const int idx = y * FW + x;
            if (depth[idx] != 0) continue;
            float wsum_d = 0.0f, wsum = 0.0f;
            int nv = 0;
            for (int dy = -kHoleFillRadius; dy <= kHoleFillRadius; ++dy) {
                const int sy = reflect(y + dy, FH);
                for (int dx = -kHoleFillRadius; dx <= kHoleFillRadius; ++dx) {
                    if (dx == 0 && dy == 0) continue;
                    const float cm = cpuDepthMeters(depth[sy * FW + reflect(x + dx, FW)], lo, hi);
                    if (cm == 0.0f) continue;
                    const int d2 = dx * dx + dy * dy;
                    const float w = 1.0f / (d2 + 1.0f);
                    wsum_d += w * cm;
                    wsum += w;
                    ++nv;
                }
            }
            if (nv > 0 && wsum > 1e-6f) out[idx] = metersToRaw(wsum_d / wsum, lo, hi);
        }
    std::copy(out.begin(), out.end(), depth);
}

// guidedDepthFilter (:637-715).
extern "C" void orc_pre_guided(uint16_t* depth, const float* luma, float lo, float hi) {
    std::vector<uint16_t> out(FW * FH);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < FH; ++y)
        for (int x = 0; x < FW; ++x) {
            const int idx = y * FW + x;
            const float cd = cpuDepthMeters(depth[idx], lo, hi);
            if (cd == 0.0f) { out[idx] = depth[idx]; continue; }
            const float cl = luma[idx];
            const float edge = depthGradient(depth, x, y, lo, hi);
            float sw = 0.0f, sd = 0.0f;
            for (int dy = -kGuidedRadius; dy <= kGuidedRadius; ++dy) {
                const int sy = reflect(y + dy, FH);
                for (int dx = -kGuidedRadius; dx <= kGuidedRadius; ++dx) {
                    const int sx = reflect(x + dx, FW);
                    const int ni = sy * FW + sx;
                    const float nd = cpuDepthMeters(depth[ni], lo, hi);
                    if (nd == 0.0f) continue;
                    const float sd2 = static_cast<float>(dx * dx + dy * dy);
                    const float gdl = luma[ni] - cl;
                    const float ddl = (cd > 0.0f) ? (nd - cd) : 0.0f;
                    const float spw = std::exp(-sd2 / (2.0f * kGuidedRadius * kGuidedRadius));
                    const float lw = std::exp(-(gdl * gdl) / (2.0f * kGuidedSigmaLuma * kGuidedSigmaLuma + 0.01f));
                    const float dw = std::exp(-(ddl * ddl) / (2.0f * kGuidedSigmaDepth * kGuidedSigmaDepth + 0.01f));
                    const float ef = 1.0f - edge * 0.5f;
                    const float w = spw * lw * dw * ef;
                    sw += w;
                    sd += w * nd;
                }
            }
            out[idx] = (sw > 1e-6f) ? metersToRaw(sd / sw, lo, hi) : depth[idx];
        }
    std::copy(out.begin(), out.end(), depth);
}

// applyDepthEma (:494-576).
extern "C" void orc_pre_ema(uint16_t* depth, float* ema, float lo, float hi) {
    std::vector<uint16_t> src(depth, depth + FW * FH);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < FW * FH; ++i) {
        const float dm = cpuDepthMeters(src[i], lo, hi);
        if (dm == 0.0f) { ema[i] = 0.0f; continue; }
        const float prev = ema[i];
        const float delta = std::fabs(dm - prev);
        bool reset = std::isnan(prev) || std::isinf(prev) || prev <= 0.0f || delta > kEmaJumpResetMeters;
        if (!reset && delta > kEmaJumpResetMeters * 0.5f) {
            const int x = i % FW, y = i / FW;
            float ns = 0.0f;
            int nc = 0;
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    if (dx == 0 && dy == 0) continue;
                    const float nd = cpuDepthMeters(src[reflect(y + dy, FH) * FW + reflect(x + dx, FW)], lo, hi);
                    if (nd != 0.0f) { ns += nd; ++nc; }
                }
            if (nc > 0) {
                const float avg = ns / nc;
                if (std::fabs(dm - avg) > kEmaJumpResetMeters) reset = true;
            }
        }
        const float filt = reset ? dm : (0.7f * dm + 0.3f * prev);
        const uint16_t enc = metersToRaw(filt, lo, hi);
        ema[i] = (enc != 0) ? filt : 0.0f;
        depth[i] = enc;
    }
}

// SignalConditioner::processCpu (:337-349).
extern "C" void orc_preprocess(uint16_t* depth, uint8_t* rgb, float* ema, float* luma_out, float lo, float hi,
                               int minimal) {
    std::vector<float> luma(FW * FH);
    orc_pre_rgb(rgb, luma.data());
    if (luma_out) std::copy(luma.begin(), luma.end(), luma_out);
    orc_pre_depth_median(depth, lo, hi);
    if (!minimal) {
        orc_pre_fill_holes(depth, lo, hi);
        orc_pre_guided(depth, luma.data(), lo, hi);
        orc_pre_ema(depth, ema, lo, hi);
    }
}
