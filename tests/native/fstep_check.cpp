// Host check of azu_gb300/csrc/fstep.cuh: the closed-form running sum equals
// the sequential chain of rounded float additions bit for bit. Prints the
// number of mismatches and the number of values compared.
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>

#include "../../azu_gb300/csrc/fstep.cuh"

using azu::fs_add;
using azu::fs_bits;
using azu::fs_float;
using azu::fs_segment;
using azu::fs_walk;

static long long g_bad = 0, g_checked = 0;

static void check_chain(float v0, float s, int N, std::mt19937_64& rng) {
    std::vector<float> c(N + 1);
    c[0] = v0;
    for (int k = 1; k <= N; ++k) c[k] = fs_add(c[k - 1], s);
    // walks from random anchors, random lengths
    std::uniform_int_distribution<int> pick(0, N);
    for (int t = 0; t < 24; ++t) {
        int a = pick(rng), b = pick(rng);
        if (a > b) std::swap(a, b);
        const float w = fs_walk(c[a], s, b - a);
        ++g_checked;
        if (fs_bits(w) != fs_bits(c[b])) {
            if (g_bad < 10)
                std::printf("walk mismatch v=%a s=%a a=%d n=%d got %a want %a\n", c[a], s, a, b - a, w, c[b]);
            ++g_bad;
        }
    }
    // every segment along the chain, checked value by value
    for (int a = 0; a < N;) {
        const azu::FSeg g = fs_segment(c[a], s);
        const int m = g.m == azu::kFsForever ? N - a : (g.m < N - a ? g.m : N - a);
        for (int j = 0; j <= m; ++j) {
            const float f = azu::fs_fma(static_cast<float>(j), g.d, c[a]);
            ++g_checked;
            if (fs_bits(f) != fs_bits(c[a + j])) {
                if (g_bad < 10)
                    std::printf("segment mismatch v=%a s=%a j=%d m=%d d=%a got %a want %a\n", c[a], s, j, g.m, g.d,
                                f, c[a + j]);
                ++g_bad;
                break;
            }
        }
        a += m > 0 ? m : 1;
    }
}

int main(int argc, char** argv) {
    const int cases = argc > 1 ? std::atoi(argv[1]) : 20000;
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<float> uni(-1.0f, 1.0f);
    std::uniform_int_distribution<int> len(1, 700);
    std::uniform_int_distribution<uint32_t> bits(0, 0xffffffffu);
    for (int i = 0; i < cases; ++i) {
        const int kind = i % 8;
        float v0, s;
        int N = len(rng);
        switch (kind) {
            case 0:  // camera coordinates of a voxel row: metres, steps of a few mm
                v0 = 3.0f * uni(rng);
                s = 0.004f * uni(rng);
                break;
            case 1: {  // rows that cross zero
                s = 0.0039f * uni(rng);
                v0 = -s * static_cast<float>(N) * (0.2f + 0.6f * std::fabs(uni(rng)));
                break;
            }
            case 2: {  // steps with few mantissa bits: rounding ties in nearby binades
                const int e = -12 + static_cast<int>(std::fabs(uni(rng)) * 6.0f);
                const uint32_t mant = bits(rng) & 0x7fe000u;  // low 13 bits zero
                s = fs_float((static_cast<uint32_t>(127 + e) << 23) | mant) * (uni(rng) < 0 ? -1.0f : 1.0f);
                v0 = 4.0f * uni(rng);
                break;
            }
            case 3: {  // exact ties: s = (k + 1/2) ulp of the start's binade
                v0 = 0.5f + std::fabs(uni(rng)) * 1.4f;
                const float u = fs_float(fs_bits(v0) & 0x7f800000u) * 0x1p-23f;
                const int k = static_cast<int>(std::fabs(uni(rng)) * 4000.0f);
                s = (static_cast<float>(k) + 0.5f) * u * (uni(rng) < 0 ? -1.0f : 1.0f);
                break;
            }
            case 4:  // powers of two (axis-aligned rotations, identity pose)
                s = std::ldexp(1.0f, -8 - static_cast<int>(std::fabs(uni(rng)) * 8.0f)) * (uni(rng) < 0 ? -1.f : 1.f);
                v0 = std::ldexp(std::floor(uni(rng) * 4096.0f), -10);
                break;
            case 5:  // steps below half an ulp (sum never moves) and tiny steps
                v0 = 2.0f * uni(rng);
                s = std::ldexp(uni(rng), -30 - static_cast<int>(std::fabs(uni(rng)) * 100.0f));
                break;
            case 6:  // zero start, zero step, subnormal step
                v0 = (i & 16) ? 0.0f : -0.0f;
                s = (i & 32) ? 0.0f : std::ldexp(uni(rng), -140);
                if (i & 64) s = 0.003f * uni(rng);
                break;
            default: {  // random bit patterns of moderate magnitude
                v0 = fs_float((bits(rng) & 0x807fffffu) | (static_cast<uint32_t>(110 + (bits(rng) % 30)) << 23));
                s = fs_float((bits(rng) & 0x807fffffu) | (static_cast<uint32_t>(100 + (bits(rng) % 25)) << 23));
                break;
            }
        }
        check_chain(v0, s, N, rng);
    }
    std::printf("%lld %lld\n", g_bad, g_checked);
    return g_bad ? 1 : 0;
}
