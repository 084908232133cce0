// Coarse-to-fine point-to-plane ICP in one persistent kernel, behind the
// azu_tracker_* C ABI. Semantics: src/tracking/ICPTracker.cpp:40-354 and the
// numeric policy of include/tracking/ICPShared.h:34-110.
//
// One cooperative launch runs every level and iteration:
//   1. each block accumulates the 21 + 6 normal-equation terms, the Huber loss
//      and 6 counters over a slice of the level's interior pixels (projective
//      association into the model image, one thread per pixel);
//   2. warp shuffles (recursive halving), then shared memory, reduce them to
//      one block partial, written to global memory value-major;
//   3. the block that arrives last at the split barrier reduces all block
//      partials in one fixed order, solves the damped 6x6 system and publishes
//      the outcome; the others wait (bounded spin; a timeout sets an error
//      word) and read it.
// Partials are double-buffered by iteration parity. The precision form
// (precision = 1) keeps the per-pixel terms in FP32 with compensated block
// sums and uses FP64 only for the cross-block sum, the Cholesky solve, the
// SE(3) exponential, the pose composition and the rotation projection.
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#include <mutex>

#include "azu_internal.h"
#include "kf_math.cuh"
#include "reduce.cuh"

namespace azu {

int launch_prepare_live(const float* d_depth, int W, int H, float fx, float fy, float cx, float cy, float* const V[3],
                        float* const N[3], float* const D[3], cudaStream_t s);

constexpr int kNF = 28;   // 21 A + 6 b + residual
constexpr int kNI = 6;    // inliers, valid_live, valid_model, projected, dist_filtered, angle_filtered
constexpr int kIcpThreads = 512;
constexpr unsigned kSpinLimit = 1u << 22;

constexpr float kHuberK = 0.02f;
constexpr float kDampingDefault = 0.1f, kDampingLevel0 = 0.01f, kDampingEscalated = 1.0f;
constexpr float kCondEscalate = 1e7f, kMinEigEscalate = 1e-4f;
constexpr float kTranslationCapStep = 0.2f, kRotationCapStep = 0.5f;
constexpr float kConvergenceStep = 5e-5f, kAcceptableFinalStep = 1e-3f;
constexpr int kMinInliersForIteration = 10, kMinInliersForOk = 100;

struct IcpLevel {
    const float* v;
    const float* n;
    int W, H;
};

struct IcpArgs {
    IcpLevel lv[3];
    const float* mv;
    const float* mn;
    int MW, MH;
    float fx, fy, cx, cy;  // camera intrinsics scaled to the model size
    float dist2, angle_cos;
    int iters[3];
    int precision;
    int build_level;  // >= 0: one association pass at this level, no solve
    const float* d_estimate;
    const float* d_ref;
    const float* d_prev;  // non-null: grade, retry from prev on Failed (pipeline)
    float* d_pose_out;    // non-null: final pose (pipeline: current pose, updated unless Failed)
    azu_icp_result* d_result;
    int* d_quality;
    int* d_gate;          // set to 1 when the frame grades Good
    double* partials;     // [2][kNF][vblocks]: double in the precision form, else float
    int* ipartials;       // [2][kNI][vblocks]
    int vblocks;          // partial slots: the pixel split and summation order (>= the launch's blocks)
    unsigned* bar;        // [0] arrivals, [1] generation
    unsigned* err;
    float* build_out;     // build mode: A[36], b[6], residual, counts[6] (as int bits)
};

// ---------------------------------------------------------------------------
// Grid barrier with a bounded spin. Co-residency comes from the cooperative
// launch. After a timeout the error word is set and every later barrier
// returns at once, so the kernel always finishes.
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// The wait limits of every barrier: the spin limit and the arrival count that
// releases a barrier (the group's block count). A testing hook may lower the
// limit and raise the count by extra arrivals that never come, so that a wait
// runs out by design; the kernel then finishes with the error word set.
__device__ unsigned g_icp_spin_limit = kSpinLimit;
__device__ unsigned g_icp_extra_arrivals = 0;

struct WaitLimits {
    unsigned spins;     // iterations before a wait gives up
    unsigned arrivals;  // arrivals that complete a barrier
};

// The arrival count (bar[0]) and the generation (bar[1]) are the two halves of
// one 64-bit word (little-endian), so the last arrival resets the count and
// advances the generation in a single atomic: adding 2^32 - arrivals takes the
// count from `arrivals` to 0 with a carry into the generation. An arrival
// releases the block's earlier stores and acquires the earlier arrivals' (the
// last block reads every partial); waiters acquire the generation, which the
// release sequence of every arrival on this word carries.
__device__ __forceinline__ unsigned long long atom_add_acq_rel(unsigned long long* p, unsigned long long v) {
    unsigned long long old;
    asm volatile("atom.add.acq_rel.gpu.global.u64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
    return old;
}

__device__ void grid_sync(unsigned* bar, unsigned* err, WaitLimits wl, unsigned& gen) {
    __syncthreads();
    if (threadIdx.x == 0) {
        if (ld_acquire(err) == 0) {
            unsigned long long* word = reinterpret_cast<unsigned long long*>(bar);
            const unsigned long long old = atom_add_acq_rel(word, 1ull);
            if (static_cast<unsigned>(old) == wl.arrivals - 1) {
                atom_add_acq_rel(word, (1ull << 32) - wl.arrivals);
            } else {
                unsigned spins = 0;
                while (ld_acquire(&bar[1]) == gen) {
                    if (++spins > wl.spins) {
                        atomicExch(err, kDevErrBarrierTimeout);
                        break;
                    }
                    __nanosleep(32);
                }
            }
        }
        gen += 1;
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Per-pixel association (ICPTracker.cpp:236-328).
struct Rel {
    float Rcw[9], Rrel[9];
    F3 tcw, trel;
};

struct Acc {
    float f[kNF];
    int i[kNI];
};

__device__ __forceinline__ bool normal_valid(F3 n) { return finite3(n) && sqnorm3(n) > 0.9f; }

__device__ __forceinline__ F3 ld3(const float* p, int i) {
    return mk3(__ldg(p + 3 * i), __ldg(p + 3 * i + 1), __ldg(p + 3 * i + 2));
}

// First half: live point into the model image. Returns the model pixel or -1.
__device__ __forceinline__ int associate_project(const IcpArgs& a, const Rel& r, F3 lv, Acc& acc) {
    if (lv.z <= 0.001f || !finite3(lv)) return -1;
    const F3 vr = add3(mv3(r.Rrel, lv), r.trel);
    if (vr.z <= 0.001f) return -1;
    acc.i[1]++;
    const float inv_z = fd(1.0f, vr.z);
    const float mxf = fa(fm(fm(a.fx, vr.x), inv_z), a.cx);
    const float myf = fa(fm(fm(a.fy, vr.y), inv_z), a.cy);
    int mx, my;
    if (!floor_to_int(fa(mxf, 0.5f), &mx) || !floor_to_int(fa(myf, 0.5f), &my)) return -1;
    if (mx < 0 || mx >= a.MW || my < 0 || my >= a.MH) return -1;
    acc.i[3]++;
    return my * a.MW + mx;
}

// Second half: filters and the normal-equation terms of one association.
__device__ __forceinline__ void associate_finish(const IcpArgs& a, const Rel& r, F3 lv, F3 ln, F3 mv, F3 mn,
                                                 Acc& acc) {
    if (!(finite3(mv) && sqnorm3(mv) > 1e-12f) || !normal_valid(mn)) return;
    acc.i[2]++;
    const F3 vw = add3(mv3(r.Rcw, lv), r.tcw);
    const F3 dvm = sub3(vw, mv);
    if (sqnorm3(dvm) > a.dist2) { acc.i[4]++; return; }
    if (!normal_valid(ln)) return;
    const F3 nw = mv3(r.Rcw, ln);
    if (fabsf(dot3(nw, mn)) < a.angle_cos) { acc.i[5]++; return; }
    const float err = dot3(mn, dvm);
    if (!isfinite(err)) return;
    const F3 nc = mtv3(r.Rcw, mn);
    const F3 cr = cross3(lv, nc);
    const float J[6] = {nc.x, nc.y, nc.z, cr.x, cr.y, cr.z};
    if (!(isfinite(J[0]) && isfinite(J[1]) && isfinite(J[2]) && isfinite(J[3]) && isfinite(J[4]) && isfinite(J[5])))
        return;
    const float ae = fabsf(err);
    const float w = (ae <= kHuberK) ? 1.0f : fd(kHuberK, ae);
    const float we = fm(err, w);
    int k = 0;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
#pragma unroll
        for (int j = i; j < 6; ++j) {
            acc.f[k] = fa(acc.f[k], fm(fm(w, J[i]), J[j]));
            ++k;
        }
        acc.f[21 + i] = fs(acc.f[21 + i], fm(J[i], we));
    }
    const float loss = (ae <= kHuberK) ? fm(ae, ae) : fs(fm(fm(2.0f, kHuberK), ae), fm(kHuberK, kHuberK));
    acc.f[27] = fa(acc.f[27], loss);
    acc.i[0]++;
}

// The interior pixels p = first, first + stride, ... of a level, two at a
// time so that the loads of both are in flight together. Accumulation order
// is the pixel order.
__device__ __forceinline__ void associate_range(const IcpArgs& a, const Rel& r, const IcpLevel& L, int first,
                                                int stride, int n, Acc& acc) {
    const int iw = L.W - 2;
    const F3 zero = mk3(0.0f, 0.0f, 0.0f);
    for (int p0 = first; p0 < n; p0 += 2 * stride) {
        const int p1 = p0 + stride;
        const bool has1 = p1 < n;
        const int i0 = (1 + p0 / iw) * L.W + 1 + p0 % iw;
        const int i1 = has1 ? (1 + p1 / iw) * L.W + 1 + p1 % iw : i0;
        const F3 lv0 = ld3(L.v, i0), ln0 = ld3(L.n, i0);
        const F3 lv1 = has1 ? ld3(L.v, i1) : zero, ln1 = has1 ? ld3(L.n, i1) : zero;
        const int m0 = associate_project(a, r, lv0, acc);
        const int m1 = has1 ? associate_project(a, r, lv1, acc) : -1;
        const F3 mv0 = m0 >= 0 ? ld3(a.mv, m0) : zero, mn0 = m0 >= 0 ? ld3(a.mn, m0) : zero;
        const F3 mv1 = m1 >= 0 ? ld3(a.mv, m1) : zero, mn1 = m1 >= 0 ? ld3(a.mn, m1) : zero;
        if (m0 >= 0) associate_finish(a, r, lv0, ln0, mv0, mn0, acc);
        if (m1 >= 0) associate_finish(a, r, lv1, ln1, mv1, mn1, acc);
    }
}


// Block reduction of one pass into global partial slot `slot` (FP32 path; no
// FP64 instruction — GB300's FP64 rate is a small fraction of its FP32 rate).
// The six counters travel as T: every per-block count is below 2^24, so exact.
// Partials are stored value-major, [slot][value][block], so the grid reduction
// reads them coalesced; the partial buffers and the shared staging are sized
// for double and reinterpreted for float.
// FP32 values take half of the staging, so consecutive slots alternate halves
// (buf) and the block needs no barrier after the partial stores: a half is
// written again two slots later, after the next slot's barrier, which every
// thread reaches only when its reads of this slot are done.
template <typename T>
__device__ __forceinline__ void reduce_block_t(const IcpArgs& a, const Acc& acc, int slot, int vb, double* s_red_raw,
                                               int buf) {
    static_assert(sizeof(T) == 4, "two staging halves hold FP32 values only");
    constexpr int kNV = kNF + kNI;  // 34
    T* s_red = reinterpret_cast<T*>(s_red_raw) + buf * (kIcpThreads / 32) * kNV;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    T v[32];
#pragma unroll
    for (int k = 0; k < kNF; ++k) v[k] = static_cast<T>(acc.f[k]);
#pragma unroll
    for (int k = kNF; k < 32; ++k) v[k] = static_cast<T>(acc.i[k - kNF]);
    const T e0 = warp_sum(static_cast<T>(acc.i[32 - kNF]));
    const T e1 = warp_sum(static_cast<T>(acc.i[33 - kNF]));
    const T mine = warp_sum_transpose32(v, lane);
    s_red[warp * kNV + lane] = mine;
    if (lane == 0) {
        s_red[warp * kNV + 32] = e0;
        s_red[warp * kNV + 33] = e1;
    }
    __syncthreads();
    const int k = threadIdx.x, nb = a.vblocks;
    if (k < kNF) {
        T sum = T(0);
        for (int w = 0; w < nw; ++w) sum += s_red[w * kNV + k];
        reinterpret_cast<T*>(a.partials)[(static_cast<size_t>(slot) * kNF + k) * nb + vb] = sum;
    } else if (k < kNV) {
        T sum = T(0);
        for (int w = 0; w < nw; ++w) sum += s_red[w * kNV + k];
        a.ipartials[(static_cast<size_t>(slot) * kNI + (k - kNF)) * nb + vb] = static_cast<int>(sum);
    }
}

// Error-free sum: s + e == a + b exactly (Knuth's TwoSum).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Precision form: the per-pixel terms and the warp sums stay FP32 (the same
// recursive halving as the plain path); the sum over the block's warps is
// compensated (each value carries the exact error of its additions), and the
// block partial is stored as the float pair (s, c) for the compensated
// cross-block sum.
__device__ void reduce_block_comp(const IcpArgs& a, const Acc& acc, int slot, int vb, double* s_red_raw) {
    constexpr int kNV = kNF + kNI;
    float* s_red = reinterpret_cast<float*>(s_red_raw);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    float v[32];
#pragma unroll
    for (int k = 0; k < kNF; ++k) v[k] = acc.f[k];
#pragma unroll
    for (int k = kNF; k < 32; ++k) v[k] = static_cast<float>(acc.i[k - kNF]);
    const float e0 = warp_sum(static_cast<float>(acc.i[32 - kNF]));
    const float e1 = warp_sum(static_cast<float>(acc.i[33 - kNF]));
    const float mine = warp_sum_transpose32(v, lane);
    s_red[warp * kNV + lane] = mine;
    if (lane == 0) {
        s_red[warp * kNV + 32] = e0;
        s_red[warp * kNV + 33] = e1;
    }
    __syncthreads();
    const int k = threadIdx.x, nb = a.vblocks;
    if (k < kNV) {
        float sum = 0.0f, c = 0.0f;
        for (int w = 0; w < nw; ++w) {
            float sn, err;
            two_sum(sum, s_red[w * kNV + k], sn, err);
            sum = sn;
            c = __fadd_rn(c, err);
        }
        if (k < kNF)
            reinterpret_cast<float2*>(a.partials)[(static_cast<size_t>(slot) * kNF + k) * nb + vb] =
                make_float2(sum, c);
        else
            a.ipartials[(static_cast<size_t>(slot) * kNI + (k - kNF)) * nb + vb] = static_cast<int>(sum);
    }
    __syncthreads();
}

template <bool kP>
__device__ void reduce_block(const IcpArgs& a, Acc& acc, int slot, int vb, double* s_red, int buf) {
    if (kP) reduce_block_comp(a, acc, slot, vb, s_red);
    else reduce_block_t<float>(a, acc, slot, vb, s_red, buf);
}

// One association pass over the pixels of every partial slot this block owns
// (slot vb: pixels vb * blockDim + t + k * vblocks * blockDim). The split and
// each slot's sum are those of a launch with vblocks blocks whatever the grid,
// so a smaller grid (several scenes tracked side by side) gives the same sums.
template <bool kP>
__device__ __forceinline__ void associate_all(const IcpArgs& a, const Rel& rel, const IcpLevel& L, int n, int slot,
                                              double* s_red, int gb, int gn) {
    int buf = 0;
    for (int vb = gb; vb < a.vblocks; vb += gn, buf ^= 1) {
        Acc acc;
#pragma unroll
        for (int k = 0; k < kNF; ++k) acc.f[k] = 0.0f;
#pragma unroll
        for (int k = 0; k < kNI; ++k) acc.i[k] = 0;
        associate_range(a, rel, L, vb * blockDim.x + threadIdx.x, a.vblocks * blockDim.x, n, acc);
        reduce_block<kP>(a, acc, slot, vb, s_red, buf);
    }
}

// Sum of all block partials of `slot` in one fixed order (lane l takes blocks
// l, l + 32, ...; then a fixed shuffle tree), so the result does not depend
// on which block computes it. The loads of several values are issued before
// any add.
// The sums land in s_sum as T (float sums in the first half of the storage).
constexpr int kMaxGridBlocks = 512;
constexpr int kPerLane = kMaxGridBlocks / 32;

template <typename T>
__device__ __forceinline__ void reduce_grid_t(const IcpArgs& a, int slot, double* s_sum_raw, int* s_isum) {
    T* s_sum = reinterpret_cast<T*>(s_sum_raw);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    const int nb = a.vblocks;
    for (int k = warp; k < kNF + kNI; k += nw) {
        if (k < kNF) {
            const T* src = reinterpret_cast<const T*>(a.partials) + (static_cast<size_t>(slot) * kNF + k) * nb;
            T v[kPerLane];
#pragma unroll
            for (int j = 0; j < kPerLane; ++j) {
                const int b = lane + 32 * j;
                v[j] = b < nb ? __ldcg(src + b) : T(0);
            }
            T sum = T(0);
#pragma unroll
            for (int j = 0; j < kPerLane; ++j) sum += v[j];
            for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
            if (lane == 0) s_sum[k] = sum;
        } else {
            const int kk = k - kNF;
            const int* src = a.ipartials + (static_cast<size_t>(slot) * kNI + kk) * nb;
            int v[kPerLane];
#pragma unroll
            for (int j = 0; j < kPerLane; ++j) {
                const int b = lane + 32 * j;
                v[j] = b < nb ? __ldcg(src + b) : 0;
            }
            int sum = 0;
#pragma unroll
            for (int j = 0; j < kPerLane; ++j) sum += v[j];
            for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
            if (lane == 0) s_isum[kk] = sum;
        }
    }
    __syncthreads();
}

// FP32 path: a warp takes kVals values per round with all their loads in
// flight (one L2 round trip per round), lane l loading slots l + 32 j for
// j < kPL; per value the same order as above (the slots beyond the grid would
// only add +0, which leaves a float sum that started at +0 unchanged), so every
// instantiation gives the same bits.
template <int kPL, int kVals>
__device__ __forceinline__ void reduce_grid_f(const IcpArgs& a, int slot, float* s_sum, int* s_isum) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    const int nb = a.vblocks;
    for (int k0 = warp; k0 < kNF + kNI; k0 += kVals * nw) {
        unsigned w[kVals][kPL];
#pragma unroll
        for (int r = 0; r < kVals; ++r) {
            const int k = k0 + r * nw;
            const unsigned* src =
                k < kNF ? reinterpret_cast<const unsigned*>(a.partials) + (static_cast<size_t>(slot) * kNF + k) * nb
                        : reinterpret_cast<const unsigned*>(a.ipartials) +
                              (static_cast<size_t>(slot) * kNI + (k - kNF)) * nb;
#pragma unroll
            for (int j = 0; j < kPL; ++j) {
                const int b = lane + 32 * j;
                w[r][j] = (b < nb && k < kNF + kNI) ? __ldcg(src + b) : 0u;
            }
        }
#pragma unroll
        for (int r = 0; r < kVals; ++r) {
            const int k = k0 + r * nw;
            if (k < kNF) {
                float sum = 0.0f;
#pragma unroll
                for (int j = 0; j < kPL; ++j) sum += __uint_as_float(w[r][j]);
                for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
                if (lane == 0) s_sum[k] = sum;
            } else if (k < kNF + kNI) {
                int sum = 0;
#pragma unroll
                for (int j = 0; j < kPL; ++j) sum += static_cast<int>(w[r][j]);
                for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
                if (lane == 0) s_isum[k - kNF] = sum;
            }
        }
    }
    __syncthreads();
}

// Up to 160 partial slots (one block per SM) and 16 warps: all 34 values in one
// round; otherwise two values per warp and round over up to kMaxGridBlocks.
template <>
__device__ __forceinline__ void reduce_grid_t<float>(const IcpArgs& a, int slot, double* s_sum_raw, int* s_isum) {
    float* s_sum = reinterpret_cast<float*>(s_sum_raw);
    if (a.vblocks <= 5 * 32 && 3 * static_cast<int>(blockDim.x >> 5) >= kNF + kNI)
        reduce_grid_f<5, 3>(a, slot, s_sum, s_isum);
    else
        reduce_grid_f<kPerLane, 2>(a, slot, s_sum, s_isum);
}

// (s, c) += (s2, c2): a float-float sum, s the rounded total and c the sum of
// the exact rounding errors (TwoSum), about 48 significant bits.
__device__ __forceinline__ void ff_add(float& s, float& c, float s2, float c2) {
    float t, e;
    two_sum(s, s2, t, e);
    s = t;
    c = __fadd_rn(c, __fadd_rn(c2, e));
}

// Precision form: the cross-block sum of the (s, c) partials in float-float,
// in the fixed order of reduce_grid_f (lane l takes slots l + 32 j, then a
// shuffle tree), all of a round's loads in flight; each value lands in s_sum
// as the double s + c. Pure FP32 instructions: GB300's FP64 rate is a small
// fraction of its FP32 rate.
template <int kPL, int kVals>
__device__ __forceinline__ void reduce_grid_ff(const IcpArgs& a, int slot, double* s_sum, int* s_isum) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    const int nb = a.vblocks;
    const float2* fp = reinterpret_cast<const float2*>(a.partials);
    for (int k0 = warp; k0 < kNF + kNI; k0 += kVals * nw) {
        float2 w[kVals][kPL];
#pragma unroll
        for (int r = 0; r < kVals; ++r) {
            const int k = k0 + r * nw;
#pragma unroll
            for (int j = 0; j < kPL; ++j) {
                const int b = lane + 32 * j;
                w[r][j] = make_float2(0.0f, 0.0f);
                if (b < nb && k < kNF) {
                    w[r][j] = __ldcg(fp + (static_cast<size_t>(slot) * kNF + k) * nb + b);
                } else if (b < nb && k < kNF + kNI) {
                    const int* src = a.ipartials + (static_cast<size_t>(slot) * kNI + (k - kNF)) * nb;
                    w[r][j].x = static_cast<float>(__ldcg(src + b));
                }
            }
        }
#pragma unroll
        for (int r = 0; r < kVals; ++r) {
            const int k = k0 + r * nw;
            if (k < kNF) {
                float sm = 0.0f, c = 0.0f;
#pragma unroll
                for (int j = 0; j < kPL; ++j) ff_add(sm, c, w[r][j].x, w[r][j].y);
                for (int o = 16; o > 0; o >>= 1) {
                    const float s2 = __shfl_down_sync(0xffffffffu, sm, o), c2 = __shfl_down_sync(0xffffffffu, c, o);
                    ff_add(sm, c, s2, c2);
                }
                if (lane == 0) s_sum[k] = static_cast<double>(sm) + static_cast<double>(c);
            } else if (k < kNF + kNI) {
                int sum = 0;
#pragma unroll
                for (int j = 0; j < kPL; ++j) sum += static_cast<int>(w[r][j].x);
                for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
                if (lane == 0) s_isum[k - kNF] = sum;
            }
        }
    }
    __syncthreads();
}

template <bool kP>
__device__ void reduce_grid(const IcpArgs& a, int slot, double* s_sum, int* s_isum) {
    if (kP) {
        if (a.vblocks <= 5 * 32 && 3 * static_cast<int>(blockDim.x >> 5) >= kNF + kNI)
            reduce_grid_ff<5, 3>(a, slot, s_sum, s_isum);
        else
            reduce_grid_ff<kPerLane, 2>(a, slot, s_sum, s_isum);
    } else {
        reduce_grid_t<float>(a, slot, s_sum, s_isum);
    }
}

// Reduced sum k as float (the storage holds floats unless in precision form).
template <bool kP>
__device__ __forceinline__ float sum_f(const IcpArgs& a, const double* sum, int k) {
    return kP ? static_cast<float>(sum[k]) : reinterpret_cast<const float*>(sum)[k];
}

// ---------------------------------------------------------------------------
// 6x6 symmetric eigenvalues by a parallel cyclic Jacobi sweep on one warp
// (round-robin pairing: 5 rounds of 3 disjoint rotations per sweep).
__constant__ int kPairs[5][3][2] = {{{0, 1}, {2, 5}, {3, 4}}, {{0, 2}, {1, 3}, {4, 5}}, {{0, 3}, {2, 4}, {1, 5}},
                                    {{0, 4}, {3, 5}, {1, 2}}, {{0, 5}, {1, 4}, {2, 3}}};

__device__ void warp_eig6(float* m /* smem 36, destroyed */, float* cs /* smem 12 */, float& mn, float& mx) {
    const int lane = threadIdx.x & 31;
    for (int sweep = 0; sweep < 8; ++sweep) {
        for (int r = 0; r < 5; ++r) {
            if (lane < 3) {
                const int p = kPairs[r][lane][0], q = kPairs[r][lane][1];
                const float apq = m[p * 6 + q];
                float c = 1.0f, s = 0.0f;
                if (apq != 0.0f) {
                    const float theta = (m[q * 6 + q] - m[p * 6 + p]) / (2.0f * apq);
                    const float t = (theta >= 0.0f ? 1.0f : -1.0f) / (fabsf(theta) + sqrtf(theta * theta + 1.0f));
                    c = rsqrtf(t * t + 1.0f);
                    s = t * c;
                }
                cs[4 * lane] = c;
                cs[4 * lane + 1] = s;
            }
            __syncwarp();
            // rows
            float nv[2];
            for (int h = 0; h < 2; ++h) {
                const int e = lane + 32 * h;
                if (e < 36) {
                    const int i = e / 6, k = e % 6;
                    int pi = 0;
                    for (int t = 0; t < 3; ++t)
                        if (kPairs[r][t][0] == i || kPairs[r][t][1] == i) pi = t;
                    const int p = kPairs[r][pi][0], q = kPairs[r][pi][1];
                    const float c = cs[4 * pi], s = cs[4 * pi + 1];
                    nv[h] = (i == p) ? c * m[p * 6 + k] - s * m[q * 6 + k] : s * m[p * 6 + k] + c * m[q * 6 + k];
                }
            }
            __syncwarp();
            for (int h = 0; h < 2; ++h) if (lane + 32 * h < 36) m[lane + 32 * h] = nv[h];
            __syncwarp();
            // columns
            for (int h = 0; h < 2; ++h) {
                const int e = lane + 32 * h;
                if (e < 36) {
                    const int k = e / 6, j = e % 6;
                    int pj = 0;
                    for (int t = 0; t < 3; ++t)
                        if (kPairs[r][t][0] == j || kPairs[r][t][1] == j) pj = t;
                    const int p = kPairs[r][pj][0], q = kPairs[r][pj][1];
                    const float c = cs[4 * pj], s = cs[4 * pj + 1];
                    nv[h] = (j == p) ? c * m[k * 6 + p] - s * m[k * 6 + q] : s * m[k * 6 + p] + c * m[k * 6 + q];
                }
            }
            __syncwarp();
            for (int h = 0; h < 2; ++h) if (lane + 32 * h < 36) m[lane + 32 * h] = nv[h];
            __syncwarp();
        }
    }
    float lo = m[0], hi = m[0];
    for (int i = 1; i < 6; ++i) {
        lo = fminf(lo, m[i * 7]);
        hi = fmaxf(hi, m[i * 7]);
    }
    mn = lo;
    mx = hi;
}

// A x = b by the LDL^T factorisation in double (precision form), unrolled on
// packed triangles. On GB300 a dependent FP64 fma takes ~64 cycles, a division
// ~430 and a square root ~700, so the factorisation's critical path is its
// pivots: LDL^T needs one division per pivot and no square root (13.2 k cycles
// for Cholesky with a square root and a reciprocal per pivot, measured on one
// thread). False when a pivot is not positive.
__device__ __noinline__ bool ldlt_solve_d(const double* Ain, const double* b, double* x) {
    double L[21], LD[21], inv[6];  // L(i, j) and L(i, j) D(j), j < i, at i (i + 1) / 2 + j
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        double s = Ain[j * 6 + j];
#pragma unroll
        for (int k = 0; k < j; ++k) s -= L[j * (j + 1) / 2 + k] * LD[j * (j + 1) / 2 + k];
        if (!(s > 0.0)) return false;
        inv[j] = 1.0 / s;
#pragma unroll
        for (int i = j + 1; i < 6; ++i) {
            double t = Ain[i * 6 + j];
#pragma unroll
            for (int k = 0; k < j; ++k) t -= L[i * (i + 1) / 2 + k] * LD[j * (j + 1) / 2 + k];
            LD[i * (i + 1) / 2 + j] = t;
            L[i * (i + 1) / 2 + j] = t * inv[j];
        }
    }
    double y[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        double s = b[i];
#pragma unroll
        for (int k = 0; k < i; ++k) s -= L[i * (i + 1) / 2 + k] * y[k];
        y[i] = s;
    }
#pragma unroll
    for (int i = 5; i >= 0; --i) {
        double s = y[i] * inv[i];
#pragma unroll
        for (int k = i + 1; k < 6; ++k) s -= L[k * (k + 1) / 2 + i] * x[k];
        x[i] = s;
    }
    return true;
}

// Nearest proper rotation of a general 3x3 matrix M (row-major, double): U V^T
// of its SVD with the direction of the smallest singular value flipped when
// det(U V^T) < 0 (projectToSO3, include/tracking/ICPShared.h:102-110). V holds
// the eigenvectors of M^T M (cyclic Jacobi), U = M V / sigma. This is the
// exact path for matrices the Newton-Schulz steps below cannot bring to a
// rotation (reflections, large scale errors); near-rotations never reach it.
__device__ __noinline__ void nearest_rotation_d(const double* M, double* R) {
    double a[9], V[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) a[3 * i + j] = M[i] * M[j] + M[3 + i] * M[3 + j] + M[6 + i] * M[6 + j];
    for (int sweep = 0; sweep < 30; ++sweep) {
        const double off = a[1] * a[1] + a[2] * a[2] + a[5] * a[5];
        if (!(off > 1e-300)) break;
        for (int pq = 0; pq < 3; ++pq) {
            const int p = pq == 2 ? 1 : 0, q = pq == 0 ? 1 : 2;
            const double apq = a[3 * p + q];
            if (apq == 0.0) continue;
            const double theta = (a[3 * q + q] - a[3 * p + p]) / (2.0 * apq);
            const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
            const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
            for (int k = 0; k < 3; ++k) {
                const double akp = a[3 * k + p], akq = a[3 * k + q];
                a[3 * k + p] = c * akp - sn * akq;
                a[3 * k + q] = sn * akp + c * akq;
            }
            for (int k = 0; k < 3; ++k) {
                const double apk = a[3 * p + k], aqk = a[3 * q + k];
                a[3 * p + k] = c * apk - sn * aqk;
                a[3 * q + k] = sn * apk + c * aqk;
            }
            for (int k = 0; k < 3; ++k) {
                const double vkp = V[3 * k + p], vkq = V[3 * k + q];
                V[3 * k + p] = c * vkp - sn * vkq;
                V[3 * k + q] = sn * vkp + c * vkq;
            }
        }
    }
    double ev[3] = {a[0], a[4], a[8]};
    int ord[3] = {0, 1, 2};  // ascending eigenvalues: ord[0] is the smallest singular value
    for (int i = 0; i < 3; ++i)
        for (int j = i + 1; j < 3; ++j)
            if (ev[ord[j]] < ev[ord[i]]) { const int t = ord[i]; ord[i] = ord[j]; ord[j] = t; }
    double U[9], Vs[9];
    for (int c = 0; c < 3; ++c) {
        const int e = ord[c];
        const double sig = sqrt(fmax(ev[e], 1e-300));
        for (int i = 0; i < 3; ++i) {
            Vs[3 * i + c] = V[3 * i + e];
            U[3 * i + c] = (M[3 * i] * V[e] + M[3 * i + 1] * V[3 + e] + M[3 * i + 2] * V[6 + e]) / sig;
        }
    }
    if (!(ev[ord[0]] > 1e-24 * ev[ord[2]])) {  // rank-deficient: complete the frame
        U[0] = U[4] * U[8] - U[7] * U[5];
        U[3] = U[7] * U[2] - U[1] * U[8];
        U[6] = U[1] * U[5] - U[4] * U[2];
    }
    for (int pass = 0; pass < 2; ++pass) {
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                R[3 * i + j] = U[3 * i] * Vs[3 * j] + U[3 * i + 1] * Vs[3 * j + 1] + U[3 * i + 2] * Vs[3 * j + 2];
        const double det = R[0] * (R[4] * R[8] - R[5] * R[7]) - R[1] * (R[3] * R[8] - R[5] * R[6]) +
                           R[2] * (R[3] * R[7] - R[4] * R[6]);
        if (det >= 0.0) break;
        for (int i = 0; i < 3; ++i) U[3 * i] = -U[3 * i];
    }
}

// True when X (row-major 3x3) is a rotation to tolerance: X^T X = I within
// tol and det > 0.
template <typename T>
__device__ __forceinline__ bool is_rotation(const T* X, T tol) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const T g = X[i] * X[j] + X[3 + i] * X[3 + j] + X[6 + i] * X[6 + j];
            if (!(fabs(g - (i == j ? T(1) : T(0))) <= tol)) return false;
        }
    const T det = X[0] * (X[4] * X[8] - X[5] * X[7]) - X[1] * (X[3] * X[8] - X[5] * X[6]) +
                  X[2] * (X[3] * X[7] - X[4] * X[6]);
    return det > T(0);
}

// sin and cos of an angle of at most 0.5 rad by their Taylor series in FP64:
// after the x^19 / x^18 terms the remainder is below 1e-25, far under half an
// ulp of the results. Larger angles (not reached by capped steps) take sincos.
__device__ __forceinline__ void sincos_small(double x, double& sn, double& cs) {
    if (!(fabs(x) <= 0.5)) {
        sincos(x, &sn, &cs);
        return;
    }
    // 1 / n!, n = 0 .. 19
    constexpr double kInvFact[20] = {
        1.0, 1.0, 1.0 / 2.0, 1.0 / 6.0, 1.0 / 24.0, 1.0 / 120.0, 1.0 / 720.0, 1.0 / 5040.0, 1.0 / 40320.0,
        1.0 / 362880.0, 1.0 / 3628800.0, 1.0 / 39916800.0, 1.0 / 479001600.0, 1.0 / 6227020800.0,
        1.0 / 87178291200.0, 1.0 / 1307674368000.0, 1.0 / 20922789888000.0, 1.0 / 355687428096000.0,
        1.0 / 6402373705728000.0, 1.0 / 121645100408832000.0};
    const double x2 = x * x;
    double ps = kInvFact[19], pc = kInvFact[18];
#pragma unroll
    for (int k = 8; k >= 0; --k) {
        ps = kInvFact[2 * k + 1] - x2 * ps;
        pc = kInvFact[2 * k] - x2 * pc;
    }
    sn = x * ps;
    cs = pc;
}

// Precision form: SE(3) exponential of the step and pose composition in FP64,
// then the nearest rotation (orthogonal polar factor, = U V^T of the SVD for
// det > 0) by a Newton-Schulz step X <- X (3 I - X^T X) / 2 in FP64.
// The rotation is Rodrigues' formula R = I + A K + B K^2 of K = [r]x with
// A = sin t / t and B = (1 - cos t) / t^2 (t = |r|), the same matrix as
// cos t I + (1 - cos t) a a^T + sin t [a]x of the unit axis a; A and B are
// their Taylor series in t^2 (remainder below 1e-25 for t <= 0.5), so neither
// a square root nor a division is on the path. The composed rotation part is
// orthogonal to the float pose's ~1e-7, and one step takes that to ~1e-14,
// below what the float result can hold.
__device__ void compose_precise(float* pose, const double* x) {
    const double rx = x[3], ry = x[4], rz = x[5];
    const double t2 = rx * rx + ry * ry + rz * rz;
    double R[9];
    if (t2 > 1e-8) {  // angle > 1e-4
        double A, B;
        if (t2 <= 0.25) {
            // 1 / (2k + 1)! and 1 / (2k + 2)!, k = 0 .. 9
            constexpr double kA[10] = {1.0, 1.0 / 6.0, 1.0 / 120.0, 1.0 / 5040.0, 1.0 / 362880.0,
                                       1.0 / 39916800.0, 1.0 / 6227020800.0, 1.0 / 1307674368000.0,
                                       1.0 / 355687428096000.0, 1.0 / 121645100408832000.0};
            constexpr double kB[10] = {1.0 / 2.0, 1.0 / 24.0, 1.0 / 720.0, 1.0 / 40320.0, 1.0 / 3628800.0,
                                       1.0 / 479001600.0, 1.0 / 87178291200.0, 1.0 / 20922789888000.0,
                                       1.0 / 6402373705728000.0, 1.0 / 2432902008176640000.0};
            A = kA[9];
            B = kB[9];
#pragma unroll
            for (int k = 8; k >= 0; --k) {
                A = kA[k] - t2 * A;
                B = kB[k] - t2 * B;
            }
        } else {  // outside the series' range (not reached by capped steps)
            const double t = sqrt(t2);
            double sn, cs;
            sincos_small(t, sn, cs);
            A = sn / t;
            B = (1.0 - cs) / t2;
        }
        R[0] = 1.0 - B * (ry * ry + rz * rz); R[1] = B * rx * ry - A * rz;        R[2] = B * rx * rz + A * ry;
        R[3] = B * rx * ry + A * rz;        R[4] = 1.0 - B * (rx * rx + rz * rz); R[5] = B * ry * rz - A * rx;
        R[6] = B * rx * rz - A * ry;        R[7] = B * ry * rz + A * rx;        R[8] = 1.0 - B * (rx * rx + ry * ry);
    } else {
        R[0] = 1.0; R[1] = -rz; R[2] = ry; R[3] = rz; R[4] = 1.0; R[5] = -rx; R[6] = -ry; R[7] = rx; R[8] = 1.0;
    }
    const double D[12] = {R[0], R[1], R[2], x[0], R[3], R[4], R[5], x[1], R[6], R[7], R[8], x[2]};
    double P[12];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            double sum = (j == 3) ? static_cast<double>(pose[4 * i + 3]) : 0.0;
#pragma unroll
            for (int k = 0; k < 3; ++k) sum += static_cast<double>(pose[4 * i + k]) * D[4 * k + j];
            P[4 * i + j] = sum;
        }
    double X[9] = {P[0], P[1], P[2], P[4], P[5], P[6], P[8], P[9], P[10]};
    {
        double G[9];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
                G[3 * i + j] = (i == j ? 3.0 : 0.0) - (X[i] * X[j] + X[3 + i] * X[3 + j] + X[6 + i] * X[6 + j]);
        double N[9];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
                N[3 * i + j] = 0.5 * (X[3 * i] * G[j] + X[3 * i + 1] * G[3 + j] + X[3 * i + 2] * G[6 + j]);
#pragma unroll
        for (int k = 0; k < 9; ++k) X[k] = N[k];
    }
    if (!is_rotation(X, 1e-9)) {
        const double M[9] = {P[0], P[1], P[2], P[4], P[5], P[6], P[8], P[9], P[10]};
        nearest_rotation_d(M, X);
    }
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) pose[4 * i + j] = static_cast<float>(X[3 * i + j]);
        pose[4 * i + 3] = static_cast<float>(P[4 * i + 3]);
    }
}

// The same projection in float by the Newton-Schulz iteration
// X <- X (3 I - X^T X) / 2, which converges quadratically to the orthogonal
// polar factor from a near-rotation (no division); two steps reach float
// precision from the composed pose. A result that is not a rotation (the
// input was a reflection or far from orthogonal) takes the exact SVD path.
__device__ void project_so3_f(float* P) {
    float X[9];
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) X[3 * i + j] = P[4 * i + j];
#pragma unroll
    for (int it = 0; it < 2; ++it) {
        float G[9];  // 3 I - X^T X
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const float g = X[i] * X[j] + X[3 + i] * X[3 + j] + X[6 + i] * X[6 + j];
                G[3 * i + j] = (i == j ? 3.0f : 0.0f) - g;
            }
        float N[9];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
                N[3 * i + j] = 0.5f * (X[3 * i] * G[j] + X[3 * i + 1] * G[3 + j] + X[3 * i + 2] * G[6 + j]);
#pragma unroll
        for (int k = 0; k < 9; ++k) X[k] = N[k];
    }
    if (!is_rotation(X, 1e-5f)) {
        double M[9], Rd[9];
        for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) M[3 * i + j] = P[4 * i + j];
        nearest_rotation_d(M, Rd);
        for (int k = 0; k < 9; ++k) X[k] = static_cast<float>(Rd[k]);
    }
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) P[4 * i + j] = X[3 * i + j];
}

// Rodrigues rotation (Eigen::AngleAxisf::toRotationMatrix) into a row-major 3x3.
__device__ void angle_axis(float angle, F3 axis, float* r) {
    const float s = sinf(angle), c = cosf(angle);
    const F3 sa = mul3(axis, s);
    const F3 ca = mul3(axis, fs(1.0f, c));
    float t = fm(ca.x, axis.y);
    r[1] = fs(t, sa.z); r[3] = fa(t, sa.z);
    t = fm(ca.x, axis.z);
    r[2] = fa(t, sa.y); r[6] = fs(t, sa.y);
    t = fm(ca.y, axis.z);
    r[5] = fs(t, sa.x); r[7] = fa(t, sa.x);
    r[0] = fa(fm(ca.x, axis.x), c); r[4] = fa(fm(ca.y, axis.y), c); r[8] = fa(fm(ca.z, axis.z), c);
}

struct LevelState {
    float pose[16];
    float error, final_step;
    int inliers, converged;
    float information[36];
    int counts[6];  // valid_live .. angle_filtered (index 1..5 used)
    int iters;
};

// Shared-memory scratch of the solve.
struct SolveSmem {
    double sum[kNF];  // reduced sums: double (precision form) or float in the first half
    int isum[kNI];
    float m[36];
    float cs[12];
    int action;    // 0 continue, 1 stop level
    int need_eig;  // the shifted-Cholesky test could not settle the damping
    float spec_pose[16];  // the pose the step with the level's default damping leads to
    float spec_step;      // that step's norm
    int spec_ok;          // 0: that step stops the level (no solution, not finite or over a cap)
    float spec2_pose[16];  // the same with the escalated damping
    float spec2_step;
    int spec2_ok;
};

// Cholesky factor of A + shift I (6x6, float), fully unrolled so that the
// factor stays in registers. False when a pivot is not positive.
__device__ __forceinline__ bool chol6_f(const float* A, float shift, float (&L)[36], float (&inv)[6]) {
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        float sj = A[j * 6 + j] + shift;
#pragma unroll
        for (int k = 0; k < j; ++k) sj -= L[j * 6 + k] * L[j * 6 + k];
        if (!(sj > 0.0f)) return false;
        const float d = sqrtf(sj);
        inv[j] = 1.0f / d;
        L[j * 6 + j] = d;
#pragma unroll
        for (int i = j + 1; i < 6; ++i) {
            float t = A[i * 6 + j];
#pragma unroll
            for (int k = 0; k < j; ++k) t -= L[i * 6 + k] * L[j * 6 + k];
            L[i * 6 + j] = t * inv[j];
        }
    }
    return true;
}

// True when A - shift I is positive definite.
__device__ bool pd_after_shift(const float* A, float shift) {
    float L[36], inv[6];
    return chol6_f(A, -shift, L, inv);
}

// (A + damp I) x = b by Cholesky (A + damp I is positive definite for a
// normal-equation matrix); NaN when the factorisation breaks down, which the
// caller's finiteness check turns into a stop.
__device__ void chol6_solve_f(const float* A, float damp, const float* b, float* x) {
    float L[36], inv[6];
    if (!chol6_f(A, damp, L, inv)) {
#pragma unroll
        for (int i = 0; i < 6; ++i) x[i] = __int_as_float(0x7fffffff);
        return;
    }
    float y[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        float t = b[i];
#pragma unroll
        for (int k = 0; k < i; ++k) t -= L[i * 6 + k] * y[k];
        y[i] = t * inv[i];
    }
#pragma unroll
    for (int i = 5; i >= 0; --i) {
        float t = y[i];
#pragma unroll
        for (int k = i + 1; k < 6; ++k) t -= L[k * 6 + i] * x[k];
        x[i] = t * inv[i];
    }
}

// Damped solve of (A + damp I) x = b from the reduced sums: Cholesky in float,
// or LDL^T in double for the precision form (the reference's LDL^T of the same
// positive definite matrix agrees to rounding). False when the
// double factorisation breaks down.
template <bool kP>
__device__ bool damped_solve(const IcpArgs& a, const SolveSmem& sm, float damp, float* x, double* xd) {
    if (kP) {
        double A[36], b[6];
        int k = 0;
        for (int i = 0; i < 6; ++i)
            for (int j = i; j < 6; ++j) { A[i * 6 + j] = A[j * 6 + i] = sm.sum[k++]; }
        for (int i = 0; i < 6; ++i) { A[i * 6 + i] += damp; b[i] = sm.sum[21 + i]; }
        if (!ldlt_solve_d(A, b, xd)) return false;
        for (int i = 0; i < 6; ++i) x[i] = static_cast<float>(xd[i]);
    } else {
        float A[36], b[6];
        int k = 0;
#pragma unroll
        for (int i = 0; i < 6; ++i)
#pragma unroll
            for (int j = i; j < 6; ++j) { A[i * 6 + j] = A[j * 6 + i] = sum_f<kP>(a, sm.sum, k++); }
#pragma unroll
        for (int i = 0; i < 6; ++i) b[i] = sum_f<kP>(a, sm.sum, 21 + i);
        chol6_solve_f(A, damp, b, x);
    }
    return true;
}

// The step of damping `damp` from the reduced sums and the pose it leads to
// (ICPTracker.cpp:86-119): false when the damped system has no solution or
// the step is not finite or exceeds a cap, which stops the level.
template <bool kP>
__device__ __noinline__ bool step_pose(const IcpArgs& a, const SolveSmem& sm, const float* pose, float damp,
                                       float* out, float& step_norm) {
    float x[6];
    double xd[6];
    if (!damped_solve<kP>(a, sm, damp, x, xd)) return false;
    bool fin = true;
    for (int i = 0; i < 6; ++i) fin = fin && isfinite(x[i]);
    const float tn = norm3(mk3(x[0], x[1], x[2])), rn = norm3(mk3(x[3], x[4], x[5]));
    if (!fin || tn > kTranslationCapStep || rn > kRotationCapStep) return false;
    float ss = 0.0f;
    for (int i = 0; i < 6; ++i) ss = fa(ss, fm(x[i], x[i]));
    step_norm = fsq(ss);
    for (int i = 0; i < 16; ++i) out[i] = pose[i];
    if (kP) {
        compose_precise(out, xd);
    } else {
        const float rx = x[3], ry = x[4], rz = x[5];
        float delta[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
        const float angle = fsq(fa(fa(fm(rx, rx), fm(ry, ry)), fm(rz, rz)));
        float R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        if (angle > 1e-4f) {
            F3 axis = mk3(rx, ry, rz);
            axis = div3(axis, norm3(axis));
            angle_axis(angle, axis, R);
        } else {
            R[1] = -rz; R[2] = ry; R[3] = rz; R[5] = -rx; R[6] = -ry; R[7] = rx;
        }
        for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) delta[4 * i + j] = R[3 * i + j];
        delta[3] = x[0]; delta[7] = x[1]; delta[11] = x[2];
        float P[16];
        mm4(pose, delta, P);
        project_so3_f(P);
        for (int i = 0; i < 16; ++i) out[i] = P[i];
    }
    return true;
}

// Barrier of warps 0, 1 and 2 only (named barrier 1, 96 threads).
__device__ __forceinline__ void sync_solve_warps() { asm volatile("bar.sync 1, 96;" ::: "memory"); }

// One solve from the reduced sums (ICPTracker.cpp:78-131), executed by warps
// 0, 1 and 2. Lanes 2..22 of warp 0 store the information matrix; lane 0 of
// warp 1 solves with the level's default damping and composes the pose it
// leads to, lane 0 of warp 2 does the same with the escalated damping, while
// lane 0 of warp 0 runs the damping test (separate warps, so the three run
// side by side rather than one after the other as divergent lanes of one
// warp would). The test then only picks one of the two steps: no solve runs
// after it (track stage on c2 0.0837 -> 0.0817 ms).
template <bool kP>
__device__ void solve_step(const IcpArgs& a, int level, SolveSmem& sm, LevelState& st) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int inl = sm.isum[0];
    const float base_damp = (level == 0) ? kDampingLevel0 : kDampingDefault;
    const bool stop = (inl <= 0 || inl < kMinInliersForIteration);
    if (warp == 1) {
        if (lane == 0 && !stop)
            sm.spec_ok = step_pose<kP>(a, sm, st.pose, base_damp, sm.spec_pose, sm.spec_step) ? 1 : 0;
        sync_solve_warps();
        return;
    }
    if (warp == 2) {
        if (lane == 0 && !stop)
            sm.spec2_ok = step_pose<kP>(a, sm, st.pose, kDampingEscalated, sm.spec2_pose, sm.spec2_step) ? 1 : 0;
        sync_solve_warps();
        return;
    }
    if (!stop && lane >= 2 && lane < 23) {
        const int k = lane - 2;  // upper-triangle entry k = (i, j), row by row
        int i = 0, r = k;
        while (r >= 6 - i) { r -= 6 - i; ++i; }
        const int j = i + r;
        const float v = sum_f<kP>(a, sm.sum, k);
        st.information[i * 6 + j] = v;
        st.information[j * 6 + i] = v;
    }
    __syncwarp();
    if (lane == 0) {
        for (int k = 1; k < 6; ++k) st.counts[k] = sm.isum[k];
        sm.action = stop ? 1 : 0;
        if (!stop) {
            // dampingForHessian (ICPShared.h:86-100) escalates when min_eig < 1e-4
            // or max_eig > 1e7 min_eig. Since max_eig <= trace, min_eig >= sigma =
            // max(1e-4, trace / 1e7) rules both out; A - sigma' I positive definite
            // proves it, with sigma' = 2 sigma + 32 eps trace covering the
            // rounding of the float factorisation. Only when that test fails do
            // the eigenvalues decide.
            float tr = 0.0f;
            for (int i = 0; i < 6; ++i) tr += st.information[i * 6 + i];
            const float sigma = fmaxf(kMinEigEscalate, tr / kCondEscalate);
            const float shift = 2.0f * sigma + 32.0f * 1.1920929e-7f * tr;
            sm.need_eig = (isfinite(tr) && pd_after_shift(st.information, shift)) ? 0 : 1;
        }
    }
    sync_solve_warps();  // warp 1's step is done, and warp 0's test
    if (sm.action != 0) return;
    float mn = 1.0f, mx = 1.0f;
    if (sm.need_eig) {
        for (int i = lane; i < 36; i += 32) sm.m[i] = st.information[i];
        __syncwarp();
        warp_eig6(sm.m, sm.cs, mn, mx);
    }
    if (lane != 0) return;
    float damp = base_damp;
    if (sm.need_eig) {
        if (!isfinite(mn) || !isfinite(mx) || mn < kMinEigEscalate) damp = kDampingEscalated;
        else if (mx > kCondEscalate * mn) damp = kDampingEscalated;
    }
    float step_norm;
    if (damp == base_damp) {
        if (!sm.spec_ok) { sm.action = 1; return; }
        for (int i = 0; i < 16; ++i) st.pose[i] = sm.spec_pose[i];
        step_norm = sm.spec_step;
    } else {
        if (!sm.spec2_ok) { sm.action = 1; return; }
        for (int i = 0; i < 16; ++i) st.pose[i] = sm.spec2_pose[i];
        step_norm = sm.spec2_step;
    }
    st.final_step = step_norm;
    st.error = fd(sum_f<kP>(a, sm.sum, 27), static_cast<float>(inl > 1 ? inl : 1));
    st.inliers = inl;
    st.iters++;
    if (step_norm < kConvergenceStep) {
        st.converged = 1;
        sm.action = 1;
    }
}

__device__ void compute_rel(const float* pose, const float* ref_inv, Rel& r) {
    rot_of(pose, r.Rcw);
    r.tcw = trans_of(pose);
    float Rrc[9];
    rot_of(ref_inv, Rrc);
    const F3 trc = trans_of(ref_inv);
    mm3(Rrc, r.Rcw, r.Rrel);
    r.trel = add3(mv3(Rrc, r.tcw), trc);
}

// classifyTracking (TrackingPolicy.h:70-112): 0 Good, 1 Poor, 2 Failed.
__device__ int classify(const azu_icp_result& r, const float* prev) {
    bool fin = true;
    for (int i = 0; i < 16; ++i) fin = fin && isfinite(r.pose[i]);
    if (!fin || !isfinite(r.error) || r.inliers < kMinInliersForOk) return 2;
    const float fit = r.valid_model_points > 0 ? fd(float(r.inliers), float(r.valid_model_points)) : 0.0f;
    const float rms = fsq(fmaxf(0.0f, r.error));
    const int q = (r.inliers >= 2000 && fit >= 0.40f && rms <= 0.015f) ? 0 : 1;
    float pinv[16], d[16];
    inverse4(prev, pinv);
    mm4(pinv, r.pose, d);
    const float trans = norm3(trans_of(d));
    const float tr = fa(fa(d[0], d[5]), d[10]);
    const float c = fmaxf(-1.0f, fminf(1.0f, fm(fs(tr, 1.0f), 0.5f)));
    const float ang = acosf(c);
    if (!(trans <= 0.15f && ang <= 0.52f)) return 2;
    return q;
}

// The whole track of one scene by a group of gn co-resident blocks (this one
// is block gb of the group): a whole grid for a single tracker, a share of one
// for scenes tracked side by side.
template <bool kP>
__device__ __forceinline__ void icp_body(const IcpArgs& a, int gb, int gn) {
    __shared__ double s_red[(kIcpThreads / 32) * (kNF + kNI)];
    __shared__ SolveSmem sm;
    __shared__ LevelState st;
    __shared__ Rel s_rel;
    __shared__ float s_refinv[16];
    __shared__ unsigned s_gen;
    __shared__ float s_start[16];
    __shared__ azu_icp_result s_res;
    __shared__ int s_retry;
    __shared__ WaitLimits s_wl;

    if (threadIdx.x == 0) {
        s_gen = ld_acquire(&a.bar[1]);
        s_wl.spins = g_icp_spin_limit;
        s_wl.arrivals = static_cast<unsigned>(gn) + g_icp_extra_arrivals;
        float ref[16];
        for (int i = 0; i < 16; ++i) ref[i] = a.d_ref[i];
        inverse4(ref, s_refinv);
        for (int i = 0; i < 16; ++i) s_start[i] = a.d_estimate[i];
    }
    __syncthreads();
    unsigned gen = s_gen;
    const WaitLimits wl = s_wl;
    int slot = 0;

    if (a.build_level >= 0) {  // single association pass (parity probe)
        const IcpLevel L = a.lv[a.build_level];
        if (threadIdx.x == 0) compute_rel(s_start, s_refinv, s_rel);
        __syncthreads();
        const Rel rel = s_rel;
        const int iw = L.W - 2, ih = L.H - 2;
        const int n = iw > 0 && ih > 0 ? iw * ih : 0;
        associate_all<kP>(a, rel, L, n, 0, s_red, gb, gn);
        grid_sync(a.bar, a.err, wl, gen);
        reduce_grid<kP>(a, 0, sm.sum, sm.isum);
        if (gb == 0 && threadIdx.x == 0) {
            int k = 0;
            for (int i = 0; i < 6; ++i)
                for (int j = i; j < 6; ++j) {
                    const float v = sum_f<kP>(a, sm.sum, k++);
                    a.build_out[i * 6 + j] = v;
                    a.build_out[j * 6 + i] = v;
                }
            for (int i = 0; i < 6; ++i) a.build_out[36 + i] = sum_f<kP>(a, sm.sum, 21 + i);
            a.build_out[42] = sum_f<kP>(a, sm.sum, 27);
            for (int i = 0; i < 6; ++i) reinterpret_cast<int*>(a.build_out)[43 + i] = sm.isum[i];
        }
        return;
    }

    for (int attempt = 0; attempt < 2; ++attempt) {
        // ICPTracker::track (ICPTracker.cpp:40-66); thread 0 keeps the result.
        if (threadIdx.x == 0) {
            for (int i = 0; i < 16; ++i) s_res.pose[i] = (attempt == 0) ? s_start[i] : a.d_prev[i];
            s_res.error = 0.0f; s_res.inliers = 0; s_res.converged = 0;
            s_res.final_step = __int_as_float(0x7f800000);
            for (int i = 0; i < 36; ++i) s_res.information[i] = 0.0f;
            s_res.valid_live_points = s_res.valid_model_points = s_res.projected_points = 0;
            s_res.dist_filtered = s_res.angle_filtered = 0;
            for (int l = 0; l < 3; ++l) s_res.iterations[l] = 0;
        }
        __syncthreads();
        for (int level = 2; level >= 0; --level) {
            const int max_iter = a.iters[level];
            if (max_iter <= 0) continue;
            const IcpLevel L = a.lv[level];
            if (threadIdx.x == 0) {
                for (int i = 0; i < 16; ++i) st.pose[i] = s_res.pose[i];
                st.error = 0.0f;
                st.final_step = __int_as_float(0x7f800000);
                st.inliers = 0;
                st.converged = 0;
                for (int i = 0; i < 36; ++i) st.information[i] = 0.0f;
                for (int i = 0; i < 6; ++i) st.counts[i] = 0;
                st.iters = 0;
            }
            __syncthreads();
            const int iw = L.W - 2, ih = L.H - 2;
            const int n = iw > 0 && ih > 0 ? iw * ih : 0;
            for (int iter = 0; iter < max_iter; ++iter) {
                if (threadIdx.x == 0) compute_rel(st.pose, s_refinv, s_rel);
                __syncthreads();
                const Rel rel = s_rel;
                associate_all<kP>(a, rel, L, n, slot, s_red, gb, gn);
                // Every block reduces the partials and solves on its own: the
                // same loads in the same order and the same code give every
                // block the same bits, so no block waits for another's result
                // after the barrier (the partial slots alternate, so the next
                // iteration's partials never overwrite ones still being read).
                grid_sync(a.bar, a.err, wl, gen);
                reduce_grid<kP>(a, slot, sm.sum, sm.isum);
                if (threadIdx.x < 96) solve_step<kP>(a, level, sm, st);
                __syncthreads();
                slot ^= 1;
                if (sm.action != 0) break;
            }
            // track(): the level result replaces the running one; final_step
            // carries the last finite value.
            if (threadIdx.x == 0) {
                const float carried = s_res.final_step;
                for (int i = 0; i < 16; ++i) s_res.pose[i] = st.pose[i];
                s_res.error = st.error;
                s_res.inliers = st.inliers;
                s_res.converged = st.converged;
                s_res.final_step = isfinite(st.final_step) ? st.final_step : carried;
                for (int i = 0; i < 36; ++i) s_res.information[i] = st.information[i];
                s_res.valid_live_points = st.counts[1];
                s_res.valid_model_points = st.counts[2];
                s_res.projected_points = st.counts[3];
                s_res.dist_filtered = st.counts[4];
                s_res.angle_filtered = st.counts[5];
                s_res.iterations[level] = st.iters;
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            bool pf = true;
            for (int i = 0; i < 16; ++i) pf = pf && isfinite(s_res.pose[i]);
            s_res.tracking_ok = pf && s_res.inliers > kMinInliersForOk &&
                                (s_res.converged || s_res.final_step <= kAcceptableFinalStep);
            s_res.status = 0;
            s_retry = (a.d_prev != nullptr && attempt == 0 && classify(s_res, a.d_prev) == 2) ? 1 : 0;
        }
        __syncthreads();
        if (!s_retry) break;
    }

    if (gb == 0 && threadIdx.x == 0) {
        azu_icp_result res = s_res;
        const bool timed_out = ld_acquire(a.err) != 0;
        res.status = timed_out ? AZU_E_TIMEOUT : AZU_OK;
        *a.d_result = res;
        if (a.d_prev) {
            // a track whose wait ran out is graded Failed: the pose stays at
            // prev and nothing is fused from this frame
            const int q = timed_out ? 2 : classify(res, a.d_prev);
            if (a.d_quality) *a.d_quality = q;
            if (a.d_gate) *a.d_gate = (q == 0) ? 1 : 0;
            if (a.d_pose_out) {
                if (q != 2) for (int i = 0; i < 16; ++i) a.d_pose_out[i] = res.pose[i];
                else for (int i = 0; i < 16; ++i) a.d_pose_out[i] = a.d_prev[i];
            }
        } else if (a.d_pose_out) {
            for (int i = 0; i < 16; ++i) a.d_pose_out[i] = res.pose[i];
        }
    }
}

// One kernel per form, so the FP32 form carries none of the precision form's
// FP64 code.
template <bool kP>
__global__ void __launch_bounds__(kIcpThreads) icp_kernel(IcpArgs a) { icp_body<kP>(a, blockIdx.x, gridDim.x); }

// Scenes tracked side by side in one cooperative launch: scene s owns blocks
// [first[s], first[s + 1]) and its own barrier words and partial slots.
__global__ void __launch_bounds__(kIcpThreads) icp_batch_kernel(const IcpArgs* __restrict__ args,
                                                                const int* __restrict__ first, int n) {
    __shared__ IcpArgs sa;
    int s = 0;
    while (s + 1 < n && static_cast<int>(blockIdx.x) >= __ldg(first + s + 1)) ++s;
    const int f0 = __ldg(first + s), f1 = __ldg(first + s + 1);
    if (threadIdx.x == 0) sa = args[s];
    __syncthreads();
    if (sa.precision) icp_body<true>(sa, static_cast<int>(blockIdx.x) - f0, f1 - f0);
    else icp_body<false>(sa, static_cast<int>(blockIdx.x) - f0, f1 - f0);
}

}  // namespace azu

// ---------------------------------------------------------------------------
struct azu_tracker {
    int device = 0;
    azu_tracker_params p{};
    azu::StreamRef stream;
    float* V[3] = {nullptr, nullptr, nullptr};
    float* N[3] = {nullptr, nullptr, nullptr};
    float* D[3] = {nullptr, nullptr, nullptr};
    int W = 0, H = 0;
    bool prepared = false;
    int nblocks = 0;  // partial slots and launch grid: the SMs' resident blocks
    double* partials = nullptr;
    int* ipartials = nullptr;
    unsigned* bar = nullptr;  // [0] arrivals [1] generation [2] error [4..] published state
    float* d_est = nullptr;   // 16 estimate, 16 ref, 16 prev
    azu_icp_result* d_result = nullptr;
    float* d_build = nullptr;
    void* d_many = nullptr;   // track_many: per-candidate scratch, estimates, refs, results, launch table
    size_t many_cap = 0;      // candidates d_many is laid out for
};

namespace azu {

static azu_tracker_params sanitize(const azu_tracker_params& in) {
    azu_tracker_params p = in;
    if (!std::isfinite(p.angle_threshold)) p.angle_threshold = 30.0f;
    else if (p.angle_threshold < 0.0f) p.angle_threshold = 0.0f;
    else if (p.angle_threshold > 85.0f) p.angle_threshold = 85.0f;
    return p;
}

static int alloc_levels(azu_tracker* t, int W, int H) {
    for (int l = 0; l < 3; ++l) {
        if (t->V[l]) cudaFree(t->V[l]);
        if (t->N[l]) cudaFree(t->N[l]);
        if (t->D[l]) cudaFree(t->D[l]);
        t->V[l] = t->N[l] = t->D[l] = nullptr;
    }
    for (int l = 0; l < 3; ++l) {
        const size_t n = static_cast<size_t>(W >> l) * (H >> l);
        AZU_TRY_CUDA(cudaMalloc(&t->V[l], n * 3 * sizeof(float)));
        AZU_TRY_CUDA(cudaMalloc(&t->N[l], n * 3 * sizeof(float)));
        AZU_TRY_CUDA(cudaMalloc(&t->D[l], n * sizeof(float)));
    }
    t->W = W;
    t->H = H;
    return AZU_OK;
}

// Fills the launch arguments; the caller sets pose pointers and outputs.
static void fill_args_p(azu_tracker* t, const azu_tracker_params& p, IcpArgs& a, const float* mv, const float* mn,
                        int MW, int MH);
static void fill_args(azu_tracker* t, IcpArgs& a, const float* mv, const float* mn, int MW, int MH) {
    fill_args_p(t, t->p, a, mv, mn, MW, MH);
}
static void fill_args_p(azu_tracker* t, const azu_tracker_params& p, IcpArgs& a, const float* mv, const float* mn,
                        int MW, int MH) {
    std::memset(&a, 0, sizeof(a));
    for (int l = 0; l < 3; ++l) a.lv[l] = IcpLevel{t->V[l], t->N[l], t->W >> l, t->H >> l};
    a.mv = mv;
    a.mn = mn;
    a.MW = MW;
    a.MH = MH;
    // scaleIntrinsics (include/sensor/CameraIntrinsics.h:33-40) to the model size.
    if (MW == 640 && MH == 480) {
        a.fx = p.fx; a.fy = p.fy; a.cx = p.cx; a.cy = p.cy;
    } else {
        const float sx = static_cast<float>(MW) / 640.0f, sy = static_cast<float>(MH) / 480.0f;
        a.fx = p.fx * sx; a.fy = p.fy * sy; a.cx = (p.cx + 0.5f) * sx - 0.5f; a.cy = (p.cy + 0.5f) * sy - 0.5f;
    }
    a.dist2 = p.dist_threshold * p.dist_threshold;
    a.angle_cos = static_cast<float>(std::cos(p.angle_threshold * M_PI / 180.0f));
    for (int l = 0; l < 3; ++l) a.iters[l] = p.max_iterations[l];
    a.precision = p.precision;
    a.build_level = -1;
    a.partials = t->partials;
    a.ipartials = t->ipartials;
    a.vblocks = t->nblocks;
    a.bar = t->bar;
    a.err = t->bar + 2;
}

// Blocks per SM that both forms' kernels can keep resident (a tracker's grid
// is sized once; its form can change with its parameters).
static cudaError_t icp_occupancy(int* occ) {
    int o0 = 0, o1 = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o0, icp_kernel<false>, kIcpThreads, 0);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o1, icp_kernel<true>, kIcpThreads, 0);
    *occ = std::min(o0, o1);
    return e;
}

int icp_launch(azu_tracker* t, const IcpArgs& a, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(t->nblocks);
    cfg.blockDim = dim3(kIcpThreads);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    AZU_TRY_CUDA(cudaLaunchKernelEx(&cfg, a.precision ? icp_kernel<true> : icp_kernel<false>, a));
    return AZU_OK;
}

// Pipeline entry: track against device poses; result/grade stay on the device.
static void track_args(azu_tracker* t, const TrackDev& d, IcpArgs& a) {
    fill_args(t, a, d.mv, d.mn, d.MW, d.MH);
    a.d_estimate = d.d_estimate;
    a.d_ref = d.d_ref;
    a.d_prev = d.d_prev;
    a.d_pose_out = d.d_pose_out;
    a.d_result = d.d_result;
    a.d_quality = d.d_quality;
    a.d_gate = d.d_gate;
}

int tracker_track_dev(azu_tracker* t, const float* mv, const float* mn, int MW, int MH, const float* d_estimate,
                      const float* d_ref, const float* d_prev, float* d_pose_out, azu_icp_result* d_result,
                      int* d_quality, int* d_gate, cudaStream_t s) {
    IcpArgs a;
    track_args(t, TrackDev{mv, mn, MW, MH, d_estimate, d_ref, d_prev, d_pose_out, d_result, d_quality, d_gate}, a);
    return icp_launch(t, a, s);
}

}  // namespace azu

// Scenes tracked side by side (the batch): one cooperative launch, the
// resident blocks split evenly, each scene's ICP on its own share. Any share
// gives the sums of the scene's own tracker (its partial slots are fixed).
struct azu_icp_batch {
    int n = 0, grid = 0;
    azu::IcpArgs* d_args = nullptr;
    int* d_first = nullptr;
};

namespace azu {

void icp_batch_destroy(azu_icp_batch* b) {
    if (!b) return;
    if (b->d_args) cudaFree(b->d_args);
    if (b->d_first) cudaFree(b->d_first);
    delete b;
}

int icp_batch_create(azu_tracker* const* t, const TrackDev* d, int n, azu_icp_batch** out) {
    AZU_CHECK_ARG(t != nullptr && d != nullptr && out != nullptr && n >= 1, "null argument");
    *out = nullptr;
    int sms = 0, occ = 0;
    AZU_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, t[0]->device));
    AZU_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, icp_batch_kernel, kIcpThreads, 0));
    const int grid = sms * std::min(occ, 2);
    AZU_CHECK_ARG(grid >= n, "more scenes than resident ICP blocks");
    std::vector<IcpArgs> args(n);
    std::vector<int> first(n + 1, 0);
    for (int i = 0; i < n; ++i) {
        AZU_CHECK_ARG(t[i] != nullptr, "null tracker");
        track_args(t[i], d[i], args[i]);
        first[i + 1] = first[i] + grid / n;
    }
    azu_icp_batch* b = new azu_icp_batch();
    b->n = n;
    b->grid = first[n];
    cudaError_t e = cudaMalloc(&b->d_args, n * sizeof(IcpArgs));
    if (!e) e = cudaMalloc(&b->d_first, (n + 1) * sizeof(int));
    if (!e) e = cudaMemcpy(b->d_args, args.data(), n * sizeof(IcpArgs), cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(b->d_first, first.data(), (n + 1) * sizeof(int), cudaMemcpyHostToDevice);
    if (e) {
        set_error("icp batch: %s", cudaGetErrorString(e));
        icp_batch_destroy(b);
        return AZU_E_NOMEM;
    }
    *out = b;
    return AZU_OK;
}

int icp_batch_launch(azu_icp_batch* b, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(b->grid);
    cfg.blockDim = dim3(kIcpThreads);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    AZU_TRY_CUDA(cudaLaunchKernelEx(&cfg, icp_batch_kernel, static_cast<const IcpArgs*>(b->d_args),
                                    static_cast<const int*>(b->d_first), b->n));
    return AZU_OK;
}

int tracker_prepare_dev(azu_tracker* t, const float* d_depth, int W, int H, cudaStream_t s) {
    return launch_prepare_live(d_depth, W, H, t->p.fx, t->p.fy, t->p.cx, t->p.cy, t->V, t->N, t->D, s);
}

// Barrier words back to their initial state (arrivals, generation, error),
// ordered on stream s after the launch that used them. After a wait ran out,
// blocks that arrived before the error was set leave the arrival count
// nonzero; the next launch would then release a barrier early.
int clear_barrier_words(unsigned* bar, cudaStream_t s) {
    AZU_TRY_CUDA(cudaMemsetAsync(bar, 0, 4 * sizeof(unsigned), s));
    return AZU_OK;
}

int tracker_clear_barrier(azu_tracker* t, cudaStream_t s) { return clear_barrier_words(t->bar, s); }

}  // namespace azu

using namespace azu;

extern "C" int azu_tracker_create(int device, const azu_tracker_params* p, void* stream, azu_tracker** out) {
    AZU_CHECK_ARG(out != nullptr && p != nullptr, "null argument");
    *out = nullptr;
    for (int l = 0; l < 3; ++l) AZU_CHECK_ARG(p->max_iterations[l] >= 0 && p->max_iterations[l] <= 1000, "max_iterations");
    if (int rc = bind_device(device)) return rc;
    azu_tracker* t = new azu_tracker();
    t->device = device;
    t->p = sanitize(*p);
    int rc = t->stream.init(stream);
    int sms = 0, occ = 0;
    if (!rc) {
        cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        if (e == cudaSuccess) e = icp_occupancy(&occ);
        if (e != cudaSuccess || occ < 1) { set_error("ICP occupancy query failed"); rc = AZU_E_CUDA; }
    }
    if (!rc) {
        t->nblocks = std::min(sms * std::min(occ, 2), kMaxGridBlocks);
        cudaError_t e = cudaMalloc(&t->partials, sizeof(double) * 2 * t->nblocks * kNF);
        if (e == cudaSuccess) e = cudaMalloc(&t->ipartials, sizeof(int) * 2 * t->nblocks * kNI);
        if (e == cudaSuccess) e = cudaMalloc(&t->bar, sizeof(unsigned) * 4);
        if (e == cudaSuccess) e = cudaMemset(t->bar, 0, sizeof(unsigned) * 4);
        if (e == cudaSuccess) e = cudaMalloc(&t->d_est, sizeof(float) * 48);
        if (e == cudaSuccess) e = cudaMalloc(&t->d_result, sizeof(azu_icp_result));
        if (e == cudaSuccess) e = cudaMalloc(&t->d_build, sizeof(float) * 64);
        if (e != cudaSuccess) { set_error("tracker allocation: %s", cudaGetErrorString(e)); rc = AZU_E_NOMEM; }
    }
    if (!rc) rc = alloc_levels(t, 640, 480);
    if (rc) { azu_tracker_destroy(t); return rc; }
    *out = t;
    return AZU_OK;
}

extern "C" int azu_tracker_destroy(azu_tracker* t) {
    if (!t) return AZU_OK;
    cudaSetDevice(t->device);
    if (t->stream.s) cudaStreamSynchronize(t->stream.s);
    for (int l = 0; l < 3; ++l) { cudaFree(t->V[l]); cudaFree(t->N[l]); cudaFree(t->D[l]); }
    cudaFree(t->partials);
    cudaFree(t->ipartials);
    cudaFree(t->bar);
    cudaFree(t->d_est);
    if (t->d_many) cudaFree(t->d_many);
    cudaFree(t->d_result);
    cudaFree(t->d_build);
    t->stream.release();
    delete t;
    return AZU_OK;
}

extern "C" int azu_tracker_set_params(azu_tracker* t, const azu_tracker_params* p) {
    AZU_CHECK_ARG(t != nullptr && p != nullptr, "null argument");
    t->p = sanitize(*p);
    return AZU_OK;
}

extern "C" int azu_tracker_prepare_live(azu_tracker* t, const float* d_depth_m, int width, int height) {
    AZU_CHECK_ARG(t != nullptr && d_depth_m != nullptr, "null argument");
    AZU_CHECK_ARG(width >= 8 && height >= 8 && width % 4 == 0 && height % 4 == 0,
                  "width and height must be multiples of 4 (>= 8)");
    AZU_TRY_CUDA(cudaSetDevice(t->device));
    if (width != t->W || height != t->H) {
        AZU_TRY_CUDA(cudaStreamSynchronize(t->stream.s));
        if (int rc = alloc_levels(t, width, height)) return rc;
    }
    if (int rc = tracker_prepare_dev(t, d_depth_m, width, height, t->stream.s)) return rc;
    t->prepared = true;
    return AZU_OK;
}

extern "C" int azu_tracker_track_prepared(azu_tracker* t, int width, int height, const float* d_model_vertices,
                                          const float* d_model_normals, int model_w, int model_h,
                                          const float estimate[16], const float ref_pose[16], azu_icp_result* out) {
    AZU_CHECK_ARG(t != nullptr && d_model_vertices != nullptr && d_model_normals != nullptr && estimate != nullptr &&
                      ref_pose != nullptr && out != nullptr,
                  "null argument");
    AZU_CHECK_ARG(model_w > 0 && model_h > 0, "model size");
    if (!t->prepared || width != t->W || height != t->H) {
        set_error("track_prepared called without a matching prepare_live");
        return AZU_E_STATE;
    }
    AZU_TRY_CUDA(cudaSetDevice(t->device));
    if (int rc = set_pose_async(t->d_est, estimate, t->stream.s)) return rc;
    if (int rc = set_pose_async(t->d_est + 16, ref_pose, t->stream.s)) return rc;
    if (int rc = tracker_track_dev(t, d_model_vertices, d_model_normals, model_w, model_h, t->d_est, t->d_est + 16,
                                   nullptr, nullptr, t->d_result, nullptr, nullptr, t->stream.s))
        return rc;
    AZU_TRY_CUDA(cudaMemcpyAsync(out, t->d_result, sizeof(azu_icp_result), cudaMemcpyDeviceToHost, t->stream.s));
    AZU_TRY_CUDA(cudaStreamSynchronize(t->stream.s));
    if (out->status == AZU_E_TIMEOUT) {
        if (int rc = clear_barrier_words(t->bar, t->stream.s)) return rc;
        AZU_TRY_CUDA(cudaStreamSynchronize(t->stream.s));
        set_error("ICP grid barrier timed out");
        return AZU_E_TIMEOUT;
    }
    return AZU_OK;
}

extern "C" int azu_tracker_track_many(azu_tracker* t, int width, int height, const float* d_model_vertices,
                                      const float* d_model_normals, int model_w, int model_h, int count,
                                      const float* estimates, const float* ref_poses,
                                      const azu_tracker_params* params, azu_icp_result* out) {
    AZU_CHECK_ARG(t != nullptr && d_model_vertices != nullptr && d_model_normals != nullptr && estimates != nullptr &&
                      out != nullptr,
                  "null argument");
    AZU_CHECK_ARG(model_w > 0 && model_h > 0 && count >= 1 && count <= 4096, "model size / count");
    if (!t->prepared || width != t->W || height != t->H) {
        set_error("track_many called without a matching prepare_live");
        return AZU_E_STATE;
    }
    AZU_TRY_CUDA(cudaSetDevice(t->device));
    const azu_tracker_params p = params ? sanitize(*params) : t->p;
    cudaStream_t s = t->stream.s;
    // Layout of d_many for cap candidates (each part 256-byte aligned): the
    // candidates' own partial slots and barrier words, then estimates,
    // reference poses, results, launch arguments and block table. The scratch
    // sits first so that its barrier words keep their place between calls.
    auto up = [](size_t x) { return (x + 255) & ~static_cast<size_t>(255); };
    const size_t nb = static_cast<size_t>(t->nblocks);
    constexpr size_t kBarWords = 4;
    const size_t sz_p = up(sizeof(double) * 2 * kNF * nb), sz_i = up(sizeof(int) * 2 * kNI * nb);
    const size_t sz_b = up(sizeof(unsigned) * kBarWords), per = sz_p + sz_i + sz_b;
    if (static_cast<size_t>(count) > t->many_cap) {
        AZU_TRY_CUDA(cudaStreamSynchronize(s));
        if (t->d_many) cudaFree(t->d_many);
        t->d_many = nullptr;
        t->many_cap = 0;
        const size_t c = static_cast<size_t>(count);
        const size_t bytes = per * c + up(32 * sizeof(float) * c) + up(sizeof(azu_icp_result) * c) +
                             up(sizeof(IcpArgs) * c) + up(sizeof(int) * (c + 1));
        AZU_TRY_CUDA(cudaMalloc(&t->d_many, bytes));
        AZU_TRY_CUDA(cudaMemsetAsync(t->d_many, 0, bytes, s));  // barrier words start at zero
        t->many_cap = c;
    }
    const size_t cap = t->many_cap;
    char* base = static_cast<char*>(t->d_many);
    float* d_est = reinterpret_cast<float*>(base + per * cap);
    float* d_ref = d_est + 16 * cap;
    azu_icp_result* d_res = reinterpret_cast<azu_icp_result*>(base + per * cap + up(32 * sizeof(float) * cap));
    IcpArgs* d_args = reinterpret_cast<IcpArgs*>(reinterpret_cast<char*>(d_res) + up(sizeof(azu_icp_result) * cap));
    int* d_first = reinterpret_cast<int*>(reinterpret_cast<char*>(d_args) + up(sizeof(IcpArgs) * cap));
    auto bar_of = [&](int k) { return reinterpret_cast<unsigned*>(base + per * k + sz_p + sz_i); };
    AZU_TRY_CUDA(cudaMemcpyAsync(d_est, estimates, 16 * count * sizeof(float), cudaMemcpyHostToDevice, s));
    AZU_TRY_CUDA(cudaMemcpyAsync(d_ref, ref_poses ? ref_poses : estimates, 16 * count * sizeof(float),
                                 cudaMemcpyHostToDevice, s));
    const size_t img = static_cast<size_t>(model_w) * model_h * 3;
    // Candidates side by side in one cooperative launch, each on an equal share
    // of the resident blocks with its own slots and barrier words. The slot
    // count is the tracker's, so every solve equals track_prepared's; more
    // candidates than resident blocks run one launch after another.
    int sms = 0, occ = 0;
    AZU_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, t->device));
    AZU_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, icp_batch_kernel, kIcpThreads, 0));
    const int grid = sms * std::min(occ, 2);
    const bool side_by_side = count > 1 && count <= grid;
    std::vector<IcpArgs> args(side_by_side ? count : 0);
    std::vector<int> first(side_by_side ? count + 1 : 0, 0);
    for (int k = 0; k < count; ++k) {
        IcpArgs a;
        fill_args_p(t, p, a, d_model_vertices + img * k, d_model_normals + img * k, model_w, model_h);
        a.d_estimate = d_est + 16 * k;
        a.d_ref = d_ref + 16 * k;
        a.d_result = d_res + k;
        if (side_by_side) {
            a.partials = reinterpret_cast<double*>(base + per * k);
            a.ipartials = reinterpret_cast<int*>(base + per * k + sz_p);
            a.bar = bar_of(k);
            a.err = a.bar + 2;
            args[k] = a;
            first[k + 1] = first[k] + grid / count;
        } else if (int rc = icp_launch(t, a, s)) {
            return rc;
        }
    }
    if (side_by_side) {
        AZU_TRY_CUDA(cudaMemcpyAsync(d_args, args.data(), count * sizeof(IcpArgs), cudaMemcpyHostToDevice, s));
        AZU_TRY_CUDA(cudaMemcpyAsync(d_first, first.data(), (count + 1) * sizeof(int), cudaMemcpyHostToDevice, s));
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(first[count]);
        cfg.blockDim = dim3(kIcpThreads);
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        AZU_TRY_CUDA(cudaLaunchKernelEx(&cfg, icp_batch_kernel, static_cast<const IcpArgs*>(d_args),
                                        static_cast<const int*>(d_first), count));
    }
    AZU_TRY_CUDA(cudaMemcpyAsync(out, d_res, count * sizeof(azu_icp_result), cudaMemcpyDeviceToHost, s));
    AZU_TRY_CUDA(cudaStreamSynchronize(s));
    bool timed_out = false;
    for (int k = 0; k < count; ++k)
        if (out[k].status == AZU_E_TIMEOUT) {
            timed_out = true;
            if (int rc = clear_barrier_words(side_by_side ? bar_of(k) : t->bar, s)) return rc;
        }
    if (timed_out) {
        AZU_TRY_CUDA(cudaStreamSynchronize(s));
        set_error("ICP grid barrier timed out");
        return AZU_E_TIMEOUT;
    }
    return AZU_OK;
}

extern "C" int azu_tracker_track(azu_tracker* t, const float* d_depth_m, int width, int height,
                                 const float* d_model_vertices, const float* d_model_normals, int model_w, int model_h,
                                 const float estimate[16], const float ref_pose[16], azu_icp_result* out) {
    if (int rc = azu_tracker_prepare_live(t, d_depth_m, width, height)) return rc;
    return azu_tracker_track_prepared(t, width, height, d_model_vertices, d_model_normals, model_w, model_h, estimate,
                                      ref_pose, out);
}

extern "C" int azu_tracker_build_system(azu_tracker* t, int level, const float* d_model_vertices,
                                        const float* d_model_normals, int model_w, int model_h, const float pose[16],
                                        const float ref_pose[16], float A[36], float b[6], float* residual,
                                        int counts[6]) {
    AZU_CHECK_ARG(t != nullptr && d_model_vertices && d_model_normals && pose && ref_pose && A && b && residual &&
                      counts,
                  "null argument");
    AZU_CHECK_ARG(level >= 0 && level < 3, "level");
    if (!t->prepared) { set_error("build_system called before prepare_live"); return AZU_E_STATE; }
    AZU_TRY_CUDA(cudaSetDevice(t->device));
    if (int rc = set_pose_async(t->d_est, pose, t->stream.s)) return rc;
    if (int rc = set_pose_async(t->d_est + 16, ref_pose, t->stream.s)) return rc;
    IcpArgs a;
    fill_args(t, a, d_model_vertices, d_model_normals, model_w, model_h);
    a.d_estimate = t->d_est;
    a.d_ref = t->d_est + 16;
    a.build_level = level;
    a.build_out = t->d_build;
    if (int rc = icp_launch(t, a, t->stream.s)) return rc;
    float out[49];
    AZU_TRY_CUDA(cudaMemcpyAsync(out, t->d_build, sizeof(out), cudaMemcpyDeviceToHost, t->stream.s));
    unsigned err = 0;
    AZU_TRY_CUDA(cudaMemcpyAsync(&err, t->bar + 2, sizeof(err), cudaMemcpyDeviceToHost, t->stream.s));
    AZU_TRY_CUDA(cudaStreamSynchronize(t->stream.s));
    if (err) {
        if (int rc = clear_barrier_words(t->bar, t->stream.s)) return rc;
        AZU_TRY_CUDA(cudaStreamSynchronize(t->stream.s));
        set_error("ICP grid barrier timed out");
        return AZU_E_TIMEOUT;
    }
    std::memcpy(A, out, 36 * sizeof(float));
    std::memcpy(b, out + 36, 6 * sizeof(float));
    *residual = out[42];
    std::memcpy(counts, out + 43, 6 * sizeof(int));
    return AZU_OK;
}

extern "C" int azu_tracker_live_maps(azu_tracker* t, int level, const float** d_vertices, const float** d_normals,
                                     const float** d_depth_m) {
    AZU_CHECK_ARG(t != nullptr && level >= 0 && level < 3, "argument");
    if (d_vertices) *d_vertices = t->V[level];
    if (d_normals) *d_normals = t->N[level];
    if (d_depth_m) *d_depth_m = t->D[level];
    return AZU_OK;
}

extern "C" int azu_tracker_load_live(azu_tracker* t, int level, const float* d_vertices, const float* d_normals,
                                     int width, int height) {
    AZU_CHECK_ARG(t != nullptr && d_vertices != nullptr && d_normals != nullptr, "null argument");
    AZU_CHECK_ARG(level >= 0 && level < 3, "level");
    AZU_CHECK_ARG(width >= 8 && height >= 8 && width % 4 == 0 && height % 4 == 0,
                  "width and height must be multiples of 4 (>= 8)");
    AZU_TRY_CUDA(cudaSetDevice(t->device));
    if (width != t->W || height != t->H) {
        AZU_TRY_CUDA(cudaStreamSynchronize(t->stream.s));
        if (int rc = alloc_levels(t, width, height)) return rc;
    }
    const size_t n = static_cast<size_t>(width >> level) * (height >> level) * 3 * sizeof(float);
    AZU_TRY_CUDA(cudaMemcpyAsync(t->V[level], d_vertices, n, cudaMemcpyDeviceToDevice, t->stream.s));
    AZU_TRY_CUDA(cudaMemcpyAsync(t->N[level], d_normals, n, cudaMemcpyDeviceToDevice, t->stream.s));
    t->prepared = true;
    return AZU_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free association + reduction pass.
//
// For callers that must not allocate device memory once they run: a real-time
// tracking loop that fixes its device-memory budget at start-up, or a host whose
// device memory belongs to its own pool or arena that this library cannot draw
// from (cudaMalloc also synchronises the device, which such loops avoid). The
// caller passes the live and model maps (device) and the host outputs; the block
// partials, barrier words, poses and result staging live in one file-scope
// device array that every GPU loading the library holds until exit.
//
// Limit: the array holds partials for kStaticMaxBlocks (512) cooperative
// blocks; the launch uses one block of kIcpThreads threads per unit of
// co-resident occupancy (at most 2 per SM, 152 on a GB300), and a device that
// would need more is rejected with AZU_E_UNSUPPORTED. Images may be up to
// 8192 x 8192.
//
// The first call on a device resolves the array's device address with that
// device current; make that first call before any stream capture. Every call
// shares the one array and leaves its contents behind: the barrier words are
// cleared at the start of each call, everything else is overwritten. Calls
// that overlap on the GPU (other streams or threads) race on the array.
namespace {
constexpr int kStaticMaxBlocks = 512;
constexpr size_t kStaticScratchBytes = 256 * 1024;
constexpr size_t kOffPoses = 0;      // 32 floats: pose, ref_pose
constexpr size_t kOffOut = 256;      // 49 words: A, b, residual, counts
constexpr size_t kOffBar = 512;      // 4 words: arrivals, generation, error
constexpr size_t kOffPartials = 1024;
constexpr size_t kOffIPartials = kOffPartials + 2ull * kStaticMaxBlocks * azu::kNF * sizeof(double);
static_assert(kOffIPartials + 2ull * kStaticMaxBlocks * azu::kNI * sizeof(int) <= kStaticScratchBytes,
              "static scratch layout");
constexpr int kStaticMaxDevices = 64;
struct StaticSlot {
    unsigned char* base = nullptr;
    int nblocks = 0;
};
std::mutex g_static_mu;
StaticSlot g_static_slot[kStaticMaxDevices];
}  // namespace

static __device__ __align__(256) unsigned char g_icp_static_scratch[kStaticScratchBytes];

static int static_slot_for_current_device(StaticSlot& out) {
    int dev = -1;
    AZU_TRY_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kStaticMaxDevices) {
        set_error("device ordinal %d beyond the %d supported", dev, kStaticMaxDevices);
        return AZU_E_UNSUPPORTED;
    }
    std::lock_guard<std::mutex> lk(g_static_mu);
    StaticSlot& s = g_static_slot[dev];
    if (!s.base) {
        cudaDeviceProp prop;
        AZU_TRY_CUDA(cudaGetDeviceProperties(&prop, dev));
        if (prop.major * 10 + prop.minor != 103) {
            set_error("device %d is sm_%d%d; this library is built for sm_103a (GB300) only", dev, prop.major,
                      prop.minor);
            return AZU_E_UNSUPPORTED;
        }
        void* p = nullptr;
        AZU_TRY_CUDA(cudaGetSymbolAddress(&p, g_icp_static_scratch));
        int occ = 0;
        AZU_TRY_CUDA(icp_occupancy(&occ));
        s.nblocks = std::min(prop.multiProcessorCount * std::min(occ, 2), azu::kMaxGridBlocks);
        s.base = static_cast<unsigned char*>(p);
    }
    out = s;
    return AZU_OK;
}

extern "C" int azu_icp_build_system_noalloc(const float* d_live_vertices, const float* d_live_normals, int width,
                                            int height, const float* d_model_vertices, const float* d_model_normals,
                                            int model_w, int model_h, const azu_tracker_params* params,
                                            const float pose[16], const float ref_pose[16], void* stream,
                                            float A[36], float b[6], float* residual, int counts[6]) {
    AZU_CHECK_ARG(d_live_vertices && d_live_normals && d_model_vertices && d_model_normals && params && pose &&
                      ref_pose && A && b && residual && counts,
                  "null argument");
    AZU_CHECK_ARG(width >= 3 && height >= 3 && width <= 8192 && height <= 8192, "live size must be in [3, 8192]");
    AZU_CHECK_ARG(model_w > 0 && model_h > 0 && model_w <= 8192 && model_h <= 8192,
                  "model size must be in [1, 8192]");
    StaticSlot slot;
    if (int rc = static_slot_for_current_device(slot)) return rc;
    if (slot.nblocks > kStaticMaxBlocks) {
        set_error("this device needs partials for %d blocks; the static scratch holds %d", slot.nblocks,
                  kStaticMaxBlocks);
        return AZU_E_UNSUPPORTED;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    float* d_poses = reinterpret_cast<float*>(slot.base + kOffPoses);
    float* d_out = reinterpret_cast<float*>(slot.base + kOffOut);
    unsigned* d_bar = reinterpret_cast<unsigned*>(slot.base + kOffBar);
    if (int rc = set_pose_async(d_poses, pose, s)) return rc;
    if (int rc = set_pose_async(d_poses + 16, ref_pose, s)) return rc;
    AZU_TRY_CUDA(cudaMemsetAsync(d_bar, 0, 4 * sizeof(unsigned), s));

    const azu_tracker_params p = sanitize(*params);
    IcpArgs a;
    std::memset(&a, 0, sizeof(a));
    for (int l = 0; l < 3; ++l) a.lv[l] = IcpLevel{d_live_vertices, d_live_normals, width, height};
    a.mv = d_model_vertices;
    a.mn = d_model_normals;
    a.MW = model_w;
    a.MH = model_h;
    if (model_w == 640 && model_h == 480) {
        a.fx = p.fx; a.fy = p.fy; a.cx = p.cx; a.cy = p.cy;
    } else {
        const float sx = static_cast<float>(model_w) / 640.0f, sy = static_cast<float>(model_h) / 480.0f;
        a.fx = p.fx * sx; a.fy = p.fy * sy; a.cx = (p.cx + 0.5f) * sx - 0.5f; a.cy = (p.cy + 0.5f) * sy - 0.5f;
    }
    a.dist2 = p.dist_threshold * p.dist_threshold;
    a.angle_cos = static_cast<float>(std::cos(p.angle_threshold * M_PI / 180.0f));
    for (int l = 0; l < 3; ++l) a.iters[l] = p.max_iterations[l];
    a.precision = p.precision;
    a.build_level = 0;
    a.d_estimate = d_poses;
    a.d_ref = d_poses + 16;
    a.partials = reinterpret_cast<double*>(slot.base + kOffPartials);
    a.ipartials = reinterpret_cast<int*>(slot.base + kOffIPartials);
    a.vblocks = slot.nblocks;
    a.bar = d_bar;
    a.err = d_bar + 2;
    a.build_out = d_out;

    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(slot.nblocks);
    cfg.blockDim = dim3(kIcpThreads);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    AZU_TRY_CUDA(cudaLaunchKernelEx(&cfg, a.precision ? icp_kernel<true> : icp_kernel<false>, a));
    float out[49];
    unsigned err = 0;
    AZU_TRY_CUDA(cudaMemcpyAsync(out, d_out, sizeof(out), cudaMemcpyDeviceToHost, s));
    AZU_TRY_CUDA(cudaMemcpyAsync(&err, d_bar + 2, sizeof(err), cudaMemcpyDeviceToHost, s));
    AZU_TRY_CUDA(cudaStreamSynchronize(s));
    if (err) {
        set_error("ICP grid barrier timed out");
        return AZU_E_TIMEOUT;
    }
    std::memcpy(A, out, 36 * sizeof(float));
    std::memcpy(b, out + 36, 6 * sizeof(float));
    *residual = out[42];
    std::memcpy(counts, out + 43, 6 * sizeof(int));
    return AZU_OK;
}

// ---------------------------------------------------------------------------
// Testing hook: the wait limits every ICP launch on the current device reads
// at its start (see WaitLimits). Lets a test make a barrier wait run out on
// purpose, through the bounded path only: no wait is left unbounded.
extern "C" int azu_testing_set_icp_wait(unsigned spin_limit, unsigned extra_arrivals) {
    AZU_CHECK_ARG(extra_arrivals <= 1024, "extra_arrivals");
    const unsigned spins = spin_limit ? spin_limit : azu::kSpinLimit;
    AZU_TRY_CUDA(cudaMemcpyToSymbol(azu::g_icp_spin_limit, &spins, sizeof(spins)));
    AZU_TRY_CUDA(cudaMemcpyToSymbol(azu::g_icp_extra_arrivals, &extra_arrivals, sizeof(extra_arrivals)));
    return AZU_OK;
}
