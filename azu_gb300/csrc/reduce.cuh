// Deterministic warp reductions shared by the ICP reduction (icp.cu) and the
// differentiable renderer (diff.cu).
#pragma once

namespace azu {

// Warp sum of 32 values per lane by recursive halving: at offset o each lane
// keeps half of its values, adds the partner's copy of that half and hands it
// the other half. After five steps lane l holds the warp sum of value l
// (31 shuffles instead of 32 x 5). Fixed pattern, so deterministic.
template <typename T>
__device__ __forceinline__ T warp_sum_transpose32(T (&v)[32], int lane) {
#pragma unroll
    for (int lvl = 0; lvl < 5; ++lvl) {
        const int o = 16 >> lvl, n = 16 >> lvl;
        const bool upper = (lane & o) != 0;
#pragma unroll
        for (int i = 0; i < n; ++i) {
            const T send = upper ? v[i] : v[i + n];
            const T keep = upper ? v[i + n] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
    return v[0];
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace azu
