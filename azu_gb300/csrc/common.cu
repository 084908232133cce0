// Shared host-side plumbing of the C ABI: error text, device binding, GPU
// selection (src/app/GpuSelect_cuda.cu:18-71 counterpart).
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "azu_internal.h"

namespace azu {

namespace {
thread_local char g_err[512] = "";
}

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int bind_device(int device) {
    int n = 0;
    AZU_TRY_CUDA(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) {
        set_error("device %d out of range (%d devices)", device, n);
        return AZU_E_INVALID;
    }
    cudaDeviceProp prop;
    AZU_TRY_CUDA(cudaGetDeviceProperties(&prop, device));
    if (prop.major * 10 + prop.minor != 103) {
        set_error("device %d is sm_%d%d; this library is built for sm_103a (GB300) only", device, prop.major,
                  prop.minor);
        return AZU_E_UNSUPPORTED;
    }
    AZU_TRY_CUDA(cudaSetDevice(device));
    return AZU_OK;
}

}  // namespace azu

extern "C" const char* azu_last_error(void) { return azu::g_err; }

extern "C" const char* azu_version(void) { return "azu_gb300 0.1 (sm_103a)"; }

extern "C" int azu_select_device(size_t min_free_bytes, int* device) {
    AZU_CHECK_ARG(device != nullptr, "device is null");
    int n = 0;
    AZU_TRY_CUDA(cudaGetDeviceCount(&n));
    int best = -1;
    size_t best_free = 0;
    for (int d = 0; d < n; ++d) {
        cudaDeviceProp prop;
        if (cudaGetDeviceProperties(&prop, d) != cudaSuccess) continue;
        if (prop.major * 10 + prop.minor != 103) continue;
        if (cudaSetDevice(d) != cudaSuccess) continue;
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) continue;
        if (fr >= min_free_bytes && fr > best_free) {
            best = d;
            best_free = fr;
        }
    }
    if (best < 0) {
        azu::set_error("no sm_103 device with %zu bytes free", min_free_bytes);
        return AZU_E_UNSUPPORTED;
    }
    *device = best;
    return AZU_OK;
}
