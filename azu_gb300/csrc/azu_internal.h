// Internal declarations shared by the translation units of libazu_gb300.so.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/azu_gpu.h"

struct azu_icp_batch;  // scenes tracked side by side (icp.cu)

namespace azu {

// Thread-local last-error text behind azu_last_error().
void set_error(const char* fmt, ...);

#define AZU_TRY_CUDA(expr)                                                                       \
    do {                                                                                         \
        cudaError_t e_ = (expr);                                                                 \
        if (e_ != cudaSuccess) {                                                                 \
            ::azu::set_error("%s failed at %s:%d: %s", #expr, __FILE__, __LINE__,                \
                             cudaGetErrorString(e_));                                            \
            return e_ == cudaErrorMemoryAllocation ? AZU_E_NOMEM : AZU_E_CUDA;                   \
        }                                                                                        \
    } while (0)

#define AZU_CHECK_ARG(cond, msg)                                                                 \
    do {                                                                                         \
        if (!(cond)) {                                                                           \
            ::azu::set_error("invalid argument: %s", msg);                                       \
            return AZU_E_INVALID;                                                                \
        }                                                                                        \
    } while (0)

#define AZU_LAUNCH_CHECK() AZU_TRY_CUDA(cudaGetLastError())

// Makes `device` current and checks that it is an sm_103 part.
int bind_device(int device);

// Stream owned or borrowed by a handle.
struct StreamRef {
    cudaStream_t s = nullptr;
    bool owned = false;
    int init(void* user) {
        if (user) { s = static_cast<cudaStream_t>(user); owned = false; return AZU_OK; }
        AZU_TRY_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        owned = true;
        return AZU_OK;
    }
    void release() {
        if (owned && s) cudaStreamDestroy(s);
        s = nullptr;
        owned = false;
    }
};

// Error word written by bounded device-side waits (ICP grid barrier).
enum : uint32_t { kDevErrNone = 0, kDevErrBarrierTimeout = 1 };

// ---- volume -------------------------------------------------------------
struct IntegrateConsts {
    float R_wc[9];
    float t_wc[3];
    float step_x[3];
    int x0, x1, y0, y1, z0, z1;
    int valid;
    // chunk culling: a stepped coordinate lies within cull_eps of its chunk's
    // line; cull_off = trunc + cull_eps + slack; voxels nearer than z_safe are
    // never culled
    float cull_eps, cull_off, z_safe;
    // brick pre-cull: a stepped coordinate lies within brick_eps of the exact
    // affine one anywhere on its row; brick_off = trunc + brick_eps + slack
    float brick_eps, brick_off;
};

// Tile-max pyramid over the depth image: level l tiles are 8 * 2^l pixels
// square, stored level after level from offset off[l].
constexpr int kMaxTileLevels = 12;
constexpr int kMaxTilePixels = 8 << (kMaxTileLevels - 1);
struct TileMip {
    int levels, total;
    int w[kMaxTileLevels], h[kMaxTileLevels], off[kMaxTileLevels];
};

struct RaycastConsts {
    float R_cw[9];
    float o[3];
};

}  // namespace azu

struct azu_volume {
    int device = 0;
    azu_volume_params p{};
    azu::StreamRef stream;
    void* vox = nullptr;        // float2 (FP32) or uint32 (FP16) per voxel
    float* color = nullptr;     // 3 floats per voxel when p.color
    float* d_pose = nullptr;    // 16 floats: pose slot for host-pose calls
    azu::IntegrateConsts* d_iconsts = nullptr;
    unsigned long long* d_counters = nullptr;  // [0] newly observed (cumulative), [1] updated (last), [2] colour (last),
                                               // [3] updated (cumulative), [4] integrate work counter,
                                               // [5 .. 5 + kIntBuckets) sizes of the integrate work buckets
    int int_blocks = 0;                        // resident blocks of the persistent integrate kernel
    // One bit per 8^3 brick that the frame being integrated may update, rows
    // of nb bricks along x in 32-bit words (int_live_words per row), rows in
    // (z, y) order: written by the brick pre-cull before every integration.
    uint32_t* int_live = nullptr;
    int int_live_words = 0;
    // The items of the integration that the pre-cull keeps, in kIntBuckets
    // buckets by their kept-brick count (bucket b of n_items slots at
    // int_list + b * n_items), taken heaviest first.
    int* int_list = nullptr;
    float* d_depth_stage = nullptr;            // host-depth staging (integrate_host)
    uint8_t* d_rgb_stage = nullptr;
    size_t stage_pixels = 0;
    int integrated_frames = 0;
    // Free-space bricks of 8^3 voxels (plus a 1-voxel apron): 1 when every voxel
    // in [8b, 8b+8]^3 is unobserved or has tsdf >= kFreeTsdf. Conservative: set
    // on reset and rebuilt from the volume after an upload; integration only
    // clears flags.
    uint8_t* bricks = nullptr;
    // Capped Chebyshev distance of every brick to the nearest brick that is
    // not free, recomputed from the flags before each raycast.
    uint8_t* brick_dist = nullptr;
    int nb = 0;
    bool skip_free = true;
    // Ray start map of the raycast: per 8x8 pixel tile a lower bound of the
    // distance from the camera to every brick that is not free and projects
    // into the tile (float bits, atomicMin), then one word that bounds every
    // tile (bricks across the camera plane).
    uint32_t* ray_start = nullptr;
    size_t ray_start_cap = 0;
    // Deepest in-band depth per 8x8 pixel tile of the frame being integrated.
    float* d_tiles = nullptr;
    size_t tile_cap = 0;
    // Differentiable rendering: per-block partials + sums + overflow counter.
    double* d_diff = nullptr;
    size_t diff_cap = 0;
};

namespace azu {
size_t voxel_bytes(int format);
// Exact free-brick flags recomputed from the voxels.
int rebuild_bricks(azu_volume* v, cudaStream_t s);
// Enqueue helpers shared with the pipeline (pose read from device memory).
// d_tiles_built: the depth map's tile pyramid from volume_build_tiles_dev, or
// null to build it here into the volume's own buffer.
int volume_integrate_dev(azu_volume* v, const float* d_depth_m, const uint8_t* d_rgb, const float* d_pose,
                         float fx, float fy, float cx, float cy, int W, int H, float min_d, float max_d,
                         const int* d_gate, cudaStream_t s, const float* d_tiles_built = nullptr);
int volume_build_tiles_dev(const float* d_depth_m, int W, int H, float min_d, float max_d, float* tiles,
                           cudaStream_t s);
TileMip make_tile_mip(int W, int H);
int volume_raycast_dev(azu_volume* v, const float* d_pose, float fx, float fy, float cx, float cy, int W, int H,
                       float* d_vertices, float* d_normals, uint8_t* d_colors, const int* d_gate, cudaStream_t s);
// Writes a host pose into a device slot with a by-value kernel argument.
int set_pose_async(float* d_pose, const float* pose, cudaStream_t s);

// What a batch needs to integrate and raycast one pipeline's frame.
struct PipelineFrameView {
    azu_volume* vol;
    const float* d_depth_m;
    const float* d_pose;
    const int* d_gate;
    int W, H;
    float fx, fy, cx, cy, min_d, max_d;
    float* d_vertices;
    float* d_normals;
};
int pipeline_create_on(int device, const azu_pipeline_params* p, cudaStream_t stream, azu_pipeline** out);
int pipeline_upload_inputs(azu_pipeline* pl, const uint16_t* depth, const uint8_t* rgb, cudaMemcpyKind kind);
int pipeline_enqueue_front(azu_pipeline* pl, bool first);
int pipeline_enqueue_front_on(azu_pipeline* pl, bool first, cudaStream_t s);
// The device buffers one pipeline frame's tracking reads and writes.
struct TrackDev {
    const float* mv;
    const float* mn;
    int MW, MH;
    const float* d_estimate;
    const float* d_ref;
    const float* d_prev;
    float* d_pose_out;
    azu_icp_result* d_result;
    int* d_quality;
    int* d_gate;
};
int icp_batch_create(azu_tracker* const* t, const TrackDev* d, int n, azu_icp_batch** out);
void icp_batch_destroy(azu_icp_batch* b);
int icp_batch_launch(azu_icp_batch* b, cudaStream_t s);
TrackDev pipeline_track_dev(azu_pipeline* pl);
int pipeline_enqueue_input_on(azu_pipeline* pl, cudaStream_t s);
int pipeline_enqueue_track_on(azu_pipeline* pl, bool first, cudaStream_t s);
int pipeline_enqueue_commit(azu_pipeline* pl);
int pipeline_read_result(azu_pipeline* pl, azu_frame_result* out);
// Resets the tracker's barrier words on stream s (after a wait ran out).
int tracker_clear_barrier(azu_tracker* t, cudaStream_t s);
PipelineFrameView pipeline_frame_view(azu_pipeline* pl);
}  // namespace azu

struct azu_volume_batch;
namespace azu {
// Several volumes integrated / raycast with one launch per stage (FP32, no colour).
int volume_batch_create(const PipelineFrameView* views, int n, azu_volume_batch** out);
void volume_batch_destroy(azu_volume_batch* b);
int volume_batch_set_shapes(azu_volume_batch* b, int int_warps, int int_parts, int ray_w, int ray_h);
void volume_batch_shapes(const azu_volume_batch* b, int* int_warps, int* int_parts, int* ray_w, int* ray_h);
int volume_batch_integrate(azu_volume_batch* b, cudaStream_t s);
int volume_batch_raycast(azu_volume_batch* b, cudaStream_t s);
}  // namespace azu
