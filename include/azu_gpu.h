/* azu_gpu.h — C ABI of the GB300 KinectFusion backend (libazu_gb300.so).
 *
 * The reference (iphands/azu) selects its GPU path at run time through
 * `--backend cuda` and `#ifdef CUDA_ENABLED` member functions of four classes:
 * sensor::Preprocessor, tracking::ICPTracker, tsdf::TSDFVolume and
 * meshing::MarchingCubes. Each entry point below replaces one of those member
 * functions; the comment names the file:line of the reference declaration. A
 * C++ adapter in the reference keeps its class and forwards to these calls.
 *
 * Conventions
 *  - Every function returns an int status: AZU_OK (0) or a negative AZU_E_*
 *    code; nothing throws across the ABI. azu_last_error() describes the last
 *    failure on the calling thread.
 *  - Handles own their device memory. Work is ordered on the handle's stream
 *    (the `stream` argument at creation, a cudaStream_t; NULL makes a private
 *    non-blocking stream). Calls that return results to the host synchronise
 *    that stream; the others only enqueue.
 *  - Poses are row-major float[16], world-from-camera (element (r, c) at
 *    [4 r + c]); Eigen's Matrix4f::data() is column-major, so an adapter passes
 *    the transpose.
 *  - Vertex / normal maps are float[3 * W * H] (packed float3 per pixel, the
 *    reference's float3 device maps), colours uint8[3 * W * H].
 *  - Images are row-major, W = 640, H = 480 at level 0.
 *  - "d_" pointers are device memory; "h_" pointers are host memory.
 */
#ifndef AZU_GPU_H
#define AZU_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    AZU_OK = 0,
    AZU_E_INVALID = -1,      /* bad argument (null handle, size, parameter) */
    AZU_E_CUDA = -2,         /* CUDA runtime error */
    AZU_E_NOMEM = -3,        /* device allocation failed */
    AZU_E_TIMEOUT = -4,      /* a bounded device-side wait gave up */
    AZU_E_UNSUPPORTED = -5,  /* no sm_103 device, or feature not built */
    AZU_E_STATE = -6         /* call out of order (e.g. track before prepare) */
};

const char* azu_last_error(void);
/* Library version string. */
const char* azu_version(void);

/* GPU selection (src/app/GpuSelect_cuda.cu:18-71 selectCudaDevice): picks the
 * sm_103 device with the most free memory that has at least `min_free_bytes`
 * free; returns its ordinal in *device. */
int azu_select_device(size_t min_free_bytes, int* device);

/* ------------------------------------------------------------------------ */
/* TSDF volume — tsdf::TSDFVolume (include/tsdf/TSDFVolume.h:69-190).        */
/* ------------------------------------------------------------------------ */

typedef struct azu_volume azu_volume;

enum { AZU_TSDF_FP32 = 0, AZU_TSDF_FP16 = 1, AZU_TSDF_FP16R = 2 };

typedef struct {
    int   resolution;   /* voxels per axis (TSDFParams::resolution) */
    float voxel_size;   /* metres */
    float truncation;   /* metres */
    float max_weight;
    float origin[3];    /* world position of voxel (0,0,0) */
    float min_depth;    /* raycast band, camera Z-depth (TSDFParams::min_depth) */
    float max_depth;    /* TSDFParams::max_depth */
    int   format;       /* AZU_TSDF_FP32: float tsdf + float weight (8 B/voxel);
                           AZU_TSDF_FP16: half tsdf + uint16 weight (4 B/voxel);
                           AZU_TSDF_FP16R: half tsdf + a 16-bit word holding the
                             weight (7 bits, max_weight <= 127) and a 9-bit residual
                             of the tsdf below half precision, which only the
                             integration fold reads (4 B/voxel). Readers (raycast,
                             marching cubes) see the half tsdf in both FP16 formats;
                             download returns the half tsdf plus residual. */
    int   color;        /* nonzero: keep float sRGB colour per voxel (12 B/voxel) */
} azu_volume_params;

/* Constructor + TSDFVolume::initGPU (TSDFVolume.h:141): allocates the volume on
 * `device` and resets it (tsdf 1, weight 0, colour 128/255). */
int azu_volume_create(int device, const azu_volume_params* p, void* stream, azu_volume** out);
/* TSDFVolume::freeGPU + destructor. */
int azu_volume_destroy(azu_volume* v);
/* TSDFVolume::reset (TSDFVolume.h:120). */
int azu_volume_reset(azu_volume* v);
/* TSDFVolume::setParams (TSDFVolume.h:82-85): any change clears the volume; a
 * resolution or format change reallocates. */
int azu_volume_set_params(azu_volume* v, const azu_volume_params* p);
int azu_volume_get_params(const azu_volume* v, azu_volume_params* p);

/* TSDFVolume::integrateGPU (TSDFVolume.h:145-153): voxel-projective update from
 * a device depth map in metres (d_rgb may be NULL). Enqueue only. */
int azu_volume_integrate(azu_volume* v, const float* d_depth_m, const uint8_t* d_rgb, const float pose[16],
                         float fx, float fy, float cx, float cy, int width, int height, float min_depth,
                         float max_depth);
/* TSDFVolume::integrate (TSDFVolume.h:92-100) with GPU enabled: host depth (and
 * optional host rgb) copied to the device, then integrateGPU. Enqueue only
 * (the host buffers are read before return). */
int azu_volume_integrate_host(azu_volume* v, const float* h_depth_m, const uint8_t* h_rgb, const float pose[16],
                              float fx, float fy, float cx, float cy, int width, int height, float min_depth,
                              float max_depth);
/* TSDFVolume::raycastGPU (TSDFVolume.h:154-158): model vertex/normal (and
 * optional colour) maps in world coordinates into device buffers. Misses are
 * zero. Enqueue only. */
int azu_volume_raycast(azu_volume* v, const float pose[16], float fx, float fy, float cx, float cy, int width,
                       int height, float* d_vertices, float* d_normals, uint8_t* d_colors);

typedef struct {
    int     integrated_frames;   /* TSDFVolume::integratedFrames */
    int64_t observed_voxels;     /* voxels first observed since reset (observedFraction numerator) */
    int64_t last_voxels_updated; /* voxels updated by the last integrate */
    int64_t last_color_updates;
    int64_t voxels;              /* res^3 */
    int64_t total_voxels_updated; /* voxel updates since reset (sum over integrations) */
} azu_volume_stats;
/* Synchronises the volume's stream. */
int azu_volume_get_stats(azu_volume* v, azu_volume_stats* s);

/* TSDFVolume::syncFromGPU / syncToGPU (TSDFVolume.h:143-144): whole-volume
 * copies as separate float arrays of res^3 (colour: 3 res^3, may be NULL).
 * FP16 volumes convert on the device. Synchronous. */
int azu_volume_download(azu_volume* v, float* h_tsdf, float* h_weight, float* h_color);
int azu_volume_upload(azu_volume* v, const float* h_tsdf, const float* h_weight, const float* h_color);
/* Free-space skipping (on by default): the raycast does not load samples whose
 * 8 corners are all unobserved or at tsdf >= 0.9995, and the marching cubes do
 * not read tiles of such bricks; results are identical either way. For A/B
 * timing. */
int azu_volume_set_free_space_skipping(azu_volume* v, int on);
/* TSDFVolume::getGPUVoxels (TSDFVolume.h:163): device voxel array (float2
 * {tsdf, weight} for FP32, uint32 {half, u16} for FP16). The free-space flags
 * follow integrate, upload and reset; a caller that writes voxels through this
 * pointer calls azu_volume_voxels_changed afterwards (on the volume's stream
 * order), or turns free-space skipping off. */
void* azu_volume_device_voxels(azu_volume* v);
/* Recomputes the free-space flags from the voxels (stream-ordered). No
 * reference counterpart: the reference's CPU and GPU paths keep no such flags. */
int azu_volume_voxels_changed(azu_volume* v);

/* The relocaliser's candidate renders (PipelineController::renderModel,
 * src/app/PipelineController.cpp:619-657, called per candidate by
 * tracking::Relocalizer, include/tracking/Relocalizer.h): count raycasts of
 * this volume at the host poses (16 floats each) into device images
 * d_vertices / d_normals of count * width * height * 3 floats, in one launch;
 * each image equals azu_volume_raycast's at that pose. Intrinsics are those of
 * the render size (the caller scales them, as scaleIntrinsics does). */
int azu_volume_raycast_many(azu_volume* v, const float* poses, int count, float fx, float fy, float cx, float cy,
                            int width, int height, float* d_vertices, float* d_normals);

/* TSDFVolume::extractGlobalPointCloud (TSDFVolume.cpp:571-632): voxels with
 * weight > 1 and |tsdf| < 0.2 whose colour quantises, in index order (z, y, x),
 * as world positions origin + (x, y, z) * voxel_size (3 floats) and sRGB bytes
 * (3 per point; 128 grey without colour). With h_points and h_colors NULL only
 * the count is returned; else capacity (points) must hold them all. */
int azu_volume_point_cloud(azu_volume* v, float* h_points, uint8_t* h_colors, int64_t capacity, int64_t* n_points);

/* ---- differentiation form (no counterpart in the reference) ------------ */
/* Depth image of the raycast at `pose` (camera z of the hit, metres; 0 where
 * the raycast returns no vertex): d_depth is a device float[width*height]. */
int azu_volume_render_depth(azu_volume* v, const float pose[16], float fx, float fy, float cx, float cy, int width,
                            int height, float* d_depth);
/* Huber loss sum_i rho(D_i - obs_i) over pixels whose raycast hits and whose
 * observed depth (device d_depth_obs, metres) lies in the raycast band, and
 * its adjoint: the pose gradient is with respect to xi of pose * Exp(xi), xi =
 * (rho, omega). Marching positions are recomputed in the backward pass.
 * sums (host, 35 doubles): [0] loss, [1..6] dL/dxi, [7..27] sum w J J^T
 * (upper triangle, row major), [28..33] sum w J r, [34] pixel count, with J =
 * dD/dxi and IRLS weights w = min(1, delta/|r|). Optional device outputs:
 * d_depth (float[W*H]), d_jacobian (float[6*W*H], dD/dxi per pixel),
 * d_grad_tsdf (float[res^3], dL/dtsdf ADDED to its contents). chain_overflow
 * (host, optional) counts pixels whose chain of f-dependent steps was longer
 * than the 24 the reverse sweep keeps at a time (their older steps are
 * recovered by marching the ray again; every term is kept). */
int azu_volume_depth_backward(azu_volume* v, const float pose[16], float fx, float fy, float cx, float cy,
                              int width, int height, const float* d_depth_obs, float huber_delta, float* d_depth,
                              float* d_jacobian, float* d_grad_tsdf, double sums[35], unsigned* chain_overflow);
/* Render-and-compare pose refinement: Levenberg-Marquardt on the IRLS
 * Gauss-Newton system of the Huber depth loss from pose_in, at most
 * max_iterations accepted steps. loss_trace (host, optional, max_iterations+1
 * doubles) receives the loss after each accepted step. */
int azu_volume_refine_pose(azu_volume* v, const float pose_in[16], float fx, float fy, float cx, float cy, int width,
                           int height, const float* d_depth_obs, float huber_delta, int max_iterations,
                           float pose_out[16], double* loss_trace, int* iterations);

/* ------------------------------------------------------------------------ */
/* ICP tracker — tracking::ICPTracker (include/tracking/ICPTracker.h:80-126). */
/* ------------------------------------------------------------------------ */

typedef struct azu_tracker azu_tracker;

typedef struct {
    int   max_iterations[3]; /* per level 0,1,2 (ICPParams: {10, 5, 4}) */
    float dist_threshold;    /* metres */
    float angle_threshold;   /* degrees, sanitised to [0, 85] like setParams */
    float min_depth, max_depth;
    float fx, fy, cx, cy;    /* camera intrinsics at 640x480 (setIntrinsics) */
    int   precision;         /* 0: FP32 reduction + FP32 solve (reference semantics);
                                1: compensated FP32 per-block sums, float-float
                                cross-block sum, FP64 LDL^T solve and SE(3) update */
} azu_tracker_params;

/* Mirrors ICPResult (ICPTracker.h:27-47); pose row-major. */
typedef struct {
    float pose[16];
    float error;
    int   inliers;
    int   converged;
    int   tracking_ok;
    float final_step;
    float information[36];
    int   valid_live_points, valid_model_points, projected_points, dist_filtered, angle_filtered;
    int   iterations[3];     /* accepted solves per level */
    int   status;            /* AZU_OK or AZU_E_TIMEOUT from the device */
} azu_icp_result;

/* initGPU (ICPTracker.h:114). */
int azu_tracker_create(int device, const azu_tracker_params* p, void* stream, azu_tracker** out);
/* freeGPU (ICPTracker.h:115). */
int azu_tracker_destroy(azu_tracker* t);
int azu_tracker_set_params(azu_tracker* t, const azu_tracker_params* p);
/* prepareLiveGPU (ICPTracker.h:101): vertices, normals and the 3-level
 * jump-guarded pyramid from a device depth map in metres (band-gated, 0 =
 * invalid). Enqueue only. */
int azu_tracker_prepare_live(azu_tracker* t, const float* d_depth_m, int width, int height);
/* trackPreparedGPU (ICPTracker.h:102-106): coarse-to-fine ICP against a model
 * image (device float3 maps of model_w x model_h, raycast at ref_pose). The
 * whole solve runs in one persistent kernel; synchronises and fills *out. */
int azu_tracker_track_prepared(azu_tracker* t, int width, int height, const float* d_model_vertices,
                               const float* d_model_normals, int model_w, int model_h, const float estimate[16],
                               const float ref_pose[16], azu_icp_result* out);
/* The relocaliser's candidate scoring (Relocalizer's solve hook, i.e.
 * ICPTracker::trackPreparedGPU, include/tracking/ICPTracker.h:104-113, once
 * per candidate): count solves of the prepared live frame, solve k against
 * model image k (model_w * model_h * 3 floats apart in d_model_vertices /
 * d_model_normals) from estimates[k] with reference pose ref_poses[k] (NULL:
 * the estimates), with `params` (NULL: the tracker's) — e.g. the coarse
 * stage's level-2-only iterations and wider gates. The solves run side by side
 * in one cooperative launch on the tracker's stream (one after another when
 * count exceeds the GPU's resident ICP blocks), each bit-identical to
 * track_prepared; results (count, host) are read back once. */
int azu_tracker_track_many(azu_tracker* t, int width, int height, const float* d_model_vertices,
                           const float* d_model_normals, int model_w, int model_h, int count, const float* estimates,
                           const float* ref_poses, const azu_tracker_params* params, azu_icp_result* out);
/* trackGPU (ICPTracker.h:94-100) = prepare_live + track_prepared. */
int azu_tracker_track(azu_tracker* t, const float* d_depth_m, int width, int height, const float* d_model_vertices,
                      const float* d_model_normals, int model_w, int model_h, const float estimate[16],
                      const float ref_pose[16], azu_icp_result* out);
/* One association + reduction pass (ICPTracker::buildLinearSystem,
 * src/tracking/ICPTracker.cpp:136-354) at a pyramid level, for parity checks:
 * A (36, row-major), b (6), residual, counts {inliers, valid_live, valid_model,
 * projected, dist_filtered, angle_filtered}. Synchronous. */
int azu_tracker_build_system(azu_tracker* t, int level, const float* d_model_vertices, const float* d_model_normals,
                             int model_w, int model_h, const float pose[16], const float ref_pose[16], float A[36],
                             float b[6], float* residual, int counts[6]);
/* Loads a prebuilt live pyramid level (device float3 vertex and normal maps of
 * (width >> level) x (height >> level)), the GPU counterpart of handing
 * ICPTracker::track a FramePyramid built elsewhere (ICPTracker.h:89-92). Marks
 * the tracker prepared for width x height. Enqueue only. */
int azu_tracker_load_live(azu_tracker* t, int level, const float* d_vertices, const float* d_normals, int width,
                          int height);
/* No counterpart in the reference. The association + reduction pass of
 * azu_tracker_build_system for callers that must not allocate device memory
 * once they run (a real-time loop with a device-memory budget fixed at
 * start-up, or a host whose device memory belongs to its own pool): it needs
 * no handle and calls no cudaMalloc. Live maps (width x height) and model maps
 * are device float3 maps; poses and outputs are host memory; `stream` may be
 * NULL (the legacy default stream). Its scratch is one file-scope device array
 * of 256 KiB (partials for at most 512 cooperative blocks) that every GPU
 * loading the library keeps until exit; a device needing more blocks is
 * rejected with AZU_E_UNSUPPORTED, images larger than 8192 x 8192 with
 * AZU_E_INVALID. The first call on a device sets the array up (with that
 * device current) and should come before any stream capture. All calls share
 * the array: calls that overlap on the GPU race. Synchronous. */
int azu_icp_build_system_noalloc(const float* d_live_vertices, const float* d_live_normals, int width, int height,
                                 const float* d_model_vertices, const float* d_model_normals, int model_w,
                                 int model_h, const azu_tracker_params* params, const float pose[16],
                                 const float ref_pose[16], void* stream, float A[36], float b[6], float* residual,
                                 int counts[6]);
/* Device pointers of the live pyramid (float3 maps and depth) at a level. */
int azu_tracker_live_maps(azu_tracker* t, int level, const float** d_vertices, const float** d_normals,
                          const float** d_depth_m);

/* ------------------------------------------------------------------------ */
/* Preprocessor — sensor::Preprocessor / CUDAPreprocessor                    */
/* (include/sensor/Preprocessor.h:23-53, :76-113).                          */
/* ------------------------------------------------------------------------ */

typedef struct azu_preprocessor azu_preprocessor;

enum { AZU_PRE_FULL = 0, AZU_PRE_MINIMAL = 1 };

/* makePreprocessor(CUDA) (Preprocessor.h:115-118). mode: AZU_PRE_FULL runs the
 * RGB guidance chain, depth median, hole fill, guided joint-bilateral filter and
 * temporal EMA; AZU_PRE_MINIMAL (AZU_PREPROCESS=minimal) the median only. */
int azu_preprocessor_create(int device, int mode, void* stream, azu_preprocessor** out);
int azu_preprocessor_destroy(azu_preprocessor* p);
/* Preprocessor::reset / resetTemporalState (Preprocessor.h:27-28). */
int azu_preprocessor_reset(azu_preprocessor* p);
int azu_preprocessor_reset_temporal(azu_preprocessor* p);
/* Preprocessor::process (Preprocessor.h:29): RawFrame depth (640x480 raw
 * Kinect codes) and rgb (640x480x3) processed in place on the host, device
 * copies left for getGPUDepthMeters/getGPURgb. Synchronous. */
int azu_preprocessor_process(azu_preprocessor* p, uint16_t* h_depth, uint8_t* h_rgb, float min_depth,
                             float max_depth);
/* Same from device buffers (no host round trip; outputs stay on the device). */
int azu_preprocessor_process_device(azu_preprocessor* p, const uint16_t* d_depth, const uint8_t* d_rgb,
                                    float min_depth, float max_depth);
/* getGPUDepthMeters (Preprocessor.h:44): band-gated metres of the processed
 * frame (what buildFrameData computes), valid until the next process/reset. */
float* azu_preprocessor_depth_meters(azu_preprocessor* p);
/* getGPURgb (Preprocessor.h:45): processed RGB (bilateral + median). */
uint8_t* azu_preprocessor_rgb(azu_preprocessor* p);
/* Processed raw depth codes and guidance luma on the device. */
uint16_t* azu_preprocessor_depth_raw(azu_preprocessor* p);
float* azu_preprocessor_luma(azu_preprocessor* p);

/* ------------------------------------------------------------------------ */
/* Marching cubes — meshing::MarchingCubes (include/meshing/MarchingCubes.h). */
/* ------------------------------------------------------------------------ */

typedef struct azu_mesher azu_mesher;

typedef struct {
    int64_t n_vertices;   /* welded vertices */
    int64_t n_indices;    /* 3 x triangles */
    int     truncated;    /* MeshData::truncated */
    int     launches;     /* kernels the extraction launched */
} azu_mesh_info;

int azu_mesher_create(int device, void* stream, azu_mesher** out);
int azu_mesher_destroy(azu_mesher* m);
/* setMaxTriangles (MarchingCubes.h:58). Default 2,000,000. */
int azu_mesher_set_max_triangles(azu_mesher* m, int64_t max_triangles);
/* extractGPU (MarchingCubes.h:62): classify, scan, emit and the exact-edge weld
 * on the device; results stay on the device until copied out. Synchronous
 * (returns the counts). */
int azu_mesher_extract(azu_mesher* m, azu_volume* v, azu_mesh_info* info);
/* Copies the last extraction into host buffers sized from azu_mesh_info
 * (positions/normals 3 floats per vertex, colours 3 bytes, indices uint32). */
int azu_mesher_copy_out(azu_mesher* m, float* h_positions, float* h_normals, uint8_t* h_colors,
                        uint32_t* h_indices);
/* Device pointers of the last extraction. */
int azu_mesher_device_buffers(azu_mesher* m, const float** d_positions, const float** d_normals,
                              const uint8_t** d_colors, const uint32_t** d_indices);

/* ------------------------------------------------------------------------ */
/* Per-frame pipeline — the GPU branch of PipelineController's tracking and  */
/* integration workers (src/app/PipelineController.cpp:1003-1406, 1624-1905) */
/* run in lockstep (the azu_replay offline mode).                            */
/* ------------------------------------------------------------------------ */

typedef struct azu_pipeline azu_pipeline;

typedef struct {
    azu_volume_params  volume;
    azu_tracker_params tracker;
    int   preprocess_mode;   /* AZU_PRE_FULL / AZU_PRE_MINIMAL */
    float min_depth;         /* depth band for preprocessing and frame building */
    float max_depth;
    int   input_is_mm;       /* 1: input depth is uint16 millimetres (skips the
                                Kinect preprocessor, depth_m = mm * 1e-3);
                                0: Kinect raw codes through the preprocessor */
    int   use_graph;         /* capture the per-frame work in a CUDA graph */
    int   width, height;     /* image size; 0 = 640 x 480. Other sizes need
                                input_is_mm (the Kinect preprocessor is
                                640 x 480) and the tracker's intrinsics for them */
} azu_pipeline_params;

typedef struct {
    float pose[16];          /* camera pose after tracking (world-from-camera) */
    azu_icp_result icp;      /* the solve that produced it */
    int   quality;           /* 0 Good (integrated), 1 Poor, 2 Failed, -1 first frame */
    int   integrated;        /* 1 when the frame was fused */
    int   frame_index;
} azu_frame_result;

int azu_pipeline_create(int device, const azu_pipeline_params* p, azu_pipeline** out);
int azu_pipeline_destroy(azu_pipeline* p);
int azu_pipeline_reset(azu_pipeline* p);
/* One frame from host buffers: H2D of depth (and rgb, may be NULL), the whole
 * frame on the device, D2H of the result. Returns once the result is known,
 * i.e. after tracking: the frame's integrate and raycast are still running on
 * the pipeline's stream (every call on the pipeline, its volume and its
 * tracker is ordered after them; synchronise that stream before touching
 * their device buffers directly). The next frame's upload, preprocessing and
 * frame maps run on a second stream beside them; results are those of
 * finishing each frame before the next. With stage profiling on, the call
 * returns after the whole frame. */
int azu_pipeline_process_frame(azu_pipeline* p, const uint16_t* h_depth, const uint8_t* h_rgb,
                               azu_frame_result* out);
/* Same from device buffers; out may be NULL (no host sync: the frame is only
 * enqueued and the result stays on the device). The input buffers may be
 * reused once the call returns with a result, or after the pipeline's stream
 * has been synchronised. */
int azu_pipeline_process_frame_device(azu_pipeline* p, const uint16_t* d_depth, const uint8_t* d_rgb,
                                      azu_frame_result* out);
/* Reads back the result of the last enqueued frame (synchronises). */
int azu_pipeline_last_result(azu_pipeline* p, azu_frame_result* out);
azu_volume* azu_pipeline_volume(azu_pipeline* p);
azu_tracker* azu_pipeline_tracker(azu_pipeline* p);
/* Model maps of the last raycast (device float3, 640x480). */
int azu_pipeline_model_maps(azu_pipeline* p, const float** d_vertices, const float** d_normals);
/* The pipeline's stream (cudaStream_t). */
void* azu_pipeline_stream(azu_pipeline* p);
/* Per-stage device timing (the reference's FrameTrace ms_preprocess / ms_icp /
 * ms_integrate / ms_raycast columns, include/app/FrameTrace.h:40-88): when on,
 * CUDA events bracket the stages of every frame and each synchronous call adds
 * the frame's stage times to running totals. Turning it on or off clears the
 * totals (and recaptures the frame graph). */
int azu_pipeline_set_profiling(azu_pipeline* p, int on);
/* Totals in ms for {input (preprocess), frame (vertices/normals/pyramid),
 * track (predict + ICP), integrate, raycast} and the frames they cover. */
int azu_pipeline_stage_times(azu_pipeline* p, double ms_total[5], int* frames);
/* 1 when frames k > 0 replay a captured CUDA graph. */
int azu_pipeline_uses_graph(azu_pipeline* p);

/* ------------------------------------------------------------------------ */
/* Sensor-side ingest (host code): fakenect recordings                         */
/* (tools/FakenectRecording.h:35-81) paired like KinectSensor::onDepth/onRgb    */
/* (src/sensor/KinectSensor.cpp:262-362: depth-led, nearest RGB within 17 ms    */
/* of the 60 MHz counter, else depth-only; a depth frame still waiting at the    */
/* end is published depth-only), read ahead into a ring of pinned slots.        */
/* ------------------------------------------------------------------------ */

typedef struct azu_recording azu_recording;
typedef struct azu_ingest azu_ingest;

int azu_recording_open(const char* dir, azu_recording** out);
void azu_recording_close(azu_recording* r);
int azu_recording_frame_count(const azu_recording* r);
int azu_recording_frame_info(const azu_recording* r, int k, uint32_t* depth_ticks, uint32_t* rgb_ticks,
                             int* rgb_valid);
/* Frame k's raw depth (640x480 uint16) and RGB (640x480x3, zeros without). */
int azu_recording_read(const azu_recording* r, int k, uint16_t* depth, uint8_t* rgb, int* rgb_valid);
/* A reader thread fills `slots` pinned slots (depth then RGB, back to back)
 * with frames first .. first+count-1 in order. */
int azu_ingest_create(azu_recording* rec, int slots, int first, int count, azu_ingest** out);
int azu_ingest_destroy(azu_ingest* g);
/* The next frame's slot (blocks until read); 1 at the end of the range. */
int azu_ingest_next(azu_ingest* g, const void** slot, int* frame_index, int* rgb_valid);
/* Hands the oldest consumed slot back to the reader. */
int azu_ingest_release(azu_ingest* g);
/* One frame from a packed host buffer (depth then RGB, as an ingest slot) with
 * a single host-to-device copy; otherwise as azu_pipeline_process_frame. */
int azu_pipeline_process_frame_packed(azu_pipeline* p, const void* h_packed, azu_frame_result* out);

/* ------------------------------------------------------------------------ */
/* Mesh export (host code; src/export/PLYExporter.cpp, GLBExporter.cpp).       */
/* The mesh is the mesher's MeshData: positions (3 floats per vertex),         */
/* optional normals (n_normals vertices: 0 or n_vertices), optional sRGB        */
/* colours (n_color_bytes: 0 or 3 n_vertices) and triangle indices. It is        */
/* validated with MeshData::validate's rules (include/meshing/MeshData.h:49-95)  */
/* before any file is opened; a rejected mesh creates no file.                   */
/* ------------------------------------------------------------------------ */

/* PLYExporter::writeBinary / writeASCII: the reference's bytes. */
int azu_mesh_write_ply(const char* path, int binary, const float* positions, int64_t n_vertices, const float* normals,
                       int64_t n_normals, const uint8_t* colors, int64_t n_color_bytes, const uint32_t* indices,
                       int64_t n_indices);
/* GLBExporter::write: vertices welded by exact position, glTF axes (x, -y, -z),
 * unit normals (fallback (0, 0, -1)), linear RGBA float colours, 4-byte
 * aligned [positions | normals | colours | indices] binary chunk. */
int azu_mesh_write_glb(const char* path, const float* positions, int64_t n_vertices, const float* normals,
                       int64_t n_normals, const uint8_t* colors, int64_t n_color_bytes, const uint32_t* indices,
                       int64_t n_indices);

/* ------------------------------------------------------------------------ */
/* Batching form (no counterpart in the reference): many independent scenes,   */
/* each with its own volume, image size and frame count, advanced together.   */
/* ------------------------------------------------------------------------ */

typedef struct azu_batch azu_batch;

typedef struct {
    azu_volume_params  volume;     /* FP32, no colour */
    azu_tracker_params tracker;    /* intrinsics for this scene's image size */
    int   width, height;           /* multiples of 4 */
    float min_depth, max_depth;    /* depth band of the millimetre input */
} azu_batch_scene;

/* n scenes (1..64), each an independent pipeline on millimetre depth. */
int azu_batch_create(int device, int n, const azu_batch_scene* scenes, azu_batch** out);
int azu_batch_destroy(azu_batch* b);
/* One frame for every scene i with depth_mm[i] != NULL (uint16 millimetres,
 * host or device memory per on_device); scenes with NULL sit this step out.
 * Per scene as the single pipeline does (first frame at identity, then ICP
 * and gated fusion); integration and raycasting of all active scenes run as
 * one launch per stage, and steps replay one CUDA graph per active set.
 * results (n entries, optional) receive the active scenes' results (sync). */
int azu_batch_process(azu_batch* b, const uint16_t* const* depth_mm, int on_device, azu_frame_result* results);
/* Times the integrate item shapes (warps per block 1, 2, 4 x x-parts per
 * 32-row item 1, 2, 4) and raycast tile shapes on the batch's own data (after
 * at least one step) and keeps the fastest; results unchanged. */
int azu_batch_autotune(azu_batch* b, float* best_integrate_ms, float* best_raycast_ms);
int azu_batch_set_shapes(azu_batch* b, int int_warps, int int_parts, int ray_w, int ray_h);
int azu_batch_get_shapes(azu_batch* b, int* int_warps, int* int_parts, int* ray_w, int* ray_h);
azu_volume* azu_batch_volume(azu_batch* b, int i);
void* azu_batch_stream(azu_batch* b);
int azu_batch_uses_graph(azu_batch* b);
int azu_batch_synchronize(azu_batch* b);

/* ------------------------------------------------------------------------ */
/* Testing hooks (no counterpart in the reference).                          */
/* ------------------------------------------------------------------------ */

/* Wait limits of every later ICP launch on the current device: each barrier
 * wait gives up after spin_limit polls (0 = the default, about a quarter of a
 * second), and a barrier completes only after extra_arrivals more arrivals
 * than the launch has blocks (0 = normal). extra_arrivals > 0 makes every
 * wait run out on purpose, so a test can check that the call reports
 * AZU_E_TIMEOUT, that the frame is graded Failed and fuses nothing, and that
 * the next call works. Synchronous; not for use while ICP work is in flight. */
int azu_testing_set_icp_wait(unsigned spin_limit, unsigned extra_arrivals);

#ifdef __cplusplus
}
#endif
#endif /* AZU_GPU_H */
