/* Oracle (test infrastructure only): C entry points of the CPU restatement of
 * Azu's per-frame KinectFusion hot path. Only tests, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg load this library, to compare results
 * against and to time the CPU path; the product never links it.
 *
 * Conventions: poses are row-major float[16] (element (r, c) at 4 r + c),
 * world-from-camera. Vertex/normal maps are float[3 * W * H] (x, y, z per pixel,
 * row-major pixels). Volumes are separate float arrays tsdf[n], weight[n] and
 * optional color[3 n] (float sRGB), n = res^3, index z*res*res + y*res + x.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int   res;
    float voxel_size;
    float truncation;
    float max_weight;
    float origin[3];
    float min_depth; /* raycast band (TSDFParams::min_depth) */
    float max_depth; /* raycast band (TSDFParams::max_depth) */
} orc_tsdf_params;

typedef struct {
    float fx, fy, cx, cy;
} orc_intrinsics;

/* TSDFVolume::reset (src/tsdf/TSDFVolume.cpp:117-122). */
void orc_tsdf_reset(const orc_tsdf_params* p, float* tsdf, float* weight, float* color);

/* TSDFVolume::integrateCPU (src/tsdf/TSDFVolume.cpp:214-346). stats[0] =
 * newly observed voxels, stats[1] = voxels updated, stats[2] = colour updates,
 * stats[3] = AABB x0, [4] x1, [5] y0, [6] y1, [7] z0, [8] z1 (-1 when the AABB
 * is not finite). */
void orc_tsdf_integrate(const orc_tsdf_params* p, float* tsdf, float* weight, float* color,
                        const float* depth_m, const uint8_t* rgb, const float pose[16],
                        orc_intrinsics K, int W, int H, float min_depth, float max_depth,
                        int64_t stats[9]);

/* Precision form of orc_tsdf_integrate (same projections and decisions):
 * half_storage != 0 stores the tsdf rounded to IEEE half after each update (the
 * FP16 + u16 volume); tsdf64 (may be NULL) carries the same running average in
 * double (the FP64 reference). No colour. */
void orc_tsdf_integrate_prec(const orc_tsdf_params* p, float* tsdf, float* weight, double* tsdf64,
                             const float* depth_m, const float pose[16], orc_intrinsics K, int W, int H,
                             float min_depth, float max_depth, int half_storage);

/* TSDFVolume::raycast (src/tsdf/TSDFVolume.cpp:348-476). colors_out may be NULL;
 * color may be NULL (every voxel then carries EMPTY_COLOR). samples_out (may
 * be NULL) receives the number of trilinear samples taken. */
void orc_tsdf_raycast(const orc_tsdf_params* p, const float* tsdf, const float* weight,
                      const float* color, const float pose[16], orc_intrinsics K, int W, int H,
                      float* vertices_out, float* normals_out, uint8_t* colors_out,
                      int64_t* samples_out);

/* sensor::buildFrameData + updateVerticesFromDepth (src/sensor/FrameData.cpp:113-194)
 * from raw Kinect codes; depth_m receives band-gated metres. */
void orc_build_frame(const uint16_t* raw, int W, int H, orc_intrinsics K, float min_depth,
                     float max_depth, float* depth_m, float* vertices, float* normals);
/* Same from metres (the reference tests' fillFrame precedent): depth_m in, vertices out. */
void orc_vertices_from_depth(const float* depth_m, int W, int H, orc_intrinsics K, float* vertices);
/* sensor::computeNormals (src/sensor/FrameData.cpp:196-251). */
void orc_compute_normals(const float* depth_m, const float* vertices, int W, int H, float* normals);
/* sensor::downsample (src/sensor/FrameData.cpp:262-334): W x H -> W/2 x H/2. */
void orc_downsample(const float* depth_m, const float* vertices, const float* normals, int W, int H,
                    float* depth_out, float* vertices_out, float* normals_out);

typedef struct {
    int   max_iterations[3];
    float dist_threshold;
    float angle_threshold;
    int   fold_threads; /* OpenMP-static partition count of the reference's fold (>= 1) */
} orc_icp_params;

typedef struct {
    float pose[16];
    float error;
    int   inliers;
    int   converged;
    int   tracking_ok;
    float final_step;
    float information[36];
    int   valid_live_points, valid_model_points, projected_points, dist_filtered, angle_filtered;
    int   iterations[3]; /* solves accepted per level (diagnostic) */
} orc_icp_result;

/* ICPTracker::buildLinearSystem (src/tracking/ICPTracker.cpp:136-354): one
 * association + reduction pass. A is 36 floats (row-major, symmetric), b 6,
 * counts = {inliers, valid_live, valid_model, projected, dist_filtered,
 * angle_filtered}. Returns inliers > 0. live_K is unused by the reference
 * (projection uses the camera intrinsics scaled to the model size). */
int orc_icp_build_system(const orc_icp_params* prm, orc_intrinsics camK,
                         const float* live_v, const float* live_n, int W, int H,
                         const float* model_v, const float* model_n, int MW, int MH,
                         const float pose[16], const float ref_pose[16],
                         float A[36], float b[6], float* residual, int counts[6]);

/* The same pass with the per-pixel float terms accumulated in double (the FP64
 * reduction oracle). */
int orc_icp_build_system_f64(const orc_icp_params* prm, orc_intrinsics camK,
                             const float* live_v, const float* live_n, int W, int H,
                             const float* model_v, const float* model_n, int MW, int MH,
                             const float pose[16], const float ref_pose[16],
                             double A[36], double b[6], int counts[6]);

/* ICPTracker::track (src/tracking/ICPTracker.cpp:40-134) over a 3-level live
 * pyramid: live_v[l], live_n[l] at (W >> l) x (H >> l). */
void orc_icp_track(const orc_icp_params* prm, orc_intrinsics camK,
                   const float* const live_v[3], const float* const live_n[3], int W, int H,
                   const float* model_v, const float* model_n, int MW, int MH,
                   const float estimate[16], const float ref_pose[16], orc_icp_result* out);

/* tracking::classifyTracking (include/tracking/TrackingPolicy.h:70-112):
 * 0 = Good, 1 = Poor, 2 = Failed. */
int orc_classify_tracking(const orc_icp_result* r, const float prev_pose[16]);

/* Constant-velocity prediction (src/app/PipelineController.cpp:1175-1177):
 * pred = cur * (last^-1 * cur). */
void orc_predict(const float cur[16], const float last[16], float pred[16]);

/* MarchingCubes::extract (src/meshing/MarchingCubes.cpp:174-382). Two-phase:
 * call with positions == NULL to get counts (n_vertices, n_indices, truncated),
 * then again with buffers of those sizes. max_triangles is the cap. */
typedef struct {
    int64_t n_vertices;
    int64_t n_indices;
    int     truncated;
} orc_mesh_info;
void orc_mc_extract(const orc_tsdf_params* p, const float* tsdf, const float* weight,
                    const float* color, int64_t max_triangles, orc_mesh_info* info,
                    float* positions, float* normals, uint8_t* colors, uint32_t* indices);

/* SignalConditioner::processCpu (src/sensor/SignalConditioner_omp.cpp:337-349)
 * on a 640x480 RawFrame: rgb (in/out, 3 B per pixel) and depth raw codes (in/out);
 * ema_state is the persistent float[W*H] EMA buffer; luma_out (may be NULL)
 * receives the guidance luma. minimal != 0 runs the depth median only. */
void orc_preprocess(uint16_t* depth, uint8_t* rgb, float* ema_state, float* luma_out,
                    float min_depth, float max_depth, int minimal);
/* The depth stages one by one (same files), for stage-level parity. */
void orc_pre_rgb(uint8_t* rgb, float* luma_out);
void orc_pre_depth_median(uint16_t* depth, float min_depth, float max_depth);
void orc_pre_fill_holes(uint16_t* depth, float min_depth, float max_depth);
void orc_pre_guided(uint16_t* depth, const float* luma, float min_depth, float max_depth);
void orc_pre_ema(uint16_t* depth, float* ema_state, float min_depth, float max_depth);

/* Depth-domain helpers (include/sensor/DepthValidity.h:73-118). */
float    orc_raw_to_meters(uint16_t raw);
float    orc_cpu_depth_meters(uint16_t raw, float min_depth, float max_depth);
uint16_t orc_meters_to_raw(float meters, float min_depth, float max_depth);

/* OpenMP threads the oracle uses (0 = library default). */
void orc_set_threads(int n);
int  orc_get_threads(void);

/* Differentiation form (no reference counterpart): depth image of the
 * reference's raycast (camera z of the hit, 0 on a miss), Huber loss on the
 * residual to depth_obs (pixels whose observed depth is in the raycast band),
 * and the adjoint with respect to xi of pose * Exp(xi) (xi = rho, omega) and to
 * the tsdf values (accumulated into grad_tsdf, res^3 doubles, when non-null).
 * jac_out (6 per pixel) receives dDepth/dxi. orc_depth_adjoint_f marches in
 * float exactly as the reference and evaluates the adjoint in double;
 * orc_depth_loss_d does everything in double at pose * Exp(xi). */
void orc_depth_adjoint_f(const orc_tsdf_params* p, const float* tsdf, const float* weight, const float pose[16],
                         orc_intrinsics K, int width, int height, const float* depth_obs, double huber_delta,
                         double* loss, double grad_xi[6], double* grad_tsdf, double* depth_out, double* jac_out,
                         int* n_valid);
void orc_depth_loss_d(const orc_tsdf_params* p, const double* tsdf, const float* weight, const double pose[16],
                      const double xi[6], orc_intrinsics K, int width, int height, const float* depth_obs,
                      double huber_delta, double* loss, double grad_xi[6], double* grad_tsdf, double* depth_out,
                      double* jac_out, int* n_valid);

/* TSDFVolume::extractGlobalPointCloud (TSDFVolume.cpp:571-632), one thread:
 * index order z, y, x. Returns the count; pts / cols (3 per point) may be NULL. */
int64_t orc_point_cloud(const orc_tsdf_params* p, const float* tsdf, const float* weight, const float* color,
                        float* pts, uint8_t* cols);

#ifdef __cplusplus
}
#endif
