// Oracle (test infrastructure only): C entry points over the reference's OWN
// hot-path classes, compiled unmodified from the reference's sources against
// the Eigen-API shim (eigen_shim/) by oracle/ref.mk into oracle/_ref/libazu_ref.so.
// Tests call these beside the CPU restatement (liborc.so, orc_api.h) with the
// same conventions — row-major float[16] poses, float3 maps, separate
// tsdf/weight/colour arrays — to pin the restatement to the reference's code.
//
// Wrapped: tsdf::TSDFVolume (integrate, raycast, point cloud), meshing::
// MarchingCubes::extract, sensor::buildFrameData / computeNormals /
// buildFramePyramid, tracking::ICPTracker (track; buildLinearSystem through
// the class's private member, opened for this translation unit only),
// tracking::classifyTracking, sensor::SignalConditioner::process, the
// export_io::PLYExporter / GLBExporter writers and sensor::KinectSensor's
// depth-led pairing (through its device-free test seam).
// Everything ICPTracker.h includes comes first, so that only that class's
// declaration is read with its private members opened.
#include <Eigen/Core>
#include <Eigen/Geometry>
#include <limits>
#include <vector>

#include "sensor/FrameData.h"
#define private public
#include "tracking/ICPTracker.h"
#undef private

#include "export/GLBExporter.h"
#include "export/PLYExporter.h"
#include "meshing/MarchingCubes.h"
#include "sensor/FrameData.h"
#include "sensor/KinectSensor.h"
#include "sensor/SignalConditioner.h"
#include "tracking/TrackingPolicy.h"
#include "tsdf/TSDFVolume.h"

#include <omp.h>

#include <cstring>
#include <memory>

#include "orc_api.h"

using namespace kfusion;

namespace {

Eigen::Matrix4f pose_of(const float* rm) {
    Eigen::Matrix4f P;
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) P(r, c) = rm[4 * r + c];
    return P;
}

void pose_to(const Eigen::Matrix4f& P, float* rm) {
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) rm[4 * r + c] = P(r, c);
}

tsdf::TSDFParams tsdf_params_of(const orc_tsdf_params* p) {
    tsdf::TSDFParams t;
    t.resolution = p->res;
    t.voxel_size = p->voxel_size;
    t.truncation = p->truncation;
    t.max_weight = p->max_weight;
    t.origin = Eigen::Vector3f(p->origin[0], p->origin[1], p->origin[2]);
    t.min_depth = p->min_depth;
    t.max_depth = p->max_depth;
    return t;
}

void load_maps(const float* v, const float* n, size_t count, std::vector<Eigen::Vector3f>& vo,
               std::vector<Eigen::Vector3f>& no) {
    vo.resize(count);
    no.resize(count);
    for (size_t i = 0; i < count; ++i) {
        vo[i] = Eigen::Vector3f(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
        no[i] = Eigen::Vector3f(n[3 * i], n[3 * i + 1], n[3 * i + 2]);
    }
}

void store_map(const std::vector<Eigen::Vector3f>& in, float* out) {
    for (size_t i = 0; i < in.size(); ++i)
        for (int k = 0; k < 3; ++k) out[3 * i + k] = in[i](k);
}

sensor::CameraIntrinsics intr_of(orc_intrinsics K, int W, int H) {
    sensor::CameraIntrinsics c{};
    c.fx = K.fx;
    c.fy = K.fy;
    c.cx = K.cx;
    c.cy = K.cy;
    (void)W;
    (void)H;
    return c;
}

}  // namespace

extern "C" {

// ---- TSDF volume -----------------------------------------------------------
void* ref_volume_create(const orc_tsdf_params* p) { return new tsdf::TSDFVolume(tsdf_params_of(p)); }
void ref_volume_destroy(void* h) { delete static_cast<tsdf::TSDFVolume*>(h); }

// TSDFVolume::setParams: any difference clears the volume.
void ref_volume_set_params(void* h, const orc_tsdf_params* p) {
    static_cast<tsdf::TSDFVolume*>(h)->setParams(tsdf_params_of(p));
}

// Voxel contents in and out (tsdf, weight, colour[3 n] or NULL), z-major.
void ref_volume_load(void* h, const float* tsdf, const float* weight, const float* color) {
    auto* v = static_cast<tsdf::TSDFVolume*>(h);
    const int r = v->params().resolution;
    size_t i = 0;
    for (int z = 0; z < r; ++z)
        for (int y = 0; y < r; ++y)
            for (int x = 0; x < r; ++x, ++i) {
                tsdf::Voxel& vx = v->voxelAt(x, y, z);
                vx.tsdf = tsdf[i];
                vx.weight = weight[i];
                if (color) {
                    vx.r = color[3 * i];
                    vx.g = color[3 * i + 1];
                    vx.b = color[3 * i + 2];
                }
            }
}

void ref_volume_store(void* h, float* tsdf, float* weight, float* color) {
    auto* v = static_cast<tsdf::TSDFVolume*>(h);
    const std::vector<tsdf::Voxel>& d = v->voxelData();
    for (size_t i = 0; i < d.size(); ++i) {
        tsdf[i] = d[i].tsdf;
        weight[i] = d[i].weight;
        if (color) {
            color[3 * i] = d[i].r;
            color[3 * i + 1] = d[i].g;
            color[3 * i + 2] = d[i].b;
        }
    }
}

// TSDFVolume::integrate (CPU path). newly_observed from the observed fraction.
void ref_volume_integrate(void* h, const float* depth_m, const uint8_t* rgb, const float pose[16], orc_intrinsics K,
                          int W, int H, float min_depth, float max_depth, int64_t* newly_observed) {
    auto* v = static_cast<tsdf::TSDFVolume*>(h);
    const double n = static_cast<double>(v->voxelData().size());
    const double before = static_cast<double>(v->observedFraction()) * n;
    v->integrate(depth_m, rgb, pose_of(pose), K.fx, K.fy, K.cx, K.cy, W, H, min_depth, max_depth);
    if (newly_observed)
        *newly_observed = static_cast<int64_t>(static_cast<double>(v->observedFraction()) * n - before + 0.5);
}

void ref_volume_raycast(void* h, const float pose[16], orc_intrinsics K, int W, int H, float* vertices,
                        float* normals, uint8_t* colors) {
    auto* v = static_cast<tsdf::TSDFVolume*>(h);
    std::vector<Eigen::Vector3f> vo(static_cast<size_t>(W) * H), no(static_cast<size_t>(W) * H);
    v->raycast(pose_of(pose), K.fx, K.fy, K.cx, K.cy, W, H, vo.data(), no.data(), colors);
    store_map(vo, vertices);
    store_map(no, normals);
}

int64_t ref_volume_point_cloud(void* h, float* pts, uint8_t* cols) {
    auto* v = static_cast<tsdf::TSDFVolume*>(h);
    std::vector<Eigen::Vector3f> p;
    std::vector<uint8_t> c;
    v->extractGlobalPointCloud(p, c);
    if (pts) store_map(p, pts);
    if (cols) std::memcpy(cols, c.data(), c.size());
    return static_cast<int64_t>(p.size());
}

// MarchingCubes::extract: call with positions == NULL for the counts.
void ref_volume_mesh(void* h, int64_t max_triangles, orc_mesh_info* info, float* positions, float* normals,
                     uint8_t* colors, uint32_t* indices) {
    auto* v = static_cast<tsdf::TSDFVolume*>(h);
    meshing::MarchingCubes mc;
    mc.setMaxTriangles(static_cast<size_t>(max_triangles));
    std::shared_ptr<meshing::MeshData> m = mc.extract(*v);
    info->n_vertices = static_cast<int64_t>(m->positions.size());
    info->n_indices = static_cast<int64_t>(m->indices.size());
    info->truncated = m->truncated ? 1 : 0;
    if (!positions) return;
    store_map(m->positions, positions);
    store_map(m->normals, normals);
    if (colors) std::memcpy(colors, m->colors.data(), m->colors.size());
    std::memcpy(indices, m->indices.data(), m->indices.size() * sizeof(uint32_t));
}

// ---- frames -------------------------------------------------------------------
// buildFrameData from 640x480 raw codes (rgb may be NULL: grey), then normals.
void ref_build_frame(const uint16_t* raw, orc_intrinsics K, float min_depth, float max_depth, float* depth_m,
                     float* vertices, float* normals) {
    sensor::FrameData f;
    std::vector<uint8_t> rgb(static_cast<size_t>(sensor::FRAME_W) * sensor::FRAME_H * 3, 128);
    sensor::buildFrameData(raw, rgb.data(), f, min_depth, max_depth, intr_of(K, sensor::FRAME_W, sensor::FRAME_H));
    std::memcpy(depth_m, f.depth_meters.data(), f.depth_meters.size() * sizeof(float));
    store_map(f.vertices, vertices);
    store_map(f.normals, normals);
}

// computeNormals + buildFramePyramid from a level-0 depth (metres) and vertex
// map: the three levels' depth, vertices and normals, level l at offsets of
// the previous levels' sizes (640x480, 320x240, 160x120).
void ref_frame_pyramid(const float* depth_m, const float* vertices, orc_intrinsics K, float* depth_out,
                       float* vertices_out, float* normals_out) {
    sensor::FrameData f;
    f.intrinsics = intr_of(K, sensor::FRAME_W, sensor::FRAME_H);
    const size_t n = static_cast<size_t>(sensor::FRAME_W) * sensor::FRAME_H;
    std::memcpy(f.depth_meters.data(), depth_m, n * sizeof(float));
    for (size_t i = 0; i < n; ++i) f.vertices[i] = Eigen::Vector3f(vertices[3 * i], vertices[3 * i + 1], vertices[3 * i + 2]);
    sensor::computeNormals(f);
    sensor::FramePyramid pyr;
    sensor::buildFramePyramid(f, pyr);
    size_t off = 0;
    for (int l = 0; l < sensor::FramePyramid::LEVELS; ++l) {
        const sensor::FrameData& L = pyr.levels[l];
        const size_t m = static_cast<size_t>(L.width) * L.height;
        std::memcpy(depth_out + off, L.depth_meters.data(), m * sizeof(float));
        store_map(L.vertices, vertices_out + 3 * off);
        store_map(L.normals, normals_out + 3 * off);
        off += m;
    }
}

// ---- ICP -------------------------------------------------------------------------
static std::unique_ptr<tracking::ICPTracker> make_tracker(const orc_icp_params* prm, orc_intrinsics K) {
    tracking::ICPParams p;
    for (int l = 0; l < 3; ++l) p.max_iterations[l] = prm->max_iterations[l];
    p.dist_threshold = prm->dist_threshold;
    p.angle_threshold = prm->angle_threshold;
    auto t = std::make_unique<tracking::ICPTracker>(p);
    t->setIntrinsics(intr_of(K, sensor::FRAME_W, sensor::FRAME_H));
    if (prm->fold_threads > 0) t->setNumThreads(prm->fold_threads);
    return t;
}

static void model_of(const float* mv, const float* mn, int MW, int MH, tracking::ModelFrame& m) {
    m.width = MW;
    m.height = MH;
    load_maps(mv, mn, static_cast<size_t>(MW) * MH, m.vertices, m.normals);
}

// ICPTracker::buildLinearSystem at one pyramid level (live maps W x H).
int ref_icp_build_system(const orc_icp_params* prm, orc_intrinsics K, const float* live_v, const float* live_n, int W,
                         int H, const float* model_v, const float* model_n, int MW, int MH, const float pose[16],
                         const float ref_pose[16], float A[36], float b[6], float* residual, int counts[6]) {
    auto t = make_tracker(prm, K);
    sensor::FrameData live;
    live.width = W;
    live.height = H;
    load_maps(live_v, live_n, static_cast<size_t>(W) * H, live.vertices, live.normals);
    tracking::ModelFrame m(MW, MH);
    model_of(model_v, model_n, MW, MH, m);
    Eigen::Matrix<float, 6, 6> Am = Eigen::Matrix<float, 6, 6>::Zero();
    Eigen::Matrix<float, 6, 1> bm = Eigen::Matrix<float, 6, 1>::Zero();
    int inl = 0;
    const bool ok = t->buildLinearSystem(live, m, pose_of(pose), pose_of(ref_pose), Am, bm, *residual, inl, counts[1],
                                        counts[2], counts[3], counts[4], counts[5]);
    counts[0] = inl;
    for (int i = 0; i < 6; ++i) {
        b[i] = bm(i);
        for (int j = 0; j < 6; ++j) A[6 * i + j] = Am(i, j);
    }
    return ok ? 1 : 0;
}

// ICPTracker::track over a 3-level live pyramid (level l: (W >> l) x (H >> l)).
void ref_icp_track(const orc_icp_params* prm, orc_intrinsics K, const float* const live_v[3],
                   const float* const live_n[3], int W, int H, const float* model_v, const float* model_n, int MW,
                   int MH, const float estimate[16], const float ref_pose[16], orc_icp_result* out) {
    auto t = make_tracker(prm, K);
    sensor::FramePyramid pyr;
    for (int l = 0; l < 3; ++l) {
        pyr.levels[l].width = W >> l;
        pyr.levels[l].height = H >> l;
        load_maps(live_v[l], live_n[l], static_cast<size_t>(W >> l) * (H >> l), pyr.levels[l].vertices,
                  pyr.levels[l].normals);
    }
    tracking::ModelFrame m(MW, MH);
    model_of(model_v, model_n, MW, MH, m);
    const tracking::ICPResult r = t->track(pyr, m, pose_of(estimate), pose_of(ref_pose));
    std::memset(out, 0, sizeof(*out));
    pose_to(r.pose, out->pose);
    out->error = r.error;
    out->inliers = r.inliers;
    out->converged = r.converged ? 1 : 0;
    out->tracking_ok = r.tracking_ok ? 1 : 0;
    out->final_step = r.final_step;
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) out->information[6 * i + j] = r.information(i, j);
    out->valid_live_points = r.valid_live_points;
    out->valid_model_points = r.valid_model_points;
    out->projected_points = r.projected_points;
    out->dist_filtered = r.dist_filtered;
    out->angle_filtered = r.angle_filtered;
}

// tracking::classifyTracking: 0 Good, 1 Poor, 2 Failed.
int ref_classify_tracking(const orc_icp_result* r, const float prev_pose[16]) {
    tracking::ICPResult x;
    x.pose = pose_of(r->pose);
    x.error = r->error;
    x.inliers = r->inliers;
    x.converged = r->converged != 0;
    x.tracking_ok = r->tracking_ok != 0;
    x.final_step = r->final_step;
    x.valid_live_points = r->valid_live_points;
    x.valid_model_points = r->valid_model_points;
    x.projected_points = r->projected_points;
    x.dist_filtered = r->dist_filtered;
    x.angle_filtered = r->angle_filtered;
    const tracking::TrackQuality q = tracking::classifyTracking(x, pose_of(prev_pose));
    return q == tracking::TrackQuality::Good ? 0 : (q == tracking::TrackQuality::Poor ? 1 : 2);
}

// ---- preprocessor -----------------------------------------------------------------
void* ref_conditioner_create(int minimal) {
    auto* c = new sensor::SignalConditioner();
    c->setMinimalDepth(minimal != 0);
    return c;
}
void ref_conditioner_destroy(void* h) { delete static_cast<sensor::SignalConditioner*>(h); }

// SignalConditioner::process on one 640x480 frame, depth raw codes and rgb in place.
void ref_conditioner_process(void* h, uint16_t* depth, uint8_t* rgb, float min_depth, float max_depth) {
    auto* c = static_cast<sensor::SignalConditioner*>(h);
    sensor::RawFrame raw;
    const size_t n = static_cast<size_t>(sensor::FRAME_W) * sensor::FRAME_H;
    std::memcpy(raw.depth.data(), depth, n * sizeof(uint16_t));
    std::memcpy(raw.rgb.data(), rgb, n * 3);
    raw.depth_valid = true;
    raw.rgb_valid = true;
    c->process(raw, nullptr, min_depth, max_depth);
    std::memcpy(depth, raw.depth.data(), n * sizeof(uint16_t));
    std::memcpy(rgb, raw.rgb.data(), n * 3);
}

// ---- export ------------------------------------------------------------------
static meshing::MeshData mesh_of(const float* pos, const float* nrm, const uint8_t* col, int64_t nv,
                                 const uint32_t* idx, int64_t ni) {
    meshing::MeshData m;
    m.positions.resize(static_cast<size_t>(nv));
    for (int64_t i = 0; i < nv; ++i) m.positions[i] = Eigen::Vector3f(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    if (nrm) {
        m.normals.resize(static_cast<size_t>(nv));
        for (int64_t i = 0; i < nv; ++i) m.normals[i] = Eigen::Vector3f(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
    }
    if (col) m.colors.assign(col, col + 3 * nv);
    m.indices.assign(idx, idx + ni);
    return m;
}

// PLYExporter::writeBinary (binary != 0) or writeASCII; GLBExporter::write.
// Normals or colours may be NULL. Returns the writer's success flag.
int ref_export_ply(const float* pos, const float* nrm, const uint8_t* col, int64_t nv, const uint32_t* idx,
                   int64_t ni, const char* path, int binary) {
    const meshing::MeshData m = mesh_of(pos, nrm, col, nv, idx, ni);
    return binary ? export_io::PLYExporter::writeBinary(m, path) : export_io::PLYExporter::writeASCII(m, path);
}

int ref_export_glb(const float* pos, const float* nrm, const uint8_t* col, int64_t nv, const uint32_t* idx,
                   int64_t ni, const char* path) {
    return export_io::GLBExporter::write(mesh_of(pos, nrm, col, nv, idx, ni), path);
}

// ---- sensor pairing ------------------------------------------------------------
// Feeds depth (kind 0) and RGB (kind 1) samples with their 60 MHz tick stamps,
// in order, through KinectSensor's pairing path. Per published frame writes
// the depth ticks and the paired RGB ticks (-1: published depth-only).
// Returns the number of frames published (at most cap are written).
int ref_sensor_pairing(const int* kinds, const uint32_t* ticks, int n, int64_t* depth_ticks, int64_t* rgb_ticks,
                       int cap) {
    static std::vector<uint16_t> depth(static_cast<size_t>(sensor::DEPTH_WIDTH) * sensor::DEPTH_HEIGHT, 0);
    static std::vector<uint8_t> rgb(static_cast<size_t>(sensor::RGB_WIDTH) * sensor::RGB_HEIGHT * 3, 0);
    sensor::KinectSensor s;
    std::vector<std::pair<int64_t, int64_t>> got;
    s.setFrameCallback([&got](std::shared_ptr<sensor::RawFrame> f) {
        got.emplace_back(f->depth_ticks, f->rgb_valid ? static_cast<int64_t>(f->rgb_ticks) : -1);
    });
    for (int i = 0; i < n; ++i) {
        if (kinds[i] == 0) s.injectDepthForTests(depth.data(), ticks[i]);
        else s.injectRgbForTests(rgb.data(), ticks[i]);
    }
    s.setFrameCallback(nullptr);
    for (size_t k = 0; k < got.size() && static_cast<int>(k) < cap; ++k) {
        depth_ticks[k] = got[k].first;
        rgb_ticks[k] = got[k].second;
    }
    return static_cast<int>(got.size());
}

void ref_set_threads(int n) {
    if (n > 0) omp_set_num_threads(n);
}

}  // extern "C"
