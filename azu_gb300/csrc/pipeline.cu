// Per-frame KinectFusion pipeline on one GPU, behind the azu_pipeline_* ABI:
// the GPU branch of the reference's tracking and integration workers run in
// lockstep, as its offline replay drives them (src/app/PipelineController.cpp:
// 1003-1406 tracking, 1624-1905 integration; tools/azu_replay.cpp).
//
// Frame 0: pose = identity, integrate, raycast the model.
// Frame k > 0, all on the device with no host round trip:
//   input      preprocess Kinect raw codes (or mm -> metres)
//   frame      vertices, normals, 3-level pyramid
//   predict    constant velocity: pred = cur * (last^-1 * cur); prev = cur; last = cur
//              (computed by the previous frame's commit)
//   track      persistent ICP from pred against the model; on a Failed grade it
//              retries from prev; Good/Poor move cur, Failed keeps it
//   integrate  only when the grade is Good (a device flag gates the kernels)
//   raycast    the new model at cur (same gate)
// A pipeline made by azu_pipeline_create runs the input and frame stages on a
// second stream: frame k+1's upload, preprocessing, frame maps and depth tiles
// overlap frame k's integrate and raycast (they only wait for frame k's
// tracking, and the depth map and its tiles alternate between two buffers),
// and a call that returns the result returns once the pose is known (read back
// on a third stream), with the fusion of the frame still running on the
// pipeline's stream. Each part replays its own captured CUDA
// graph (frames k > 0); host inputs and the result are copied outside them.
// Results are those of the strictly sequential schedule: every stage reads
// what it read there.
#include <cstring>

#include "azu_internal.h"
#include "kf_math.cuh"

struct azu_preprocessor;

namespace azu {
int preprocess_enqueue(azu_preprocessor* p, float lo, float hi, cudaStream_t s);
int mm_to_meters_enqueue(const uint16_t* d_mm, float* d_out, int n, float lo, float hi, cudaStream_t s);
uint16_t* preprocess_input(azu_preprocessor* p);
uint8_t* preprocess_rgb_input(azu_preprocessor* p);
float* preprocess_depth_m(azu_preprocessor* p);
int tracker_prepare_dev(azu_tracker* t, const float* d_depth, int W, int H, cudaStream_t s);
int tracker_track_dev(azu_tracker* t, const float* mv, const float* mn, int MW, int MH, const float* d_estimate,
                      const float* d_ref, const float* d_prev, float* d_pose_out, azu_icp_result* d_result,
                      int* d_quality, int* d_gate, cudaStream_t s);

// Device-resident pose state of the pipeline.
struct PoseState {
    float cur[16];
    float last[16];
    float pred[16];
    float prev[16];
    float model_pose[16];
    int quality;
    int gate;
    int frame_index;
    int integrated;
};

// After a gated integrate + raycast: the model now shows the scene at cur.
// Then the next frame's prediction, PipelineController.cpp:1175-1177 (velocity
// model off, the default): prev = cur; pred = cur * (last^-1 * cur); last = cur.
// cur is final once this frame's tracking has run, so it is done here rather
// than in a launch of its own at the next frame's start.
__global__ void commit_kernel(PoseState* st) {
    if (threadIdx.x != 0) return;
    st->integrated = st->gate;
    if (st->gate)
        for (int i = 0; i < 16; ++i) st->model_pose[i] = st->cur[i];
    st->frame_index += 1;
    float inv[16], m[16];
    for (int i = 0; i < 16; ++i) st->prev[i] = st->cur[i];
    inverse4(st->last, inv);
    mm4(inv, st->cur, m);
    mm4(st->cur, m, st->pred);
    for (int i = 0; i < 16; ++i) st->last[i] = st->cur[i];
}

__global__ void first_frame_kernel(PoseState* st) {
    if (threadIdx.x != 0) return;
    for (int i = 0; i < 16; ++i) {
        const float v = (i % 5 == 0) ? 1.0f : 0.0f;
        st->cur[i] = st->last[i] = st->pred[i] = st->prev[i] = st->model_pose[i] = v;
    }
    st->quality = -1;
    st->gate = 1;
    st->frame_index = 0;
    st->integrated = 0;
}

}  // namespace azu

struct azu_pipeline {
    int device = 0;
    azu_pipeline_params p{};
    cudaStream_t s = nullptr;
    azu_preprocessor* pre = nullptr;
    azu_tracker* trk = nullptr;
    azu_volume* vol = nullptr;
    uint16_t* d_in = nullptr;   // mm input when input_is_mm
    float* d_depth_m = nullptr; // mm path output
    float* d_model_v = nullptr;
    float* d_model_n = nullptr;
    azu::PoseState* d_st = nullptr;
    azu_icp_result* d_icp = nullptr;
    int frames = 0;
    int W = 640, H = 480;
    uint8_t* d_packed = nullptr;  // one frame's depth | rgb, for the single-copy input
    bool own_stream = true;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    // two-stream schedule (standalone pipelines)
    cudaStream_t s2 = nullptr;                    // inputs, preprocessing, frame maps
    cudaStream_t s3 = nullptr;                    // result read-back beside the fusion
    cudaEvent_t ev_front = nullptr, ev_track = nullptr, ev_result = nullptr;
    cudaEvent_t ev_fused = nullptr;               // the frame's integrate is done
    float* d_depth2[2] = {nullptr, nullptr};      // the frame's depth (metres), alternating
    float* d_tiles2[2] = {nullptr, nullptr};      // its depth tile pyramid
    int buf = 0;
    cudaGraph_t g_part[5] = {};                   // front[2], track, tail[2]
    cudaGraphExec_t x_part[5] = {};
    azu::PoseState* h_st = nullptr;               // pinned result staging
    azu_icp_result* h_icp = nullptr;
    cudaEvent_t ev[6] = {};
    double stage_ms[5] = {0, 0, 0, 0, 0};
    int stage_frames = 0;
    bool profiling = false;
    int graph_failed = 0;
};

namespace azu {

static bool two_streams(const azu_pipeline* pl) { return pl->s2 != nullptr; }
static cudaStream_t front_stream(const azu_pipeline* pl) { return pl->s2 ? pl->s2 : pl->s; }

static const float* depth_source(azu_pipeline* pl) {
    if (two_streams(pl)) return pl->d_depth2[pl->buf];
    return pl->p.input_is_mm ? pl->d_depth_m : preprocess_depth_m(pl->pre);
}

static int mark(azu_pipeline* pl, int k, cudaStream_t s) {
    if (!pl->profiling) return AZU_OK;
    // External records stay ordinary, host-visible events when captured into a
    // graph; outside a capture the record is a plain one.
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    AZU_TRY_CUDA(cudaStreamIsCapturing(s, &cs));
    if (cs == cudaStreamCaptureStatusActive)
        AZU_TRY_CUDA(cudaEventRecordWithFlags(pl->ev[k], s, cudaEventRecordExternal));
    else
        AZU_TRY_CUDA(cudaEventRecord(pl->ev[k], s));
    return AZU_OK;
}

// Input stage: depth in metres (preprocessed Kinect codes or mm), then the
// tracker's live frame maps.
static int enqueue_input(azu_pipeline* pl, cudaStream_t s) {
    const azu_pipeline_params& P = pl->p;
    const float lo = P.min_depth, hi = P.max_depth;
    const int W = pl->W, H = pl->H;
    if (int rc = mark(pl, 0, s)) return rc;
    if (P.input_is_mm) {
        float* out = two_streams(pl) ? pl->d_depth2[pl->buf] : pl->d_depth_m;
        if (int rc = mm_to_meters_enqueue(pl->d_in, out, W * H, lo, hi, s)) return rc;
    } else {
        if (int rc = preprocess_enqueue(pl->pre, lo, hi, s)) return rc;
        // the next frame's preprocessing overwrites the preprocessor's output
        if (two_streams(pl))
            AZU_TRY_CUDA(cudaMemcpyAsync(pl->d_depth2[pl->buf], preprocess_depth_m(pl->pre),
                                         static_cast<size_t>(W) * H * 4, cudaMemcpyDeviceToDevice, s));
    }
    if (int rc = mark(pl, 1, s)) return rc;
    if (int rc = tracker_prepare_dev(pl->trk, depth_source(pl), W, H, s)) return rc;
    // the integration's depth tiles depend on the depth only
    if (two_streams(pl))
        if (int rc = volume_build_tiles_dev(depth_source(pl), W, H, lo, hi, pl->d_tiles2[pl->buf], s)) return rc;
    return mark(pl, 2, s);
}

// Tracking (or the first-frame pose); the prediction it starts from was made
// by the previous frame's commit.
static int enqueue_track(azu_pipeline* pl, bool first, cudaStream_t s) {
    PoseState* st = pl->d_st;
    if (first) {
        first_frame_kernel<<<1, 32, 0, s>>>(st);
        AZU_LAUNCH_CHECK();
    } else {
        // pred / prev / last were set by the previous frame's commit
        if (int rc = tracker_track_dev(pl->trk, pl->d_model_v, pl->d_model_n, pl->W, pl->H, st->pred, st->model_pose,
                                       st->prev, st->cur, pl->d_icp, &st->quality, &st->gate, s))
            return rc;
    }
    return mark(pl, 3, s);
}

int pipeline_enqueue_input_on(azu_pipeline* pl, cudaStream_t s) { return enqueue_input(pl, s); }
int pipeline_enqueue_track_on(azu_pipeline* pl, bool first, cudaStream_t s) { return enqueue_track(pl, first, s); }

// What this pipeline's tracking of a frame reads and writes (a batch tracks
// its scenes together with it).
TrackDev pipeline_track_dev(azu_pipeline* pl) {
    PoseState* st = pl->d_st;
    return TrackDev{pl->d_model_v, pl->d_model_n, pl->W, pl->H, st->pred, st->model_pose, st->prev, st->cur,
                    pl->d_icp, &st->quality, &st->gate};
}

// Front of one frame after the inputs are on the device, on stream s (the
// pipeline's own by default): depth, frame maps and tracking.
int pipeline_enqueue_front_on(azu_pipeline* pl, bool first, cudaStream_t s) {
    if (int rc = enqueue_input(pl, s)) return rc;
    return enqueue_track(pl, first, s);
}
int pipeline_enqueue_front(azu_pipeline* pl, bool first) { return pipeline_enqueue_front_on(pl, first, pl->s); }

// The model commit that closes a frame (after the gated integrate + raycast).
int pipeline_enqueue_commit(azu_pipeline* pl) {
    commit_kernel<<<1, 32, 0, pl->s>>>(pl->d_st);
    AZU_LAUNCH_CHECK();
    return AZU_OK;
}

// Everything a batch needs to integrate and raycast this pipeline's frame.
PipelineFrameView pipeline_frame_view(azu_pipeline* pl) {
    const azu_tracker_params& T = pl->p.tracker;
    return PipelineFrameView{pl->vol, depth_source(pl), pl->d_st->cur, &pl->d_st->gate, pl->W, pl->H, T.fx, T.fy,
                             T.cx, T.cy, pl->p.min_depth, pl->p.max_depth, pl->d_model_v, pl->d_model_n};
}

// Gated integrate + raycast of the frame and the model commit.
static int enqueue_tail(azu_pipeline* pl, cudaStream_t s) {
    const azu_pipeline_params& P = pl->p;
    const azu_tracker_params& T = P.tracker;
    const int W = pl->W, H = pl->H;
    PoseState* st = pl->d_st;
    if (int rc = volume_integrate_dev(pl->vol, depth_source(pl), nullptr, st->cur, T.fx, T.fy, T.cx, T.cy, W, H,
                                      P.min_depth, P.max_depth, &st->gate, s,
                                      two_streams(pl) ? pl->d_tiles2[pl->buf] : nullptr))
        return rc;
    if (two_streams(pl)) {
        // an external record node when captured, so the next frame's input
        // stage can wait for it from outside the graph
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        AZU_TRY_CUDA(cudaStreamIsCapturing(s, &cs));
        if (cs == cudaStreamCaptureStatusActive)
            AZU_TRY_CUDA(cudaEventRecordWithFlags(pl->ev_fused, s, cudaEventRecordExternal));
        else
            AZU_TRY_CUDA(cudaEventRecord(pl->ev_fused, s));
    }
    if (int rc = mark(pl, 4, s)) return rc;
    if (int rc = volume_raycast_dev(pl->vol, st->cur, T.fx, T.fy, T.cx, T.cy, W, H, pl->d_model_v, pl->d_model_n,
                                    nullptr, &st->gate, s))
        return rc;
    if (int rc = pipeline_enqueue_commit(pl)) return rc;
    return mark(pl, 5, s);
}

// Runs `enqueue` on stream s through the captured graph in (graph, exec),
// capturing it on first use. A capture that fails turns graphs off for the
// pipeline and runs the work eagerly (capture is an optimisation only).
template <typename F>
static int run_part(azu_pipeline* pl, cudaGraph_t& graph, cudaGraphExec_t& exec, cudaStream_t s, F enqueue) {
    if (!pl->p.use_graph) return enqueue();
    if (!exec) {
        AZU_TRY_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue();
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(s, &g);
        cudaError_t ei = cudaErrorUnknown;
        if (!rc && e == cudaSuccess) ei = cudaGraphInstantiate(&exec, g, 0);
        if (rc || e != cudaSuccess || ei != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            exec = nullptr;
            cudaGetLastError();
            pl->p.use_graph = 0;
            pl->graph_failed = 1;
            return enqueue();
        }
        graph = g;
    }
    AZU_TRY_CUDA(cudaGraphLaunch(exec, s));
    return AZU_OK;
}

static int run_frame(azu_pipeline* pl, bool stage_result = false) {
    const bool first = pl->frames == 0;
    if (two_streams(pl)) {
        // input stage on s2 once frame k-1's tracking no longer needs the live
        // maps (and frame k-2's fusion no longer needs this depth buffer), and
        // not before frame k-1's integrate is done: beside the persistent
        // integrate its kernels only slow it, while the raycast's tail leaves
        // SMs idle (frame period 0.542 -> 0.535 ms on c2 raw codes)
        const int b = pl->buf;
        cudaStream_t s = pl->s, s2 = pl->s2;
        AZU_TRY_CUDA(cudaStreamWaitEvent(s2, pl->ev_track, 0));
        AZU_TRY_CUDA(cudaStreamWaitEvent(s2, pl->ev_fused, 0));
        int rc = first ? enqueue_input(pl, s2)
                       : run_part(pl, pl->g_part[b], pl->x_part[b], s2, [&] { return enqueue_input(pl, s2); });
        if (rc) return rc;
        AZU_TRY_CUDA(cudaEventRecord(pl->ev_front, s2));
        AZU_TRY_CUDA(cudaStreamWaitEvent(s, pl->ev_front, 0));
        rc = first ? enqueue_track(pl, true, s)
                   : run_part(pl, pl->g_part[2], pl->x_part[2], s, [&] { return enqueue_track(pl, false, s); });
        if (rc) return rc;
        AZU_TRY_CUDA(cudaEventRecord(pl->ev_track, s));
        if (stage_result) {
            // on a third stream, so the fusion does not wait for the copies; only
            // what the tracking wrote and the fusion does not touch is read
            cudaStream_t s3 = pl->s3;
            AZU_TRY_CUDA(cudaStreamWaitEvent(s3, pl->ev_track, 0));
            AZU_TRY_CUDA(cudaMemcpyAsync(pl->h_st->cur, pl->d_st->cur, sizeof(pl->h_st->cur), cudaMemcpyDeviceToHost,
                                         s3));
            AZU_TRY_CUDA(cudaMemcpyAsync(&pl->h_st->quality, &pl->d_st->quality, 2 * sizeof(int),
                                         cudaMemcpyDeviceToHost, s3));  // quality, gate
            AZU_TRY_CUDA(cudaMemcpyAsync(pl->h_icp, pl->d_icp, sizeof(azu_icp_result), cudaMemcpyDeviceToHost, s3));
            AZU_TRY_CUDA(cudaEventRecord(pl->ev_result, s3));
        }
        rc = first ? enqueue_tail(pl, s)
                   : run_part(pl, pl->g_part[3 + b], pl->x_part[3 + b], s, [&] { return enqueue_tail(pl, s); });
        if (rc) return rc;
        pl->buf ^= 1;
    } else if (first || !pl->p.use_graph) {
        if (int rc = pipeline_enqueue_front(pl, first)) return rc;
        if (int rc = enqueue_tail(pl, pl->s)) return rc;
    } else {
        if (int rc = run_part(pl, pl->graph, pl->exec, pl->s, [&] {
                if (int r = pipeline_enqueue_front(pl, false)) return r;
                return enqueue_tail(pl, pl->s);
            }))
            return rc;
    }
    pl->frames++;
    pl->vol->integrated_frames++;
    return AZU_OK;
}

int pipeline_upload_inputs(azu_pipeline* pl, const uint16_t* depth, const uint8_t* rgb, cudaMemcpyKind kind) {
    const size_t n = static_cast<size_t>(pl->W) * pl->H;
    cudaStream_t s = front_stream(pl);
    if (pl->p.input_is_mm) {
        AZU_TRY_CUDA(cudaMemcpyAsync(pl->d_in, depth, n * 2, kind, s));
    } else {
        AZU_TRY_CUDA(cudaMemcpyAsync(preprocess_input(pl->pre), depth, n * 2, kind, s));
        if (rgb) AZU_TRY_CUDA(cudaMemcpyAsync(preprocess_rgb_input(pl->pre), rgb, n * 3, kind, s));
    }
    return AZU_OK;
}

// The result of the frame just run with stage_result: it is known once the
// tracking is done (integrated = the gate the fusion runs under), so this
// waits for that point only.
static int read_staged_result(azu_pipeline* pl, azu_frame_result* out) {
    AZU_TRY_CUDA(cudaEventSynchronize(pl->ev_result));
    const PoseState& st = *pl->h_st;
    std::memcpy(out->pose, st.cur, sizeof(out->pose));
    out->icp = *pl->h_icp;
    out->quality = st.quality;
    out->integrated = st.gate;
    out->frame_index = pl->frames - 1;  // run_frame has counted this frame
    if (st.quality == -1) std::memset(&out->icp, 0, sizeof(out->icp));
    if (out->icp.status == AZU_E_TIMEOUT) {
        // the frame was graded Failed on the device; the next frame's tracking
        // (after this on the pipeline's stream) starts from clean barrier words
        if (int rc = tracker_clear_barrier(pl->trk, pl->s)) return rc;
        set_error("ICP grid barrier timed out");
        return AZU_E_TIMEOUT;
    }
    return AZU_OK;
}

// One frame whose inputs are being uploaded, with its result read back.
static int run_frame_with_result(azu_pipeline* pl, azu_frame_result* out) {
    if (two_streams(pl) && !pl->profiling) {
        if (int rc = run_frame(pl, true)) return rc;
        return read_staged_result(pl, out);
    }
    if (int rc = run_frame(pl)) return rc;
    return pipeline_read_result(pl, out);
}

int pipeline_read_result(azu_pipeline* pl, azu_frame_result* out) {
    PoseState st;
    AZU_TRY_CUDA(cudaMemcpyAsync(&st, pl->d_st, sizeof(st), cudaMemcpyDeviceToHost, pl->s));
    AZU_TRY_CUDA(cudaMemcpyAsync(&out->icp, pl->d_icp, sizeof(azu_icp_result), cudaMemcpyDeviceToHost, pl->s));
    AZU_TRY_CUDA(cudaStreamSynchronize(pl->s));
    if (pl->profiling) {
        float ms[5];
        bool ok = true;
        for (int k = 0; k < 5 && ok; ++k) ok = cudaEventElapsedTime(&ms[k], pl->ev[k], pl->ev[k + 1]) == cudaSuccess;
        if (ok) {
            for (int k = 0; k < 5; ++k) pl->stage_ms[k] += ms[k];
            pl->stage_frames++;
        } else {
            cudaGetLastError();  // an unreadable frame is skipped, not a sticky error
        }
    }
    std::memcpy(out->pose, st.cur, sizeof(out->pose));
    out->quality = st.quality;
    out->integrated = st.integrated;
    out->frame_index = st.frame_index - 1;
    if (st.quality == -1) std::memset(&out->icp, 0, sizeof(out->icp));
    if (out->icp.status == AZU_E_TIMEOUT) {
        if (int rc = tracker_clear_barrier(pl->trk, pl->s)) return rc;
        set_error("ICP grid barrier timed out");
        return AZU_E_TIMEOUT;
    }
    return AZU_OK;
}

}  // namespace azu

using namespace azu;

static void drop_graphs(azu_pipeline* pl) {
    if (pl->exec) cudaGraphExecDestroy(pl->exec);
    if (pl->graph) cudaGraphDestroy(pl->graph);
    pl->exec = nullptr;
    pl->graph = nullptr;
    for (int k = 0; k < 5; ++k) {
        if (pl->x_part[k]) cudaGraphExecDestroy(pl->x_part[k]);
        if (pl->g_part[k]) cudaGraphDestroy(pl->g_part[k]);
        pl->x_part[k] = nullptr;
        pl->g_part[k] = nullptr;
    }
}

extern "C" int azu_pipeline_destroy(azu_pipeline* pl) {
    if (!pl) return AZU_OK;
    cudaSetDevice(pl->device);
    if (pl->s2) cudaStreamSynchronize(pl->s2);
    if (pl->s3) cudaStreamSynchronize(pl->s3);
    if (pl->s) cudaStreamSynchronize(pl->s);
    drop_graphs(pl);
    azu_preprocessor_destroy(pl->pre);
    azu_tracker_destroy(pl->trk);
    azu_volume_destroy(pl->vol);
    for (void* q : {(void*)pl->d_in, (void*)pl->d_depth_m, (void*)pl->d_model_v, (void*)pl->d_model_n,
                    (void*)pl->d_st, (void*)pl->d_icp, (void*)pl->d_packed, (void*)pl->d_depth2[0],
                    (void*)pl->d_depth2[1], (void*)pl->d_tiles2[0], (void*)pl->d_tiles2[1]})
        if (q) cudaFree(q);
    if (pl->h_st) cudaFreeHost(pl->h_st);
    if (pl->h_icp) cudaFreeHost(pl->h_icp);
    for (cudaEvent_t e : pl->ev) if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : {pl->ev_front, pl->ev_track, pl->ev_result, pl->ev_fused}) if (e) cudaEventDestroy(e);
    if (pl->s2) cudaStreamDestroy(pl->s2);
    if (pl->s3) cudaStreamDestroy(pl->s3);
    if (pl->s && pl->own_stream) cudaStreamDestroy(pl->s);
    delete pl;
    return AZU_OK;
}

namespace azu {
// A pipeline on the given stream (not owned), or on its own when null.
int pipeline_create_on(int device, const azu_pipeline_params* p, cudaStream_t stream, azu_pipeline** out) {
    AZU_CHECK_ARG(p != nullptr && out != nullptr, "null argument");
    *out = nullptr;
    const int W = p->width > 0 ? p->width : 640, H = p->height > 0 ? p->height : 480;
    AZU_CHECK_ARG(W >= 8 && H >= 8 && W <= 8192 && H <= 8192 && W % 4 == 0 && H % 4 == 0,
                  "image size must be multiples of 4 in [8, 8192]");
    AZU_CHECK_ARG(p->input_is_mm || (W == 640 && H == 480), "the Kinect raw-code path is 640 x 480");
    if (int rc = bind_device(device)) return rc;
    azu_pipeline* pl = new azu_pipeline();
    pl->device = device;
    pl->p = *p;
    pl->W = W;
    pl->H = H;
    int rc = AZU_OK;
    cudaError_t e = cudaSuccess;
    if (stream) {
        pl->s = stream;
        pl->own_stream = false;
    } else {
        // the frame's critical path (tracking, fusion) gets the highest
        // priority; the next frame's input stage (second stream) fills the gaps
        int least = 0, greatest = 0;
        e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
        if (!e) e = cudaStreamCreateWithPriority(&pl->s, cudaStreamNonBlocking, greatest);
    }
    if (e) { set_error("stream: %s", cudaGetErrorString(e)); rc = AZU_E_CUDA; }
    if (!rc) rc = azu_volume_create(device, &p->volume, pl->s, &pl->vol);
    if (!rc) rc = azu_tracker_create(device, &p->tracker, pl->s, &pl->trk);
    if (!rc && !p->input_is_mm) rc = azu_preprocessor_create(device, p->preprocess_mode, pl->s, &pl->pre);
    if (!rc) {
        const size_t n = static_cast<size_t>(W) * H;
        e = cudaMalloc(&pl->d_in, n * 2);
        if (!e) e = cudaMalloc(&pl->d_depth_m, n * 4);
        if (!e) e = cudaMalloc(&pl->d_model_v, n * 12);
        if (!e) e = cudaMalloc(&pl->d_model_n, n * 12);
        if (!e) e = cudaMalloc(&pl->d_st, sizeof(PoseState));
        if (!e) e = cudaMalloc(&pl->d_icp, sizeof(azu_icp_result));
        if (!e) e = cudaMemsetAsync(pl->d_icp, 0, sizeof(azu_icp_result), pl->s);
        for (int k = 0; !e && k < 6; ++k) e = cudaEventCreate(&pl->ev[k]);
        if (!e && pl->own_stream) {
            // the second stream of the two-stream schedule
            int least = 0, greatest = 0;
            e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
            if (!e) e = cudaStreamCreateWithPriority(&pl->s2, cudaStreamNonBlocking, least);
            if (!e) e = cudaStreamCreateWithFlags(&pl->s3, cudaStreamNonBlocking);
            for (cudaEvent_t* ev : {&pl->ev_front, &pl->ev_track, &pl->ev_result, &pl->ev_fused})
                if (!e) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
            for (int k = 0; !e && k < 2; ++k) e = cudaMalloc(&pl->d_depth2[k], n * 4);
            const size_t nt = static_cast<size_t>(make_tile_mip(W, H).total);
            for (int k = 0; !e && k < 2; ++k) e = cudaMalloc(&pl->d_tiles2[k], nt * 4);
            if (!e) e = cudaHostAlloc(&pl->h_st, sizeof(PoseState), cudaHostAllocDefault);
            if (!e) e = cudaHostAlloc(&pl->h_icp, sizeof(azu_icp_result), cudaHostAllocDefault);
        }
        if (e) { set_error("pipeline allocation: %s", cudaGetErrorString(e)); rc = AZU_E_NOMEM; }
    }
    if (rc) { azu_pipeline_destroy(pl); return rc; }
    *out = pl;
    return AZU_OK;
}
}  // namespace azu

extern "C" int azu_pipeline_create(int device, const azu_pipeline_params* p, azu_pipeline** out) {
    return pipeline_create_on(device, p, nullptr, out);
}

extern "C" int azu_pipeline_reset(azu_pipeline* pl) {
    AZU_CHECK_ARG(pl != nullptr, "null handle");
    AZU_TRY_CUDA(cudaSetDevice(pl->device));
    if (pl->s2) AZU_TRY_CUDA(cudaStreamSynchronize(pl->s2));
    if (pl->s3) AZU_TRY_CUDA(cudaStreamSynchronize(pl->s3));
    AZU_TRY_CUDA(cudaStreamSynchronize(pl->s));
    if (int rc = azu_volume_reset(pl->vol)) return rc;
    if (pl->pre) if (int rc = azu_preprocessor_reset(pl->pre)) return rc;
    if (int rc = tracker_clear_barrier(pl->trk, pl->s)) return rc;
    AZU_TRY_CUDA(cudaStreamSynchronize(pl->s));
    pl->frames = 0;
    pl->buf = 0;
    pl->vol->integrated_frames = 0;
    return AZU_OK;
}

extern "C" int azu_pipeline_process_frame(azu_pipeline* pl, const uint16_t* h_depth, const uint8_t* h_rgb,
                                          azu_frame_result* out) {
    AZU_CHECK_ARG(pl != nullptr && h_depth != nullptr && out != nullptr, "null argument");
    AZU_CHECK_ARG(pl->p.input_is_mm || h_rgb != nullptr, "the raw-code path needs the RGB frame for guidance");
    AZU_TRY_CUDA(cudaSetDevice(pl->device));
    if (int rc = pipeline_upload_inputs(pl, h_depth, h_rgb, cudaMemcpyHostToDevice)) return rc;
    return run_frame_with_result(pl, out);
}

extern "C" int azu_pipeline_process_frame_device(azu_pipeline* pl, const uint16_t* d_depth, const uint8_t* d_rgb,
                                                 azu_frame_result* out) {
    AZU_CHECK_ARG(pl != nullptr && d_depth != nullptr, "null argument");
    AZU_CHECK_ARG(pl->p.input_is_mm || d_rgb != nullptr, "the raw-code path needs the RGB frame for guidance");
    AZU_TRY_CUDA(cudaSetDevice(pl->device));
    if (int rc = pipeline_upload_inputs(pl, d_depth, d_rgb, cudaMemcpyDeviceToDevice)) return rc;
    if (out) return run_frame_with_result(pl, out);
    return run_frame(pl);
}

extern "C" int azu_pipeline_process_frame_packed(azu_pipeline* pl, const void* h_packed, azu_frame_result* out) {
    AZU_CHECK_ARG(pl != nullptr && h_packed != nullptr && out != nullptr, "null argument");
    AZU_TRY_CUDA(cudaSetDevice(pl->device));
    const size_t n = static_cast<size_t>(pl->W) * pl->H;
    const size_t bytes = n * (pl->p.input_is_mm ? 2 : 5);
    if (!pl->d_packed) AZU_TRY_CUDA(cudaMalloc(&pl->d_packed, n * 5));
    // the one host-to-device copy of the frame; the split happens on the device
    AZU_TRY_CUDA(cudaMemcpyAsync(pl->d_packed, h_packed, bytes, cudaMemcpyHostToDevice, front_stream(pl)));
    const uint16_t* d_depth = reinterpret_cast<const uint16_t*>(pl->d_packed);
    const uint8_t* d_rgb = pl->p.input_is_mm ? nullptr : pl->d_packed + n * 2;
    if (int rc = pipeline_upload_inputs(pl, d_depth, d_rgb, cudaMemcpyDeviceToDevice)) return rc;
    return run_frame_with_result(pl, out);
}

extern "C" int azu_pipeline_last_result(azu_pipeline* pl, azu_frame_result* out) {
    AZU_CHECK_ARG(pl != nullptr && out != nullptr, "null argument");
    AZU_TRY_CUDA(cudaSetDevice(pl->device));
    return pipeline_read_result(pl, out);
}

extern "C" azu_volume* azu_pipeline_volume(azu_pipeline* pl) { return pl ? pl->vol : nullptr; }
extern "C" azu_tracker* azu_pipeline_tracker(azu_pipeline* pl) { return pl ? pl->trk : nullptr; }

extern "C" int azu_pipeline_model_maps(azu_pipeline* pl, const float** d_vertices, const float** d_normals) {
    AZU_CHECK_ARG(pl != nullptr, "null handle");
    if (d_vertices) *d_vertices = pl->d_model_v;
    if (d_normals) *d_normals = pl->d_model_n;
    return AZU_OK;
}

extern "C" void* azu_pipeline_stream(azu_pipeline* pl) { return pl ? static_cast<void*>(pl->s) : nullptr; }

extern "C" int azu_pipeline_set_profiling(azu_pipeline* pl, int on) {
    AZU_CHECK_ARG(pl != nullptr, "null handle");
    if ((on != 0) != pl->profiling) {
        // Event records are part of the captured graphs: recapture.
        if (pl->s2) AZU_TRY_CUDA(cudaStreamSynchronize(pl->s2));
        if (pl->s3) AZU_TRY_CUDA(cudaStreamSynchronize(pl->s3));
        AZU_TRY_CUDA(cudaStreamSynchronize(pl->s));
        drop_graphs(pl);
    }
    pl->profiling = on != 0;
    for (double& v : pl->stage_ms) v = 0.0;
    pl->stage_frames = 0;
    return AZU_OK;
}

extern "C" int azu_pipeline_stage_times(azu_pipeline* pl, double ms_total[5], int* frames) {
    AZU_CHECK_ARG(pl != nullptr && ms_total != nullptr, "null argument");
    for (int k = 0; k < 5; ++k) ms_total[k] = pl->stage_ms[k];
    if (frames) *frames = pl->stage_frames;
    return AZU_OK;
}

extern "C" int azu_pipeline_uses_graph(azu_pipeline* pl) {
    return pl ? (pl->p.use_graph && !pl->graph_failed ? 1 : 0) : 0;
}
