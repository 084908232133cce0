// Batching form (no counterpart in the reference): many independent scenes,
// each with its own volume, image size and frame count, advanced one frame at
// a time together. The scenes' input stages (millimetre depth -> metres,
// vertices/normals/pyramid, depth tiles) run side by side, each on its own
// stream; then ONE cooperative ICP launch tracks every scene on an equal
// share of the SMs (the ICP's partial slots, hence its sums, do not depend on
// the blocks it runs on); integration and raycasting of all active scenes run
// as ONE launch per stage (tsdf.cu batches), and the whole step replays as one
// CUDA graph per set of active scenes. Every scene's result equals its result
// through the single pipeline bit for bit.
//
// Autotuner: the integrate block size (1, 2 or 4 warps) and the raycast tile
// shape are timed on the batch's own data — raycasts as they are (they are
// idempotent at a fixed pose), integrations on a scratch copy of the voxels
// that is restored afterwards — and the fastest pair is kept.
#include <algorithm>
#include <cstring>
#include <functional>
#include <map>
#include <vector>

#include "azu_internal.h"

struct azu_batch {
    int device = 0;
    cudaStream_t s = nullptr;
    std::vector<azu_pipeline*> scenes;
    std::vector<cudaStream_t> fs;    // per scene: the stream of its front
    std::vector<cudaEvent_t> fdone;  // per scene: its front is done
    cudaEvent_t fork = nullptr;
    std::vector<int> frames;
    std::map<unsigned long long, azu_volume_batch*> vbatch;  // by active mask (first 64 scenes)
    std::map<unsigned long long, azu_icp_batch*> ibatch;
    std::map<unsigned long long, cudaGraphExec_t> graphs;
    int int_warps = 4, int_parts = 2, ray_w = 32, ray_h = 8;
    bool tuned = false;
    bool use_graph = true;
    std::vector<azu_frame_result> host_results;
};

namespace azu {

static unsigned long long mask_of(const std::vector<int>& active) {
    unsigned long long m = 0;
    for (int i : active) m |= 1ull << (i & 63);
    return m ^ (static_cast<unsigned long long>(active.size()) << 58);
}

static int icp_batch_for(azu_batch* b, const std::vector<int>& active, azu_icp_batch** out) {
    const unsigned long long key = mask_of(active);
    auto it = b->ibatch.find(key);
    if (it != b->ibatch.end()) {
        *out = it->second;
        return AZU_OK;
    }
    std::vector<azu_tracker*> t;
    std::vector<TrackDev> d;
    for (int i : active) {
        t.push_back(azu_pipeline_tracker(b->scenes[i]));
        d.push_back(pipeline_track_dev(b->scenes[i]));
    }
    azu_icp_batch* ib = nullptr;
    if (int rc = icp_batch_create(t.data(), d.data(), static_cast<int>(active.size()), &ib)) return rc;
    b->ibatch[key] = ib;
    *out = ib;
    return AZU_OK;
}

static int volume_batch_for(azu_batch* b, const std::vector<int>& active, azu_volume_batch** out) {
    const unsigned long long key = mask_of(active);
    auto it = b->vbatch.find(key);
    if (it != b->vbatch.end()) {
        *out = it->second;
        return AZU_OK;
    }
    std::vector<PipelineFrameView> views;
    for (int i : active) views.push_back(pipeline_frame_view(b->scenes[i]));
    azu_volume_batch* vb = nullptr;
    if (int rc = volume_batch_create(views.data(), static_cast<int>(views.size()), &vb)) return rc;
    if (int rc = volume_batch_set_shapes(vb, b->int_warps, b->int_parts, b->ray_w, b->ray_h)) {
        volume_batch_destroy(vb);
        return rc;
    }
    b->vbatch[key] = vb;
    *out = vb;
    return AZU_OK;
}

// The device work of one step for the given scenes (inputs already uploaded).
static int enqueue_step(azu_batch* b, const std::vector<int>& active, bool first, azu_volume_batch* vb,
                        azu_icp_batch* ib) {
    AZU_TRY_CUDA(cudaEventRecord(b->fork, b->s));
    for (int i : active) {
        AZU_TRY_CUDA(cudaStreamWaitEvent(b->fs[i], b->fork, 0));
        if (int rc = pipeline_enqueue_input_on(b->scenes[i], b->fs[i])) return rc;
        AZU_TRY_CUDA(cudaEventRecord(b->fdone[i], b->fs[i]));
        AZU_TRY_CUDA(cudaStreamWaitEvent(b->s, b->fdone[i], 0));
    }
    if (first) {
        for (int i : active)
            if (int rc = pipeline_enqueue_track_on(b->scenes[i], true, b->s)) return rc;
    } else if (int rc = icp_batch_launch(ib, b->s)) {
        return rc;
    }
    if (int rc = volume_batch_integrate(vb, b->s)) return rc;
    if (int rc = volume_batch_raycast(vb, b->s)) return rc;
    for (int i : active)
        if (int rc = pipeline_enqueue_commit(b->scenes[i])) return rc;
    return AZU_OK;
}

static void drop_graphs(azu_batch* b) {
    for (auto& g : b->graphs) cudaGraphExecDestroy(g.second);
    b->graphs.clear();
}

static int apply_shapes(azu_batch* b) {
    for (auto& v : b->vbatch)
        if (int rc = volume_batch_set_shapes(v.second, b->int_warps, b->int_parts, b->ray_w, b->ray_h)) return rc;
    drop_graphs(b);  // captured launches carry the old shapes
    return AZU_OK;
}

static int time_ms(cudaStream_t s, float* ms, const std::function<int()>& f, int reps) {
    cudaEvent_t e0, e1;
    AZU_TRY_CUDA(cudaEventCreate(&e0));
    AZU_TRY_CUDA(cudaEventCreate(&e1));
    int rc = f();  // warm-up
    if (!rc) rc = cudaEventRecord(e0, s) == cudaSuccess ? AZU_OK : AZU_E_CUDA;
    for (int r = 0; r < reps && !rc; ++r) rc = f();
    if (!rc) rc = cudaEventRecord(e1, s) == cudaSuccess ? AZU_OK : AZU_E_CUDA;
    if (!rc) rc = cudaEventSynchronize(e1) == cudaSuccess ? AZU_OK : AZU_E_CUDA;
    if (!rc) rc = cudaEventElapsedTime(ms, e0, e1) == cudaSuccess ? AZU_OK : AZU_E_CUDA;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) set_error("autotune timing failed");
    *ms /= reps;
    return rc;
}

}  // namespace azu

using namespace azu;

extern "C" int azu_batch_destroy(azu_batch* b) {
    if (!b) return AZU_OK;
    cudaSetDevice(b->device);
    if (b->s) cudaStreamSynchronize(b->s);
    drop_graphs(b);
    for (auto& v : b->vbatch) volume_batch_destroy(v.second);
    for (auto& v : b->ibatch) icp_batch_destroy(v.second);
    for (azu_pipeline* pl : b->scenes) azu_pipeline_destroy(pl);
    for (cudaStream_t q : b->fs) if (q) cudaStreamDestroy(q);
    for (cudaEvent_t e : b->fdone) if (e) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->s) cudaStreamDestroy(b->s);
    delete b;
    return AZU_OK;
}

extern "C" int azu_batch_create(int device, int n, const azu_batch_scene* scenes, azu_batch** out) {
    AZU_CHECK_ARG(out != nullptr && scenes != nullptr && n >= 1 && n <= 64, "batch of 1..64 scenes");
    *out = nullptr;
    if (int rc = bind_device(device)) return rc;
    azu_batch* b = new azu_batch();
    b->device = device;
    int rc = AZU_OK;
    if (cudaStreamCreateWithFlags(&b->s, cudaStreamNonBlocking) != cudaSuccess) {
        set_error("batch stream");
        rc = AZU_E_CUDA;
    }
    for (int i = 0; i < n && !rc; ++i) {
        const azu_batch_scene& sc = scenes[i];
        if (sc.volume.format != AZU_TSDF_FP32 || sc.volume.color) {
            set_error("batched volumes are FP32 without colour");
            rc = AZU_E_INVALID;
            break;
        }
        azu_pipeline_params pp{};
        pp.volume = sc.volume;
        pp.tracker = sc.tracker;
        pp.preprocess_mode = AZU_PRE_FULL;
        pp.min_depth = sc.min_depth;
        pp.max_depth = sc.max_depth;
        pp.input_is_mm = 1;
        pp.use_graph = 0;
        pp.width = sc.width;
        pp.height = sc.height;
        azu_pipeline* pl = nullptr;
        rc = pipeline_create_on(device, &pp, b->s, &pl);
        if (!rc) b->scenes.push_back(pl);
        cudaStream_t q = nullptr;
        cudaEvent_t e = nullptr;
        if (!rc && (cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking) != cudaSuccess ||
                    cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)) {
            set_error("batch front stream");
            rc = AZU_E_CUDA;
        }
        b->fs.push_back(q);
        b->fdone.push_back(e);
    }
    if (!rc && cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess) {
        set_error("batch fork event");
        rc = AZU_E_CUDA;
    }
    if (rc) {
        azu_batch_destroy(b);
        return rc;
    }
    b->frames.assign(n, 0);
    b->host_results.resize(n);
    *out = b;
    return AZU_OK;
}

extern "C" int azu_batch_set_shapes(azu_batch* b, int int_warps, int int_parts, int ray_w, int ray_h) {
    AZU_CHECK_ARG(b != nullptr, "null handle");
    AZU_CHECK_ARG(int_warps == 1 || int_warps == 2 || int_warps == 4, "integrate warps per block: 1, 2 or 4");
    AZU_CHECK_ARG(int_parts == 1 || int_parts == 2 || int_parts == 4, "integrate x-parts per row: 1, 2 or 4");
    AZU_CHECK_ARG(ray_w >= 8 && ray_h >= 1 && ray_w * ray_h <= 256 && (ray_w * ray_h) % 32 == 0,
                  "raycast tile: at most 256 threads, whole warps");
    AZU_TRY_CUDA(cudaSetDevice(b->device));
    AZU_TRY_CUDA(cudaStreamSynchronize(b->s));
    b->int_warps = int_warps;
    b->int_parts = int_parts;
    b->ray_w = ray_w;
    b->ray_h = ray_h;
    b->tuned = true;
    return apply_shapes(b);
}

extern "C" int azu_batch_get_shapes(azu_batch* b, int* int_warps, int* int_parts, int* ray_w, int* ray_h) {
    AZU_CHECK_ARG(b != nullptr, "null handle");
    if (int_warps) *int_warps = b->int_warps;
    if (int_parts) *int_parts = b->int_parts;
    if (ray_w) *ray_w = b->ray_w;
    if (ray_h) *ray_h = b->ray_h;
    return AZU_OK;
}

extern "C" int azu_batch_autotune(azu_batch* b, float* best_integrate_ms, float* best_raycast_ms) {
    AZU_CHECK_ARG(b != nullptr, "null handle");
    AZU_TRY_CUDA(cudaSetDevice(b->device));
    std::vector<int> all;
    for (size_t i = 0; i < b->scenes.size(); ++i)
        if (b->frames[i] > 0) all.push_back(static_cast<int>(i));
    AZU_CHECK_ARG(!all.empty(), "autotune needs at least one processed frame");
    azu_volume_batch* vb = nullptr;
    if (int rc = volume_batch_for(b, all, &vb)) return rc;
    AZU_TRY_CUDA(cudaStreamSynchronize(b->s));
    // raycast tiles: idempotent at the current poses
    const int tiles[][2] = {{32, 8}, {32, 4}, {64, 4}, {16, 16}, {32, 2}, {128, 2}};
    float best_r = 1e30f;
    int bw = b->ray_w, bh = b->ray_h;
    for (const auto& t : tiles) {
        if (int rc = volume_batch_set_shapes(vb, b->int_warps, b->int_parts, t[0], t[1])) return rc;
        float ms = 0.0f;
        if (int rc = time_ms(b->s, &ms, [&] { return volume_batch_raycast(vb, b->s); }, 5)) return rc;
        if (ms < best_r) { best_r = ms; bw = t[0]; bh = t[1]; }
    }
    // integrate block sizes: on the voxels as they are, restored after every trial
    std::vector<void*> saved(all.size(), nullptr);
    std::vector<size_t> bytes(all.size(), 0);
    std::vector<int> frames_saved(all.size(), 0);
    std::vector<unsigned long long> counters_saved(4 * all.size(), 0);
    int rc = AZU_OK;
    for (size_t k = 0; k < all.size() && !rc; ++k) {
        azu_volume* v = azu_pipeline_volume(b->scenes[all[k]]);
        frames_saved[k] = v->integrated_frames;
        if (cudaMemcpyAsync(&counters_saved[4 * k], v->d_counters, 4 * sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, b->s) != cudaSuccess)
            rc = AZU_E_CUDA;
        const size_t n = static_cast<size_t>(v->p.resolution) * v->p.resolution * v->p.resolution;
        bytes[k] = n * voxel_bytes(v->p.format);
        if (cudaMalloc(&saved[k], bytes[k]) != cudaSuccess) { set_error("autotune scratch"); rc = AZU_E_NOMEM; break; }
        if (cudaMemcpyAsync(saved[k], v->vox, bytes[k], cudaMemcpyDeviceToDevice, b->s) != cudaSuccess) rc = AZU_E_CUDA;
    }
    auto restore = [&]() {
        for (size_t k = 0; k < all.size(); ++k) {
            azu_volume* v = azu_pipeline_volume(b->scenes[all[k]]);
            if (cudaMemcpyAsync(v->vox, saved[k], bytes[k], cudaMemcpyDeviceToDevice, b->s) != cudaSuccess)
                return AZU_E_CUDA;
        }
        return AZU_OK;
    };
    // integrate item shapes: warps per block x x-parts per 32-row item
    float best_i = 1e30f;
    int bwarps = b->int_warps, bparts = b->int_parts;
    for (int warps : {1, 2, 4}) {
        for (int parts : {1, 2, 4}) {
            if (rc) break;
            rc = volume_batch_set_shapes(vb, warps, parts, bw, bh);
            float ms = 0.0f;
            if (!rc) rc = time_ms(b->s, &ms, [&] { return volume_batch_integrate(vb, b->s); }, 3);
            if (!rc) rc = restore();
            if (!rc && ms < best_i) { best_i = ms; bwarps = warps; bparts = parts; }
        }
    }
    // integrations changed counters and free-brick flags: recompute flags from
    // the restored voxels (conservative flags stay exact for the raycast)
    for (size_t k = 0; k < all.size() && !rc; ++k) rc = rebuild_bricks(azu_pipeline_volume(b->scenes[all[k]]), b->s);
    if (cudaStreamSynchronize(b->s) != cudaSuccess && !rc) rc = AZU_E_CUDA;
    for (void* p : saved) if (p) cudaFree(p);
    // the trials' frames and counters are not the volumes'
    for (size_t k = 0; k < all.size() && !rc; ++k) {
        azu_volume* v = azu_pipeline_volume(b->scenes[all[k]]);
        v->integrated_frames = frames_saved[k];
        if (cudaMemcpy(v->d_counters, &counters_saved[4 * k], 4 * sizeof(unsigned long long),
                       cudaMemcpyHostToDevice) != cudaSuccess)
            rc = AZU_E_CUDA;
    }
    if (rc) return rc;
    b->int_warps = bwarps;
    b->int_parts = bparts;
    b->ray_w = bw;
    b->ray_h = bh;
    b->tuned = true;
    if (best_integrate_ms) *best_integrate_ms = best_i;
    if (best_raycast_ms) *best_raycast_ms = best_r;
    return apply_shapes(b);
}

extern "C" int azu_batch_process(azu_batch* b, const uint16_t* const* depth_mm, int on_device,
                                 azu_frame_result* results) {
    AZU_CHECK_ARG(b != nullptr && depth_mm != nullptr, "null argument");
    AZU_TRY_CUDA(cudaSetDevice(b->device));
    std::vector<int> active;
    for (size_t i = 0; i < b->scenes.size(); ++i)
        if (depth_mm[i]) active.push_back(static_cast<int>(i));
    if (active.empty()) return AZU_OK;
    bool first = b->frames[active[0]] == 0;
    for (int i : active)
        AZU_CHECK_ARG((b->frames[i] == 0) == first, "scenes of one step must all be at their first frame or none");
    for (int i : active)
        if (int rc = pipeline_upload_inputs(b->scenes[i], depth_mm[i], nullptr,
                                            on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice))
            return rc;
    azu_volume_batch* vb = nullptr;
    if (int rc = volume_batch_for(b, active, &vb)) return rc;
    azu_icp_batch* ib = nullptr;
    if (int rc = icp_batch_for(b, active, &ib)) return rc;
    if (first || !b->use_graph) {
        if (int rc = enqueue_step(b, active, first, vb, ib)) return rc;
    } else {
        const unsigned long long key = mask_of(active);
        auto it = b->graphs.find(key);
        cudaGraphExec_t exec = nullptr;
        if (it == b->graphs.end()) {
            AZU_TRY_CUDA(cudaStreamBeginCapture(b->s, cudaStreamCaptureModeThreadLocal));
            const int rc = enqueue_step(b, active, false, vb, ib);
            cudaGraph_t g = nullptr;
            const cudaError_t e = cudaStreamEndCapture(b->s, &g);
            cudaError_t ei = cudaErrorUnknown;
            if (!rc && e == cudaSuccess) ei = cudaGraphInstantiate(&exec, g, 0);
            if (g) cudaGraphDestroy(g);
            if (rc || e != cudaSuccess || ei != cudaSuccess) {
                cudaGetLastError();
                b->use_graph = false;  // capture is an optimisation only
                if (int rc2 = enqueue_step(b, active, false, vb, ib)) return rc2;
                exec = nullptr;
            } else {
                b->graphs[key] = exec;
            }
        } else {
            exec = it->second;
        }
        if (exec) {
            AZU_TRY_CUDA(cudaGraphLaunch(exec, b->s));
            // the captured integrate counted one frame per volume at capture time only
            for (int i : active) azu_pipeline_volume(b->scenes[i])->integrated_frames += (it == b->graphs.end()) ? 0 : 1;
        }
    }
    for (int i : active) b->frames[i]++;
    if (results) {
        for (int i : active)
            if (int rc = pipeline_read_result(b->scenes[i], &results[i])) return rc;
    }
    return AZU_OK;
}

extern "C" azu_volume* azu_batch_volume(azu_batch* b, int i) {
    return (b && i >= 0 && i < static_cast<int>(b->scenes.size())) ? azu_pipeline_volume(b->scenes[i]) : nullptr;
}

extern "C" void* azu_batch_stream(azu_batch* b) { return b ? static_cast<void*>(b->s) : nullptr; }

extern "C" int azu_batch_uses_graph(azu_batch* b) { return b && b->use_graph ? 1 : 0; }

extern "C" int azu_batch_synchronize(azu_batch* b) {
    AZU_CHECK_ARG(b != nullptr, "null handle");
    AZU_TRY_CUDA(cudaSetDevice(b->device));
    AZU_TRY_CUDA(cudaStreamSynchronize(b->s));
    return AZU_OK;
}
