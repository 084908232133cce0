"""The whole per-frame GPU pipeline (preprocess -> pyramid -> ICP -> integrate ->
raycast, CUDA-graph replayed) against the oracle's lockstep CPU pipeline on
the same frames: identical grades and integration decisions, and poses within
5e-4 rad / 5e-4 m along the sequence. The per-frame bound on one input pose is
1e-6 (test_gpu_icp); chained over frames, a solve that stops one iteration
earlier on one side (its step is below the 5e-5 convergence threshold) moves
that frame's pose by up to the threshold, and the next frames start from it."""
import numpy as np
import pytest

import fixtures as F

pytestmark = pytest.mark.gpu


def _pipeline(seq, input_is_mm, use_graph=True, precision=0):
    from azu_gb300 import api
    v = seq.volume
    vp = api.volume_params(v["resolution"], v["voxel_size"], v["truncation"], v["max_weight"], v["origin"],
                           seq.min_depth, seq.max_depth, v["format"])
    tp = api.tracker_params(min_depth=seq.min_depth, max_depth=seq.max_depth, precision=precision)
    return api.Pipeline(api.pipeline_params(vp, tp, 0, seq.min_depth, seq.max_depth, input_is_mm, use_graph))


@pytest.fixture(scope="module")
def seq():
    from azu_gb300 import synth
    return synth.sequence("c1", frames=10)


@pytest.mark.parametrize("input_is_mm", [False, True])
def test_pipeline_matches_lockstep_oracle(cuda_lib, orc, seq, input_is_mm):
    from azu_gb300 import synth
    pl = _pipeline(seq, input_is_mm)
    L = orc.Lockstep(seq.volume, input_is_mm=input_is_mm, fold_threads=0)
    rgb = synth.grey_rgb()
    for k in range(len(seq.poses)):
        d = seq.depth_mm[k] if input_is_mm else synth.encode_raw(seq.depth_mm[k])
        g = pl.process_frame(d, None if input_is_mm else rgb)
        o = L.process(d, rgb)
        assert g["frame_index"] == k
        assert g["quality"] == o["quality"], k
        assert g["integrated"] == o["integrated"], k
        rot, trans = F.rel_pose_error(g["pose"], o["pose"])
        assert rot <= 5e-4 and trans <= 5e-4, (k, rot, trans)
        if k:
            assert g["icp"]["status"] == 0
            # association counts follow the (slightly different) poses: within 1 %
            assert abs(g["icp"]["inliers"] - o["icp"]["inliers"]) <= max(5, 1e-2 * o["icp"]["inliers"])
            rot_gt, trans_gt = F.rel_pose_error(g["pose"], seq.poses[k])
            assert rot_gt < 5e-3 and trans_gt < 1e-2, (k, rot_gt, trans_gt)


def test_graph_replay_equals_eager(cuda_lib, seq):
    a = _pipeline(seq, True, use_graph=True)
    b = _pipeline(seq, True, use_graph=False)
    for k in range(5):
        ra = a.process_frame(seq.depth_mm[k])
        rb = b.process_frame(seq.depth_mm[k])
        assert np.array_equal(ra["pose"], rb["pose"]) and ra["quality"] == rb["quality"]
    assert a.lib.azu_pipeline_uses_graph(a.h) == 1


@pytest.mark.parametrize("input_is_mm", [False, True])
def test_overlapped_schedule_equals_sequential(cuda_lib, seq, input_is_mm):
    """Frame k+1's input stage runs beside frame k's fusion and results come
    back once the pose is known; that must give exactly what a schedule that
    finishes every frame before the next gives: the same poses every frame and
    the same volume at the end, also when frames are only enqueued."""
    import torch
    from azu_gb300 import api, synth
    rgb = synth.grey_rgb()
    frames = [seq.depth_mm[k] if input_is_mm else synth.encode_raw(seq.depth_mm[k]) for k in range(len(seq.poses))]
    seqp = _pipeline(seq, input_is_mm)
    seqp.set_profiling(True)  # stage timing reads every frame back whole
    fast = _pipeline(seq, input_is_mm)
    ref = [seqp.process_frame(d, None if input_is_mm else rgb) for d in frames]
    got = [fast.process_frame(d, None if input_is_mm else rgb) for d in frames]
    for a, b in zip(ref, got):
        assert np.array_equal(a["pose"].view(np.uint32), b["pose"].view(np.uint32))
        assert (a["quality"], a["integrated"], a["frame_index"]) == (b["quality"], b["integrated"], b["frame_index"])
        assert a["icp"]["inliers"] == b["icp"]["inliers"]
    # enqueue only, no host round trip between frames
    queued = _pipeline(seq, input_is_mm)
    d_in = torch.from_numpy(np.stack(frames).astype(np.uint16).view(np.int16)).cuda()
    d_rgb = torch.from_numpy(rgb).cuda()
    for k in range(len(frames)):
        queued.process_frame_device(d_in[k].data_ptr(), None if input_is_mm else d_rgb.data_ptr())
    last = queued.last_result()
    assert np.array_equal(last["pose"].view(np.uint32), ref[-1]["pose"].view(np.uint32))
    vp = api.volume_params(seq.volume["resolution"], seq.volume["voxel_size"], seq.volume["truncation"],
                           seq.volume["max_weight"], seq.volume["origin"], seq.min_depth, seq.max_depth,
                           seq.volume["format"])
    vols = [api.TSDFVolume.borrowed(p.volume_handle(), vp).download() for p in (seqp, fast, queued)]
    for t, w in vols[1:]:
        assert np.array_equal(t.view(np.uint32), vols[0][0].view(np.uint32))
        assert np.array_equal(w, vols[0][1])
    for p in (seqp, fast, queued):
        p.close()


def test_reset_replays_the_sequence(cuda_lib, seq):
    """After a reset in the middle of a run (frames still in flight on both
    streams), the pipeline gives exactly what a fresh one gives."""
    from azu_gb300 import api
    fresh = _pipeline(seq, True)
    ref = [fresh.process_frame(seq.depth_mm[k]) for k in range(6)]
    pl = _pipeline(seq, True)
    for k in range(3):
        pl.process_frame(seq.depth_mm[9 - k])
    pl.reset()
    got = [pl.process_frame(seq.depth_mm[k]) for k in range(6)]
    for a, b in zip(ref, got):
        assert np.array_equal(a["pose"].view(np.uint32), b["pose"].view(np.uint32))
        assert (a["quality"], a["frame_index"]) == (b["quality"], b["frame_index"])
    vp = api.volume_params(seq.volume["resolution"], seq.volume["voxel_size"], seq.volume["truncation"],
                           seq.volume["max_weight"], seq.volume["origin"], seq.min_depth, seq.max_depth,
                           seq.volume["format"])
    ta, wa = api.TSDFVolume.borrowed(fresh.volume_handle(), vp).download()
    tb, wb = api.TSDFVolume.borrowed(pl.volume_handle(), vp).download()
    assert np.array_equal(ta.view(np.uint32), tb.view(np.uint32)) and np.array_equal(wa, wb)
    fresh.close()
    pl.close()
