"""Bounded device waits: a barrier wait that runs out is reported, and the
next call works.

The ICP's grid barriers spin with an iteration limit; when it is reached the
kernel sets an error word, finishes, and the call returns AZU_E_TIMEOUT (the
status convention of the C ABI). Here the testing hook makes every barrier
need one arrival more than the launch has blocks, so each wait runs out by
design after a short limit — no wait is unbounded and nothing faults. After
the hook is undone:

  track_prepared / build_system / track_many   equal a fresh tracker's results
                                               bit for bit
  pipeline                                     the timed-out frame is graded
                                               Failed and fuses nothing; the
                                               frames after it equal those of a
                                               pipeline whose frame there had no
                                               depth (also graded Failed)
"""
import contextlib
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SPIN_LIMIT = 2000  # polls before a wait gives up (the default is 1 << 22)


@contextlib.contextmanager
def waits_run_out(lib):
    from azu_gb300 import _abi
    _abi.check(lib.azu_testing_set_icp_wait(SPIN_LIMIT, 1), "azu_testing_set_icp_wait")
    try:
        yield
    finally:
        _abi.check(lib.azu_testing_set_icp_wait(0, 0), "azu_testing_set_icp_wait")


@pytest.fixture(scope="module")
def scene():
    import torch
    from azu_gb300 import api, synth
    s = synth.sequence("c1", frames=8)
    v = s.volume
    g = api.TSDFVolume(api.volume_params(v["resolution"], v["voxel_size"], v["truncation"], v["max_weight"],
                                         v["origin"], s.min_depth, s.max_depth))
    K = (s.fx, s.fy, s.cx, s.cy)
    for k in range(7):
        g.integrate(synth.mm_to_meters(s.depth_mm[k]), s.poses[k], K, s.width, s.height, s.min_depth, s.max_depth)
    r = g.raycast(s.poses[6], K, s.width, s.height)
    mv = torch.from_numpy(np.ascontiguousarray(r["vertices"])).cuda()
    mn = torch.from_numpy(np.ascontiguousarray(r["normals"])).cuda()
    live = torch.from_numpy(synth.mm_to_meters(s.depth_mm[7])).cuda()
    return s, g, mv, mn, live


def _tracker(s, live, **kw):
    from azu_gb300 import api
    t = api.ICPTracker(api.tracker_params(min_depth=s.min_depth, max_depth=s.max_depth, **kw))
    t.prepare_live(live, s.width, s.height)
    return t


def _same(a, b):
    assert np.array_equal(np.asarray(a["pose"]).view(np.uint32), np.asarray(b["pose"]).view(np.uint32))
    for k in ("inliers", "valid_live_points", "valid_model_points", "projected_points", "dist_filtered",
              "angle_filtered", "iterations", "converged", "tracking_ok", "status"):
        assert a[k] == b[k], k
    assert np.array_equal(np.asarray(a["information"]).view(np.uint32),
                          np.asarray(b["information"]).view(np.uint32))


def test_track_prepared_recovers_after_timeout(cuda_lib, scene):
    from azu_gb300 import _abi, api
    lib = cuda_lib
    s, _, mv, mn, live = scene
    want = _tracker(s, live).track_prepared(s.width, s.height, mv, mn, s.width, s.height, s.poses[6], s.poses[6])
    assert want["status"] == 0 and want["tracking_ok"]
    trk = _tracker(s, live)
    for _ in range(2):  # twice: the second timeout starts from the words the first one left
        r = _abi.IcpResult()
        api._ready()
        with waits_run_out(lib):
            rc = lib.azu_tracker_track_prepared(trk.h, s.width, s.height, api._ptr(mv), api._ptr(mn), s.width,
                                                s.height, api._pose(s.poses[6]), api._pose(s.poses[6]),
                                                C.byref(r))
        assert rc == _abi.AZU_E_TIMEOUT and r.status == _abi.AZU_E_TIMEOUT
        assert b"timed out" in lib.azu_last_error()
        for _ in range(2):
            _same(trk.track_prepared(s.width, s.height, mv, mn, s.width, s.height, s.poses[6], s.poses[6]), want)


def test_build_system_recovers_after_timeout(cuda_lib, scene):
    from azu_gb300 import _abi, api
    lib = cuda_lib
    s, _, mv, mn, live = scene
    want = _tracker(s, live).build_system(0, mv, mn, s.width, s.height, s.poses[6], s.poses[6])
    trk = _tracker(s, live)
    A, b, res, cnt = (C.c_float * 36)(), (C.c_float * 6)(), C.c_float(), (C.c_int * 6)()
    api._ready()
    with waits_run_out(lib):
        rc = lib.azu_tracker_build_system(trk.h, 0, api._ptr(mv), api._ptr(mn), s.width, s.height,
                                          api._pose(s.poses[6]), api._pose(s.poses[6]), A, b, C.byref(res), cnt)
    assert rc == _abi.AZU_E_TIMEOUT
    got = trk.build_system(0, mv, mn, s.width, s.height, s.poses[6], s.poses[6])
    assert np.array_equal(got["A"].view(np.uint32), want["A"].view(np.uint32))
    assert np.array_equal(got["b"].view(np.uint32), want["b"].view(np.uint32))
    assert got["inliers"] == want["inliers"] > 10000


def test_track_many_recovers_after_timeout(cuda_lib, scene):
    from azu_gb300 import _abi, api
    lib = cuda_lib
    s, g, _, _, live = scene
    poses = np.stack([s.poses[6], s.poses[5], s.poses[7], s.poses[4]]).astype(np.float32)
    K160 = (s.fx / 4, s.fy / 4, (s.cx + 0.5) / 4 - 0.5, (s.cy + 0.5) / 4 - 0.5)
    mv, mn = g.raycast_many(poses, K160, 160, 120)
    coarse = api.tracker_params(iters=(0, 0, 12), dist=0.5, angle=45.0, min_depth=s.min_depth,
                                max_depth=s.max_depth)
    fresh = _tracker(s, live, iters=(0, 0, 12), dist=0.5, angle=45.0)
    want = fresh.track_many(s.width, s.height, mv, mn, 160, 120, poses, params=coarse)
    trk = _tracker(s, live, iters=(0, 0, 12), dist=0.5, angle=45.0)
    out = (_abi.IcpResult * len(poses))()
    api._ready()
    with waits_run_out(lib):
        rc = lib.azu_tracker_track_many(trk.h, s.width, s.height, api._ptr(mv), api._ptr(mn), 160, 120,
                                        len(poses), poses.ctypes.data_as(_abi.fp), None, C.byref(coarse), out)
    assert rc == _abi.AZU_E_TIMEOUT
    assert all(out[k].status == _abi.AZU_E_TIMEOUT for k in range(len(poses)))
    got = trk.track_many(s.width, s.height, mv, mn, 160, 120, poses, params=coarse)
    for a, b in zip(got, want):
        _same(a, b)
        assert a["inliers"] > 500


@pytest.mark.parametrize("use_graph", [True, False])
def test_pipeline_frame_timeout_is_a_failed_frame(cuda_lib, use_graph):
    from azu_gb300 import _abi, api, synth
    lib = cuda_lib
    s = synth.sequence("c1", frames=9)
    v = s.volume

    vp = api.volume_params(v["resolution"], v["voxel_size"], v["truncation"], v["max_weight"], v["origin"],
                           s.min_depth, s.max_depth, v["format"])

    def make():
        tp = api.tracker_params(min_depth=s.min_depth, max_depth=s.max_depth)
        return api.Pipeline(api.pipeline_params(vp, tp, 0, s.min_depth, s.max_depth, True, use_graph))

    timed, blank = make(), make()
    bad = 4
    for k in range(len(s.poses)):
        if k == bad:
            r = _abi.FrameResult()
            d = np.ascontiguousarray(s.depth_mm[k], np.uint16)
            with waits_run_out(lib):
                rc = lib.azu_pipeline_process_frame(timed.h, d.ctypes.data_as(C.c_void_p), None, C.byref(r))
            assert rc == _abi.AZU_E_TIMEOUT and r.icp.status == _abi.AZU_E_TIMEOUT
            assert r.quality == 2 and not r.integrated  # Failed: pose kept, nothing fused
            ra = timed._frame(r)
            rb = blank.process_frame(np.zeros_like(s.depth_mm[k]))
            assert rb["quality"] == 2 and not rb["integrated"]
        else:
            ra = timed.process_frame(s.depth_mm[k])
            rb = blank.process_frame(s.depth_mm[k])
            assert ra["icp"]["status"] == 0
            _same(ra["icp"], rb["icp"])
            assert (ra["quality"], ra["integrated"]) == (rb["quality"], rb["integrated"]), k
        assert np.array_equal(ra["pose"].view(np.uint32), rb["pose"].view(np.uint32)), k
    assert ra["integrated"]  # fusion resumes after the timed-out frame
    ta, wa = api.TSDFVolume.borrowed(timed.volume_handle(), vp).download()
    tb, wb = api.TSDFVolume.borrowed(blank.volume_handle(), vp).download()
    assert np.array_equal(wa, wb) and np.array_equal(ta.view(np.uint32), tb.view(np.uint32))
    # a timed-out frame whose result is never read, then a reset: the reset
    # clears the barrier words as well
    import torch
    d = torch.from_numpy(np.ascontiguousarray(s.depth_mm[1], np.uint16).view(np.int16)).cuda()
    torch.cuda.synchronize()
    with waits_run_out(lib):
        timed.process_frame_device(d.data_ptr())
        torch.cuda.ExternalStream(timed.stream).synchronize()
    timed.reset()
    blank.reset()
    for k in range(3):
        ra, rb = timed.process_frame(s.depth_mm[k]), blank.process_frame(s.depth_mm[k])
        assert np.array_equal(ra["pose"].view(np.uint32), rb["pose"].view(np.uint32)), k
    timed.close()
    blank.close()
