"""The allocation-free ICP pass (azu_icp_build_system_noalloc) against the
allocating one (azu_tracker_build_system) on the same inputs.

The no-allocation entry point serves callers that must not allocate device
memory while they run — a real-time tracking loop whose device-memory budget is
fixed at start-up, or a host whose device memory belongs to its own pool.
It keeps its scratch in one static device array shared by all calls, so two
calls in a row with different poses must each match the handle-based pass:
nothing of the first call may leak into the second. Collected last (file name)
so a failure here does not hide the other tests; it also runs alone.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def test_noalloc_pass_matches_tracker_pass_twice(cuda_lib):
    import torch

    from azu_gb300 import _abi, api, synth

    lib = _abi.load()
    s = synth.sequence("c1", frames=7)
    v = s.volume
    vol = api.TSDFVolume(api.volume_params(v["resolution"], v["voxel_size"], v["truncation"], v["max_weight"],
                                           v["origin"], s.min_depth, s.max_depth))
    K = (s.fx, s.fy, s.cx, s.cy)
    for k in range(5):
        vol.integrate(synth.mm_to_meters(s.depth_mm[k]), s.poses[k], K, 640, 480, s.min_depth, s.max_depth)
    mv, mn, _ = vol.raycast_gpu(s.poses[4], K, 640, 480)
    params = api.tracker_params()
    tracker = api.ICPTracker(params)
    tracker.prepare_live(torch.from_numpy(synth.mm_to_meters(s.depth_mm[5])).cuda(), 640, 480)
    lv, ln, ld = C.c_void_p(), C.c_void_p(), C.c_void_p()
    _abi.check(lib.azu_tracker_live_maps(tracker.h, 0, C.byref(lv), C.byref(ln), C.byref(ld)), "live_maps")
    stream = C.c_void_p(api.lib_stream().cuda_stream)

    perturbed = s.poses[5].copy()
    perturbed[:3, 3] += np.float32([0.004, -0.002, 0.003])
    for pose in (s.poses[5], perturbed):
        want = tracker.build_system(0, mv, mn, 640, 480, pose, s.poses[4])
        A = (C.c_float * 36)()
        b = (C.c_float * 6)()
        res = C.c_float()
        cnt = (C.c_int * 6)()
        rc = lib.azu_icp_build_system_noalloc(lv, ln, 640, 480, _ptr(mv), _ptr(mn), 640, 480, C.byref(params),
                                              api._pose(pose), api._pose(s.poses[4]), stream, A, b, C.byref(res),
                                              cnt)
        assert rc == _abi.AZU_OK, lib.azu_last_error()
        got_counts = list(cnt)
        assert got_counts == [want[k] for k in ("inliers", "valid_live", "valid_model", "projected",
                                                "dist_filtered", "angle_filtered")]
        assert got_counts[0] > 1000
        gA = np.array(A, np.float32).reshape(6, 6)
        gb = np.array(b, np.float32)
        scale = np.abs(want["A"]).max()
        assert np.abs(gA - want["A"]).max() <= 2e-6 * scale
        assert np.abs(gb - want["b"]).max() <= 2e-6 * max(np.abs(want["b"]).max(), 1e-3 * scale)
        assert abs(res.value - want["residual"]) <= 2e-6 * abs(want["residual"]) + 1e-12


def test_noalloc_rejects_oversized_images(cuda_lib):
    import torch

    from azu_gb300 import _abi, api

    lib = _abi.load()
    d = torch.zeros(16 * 3, dtype=torch.float32, device="cuda")
    A, b, res, cnt = (C.c_float * 36)(), (C.c_float * 6)(), C.c_float(), (C.c_int * 6)()
    rc = lib.azu_icp_build_system_noalloc(_ptr(d), _ptr(d), 9000, 4, _ptr(d), _ptr(d), 4, 4,
                                          C.byref(api.tracker_params()), api._pose(np.eye(4)),
                                          api._pose(np.eye(4)), None, A, b, C.byref(res), cnt)
    assert rc == _abi.AZU_E_INVALID
    assert b"8192" in lib.azu_last_error()
