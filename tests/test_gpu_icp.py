"""GPU parity of frame geometry (vertices, normals, pyramid) and ICP against the
oracle. Geometry and association counts are bit-exact; the normal equations
are within float reduction-order tolerance; the tracked pose within 1e-6
rad / 1e-6 m of the oracle's from the same input pose."""
import numpy as np
import pytest

import fixtures as F

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def seq():
    from azu_gb300 import synth
    return synth.sequence("c1", frames=12)


@pytest.fixture(scope="module")
def model(seq, orc):
    """Oracle volume of the first 8 frames and its raycast at frame 8."""
    from azu_gb300 import synth
    s = seq
    prm = dict(s.volume, min_depth=s.min_depth, max_depth=s.max_depth)
    prm.pop("format")
    o = orc.Volume(orc.tsdf_params(**prm))
    K = orc.intr(s.fx, s.fy, s.cx, s.cy)
    for k in range(9):
        o.integrate(synth.mm_to_meters(s.depth_mm[k]), s.poses[k], K, 640, 480, s.min_depth, s.max_depth)
    r = o.raycast(s.poses[8], K, 640, 480)
    return r["vertices"], r["normals"], s.poses[8]


def _tracker(**kw):
    from azu_gb300 import api
    return api.ICPTracker(api.tracker_params(**kw))


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_frame_pyramid_bit_exact(cuda_lib, orc, seq):
    from azu_gb300 import synth
    dm = synth.mm_to_meters(seq.depth_mm[3])
    t = _tracker()
    t.prepare_live(_dev(dm), 640, 480)
    levels = orc.frame_pyramid_from_depth(dm, orc.intr(525, 525, 319.5, 239.5))
    for l in range(3):
        d, v, n = t.live_maps(l, 640, 480)
        od, ov, on = levels[l]
        assert np.array_equal(d.view(np.uint32), od.view(np.uint32)), l
        assert np.array_equal(v.view(np.uint32), ov.view(np.uint32)), l
        assert np.array_equal(n.view(np.uint32), on.view(np.uint32)), l


def test_build_system_counts_exact(cuda_lib, orc, seq, model):
    from azu_gb300 import synth
    mv, mn, ref = model
    dm = synth.mm_to_meters(seq.depth_mm[9])
    t = _tracker()
    t.prepare_live(_dev(dm), 640, 480)
    levels = orc.frame_pyramid_from_depth(dm, orc.intr(525, 525, 319.5, 239.5))
    prm = orc.icp_params(fold_threads=1)
    K = orc.intr(525, 525, 319.5, 239.5)
    dmv, dmn = _dev(mv), _dev(mn)
    for level in range(3):
        for pose in (ref, seq.poses[9]):
            g = t.build_system(level, dmv, dmn, 640, 480, pose, ref)
            o = orc.icp_build_system(prm, K, levels[level][1], levels[level][2], mv, mn, pose, ref)
            for key in ("inliers", "valid_live", "valid_model", "projected", "dist_filtered", "angle_filtered"):
                assert g[key] == o[key], (level, key)
            assert g["inliers"] > 100
            # Normal equations against the FP64 reduction of the same float
            # terms: the GPU tree sum must be at least as close to it as the
            # reference's own serial float fold is.
            t64 = orc.icp_build_system_f64(prm, K, levels[level][1], levels[level][2], mv, mn, pose, ref)
            scale = np.abs(t64["A"]).max()
            err_gpu = np.abs(g["A"] - t64["A"]).max()
            err_ref = np.abs(o["A"] - t64["A"]).max()
            assert err_gpu <= max(err_ref, 2e-6 * scale), (err_gpu, err_ref, scale)
            bscale = max(np.abs(t64["b"]).max(), 1e-3 * scale)
            assert np.abs(g["b"] - t64["b"]).max() <= max(np.abs(o["b"] - t64["b"]).max(), 2e-6 * bscale)


@pytest.mark.parametrize("precision", [0, 1])
def test_track_pose_parity(cuda_lib, orc, seq, model, precision):
    from azu_gb300 import synth
    mv, mn, ref = model
    K = orc.intr(525, 525, 319.5, 239.5)
    prm = orc.icp_params(fold_threads=0)  # FP64 reduction of the float terms
    t = _tracker(precision=precision)
    for k in (9, 10):
        dm = synth.mm_to_meters(seq.depth_mm[k])
        t.prepare_live(_dev(dm), 640, 480)
        g = t.track_prepared(640, 480, _dev(mv), _dev(mn), 640, 480, seq.poses[8], ref)
        o = orc.icp_track(prm, K, orc.frame_pyramid_from_depth(dm, K), mv, mn, seq.poses[8], ref).as_dict()
        assert g["status"] == 0
        assert g["tracking_ok"] == o["tracking_ok"] and g["converged"] == o["converged"]
        rot, trans = F.rel_pose_error(g["pose"], o["pose"])
        assert rot <= 1e-6 and trans <= 1e-6, (rot, trans)
        assert abs(g["inliers"] - o["inliers"]) <= max(3, 1e-4 * o["inliers"])
        # and against the ground-truth trajectory, tracking works
        rot_gt, trans_gt = F.rel_pose_error(g["pose"], seq.poses[k])
        assert rot_gt < 2e-3 and trans_gt < 5e-3


def test_icp_weighting_contract_gpu(cuda_lib):
    lv, ln, mv, mn = F.icp_weighting_fixture()
    t = _tracker(iters=(1, 0, 0))
    z1 = np.zeros((240, 320, 3), np.float32)
    z2 = np.zeros((120, 160, 3), np.float32)
    t.load_live(0, _dev(lv), _dev(ln), 640, 480)
    t.load_live(1, _dev(z1), _dev(z1), 640, 480)
    t.load_live(2, _dev(z2), _dev(z2), 640, 480)
    r = t.track_prepared(640, 480, _dev(mv), _dev(mn), 640, 480, np.eye(4), np.eye(4))
    assert r["valid_live_points"] == 11 and r["valid_model_points"] == 11 and r["projected_points"] == 11
    assert r["inliers"] == 11 and r["dist_filtered"] == 0 and r["angle_filtered"] == 0
    assert abs(r["pose"][2, 3] - F.ICP_TZ) <= 5e-6
    assert abs(r["error"] - F.ICP_ERR) <= 5e-6
    r2 = t.track_prepared(640, 480, _dev(mv), _dev(mn), 640, 480, np.eye(4), np.eye(4))
    assert np.array_equal(r["pose"], r2["pose"]) and r["error"] == r2["error"]


def test_track_without_prepare_is_a_state_error(cuda_lib):
    from azu_gb300 import _abi
    t = _tracker()
    mv = _dev(np.zeros((480, 640, 3), np.float32))
    with pytest.raises(_abi.AzuError) as e:
        t.track_prepared(640, 480, mv, mv, 640, 480, np.eye(4), np.eye(4))
    assert e.value.code == _abi.AZU_E_STATE


def test_counts_exact_at_the_gpu_own_poses(cuda_lib, orc, seq, model):
    """The counters a track reports come from the association of its last
    accepted iteration (ICPTracker.cpp:77-128: inliers, valid live/model,
    projected, distance- and angle-filtered). Iteration j of level l runs at
    the pose the tracker reached after j - 1 iterations, which a track whose
    level l stops after j - 1 iterations returns bit for bit (the iterations
    before it are the same code on the same inputs). So every counter the GPU
    reports after iteration j must equal the oracle's association at the
    GPU's own pose after j - 1: the counts are exact, and any difference from
    an oracle track is in the float pose alone."""
    from azu_gb300 import synth
    mv, mn, ref = model
    K = orc.intr(525, 525, 319.5, 239.5)
    prm = orc.icp_params(fold_threads=0)
    # GPU result key -> oracle association key
    keys = {"inliers": "inliers", "valid_live_points": "valid_live", "valid_model_points": "valid_model",
            "projected_points": "projected", "dist_filtered": "dist_filtered", "angle_filtered": "angle_filtered"}
    checked = 0
    for k in (9, 11):
        dm = synth.mm_to_meters(seq.depth_mm[k])
        levels = orc.frame_pyramid_from_depth(dm, K)
        full = (10, 5, 4)
        for lvl in (2, 1, 0):
            # the pose iteration 1 of this level starts from: the estimate, or
            # what a track whose finer levels run no iterations returns
            prev = dict(pose=np.asarray(seq.poses[8], np.float32)) if lvl == 2 else None
            for j in range(0 if lvl < 2 else 1, full[lvl] + 1):
                iters = tuple(full[i] if i > lvl else (j if i == lvl else 0) for i in range(3))
                t = _tracker(iters=iters)
                t.prepare_live(_dev(dm), 640, 480)
                g = t.track_prepared(640, 480, _dev(mv), _dev(mn), 640, 480, seq.poses[8], ref)
                assert g["status"] == 0
                if prev is not None:
                    if np.array_equal(np.asarray(g["pose"]).view(np.uint32), np.asarray(prev["pose"]).view(np.uint32)):
                        break  # iteration j made no update (converged or stopped before it): the level is done
                    lv = levels[lvl]
                    o = orc.icp_build_system(prm, K, lv[1], lv[2], mv, mn, prev["pose"], ref)
                    for key, okey in keys.items():
                        assert g[key] == o[okey], (k, lvl, j, key, g[key], o[okey])
                    checked += 1
                prev = g
    assert checked >= 10
