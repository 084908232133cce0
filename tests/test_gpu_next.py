"""The consumers either side of the hot path: the relocaliser's batched
candidate renders and scoring solves, and the global point cloud.

  raycast_many   every image equals the single raycast at that pose and the
                 oracle's raycast of the same volume at 160x120 (bit-exact)
  track_many     every solve equals track_prepared on the same image
                 (bit-exact) and the oracle's association and track of the
                 160x120 model (counters exact at the GPU's own poses, end
                 poses within 5e-4)
  point cloud    equals the oracle's one-thread extraction (order and values)
"""
import numpy as np
import pytest

import fixtures as F

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def model():
    from azu_gb300 import api, synth
    s = synth.sequence("c1", frames=8)
    v = s.volume
    vp = api.volume_params(v["resolution"], v["voxel_size"], v["truncation"], v["max_weight"], v["origin"],
                           s.min_depth, s.max_depth)
    g = api.TSDFVolume(vp)
    K = (s.fx, s.fy, s.cx, s.cy)
    for k in range(8):
        g.integrate(synth.mm_to_meters(s.depth_mm[k]), s.poses[k], K, s.width, s.height, s.min_depth, s.max_depth)
    return s, g, vp


def _candidates(s, n=6):
    rng = np.random.default_rng(5)
    out = []
    for k in range(n):
        P = s.poses[7].astype(np.float64).copy()
        a = np.radians(rng.uniform(-6, 6))
        R = np.array([[np.cos(a), 0, np.sin(a)], [0, 1, 0], [-np.sin(a), 0, np.cos(a)]])
        P[:3, :3] = P[:3, :3] @ R
        P[:3, 3] += rng.uniform(-0.03, 0.03, 3)
        out.append(P.astype(np.float32))
    return np.stack(out)


def test_raycast_many_equals_single_raycasts(cuda_lib, model):
    s, g, _ = model
    poses = _candidates(s)
    K160 = (s.fx / 4, s.fy / 4, (s.cx + 0.5) / 4 - 0.5, (s.cy + 0.5) / 4 - 0.5)
    v, n = g.raycast_many(poses, K160, 160, 120)
    v, n = v.cpu().numpy(), n.cpu().numpy()
    for k, P in enumerate(poses):
        r = g.raycast(P, K160, 160, 120)
        assert np.array_equal(v[k].view(np.uint32), r["vertices"].view(np.uint32)), k
        assert np.array_equal(n[k].view(np.uint32), r["normals"].view(np.uint32)), k
        assert (r["vertices"] != 0).any(-1).sum() > 2000


def test_track_many_equals_track_prepared(cuda_lib, model):
    import torch
    from azu_gb300 import api, synth
    s, g, _ = model
    poses = _candidates(s)
    K160 = (s.fx / 4, s.fy / 4, (s.cx + 0.5) / 4 - 0.5, (s.cy + 0.5) / 4 - 0.5)
    mv, mn = g.raycast_many(poses, K160, 160, 120)
    # the coarse stage: level 2 only, wider gates (Relocalizer.h RelocParams)
    coarse = api.tracker_params(iters=(0, 0, 12), dist=0.5, angle=45.0, min_depth=s.min_depth,
                                max_depth=s.max_depth)
    trk = api.ICPTracker(coarse)
    live = torch.from_numpy(synth.mm_to_meters(s.depth_mm[7])).cuda()
    trk.prepare_live(live, s.width, s.height)
    many = trk.track_many(s.width, s.height, mv, mn, 160, 120, poses, params=coarse)
    for k, P in enumerate(poses):
        one = trk.track_prepared(s.width, s.height, mv[k], mn[k], 160, 120, P, P)
        assert np.array_equal(np.asarray(many[k]["pose"]).view(np.uint32), np.asarray(one["pose"]).view(np.uint32))
        assert many[k]["inliers"] == one["inliers"] and many[k]["inliers"] > 500
    # the candidates pull toward the true pose
    err0 = np.mean([np.linalg.norm(P[:3, 3] - s.poses[7][:3, 3]) for P in poses])
    err1 = np.mean([np.linalg.norm(np.asarray(r["pose"])[:3, 3] - s.poses[7][:3, 3]) for r in many])
    assert err1 < 0.5 * err0


def test_point_cloud_equals_oracle(cuda_lib, orc, model):
    s, g, vp = model
    pts, col = g.point_cloud()
    t, w = g.download()
    o = orc.Volume(orc.tsdf_params(resolution=vp.resolution, voxel_size=vp.voxel_size, truncation=vp.truncation,
                                   max_weight=vp.max_weight, origin=tuple(vp.origin)))
    o.tsdf[:] = t
    o.weight[:] = w
    op, oc = o.point_cloud()
    assert len(op) > 10000
    assert np.array_equal(pts.view(np.uint32), op.view(np.uint32))
    assert np.array_equal(col, oc)


def _oracle_volume(orc, g, vp):
    t, w = g.download()
    o = orc.Volume(orc.tsdf_params(resolution=vp.resolution, voxel_size=vp.voxel_size, truncation=vp.truncation,
                                   max_weight=vp.max_weight, origin=tuple(vp.origin), min_depth=vp.min_depth,
                                   max_depth=vp.max_depth))
    o.tsdf[:] = t
    o.weight[:] = w
    return o


def test_raycast_many_equals_oracle_at_160x120(cuda_lib, orc, model):
    """The relocaliser's candidate renders (the model at 160x120 with the
    intrinsics scaled as CameraIntrinsics.h:33-40 scales them) against the
    oracle's raycast of the same volume: bit for bit."""
    s, g, vp = model
    o = _oracle_volume(orc, g, vp)
    poses = _candidates(s)
    K160 = (s.fx / 4, s.fy / 4, (s.cx + 0.5) / 4 - 0.5, (s.cy + 0.5) / 4 - 0.5)
    v, n = g.raycast_many(poses, K160, 160, 120)
    v, n = v.cpu().numpy(), n.cpu().numpy()
    for k, P in enumerate(poses):
        r = o.raycast(P, orc.intr(*K160), 160, 120)
        assert np.array_equal(v[k].view(np.uint32), r["vertices"].view(np.uint32)), k
        assert np.array_equal(n[k].view(np.uint32), r["normals"].view(np.uint32)), k


def test_track_many_equals_oracle_at_160x120(cuda_lib, orc, model):
    """The coarse scoring solves of the relocaliser (level 2 only, 12
    iterations, 0.5 m / 45 deg gates) against a 160x120 model, each candidate
    against the oracle's association and track of the same low-resolution
    model (icp_lowres_model_contract: intrinsics scaled to the model size):
    every counter exact at the GPU's own pose iteration by iteration (the
    association of iteration j runs at the pose a solve stopped after j - 1
    iterations returns), the same grades, end poses within 5e-4."""
    import torch
    from azu_gb300 import api, synth
    s, g, _ = model
    poses = _candidates(s)
    K = orc.intr(s.fx, s.fy, s.cx, s.cy)
    K160 = (s.fx / 4, s.fy / 4, (s.cx + 0.5) / 4 - 0.5, (s.cy + 0.5) / 4 - 0.5)
    mv, mn = g.raycast_many(poses, K160, 160, 120)
    mvh, mnh = mv.cpu().numpy(), mn.cpu().numpy()
    dm = synth.mm_to_meters(s.depth_mm[7])
    levels = orc.frame_pyramid_from_depth(dm, K)
    live = torch.from_numpy(dm).cuda()

    def coarse(n):
        return api.tracker_params(iters=(0, 0, n), dist=0.5, angle=45.0, min_depth=s.min_depth,
                                  max_depth=s.max_depth)

    trk = api.ICPTracker(coarse(12))
    trk.prepare_live(live, s.width, s.height)
    many = trk.track_many(s.width, s.height, mv, mn, 160, 120, poses, params=coarse(12))
    prm = orc.icp_params(iters=(0, 0, 12), dist=0.5, angle=45.0, fold_threads=0)
    keys = {"inliers": "inliers", "valid_live_points": "valid_live", "valid_model_points": "valid_model",
            "projected_points": "projected", "dist_filtered": "dist_filtered", "angle_filtered": "angle_filtered"}
    prev = [dict(pose=np.asarray(P, np.float32)) for P in poses]
    done = [False] * len(poses)
    checked = 0
    for j in range(1, 13):
        cur = trk.track_many(s.width, s.height, mv, mn, 160, 120, poses, params=coarse(j))
        for k, P in enumerate(poses):
            if done[k]:
                continue
            if np.array_equal(np.asarray(cur[k]["pose"]).view(np.uint32),
                              np.asarray(prev[k]["pose"]).view(np.uint32)):
                done[k] = True  # no update at iteration j: this solve has stopped
                continue
            ob = orc.icp_build_system(prm, K, levels[2][1], levels[2][2], mvh[k], mnh[k], prev[k]["pose"], P)
            for key, okey in keys.items():
                assert cur[k][key] == ob[okey], (k, j, key, cur[k][key], ob[okey])
            checked += 1
        prev = cur
    assert checked >= 2 * len(poses)
    # The end poses: twelve coarse iterations from up to 6 deg and 3 cm off do
    # not converge, so the float reduction order (the oracle folds in FP64
    # here) shows in the last digits of the pose; the grades agree.
    for k, P in enumerate(poses):
        o = orc.icp_track(prm, K, levels, mvh[k], mnh[k], P, P).as_dict()
        assert many[k]["tracking_ok"] == o["tracking_ok"] and many[k]["converged"] == o["converged"], k
        rot, trans = F.rel_pose_error(many[k]["pose"], o["pose"])
        assert rot <= 5e-4 and trans <= 5e-4, (k, rot, trans)
