"""The consumers either side of the hot path: the relocaliser's batched
candidate renders and scoring solves, and the global point cloud.

  raycast_many   every image equals the single raycast at that pose (bit-exact)
  track_many     every solve equals track_prepared on the same image (bit-exact)
  point cloud    equals the oracle's one-thread extraction (order and values)
"""
import numpy as np
import pytest

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
