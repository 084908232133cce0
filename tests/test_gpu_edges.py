"""Edge cases of the hot path on the GPU, against the oracle:

  ragged sizes   a 77^3 volume (fills no 8-voxel brick, 32-row item or
                 16-voxel piece evenly) with a voxel size that is not a power of
                 two (the division path of the voxel transform), 203x151 frames
  no depth       all-zero frames: nothing integrates, an empty volume renders
                 nothing, and the pipeline grades and skips such frames as the
                 lockstep oracle does
"""
import math

import numpy as np
import pytest

import fixtures as F

pytestmark = pytest.mark.gpu

ODD_W, ODD_H = 203, 151


def _odd_scene(n=4):
    from azu_gb300 import synth
    scene = synth.base_scene()
    sc = ODD_W / 640.0
    K = (synth.FX * sc, synth.FY * sc, (synth.CX + 0.5) * sc - 0.5, (synth.CY + 0.5) * sc - 0.5)
    poses = [synth.orbit_pose(math.radians(2.0 * k)) for k in range(n)]
    world0 = np.linalg.inv(poses[0])
    depth = [synth.mm_to_meters(synth.render(scene, poses[k], 5, k, w=ODD_W, h=ODD_H, fx=K[0], fy=K[1], cx=K[2],
                                             cy=K[3])) for k in range(n)]
    rel = [(world0 @ p).astype(np.float32) for p in poses]
    return depth, rel, K


def _pair(orc, res, side):
    from azu_gb300 import api, synth
    v = synth._volume(res, side)
    g = api.TSDFVolume(api.volume_params(v["resolution"], v["voxel_size"], v["truncation"], v["max_weight"],
                                         v["origin"], synth.MIN_DEPTH, synth.MAX_DEPTH))
    o = orc.Volume(orc.tsdf_params(resolution=v["resolution"], voxel_size=v["voxel_size"],
                                   truncation=v["truncation"], max_weight=v["max_weight"],
                                   origin=tuple(v["origin"]), min_depth=synth.MIN_DEPTH,
                                   max_depth=synth.MAX_DEPTH))
    return g, o, v


def test_ragged_volume_and_image(cuda_lib, orc):
    from azu_gb300 import synth
    g, o, v = _pair(orc, 77, 2.0)
    vs = v["voxel_size"]
    assert math.frexp(vs)[0] != 0.5  # not a power of two
    depth, poses, K = _odd_scene()
    for k in range(3):
        g.integrate(depth[k], poses[k], K, ODD_W, ODD_H, synth.MIN_DEPTH, synth.MAX_DEPTH)
        st = o.integrate(depth[k], poses[k], orc.intr(*K), ODD_W, ODD_H, synth.MIN_DEPTH, synth.MAX_DEPTH)
        assert g.stats()["last_voxels_updated"] == st["voxels_updated"] > 1000, k
    t, w = g.download()
    assert np.array_equal(w, o.weight)
    assert np.array_equal(t.view(np.uint32), o.tsdf.view(np.uint32))
    for k in (2, 3):
        rg = g.raycast(poses[k], K, ODD_W, ODD_H)
        ro = o.raycast(poses[k], orc.intr(*K), ODD_W, ODD_H)
        assert (ro["vertices"] != 0).any(-1).sum() > 2000
        assert np.array_equal(rg["vertices"].view(np.uint32), ro["vertices"].view(np.uint32))
        assert np.array_equal(rg["normals"].view(np.uint32), ro["normals"].view(np.uint32))


def test_zero_depth_and_empty_volume(cuda_lib, orc):
    from azu_gb300 import synth
    g, o, _ = _pair(orc, 64, 2.0)
    K = (synth.FX, synth.FY, synth.CX, synth.CY)
    pose = np.eye(4, dtype=np.float32)
    empty = g.raycast(pose, K, 640, 480)
    assert not empty["vertices"].any() and not empty["normals"].any()
    t0, w0 = g.download()
    zero = np.zeros((480, 640), np.float32)
    g.integrate(zero, pose, K, 640, 480, synth.MIN_DEPTH, synth.MAX_DEPTH)
    st = o.integrate(zero, pose, orc.intr(*K), 640, 480, synth.MIN_DEPTH, synth.MAX_DEPTH)
    assert g.stats()["last_voxels_updated"] == st["voxels_updated"] == 0
    t1, w1 = g.download()
    assert np.array_equal(t1.view(np.uint32), t0.view(np.uint32)) and np.array_equal(w1, w0)
    assert np.array_equal(w1, o.weight) and np.array_equal(t1.view(np.uint32), o.tsdf.view(np.uint32))


@pytest.mark.parametrize("input_is_mm", [True, False])
def test_pipeline_frames_without_depth(cuda_lib, orc, input_is_mm):
    """Frames with no valid depth in the middle of a sequence (a covered
    sensor): each is graded and left out of the model exactly as by the
    lockstep oracle, and tracking resumes on the next good frame."""
    from azu_gb300 import api, synth
    s = synth.sequence("c1", frames=7)
    v = s.volume
    vp = api.volume_params(v["resolution"], v["voxel_size"], v["truncation"], v["max_weight"], v["origin"],
                           s.min_depth, s.max_depth, v["format"])
    tp = api.tracker_params(min_depth=s.min_depth, max_depth=s.max_depth)
    pl = api.Pipeline(api.pipeline_params(vp, tp, 0, s.min_depth, s.max_depth, input_is_mm, True))
    L = orc.Lockstep(s.volume, input_is_mm=input_is_mm, fold_threads=0)
    rgb = synth.grey_rgb()
    blank = {3, 4}
    grades = []
    for k in range(len(s.poses)):
        mm = np.zeros_like(s.depth_mm[k]) if k in blank else s.depth_mm[k]
        d = mm if input_is_mm else synth.encode_raw(mm)
        gr = pl.process_frame(d, None if input_is_mm else rgb)
        orr = L.process(d, rgb)
        assert (gr["quality"], gr["integrated"]) == (orr["quality"], orr["integrated"]), k
        rot, trans = F.rel_pose_error(gr["pose"], orr["pose"])
        assert rot <= 5e-4 and trans <= 5e-4, (k, rot, trans)
        grades.append((gr["quality"], gr["integrated"]))
    assert all(not grades[k][1] for k in blank)
    assert grades[-1][1]  # fusion resumes after the blank frames
    pl.close()
