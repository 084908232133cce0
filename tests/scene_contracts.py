"""Scenarios of the reference's room-scene contracts, with their tolerances:

  tests/icp_refpose_contract.cpp        tracking against the model's raycast
                                        pose converges to 1 mm / 0.05 deg; the
                                        previous pose as reference is worse
  tests/icp_lowres_model_contract.cpp   models rendered at 640x480, 320x240 and
                                        160x120 with scaled intrinsics track to
                                        1 mm / 0.05 deg, 2 mm / 0.1 deg and (a
                                        coarse level-2 solve from 8 deg / 3 cm)
                                        10 mm / 0.5 deg; unscaled intrinsics
                                        are measurably wrong

Written against a backend with volume(params) -> vol, vol.integrate(depth,
pose), vol.raycast(pose, K, w, h) -> (vertices, normals) and track(depth_live,
model_v, model_n, mw, mh, estimate, ref_pose, iters, dist, angle) -> result
dict, so the CPU restatement and the CUDA path run the same checks. Depth
comes from the contracts' room scene (synth.room_depth).
"""
import math

import numpy as np

from azu_gb300 import synth

K640 = (525.0, 525.0, 319.5, 239.5)
# TSDFParams defaults with the contracts' depth band [0.3, 3.0]
VOLUME = dict(resolution=256, voxel_size=0.010, truncation=0.030, max_weight=128.0, origin=(-1.28, -1.28, 0.0),
              min_depth=0.3, max_depth=3.0)


def scale_k(K, w, h):
    """scaleIntrinsics (include/sensor/CameraIntrinsics.h:33-40) from 640x480."""
    sx, sy = np.float32(w / 640.0), np.float32(h / 480.0)
    f = np.float32
    return (float(f(K[0]) * sx), float(f(K[1]) * sy), float((f(K[2]) + f(0.5)) * sx - f(0.5)),
            float((f(K[3]) + f(0.5)) * sy - f(0.5)))


def pose_error(a, b):
    """(translation m, rotation deg) of a^-1 b (the contracts' poseError)."""
    d = np.linalg.inv(np.asarray(a, np.float64)) @ np.asarray(b, np.float64)
    c = max(-1.0, min(1.0, (np.trace(d[:3, :3]) - 1.0) * 0.5))
    return float(np.linalg.norm(d[:3, 3])), math.degrees(math.acos(c))


def _model_volume(backend):
    P_model = synth.axis_angle_pose((0.0, 0.05, 0.0), (0.02, 0.0, 0.1))
    vol = backend.volume(VOLUME)
    d_model = synth.room_depth(P_model)
    for _ in range(5):
        vol.integrate(d_model, P_model)
    return vol, P_model


def refpose(backend):
    vol, P_model = _model_volume(backend)
    mv, mn = vol.raycast(P_model, K640, 640, 480)
    P_prev = P_model @ synth.axis_angle_pose((0.02, 0.1, 0.0), (0.03, 0.0, 0.01))
    P_live = P_prev @ synth.axis_angle_pose((0.0, 0.015, 0.003), (0.004, 0.0, 0.002))
    live = synth.room_depth(P_live)
    good = backend.track(live, mv, mn, 640, 480, P_prev, P_model)
    t, r = pose_error(good["pose"], P_live)
    assert good["tracking_ok"], good
    assert t < 1e-3 and r < 0.05, (t, r)
    bad = backend.track(live, mv, mn, 640, 480, P_prev, P_prev)
    tb, rb = pose_error(bad["pose"], P_live)
    assert (not bad["tracking_ok"]) or tb > 5e-3 or rb > 0.25, (tb, rb)
    return (t, r), (tb, rb)


def lowres_model(backend):
    vol, P_model = _model_volume(backend)
    P_live = P_model @ synth.axis_angle_pose((0.0, 0.02, 0.004), (0.006, 0.0, 0.003))
    live = synth.room_depth(P_live)
    out = {}
    for w, h, tol_t, tol_r in ((640, 480, 1e-3, 0.05), (320, 240, 2e-3, 0.1)):
        mv, mn = vol.raycast(P_model, scale_k(K640, w, h), w, h)
        r = backend.track(live, mv, mn, w, h, P_model, P_model)
        out[w] = pose_error(r["pose"], P_live)
        assert out[w][0] < tol_t and out[w][1] < tol_r, (w, out[w])
    # a relocalisation-style coarse solve from 8 deg / 3 cm, level 2 only
    P_far = P_model @ synth.axis_angle_pose((0.0, 0.1396, 0.0), (0.03, 0.0, 0.0))
    live_far = synth.room_depth(P_far)
    coarse = dict(iters=(0, 0, 30), dist=0.25, angle=45.0)
    mv, mn = vol.raycast(P_model, scale_k(K640, 160, 120), 160, 120)
    r = backend.track(live_far, mv, mn, 160, 120, P_model, P_model, **coarse)
    out["coarse"] = pose_error(r["pose"], P_far)
    assert out["coarse"][0] < 0.01 and out["coarse"][1] < 0.5, out["coarse"]
    mv, mn = vol.raycast(P_model, K640, 160, 120)  # unscaled intrinsics: the wrong model
    r = backend.track(live_far, mv, mn, 160, 120, P_model, P_model, **coarse)
    e = pose_error(r["pose"], P_far)
    assert r["inliers"] < 100 or e[0] > 0.02 or e[1] > 1.0, e
    return out
