"""Differentiation form on the GPU: the depth adjoint (pose and voxel
gradients of a Huber depth loss) against the FP64 CPU adjoint of the same
float march, against FP64 central finite differences, and render-and-compare
pose refinement.

Tolerances: the rendered hit set equals the reference raycast's exactly; the
GPU evaluates the adjoint in float, so per-pixel dD/dxi agrees with the FP64
adjoint to 1e-3 relative (1e-5 absolute) and the summed gradients to 1e-3; the
FP64 finite differences march in double, whose sample positions differ from
the float march by rounding, hence 2e-2 there."""
import numpy as np
import pytest

import fixtures as F

pytestmark = pytest.mark.gpu


def _scene(orc):
    from azu_gb300 import api
    t, w, prm = F.sphere_volume(res=48, vs=0.025, radius=0.3, trunc=0.075)
    prm = dict(prm, min_depth=0.1, max_depth=3.0)
    p = orc.tsdf_params(**prm)
    c = (48 - 1) * 0.025 / 2.0
    pose = np.eye(4, dtype=np.float32)
    pose[:3, 3] = (c + 0.03, c - 0.02, -0.4)
    K = (60.0, 60.0, 31.5, 23.5)
    g = api.TSDFVolume(api.volume_params(prm["resolution"], prm["voxel_size"], prm["truncation"],
                                         prm["max_weight"], prm["origin"], prm["min_depth"], prm["max_depth"]))
    g.upload(t, w)
    moved = pose.copy()
    moved[:3, 3] += (0.004, -0.003, 0.006)
    obs = orc.depth_loss_d(p, t.astype(np.float64), w, moved.astype(np.float64), np.zeros(6), orc.intr(*K),
                           64, 48)["depth"].astype(np.float32)
    return g, t, w, p, pose, K, obs


def test_adjoint_matches_fp64_cpu_adjoint(cuda_lib, orc):
    g, t, w, p, pose, K, obs = _scene(orc)
    r = g.depth_backward(pose, K, 64, 48, obs, 0.01, grad_tsdf=True, jacobian=True)
    o = orc.depth_adjoint_f(p, t, w, pose, orc.intr(*K), 64, 48, depth_obs=obs, huber_delta=0.01,
                            grad_tsdf=True, jac=True)
    assert np.array_equal(r["depth"] > 0, o["depth"] > 0)
    hit = o["depth"] > 0
    assert hit.sum() > 600 and r["n_valid"] == o["n_valid"]
    assert np.max(np.abs(r["depth"][hit] - o["depth"][hit])) <= 2e-6
    Jg, Jo = r["jacobian"][hit], o["jac"][hit]
    assert np.all(np.abs(Jg - Jo) <= 1e-5 + 1e-3 * np.abs(Jo))
    assert abs(r["loss"] - o["loss"]) <= 1e-4 * o["loss"]
    assert np.allclose(r["grad_xi"], o["grad_xi"], rtol=1e-3, atol=1e-5)
    gv, ov = r["grad_tsdf"], o["grad_tsdf"]
    touched = np.flatnonzero(ov)
    assert touched.size > 100
    both = np.union1d(touched, np.flatnonzero(gv))
    assert np.allclose(gv[both], ov[both], rtol=1e-3, atol=1e-7)
    assert r["chain_overflow"] == 0


def test_adjoint_matches_fp64_central_differences(cuda_lib, orc):
    g, t, w, p, pose, K, obs = _scene(orc)
    r = g.depth_backward(pose, K, 64, 48, obs, 0.01)
    t64 = t.astype(np.float64)
    P = pose.astype(np.float64)
    fd = np.zeros(6)
    for j in range(6):
        xi = np.zeros(6)
        xi[j] = 1e-6
        lp = orc.depth_loss_d(p, t64, w, P, xi, orc.intr(*K), 64, 48, depth_obs=obs)["loss"]
        lm = orc.depth_loss_d(p, t64, w, P, -xi, orc.intr(*K), 64, 48, depth_obs=obs)["loss"]
        fd[j] = (lp - lm) / 2e-6
    assert np.allclose(r["grad_xi"], fd, rtol=2e-2, atol=1e-3), (r["grad_xi"], fd)


def test_render_and_compare_refinement(cuda_lib, orc):
    """From a pose off by ~1 cm / 1 deg, refinement on the c1 model recovers the
    pose the observed depth was taken from."""
    from azu_gb300 import api, synth
    s = synth.sequence("c1", frames=12)
    v = s.volume
    g = api.TSDFVolume(api.volume_params(v["resolution"], v["voxel_size"], v["truncation"], v["max_weight"],
                                         v["origin"], s.min_depth, s.max_depth))
    K = (s.fx, s.fy, s.cx, s.cy)
    for k in range(12):
        g.integrate(synth.mm_to_meters(s.depth_mm[k]), s.poses[k], K, s.width, s.height, s.min_depth, s.max_depth)
    k = 11
    truth = s.poses[k].astype(np.float32)
    obs = g.render_depth(truth, K, s.width, s.height)
    ang = np.radians(1.0)
    R = np.array([[np.cos(ang), 0, np.sin(ang)], [0, 1, 0], [-np.sin(ang), 0, np.cos(ang)]], np.float32)
    start = truth.copy()
    start[:3, :3] = truth[:3, :3] @ R
    start[:3, 3] += (0.008, -0.005, 0.006)
    pose, trace, its = g.refine_pose(start, K, s.width, s.height, obs, 0.01, 30)
    assert its >= 1 and trace[-1] < 0.01 * trace[0]
    dp = np.linalg.inv(truth.astype(np.float64)) @ pose.astype(np.float64)
    assert np.linalg.norm(dp[:3, 3]) < 5e-4
    assert np.degrees(np.arccos(np.clip((np.trace(dp[:3, :3]) - 1) / 2, -1, 1))) < 0.05
