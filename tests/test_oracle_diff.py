"""The differentiation form's CPU reference: the adjoint of depth rendering
(pose and voxel gradients of a Huber depth loss) against central finite
differences of the all-double forward (step 1e-6), and the float-march adjoint
against the double one. CPU only: this pins the oracle the GPU adjoint is
checked against."""
import numpy as np
import pytest

import fixtures as F

H_STEP = 1e-6


def _scene(orc):
    t, w, prm = F.sphere_volume(res=48, vs=0.025, radius=0.3, trunc=0.075)
    prm = dict(prm, min_depth=0.1, max_depth=3.0)
    p = orc.tsdf_params(**prm)
    c = (48 - 1) * 0.025 / 2.0
    pose = np.eye(4, dtype=np.float32)
    pose[:3, 3] = (c + 0.03, c - 0.02, -0.4)   # outside the box: t_near is the box entry
    K = orc.intr(60.0, 60.0, 31.5, 23.5)
    return t, w, p, pose, K, 64, 48


def _obs(orc, t, w, p, pose, K, W, H):
    moved = pose.copy()
    moved[:3, 3] += (0.004, -0.003, 0.006)
    return orc.depth_loss_d(p, t.astype(np.float64), w, moved.astype(np.float64), np.zeros(6), K, W, H)["depth"] \
        .astype(np.float32)


def test_pose_jacobian_matches_central_differences(orc):
    t, w, p, pose, K, W, H = _scene(orc)
    t64 = t.astype(np.float64)
    base = orc.depth_loss_d(p, t64, w, pose.astype(np.float64), np.zeros(6), K, W, H, jac=True)
    hit = base["depth"] > 0
    assert hit.sum() > 600
    ok = 0
    total = 0
    for j in range(6):
        xi = np.zeros(6)
        xi[j] = H_STEP
        dp = orc.depth_loss_d(p, t64, w, pose.astype(np.float64), xi, K, W, H)["depth"]
        dm = orc.depth_loss_d(p, t64, w, pose.astype(np.float64), -xi, K, W, H)["depth"]
        m = hit & (dp > 0) & (dm > 0)
        fd = (dp - dm)[m] / (2 * H_STEP)
        jac = base["jac"][..., j][m]
        good = np.abs(fd - jac) <= 1e-5 + 1e-4 * np.abs(jac)
        ok += good.sum()
        total += m.sum()
        assert np.median(np.abs(fd - jac)) <= 1e-6, j
    assert ok >= 0.98 * total, (ok, total)


def test_loss_gradients_match_central_differences(orc):
    t, w, p, pose, K, W, H = _scene(orc)
    obs = _obs(orc, t, w, p, pose, K, W, H)
    t64 = t.astype(np.float64)
    P = pose.astype(np.float64)
    base = orc.depth_loss_d(p, t64, w, P, np.zeros(6), K, W, H, depth_obs=obs, grads=True, grad_tsdf=True)
    assert base["n_valid"] > 500 and base["loss"] > 0
    g = base["grad_xi"]
    for j in range(6):
        xi = np.zeros(6)
        xi[j] = H_STEP
        lp = orc.depth_loss_d(p, t64, w, P, xi, K, W, H, depth_obs=obs)["loss"]
        lm = orc.depth_loss_d(p, t64, w, P, -xi, K, W, H, depth_obs=obs)["loss"]
        fd = (lp - lm) / (2 * H_STEP)
        assert abs(fd - g[j]) <= 1e-3 * max(1.0, abs(g[j])), (j, fd, g[j])
    gv = base["grad_tsdf"]
    touched = np.flatnonzero(gv)
    assert touched.size > 100
    pick = touched[np.argsort(-np.abs(gv[touched]))[:12]]
    for i in pick:
        tp = t64.copy()
        tp[i] += H_STEP
        tm = t64.copy()
        tm[i] -= H_STEP
        lp = orc.depth_loss_d(p, tp, w, P, np.zeros(6), K, W, H, depth_obs=obs)["loss"]
        lm = orc.depth_loss_d(p, tm, w, P, np.zeros(6), K, W, H, depth_obs=obs)["loss"]
        fd = (lp - lm) / (2 * H_STEP)
        assert abs(fd - gv[i]) <= 1e-4 + 1e-3 * abs(gv[i]), (i, fd, gv[i])


def test_float_march_adjoint_is_the_reference_raycast(orc):
    """The float-march adjoint's depth image is the reference raycast's hits."""
    t, w, p, pose, K, W, H = _scene(orc)
    obs = _obs(orc, t, w, p, pose, K, W, H)
    a = orc.depth_adjoint_f(p, t, w, pose, K, W, H, depth_obs=obs, grad_tsdf=True, jac=True)
    v = orc.Volume(p)
    v.tsdf[:] = t
    v.weight[:] = w
    r = v.raycast(pose, K, W, H)
    hit = (r["vertices"] != 0).any(-1)
    assert np.array_equal(hit, a["depth"] > 0)
    # depth = camera z of the hit vertex (same float march; z recomputed in double)
    R, c = pose[:3, :3].astype(np.float64), pose[:3, 3].astype(np.float64)
    zc = ((r["vertices"].astype(np.float64) - c) @ R)[..., 2]
    assert np.max(np.abs(zc[hit] - a["depth"][hit])) <= 1e-5
    d = orc.depth_loss_d(p, t.astype(np.float64), w, pose.astype(np.float64), np.zeros(6), K, W, H,
                         depth_obs=obs, grads=True)
    assert np.allclose(a["grad_xi"], d["grad_xi"], rtol=2e-2, atol=1e-3)
