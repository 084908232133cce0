"""The scenarios of the reference's ICP numeric-policy contract
(tests/icp_numeric_policy_contract.cpp), each with that contract's
hand-derived expectations, written once against a `run` callable so the same
checks drive the CPU restatement (test_icp_policy_oracle.py) and the CUDA
tracker (test_gpu_icp_policy.py).

run(correspondences, iters=(1, 0, 0), dist=0.1, angle=30.0, estimate=I) must
track the level-0 maps of fixtures.corr_maps (coarser levels empty, reference
pose identity) and return a dict with pose (4x4), error, inliers, converged,
tracking_ok, final_step and the five counters.
"""
import math

import numpy as np

import fixtures as F

TOL = F.ICP_TOL_MATCH
I4 = np.eye(4, dtype=np.float32)


def _counters(r, live, model, projected, dist_f, angle_f):
    got = (r["valid_live_points"], r["valid_model_points"], r["projected_points"], r["dist_filtered"],
           r["angle_filtered"])
    assert got == (live, model, projected, dist_f, angle_f), got


def _twice(run, cs, **kw):
    """The contract runs every scenario twice and wants the same bits."""
    a, b = run(cs, **kw), run(cs, **kw)
    assert np.array_equal(np.asarray(a["pose"], np.float32).view(np.uint32),
                          np.asarray(b["pose"], np.float32).view(np.uint32))
    for k in ("error", "inliers", "converged", "tracking_ok", "final_step", "valid_live_points",
              "valid_model_points", "projected_points", "dist_filtered", "angle_filtered"):
        assert a[k] == b[k] or (k == "final_step" and math.isinf(a[k]) and math.isinf(b[k])), k
    return a


def _pose_is(r, P):
    return np.array_equal(np.asarray(r["pose"], np.float32).view(np.uint32), np.asarray(P, np.float32).view(np.uint32))


def acceptable_final_step_is_success(run):  # :240-270
    r = _twice(run, F.grid_fixture(300, 339, 237, 242, 1.0, 5e-4))
    _counters(r, 240, 240, 240, 0, 0)
    assert r["inliers"] == 240 and not r["converged"]
    assert 5e-5 < r["final_step"] <= 1e-3 and r["tracking_ok"]
    P = np.asarray(r["pose"], np.float64)
    assert abs(P[2, 3] - (-240.0 * 5e-4 / 241.0)) <= TOL
    assert abs(P[0, 3]) <= TOL and abs(P[1, 3]) <= TOL
    assert abs(r["error"] - 5e-4 * 5e-4) <= TOL


def inlier_floor(run):  # :272-304
    cs = F.grid_fixture(310, 329, 237, 241, 1.0, 5e-4)
    assert len(cs) == 100
    r = _twice(run, cs)
    _counters(r, 100, 100, 100, 0, 0)
    assert r["inliers"] == 100 and not r["converged"] and r["final_step"] <= 1e-3
    assert not r["tracking_ok"]  # 100 is not > 100
    assert abs(float(np.asarray(r["pose"])[2, 3]) - (-100.0 * 5e-4 / 101.0)) <= TOL
    r101 = _twice(run, cs + [F.make_corr(200, 200, 1.0, (0, 0, 1), 2, 5e-4)])
    assert r101["inliers"] == 101 and r101["final_step"] <= 1e-3 and r101["tracking_ok"]


def rotation_cap(run):  # :328-384
    r = _twice(run, F.rotation_leak_fixture(100), dist=3.0)
    _counters(r, 200, 200, 200, 0, 0)
    assert r["inliers"] == 0 and not r["converged"] and not r["tracking_ok"]
    assert math.isinf(r["final_step"]) and r["final_step"] > 0
    assert _pose_is(r, I4)  # rejected, not clamped
    vy = F.ICP_ROW_VY
    assert 200 * F.ICP_HUBER_K * vy / (200 * F.ICP_HUBER_K * vy * vy + 1.0) > 0.8
    s = _twice(run, F.rotation_leak_fixture(10), dist=3.0)
    assert s["inliers"] == 20
    oracle = 20 * F.ICP_HUBER_K * vy / (20 * F.ICP_HUBER_K * vy * vy + 1.0)
    assert abs(s["final_step"] - oracle) <= TOL
    P = np.asarray(s["pose"], np.float64)
    assert max(abs(P[0, 3]), abs(P[1, 3]), abs(P[2, 3])) <= TOL
    assert abs(P[2, 1]) >= 0.2


def translation_cap(run):  # :395-425
    r = _twice(run, F.grid_fixture(300, 339, 237, 242, 2.0, 1.0), dist=3.0)
    _counters(r, 240, 240, 240, 0, 0)
    assert r["inliers"] == 0 and _pose_is(r, I4)
    assert math.isinf(r["final_step"]) and not r["converged"] and not r["tracking_ok"]
    s = _twice(run, F.grid_fixture(317, 322, 239, 240, 2.0, 1.0), dist=3.0)
    assert s["inliers"] == 12
    assert abs(float(np.asarray(s["pose"])[2, 3]) - (-0.24 / 1.24)) <= TOL


def damping_escalates(run):  # :455-474
    r = _twice(run, F.escalation_fixture())
    _counters(r, 13, 13, 13, 0, 0)
    tz = float(np.asarray(r["pose"])[2, 3])
    assert abs(tz - (-0.14 / 13.25)) <= TOL
    assert abs(tz - (-0.14 / 12.35)) >= 2e-4 and abs(tz - (-0.14 / 12.26)) >= 2e-4


def damping_level0_without_escalation(run):  # :476-509
    r = _twice(run, F.three_wall_fixture())
    assert r["inliers"] == 3224 and r["angle_filtered"] == 0 and r["dist_filtered"] == 0
    tz = float(np.asarray(r["pose"])[2, 3])
    assert abs(tz - (-0.24 / 24.01)) <= TOL
    assert abs(tz - (-0.24 / 24.1)) >= 1e-5 and abs(tz - (-0.24 / 25.0)) >= 1e-5
    assert abs(r["final_step"] - 0.24 / 24.01) <= TOL


def model_normal_gate(run):  # :554-609
    base = _twice(run, F.model_normal_fixture((0, 0, -1)))
    assert base["inliers"] == 11
    clean = _twice(run, F.model_normal_fixture(None))
    assert clean["inliers"] == 10
    assert abs(float(np.asarray(clean["pose"])[2, 3]) - (-0.1 / 11.0)) <= TOL
    _counters(clean, 10, 10, 10, 0, 0)
    nan, inf = float("nan"), float("inf")
    for n, accepted in (((0, 0, 1), True), ((0, 0, 0.95), True), ((0, 0, 0.94), False), ((0, 0, 0.5), False),
                        ((0, 0, 0), False), ((0, 0, nan), False), ((0, 0, inf), False), ((nan, 0, 1), False)):
        r = _twice(run, F.model_normal_fixture(n))
        _counters(r, 11, 11 if accepted else 10, 11, 0, 0)
        assert r["inliers"] == (11 if accepted else 10), n
        if not accepted:
            assert _pose_is(r, clean["pose"]) and r["error"] == clean["error"], n
    nv = F.model_normal_fixture((0, 0, -1))
    nv[-1]["mv"][2] = np.float32(nan)
    r = _twice(run, nv)
    _counters(r, 11, 10, 11, 0, 0)
    assert r["inliers"] == 10


def live_normal_gate(run):  # :653-692
    r = _twice(run, F.live_normal_fixture((1, 0, 0)))
    _counters(r, 10, 10, 10, 0, 0)
    assert r["inliers"] == 10
    tx = float(np.asarray(r["pose"])[0, 3])
    assert abs(tx) > 1e-4 and abs(tx + 0.1 / 21.0) <= TOL
    for n in ((0, 0, 0), (float("nan"), 0, 0), (float("inf"), 0, 0)):
        s = _twice(run, F.live_normal_fixture(n))
        assert s["inliers"] == 0, n
        _counters(s, 10, 10, 10, 0, 0)
        assert _pose_is(s, I4) and math.isinf(s["final_step"]) and not s["converged"] and not s["tracking_ok"]
    o = _twice(run, F.live_normal_fixture((float("nan"), 0, 0), 0.01, 0.5))
    _counters(o, 10, 10, 10, 10, 0)  # the distance gate runs first
    assert o["inliers"] == 0


def angle_threshold_clamp_and_gate(run):  # :731-757
    r = _twice(run, F.orthogonal_fixture(), angle=120.0)  # clamped to 85 degrees
    _counters(r, 10, 10, 10, 0, 10)
    assert r["inliers"] == 0 and _pose_is(r, I4)
    c = _twice(run, F.grid_fixture(315, 324, 235, 244, 1.0, 0.01), angle=120.0)
    assert c["angle_filtered"] == 0 and c["inliers"] >= 10
    for a in (float("nan"), float("inf"), -5.0):  # 30, 30, 0 degrees: the orthogonal wall stays filtered
        s = _twice(run, F.orthogonal_fixture(), angle=a)
        assert s["angle_filtered"] == 10 and s["inliers"] == 0, a


def svd_returns_proper_rotation(run):  # :781-820
    r = _twice(run, F.reflection_fixture(), estimate=F.REFLECTED_ESTIMATE)
    assert r["inliers"] == 12 and r["converged"] and abs(r["final_step"]) < 1e-20
    _counters(r, 12, 12, 12, 0, 0)
    P = np.asarray(r["pose"], np.float64)
    R = P[:3, :3]
    assert abs(np.linalg.det(R) - 1.0) <= 1e-5
    assert np.abs(R.T @ R - np.eye(3)).max() <= 1e-4
    assert np.allclose(P[:, 3], (0, 0, 0, 1), atol=1e-6)


SCENARIOS = [acceptable_final_step_is_success, inlier_floor, rotation_cap, translation_cap, damping_escalates,
             damping_level0_without_escalation, model_normal_gate, live_normal_gate,
             angle_threshold_clamp_and_gate, svd_returns_proper_rotation]


def non_finite_live_vertex(run):  # coordinate_rounding_contract.cpp:352-400
    z = np.zeros(3, np.float32)
    nz = np.array([0, 0, 1], np.float32)
    cs = [dict(lp=lp, mp=(0, 0), lv=np.array(v, np.float32), ln=nz, mv=z, mn=z)
          for lp, v in (((100, 100), (0.1, 0.05, 0.5)), ((200, 200), (0.1, 0.05, float("nan"))),
                        ((300, 300), (float("inf"), 0.05, 0.5)))]
    r = _twice(run, cs, iters=(10, 5, 4))
    assert r["valid_live_points"] == 1 and r["projected_points"] == 1 and r["inliers"] == 0
    assert _pose_is(r, I4)


SCENARIOS.append(non_finite_live_vertex)
