"""Comparison of results with tests/golden/reference_outputs.npz, the outputs
of the reference's own code on the contract fixtures (tests/golden/make_golden.py):

  icp_checker(scenario)    a `run` wrapper for tests/icp_policy.py scenarios
                           that checks every call against the reference's
                           result: counts and flags equal, pose within 1e-6,
                           error / final step within 1e-6 relative
  tsdf_recorder(scenario)  digests of the scenario's array / raycast / mesh
                           outputs, compared in order with the reference's
  mesh(name)               the reference's mesh of a tests/mesh_fixtures.py volume
"""
import hashlib
import math
import os

import numpy as np

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_outputs.npz")
_G = None


def golden():
    global _G
    if _G is None:
        _G = dict(np.load(PATH))
    return _G


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def check_result(got: dict, prefix: str, pose_tol=1e-6):
    g = golden()
    want_ints = g[prefix + "/ints"]
    got_ints = [got["inliers"], int(got["converged"]), int(got["tracking_ok"]), got["valid_live_points"],
                got["valid_model_points"], got["projected_points"], got["dist_filtered"], got["angle_filtered"]]
    assert list(want_ints) == got_ints, (prefix, list(want_ints), got_ints)
    assert np.abs(np.asarray(got["pose"], np.float64) - g[prefix + "/pose"]).max() <= pose_tol, prefix
    for k, w in zip(("error", "final_step"), g[prefix + "/scalars"]):
        v = float(got[k])
        if math.isinf(w) or math.isinf(v):
            assert math.isinf(w) and math.isinf(v), (prefix, k)
        else:
            assert abs(v - float(w)) <= 1e-6 * max(1.0, abs(float(w))), (prefix, k, v, w)


def icp_checker(run, name, group="icp", pose_tol=1e-6):
    calls = [0]

    def wrapped(*a, **kw):
        r = run(*a, **kw)
        check_result(r, f"{group}/{name}/{calls[0]}", pose_tol)
        calls[0] += 1
        return r

    return wrapped, calls


def tsdf_digests(name):
    return list(golden()[f"tsdf/{name}"])


def mesh(name):
    g = golden()
    return {k: g[f"mesh/{name}/{k}"] for k in ("positions", "normals", "colors", "indices", "truncated")}
