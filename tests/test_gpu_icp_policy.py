"""The CUDA tracker against the reference's ICP numeric-policy contract
(tests/icp_numeric_policy_contract.cpp), scenario by scenario with the
contract's hand-derived expectations (tests/icp_policy.py): success rule,
inlier floor, rotation and translation caps, damping escalation and level-0
damping, normal gates and their order, the angle clamp, and the
determinant-corrected SO(3) projection of a reflected estimate."""
import numpy as np
import pytest

import fixtures as F
import icp_policy as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def run(cuda_lib):
    import torch
    from azu_gb300 import api
    zeros = {l: torch.zeros((480 >> l) * (640 >> l) * 3, dtype=torch.float32, device="cuda") for l in (1, 2)}

    def go(cs, iters=(1, 0, 0), dist=0.1, angle=30.0, estimate=P.I4):
        lv, ln, mv, mn = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in F.corr_maps(cs))
        trk = api.ICPTracker(api.tracker_params(iters=iters, dist=dist, angle=angle))
        trk.load_live(0, lv, ln, 640, 480)
        for l in (1, 2):
            trk.load_live(l, zeros[l], zeros[l], 640, 480)
        r = trk.track_prepared(640, 480, mv, mn, 640, 480, estimate, P.I4)
        trk.close()
        assert r["status"] == 0
        return r

    return go


@pytest.mark.parametrize("scenario", P.SCENARIOS, ids=lambda f: f.__name__)
def test_icp_numeric_policy(run, scenario):
    scenario(run)
