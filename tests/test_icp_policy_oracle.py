"""The CPU restatement against the reference's ICP numeric-policy contract
(tests/icp_numeric_policy_contract.cpp): success rule, inlier floor, rotation
and translation caps (reject, not clamp), damping escalation and the level-0
damping, model- and live-normal gates with their order, the angle-threshold
clamp, and the determinant-corrected SO(3) projection — each scenario with the
contract's own hand-derived expectations (tests/icp_policy.py)."""
import numpy as np
import pytest

import fixtures as F
import icp_policy as P


@pytest.fixture(scope="module")
def run(orc):
    K = orc.intr(F.FX, F.FY, F.CX, F.CY)

    def go(cs, iters=(1, 0, 0), dist=0.1, angle=30.0, estimate=P.I4):
        lv, ln, mv, mn = F.corr_maps(cs)
        levels = [(np.zeros((480, 640), np.float32), lv, ln)]
        for l in (1, 2):
            z = np.zeros((480 >> l, 640 >> l, 3), np.float32)
            levels.append((z[..., 0], z, z))
        prm = orc.icp_params(iters=iters, dist=dist, angle=angle, fold_threads=1)
        return orc.icp_track(prm, K, levels, mv, mn, estimate, P.I4).as_dict()

    return go


@pytest.mark.parametrize("scenario", P.SCENARIOS, ids=lambda f: f.__name__)
def test_icp_numeric_policy(run, scenario):
    scenario(run)
