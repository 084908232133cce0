"""The CPU restatement against the reference's own outputs on the contract
fixtures (tests/golden/reference_outputs.npz), as tests/test_gpu_golden.py
checks the CUDA path: ICP calls, TSDF output digests, meshes bit for bit."""
import numpy as np
import pytest

import golden_check as G
import icp_policy as P
import mesh_fixtures as MF
import tsdf_contracts as TC
from test_gpu_golden import _Recording
from test_icp_policy_oracle import run  # noqa: F401  (the restatement runner fixture)
from test_tsdf_contracts_oracle import OracleBackend


@pytest.mark.parametrize("scenario", P.SCENARIOS, ids=lambda f: f.__name__)
def test_icp_policy_equals_reference(run, scenario):
    checked, calls = G.icp_checker(run, scenario.__name__)
    scenario(checked)
    assert calls[0] > 0


@pytest.mark.parametrize("scenario", [TC.min_depth_gates, TC.fusion_bias, TC.raycast_accuracy,
                                      TC.subvoxel_thin_feature, TC.raycast_negative_origin],
                         ids=lambda f: f.__name__)
def test_tsdf_contract_outputs_equal_reference(orc, scenario):
    rec = []
    scenario(_Recording(OracleBackend(orc), rec))
    assert rec == G.tsdf_digests(scenario.__name__)


@pytest.mark.parametrize("name", list(MF.FIXTURES), ids=str)
def test_mesh_fixture_equals_reference(orc, name):
    prm, t, w, c = MF.FIXTURES[name]()
    o = orc.Volume(orc.tsdf_params(**prm), color=True)
    o.tsdf[:], o.weight[:], o.color[:] = t, w, c
    m = o.extract_mesh()
    want = G.mesh(name)
    for k in ("positions", "normals"):
        assert np.array_equal(np.asarray(m[k], np.float32).reshape(-1, 3).view(np.uint32), want[k].view(np.uint32)), k
    assert np.array_equal(np.asarray(m["colors"]).reshape(-1, 3), want["colors"])
    assert np.array_equal(np.asarray(m["indices"]).reshape(-1), want["indices"])
    if name == "weld_sphere":
        assert len(want["positions"]) == MF.welded_edge_count(prm, t, w, MF.tri_table())
