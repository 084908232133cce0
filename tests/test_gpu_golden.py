"""The CUDA path against the reference's OWN outputs on the contract fixtures
(tests/golden/reference_outputs.npz, written by tests/golden/make_golden.py
from the reference's sources built unmodified here):

  ICP numeric policy   every tracker call of every scenario: counts and flags
                       equal, pose within 1e-6 (the solvers differ in rounding)
  TSDF contracts       min-depth band and fold, fused plane (volume after 1, 3,
                       70 frames, mesh), raycast accuracy, sub-voxel plates,
                       negative origin: every volume, raycast and mesh output
                       bit for bit (sha256 of the bytes)
  room-scene ICP       ref-pose and low-res model solves: pose within 1e-4,
                       same tracking_ok
  mesh contracts       every frontier and welding fixture: positions, normals,
                       colours and welded indices bit for bit; the welded vertex
                       count equals the distinct-edge oracle
Each scenario also asserts the contract's own expectations."""
import numpy as np
import pytest

import golden_check as G
import icp_policy as P
import mesh_fixtures as MF
import scene_contracts as SC
import tsdf_contracts as TC
from test_gpu_icp_policy import run as _icp_run_fixture  # noqa: F401  (the GPU tracker runner)
from test_gpu_scene_contracts import GpuBackend as SceneGpu
from test_gpu_tsdf_contracts import GpuBackend as TsdfGpu

pytestmark = pytest.mark.gpu
run = _icp_run_fixture


@pytest.mark.parametrize("scenario", P.SCENARIOS, ids=lambda f: f.__name__)
def test_icp_policy_equals_reference(run, scenario):
    checked, calls = G.icp_checker(run, scenario.__name__)
    scenario(checked)
    assert calls[0] > 0


class _Recording:
    """Wraps a TSDF backend; every array / raycast / mesh output is digested."""

    def __init__(self, inner, rec):
        self.inner, self.rec = inner, rec

    def volume(self, prm, color=False):
        v, rec = self.inner.volume(prm, color), self.rec

        class V:
            def integrate(self, *a):
                v.integrate(*a)

            def arrays(self):
                out = v.arrays()
                rec.append(G.digest(*out) if color else G.digest(out[0], out[1]))
                return out

            def raycast(self, *a, **kw):
                out = v.raycast(*a, **kw)
                rec.append(G.digest(*out))
                return out

            def mesh(self):
                m = v.mesh()
                rec.append(G.digest(m["positions"], m["normals"], m["colors"], m["indices"]))
                return m

            def load(self, *a):
                v.load(*a)

            def set_params(self, p):
                v.set_params(p)

        return V()


@pytest.mark.parametrize("scenario", [TC.min_depth_gates, TC.fusion_bias, TC.raycast_accuracy,
                                      TC.subvoxel_thin_feature, TC.raycast_negative_origin],
                         ids=lambda f: f.__name__)
def test_tsdf_contract_outputs_equal_reference(cuda_lib, scenario):
    rec = []
    scenario(_Recording(TsdfGpu(), rec))
    want = G.tsdf_digests(scenario.__name__)
    assert len(rec) == len(want)
    bad = [k for k, (a, b) in enumerate(zip(rec, want)) if a != b]
    assert not bad, f"outputs {bad} of {len(want)} differ from the reference's"


@pytest.mark.parametrize("scenario", [SC.refpose, SC.lowres_model], ids=lambda f: f.__name__)
def test_scene_contract_solves_match_reference(cuda_lib, scenario):
    gpu = SceneGpu()
    calls = []

    class Checked:
        def volume(self, prm):
            return gpu.volume(prm)

        def track(self, *a, **kw):
            r = gpu.track(*a, **kw)
            pre = f"scene/{scenario.__name__}/{len(calls)}"
            g = G.golden()
            assert np.abs(np.asarray(r["pose"], np.float64) - g[pre + "/pose"]).max() <= 1e-4, pre
            assert int(r["tracking_ok"]) == int(g[pre + "/ints"][2]), pre
            calls.append(r)
            return r

    scenario(Checked())
    assert len(calls) >= 2


@pytest.mark.parametrize("name", list(MF.FIXTURES), ids=str)
def test_mesh_fixture_equals_reference(cuda_lib, name):
    from azu_gb300 import api
    prm, t, w, c = MF.FIXTURES[name]()
    g = api.TSDFVolume(api.volume_params(prm["resolution"], prm["voxel_size"], prm["truncation"], prm["max_weight"],
                                         prm["origin"], prm["min_depth"], prm["max_depth"], color=True))
    g.upload(t, w, c)
    m = api.MarchingCubes().extract(g)
    want = G.mesh(name)
    assert len(want["positions"]) == len(m["positions"]) and len(want["indices"]) == len(m["indices"])
    for k in ("positions", "normals"):
        assert np.array_equal(np.asarray(m[k], np.float32).view(np.uint32), want[k].view(np.uint32)), k
    assert np.array_equal(m["colors"], want["colors"]) and np.array_equal(m["indices"], want["indices"])
    assert bool(m["truncated"]) == bool(want["truncated"])
    if name.startswith("weld_sphere"):
        assert len(m["positions"]) == MF.welded_edge_count(prm, t, w, MF.tri_table())
