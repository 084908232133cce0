"""The CUDA path against the reference's room-scene contracts
(tests/scene_contracts.py): ICP with the model's reference pose
(icp_refpose_contract) and with models rendered at 640x480, 320x240 and
160x120 with scaled intrinsics, including the coarse level-2 relocalisation
solve (icp_lowres_model_contract)."""
import numpy as np
import pytest

import scene_contracts as SC

pytestmark = pytest.mark.gpu


class GpuBackend:
    def volume(self, prm):
        from azu_gb300 import api
        g = api.TSDFVolume(api.volume_params(prm["resolution"], prm["voxel_size"], prm["truncation"],
                                             prm["max_weight"], prm["origin"], prm["min_depth"], prm["max_depth"]))

        class V:
            def integrate(self, depth, pose):
                g.integrate(depth, pose, SC.K640, 640, 480, prm["min_depth"], prm["max_depth"])

            def raycast(self, pose, K, w, h):
                r = g.raycast(pose, K, w, h)
                return r["vertices"], r["normals"]

        return V()

    def track(self, live, mv, mn, mw, mh, est, ref, iters=(10, 5, 4), dist=0.1, angle=30.0):
        import torch
        from azu_gb300 import api
        trk = api.ICPTracker(api.tracker_params(iters=iters, dist=dist, angle=angle, min_depth=0.3, max_depth=3.0))
        trk.prepare_live(torch.from_numpy(np.ascontiguousarray(live, np.float32)).cuda(), 640, 480)
        r = trk.track_prepared(640, 480, torch.from_numpy(np.ascontiguousarray(mv)).cuda(),
                               torch.from_numpy(np.ascontiguousarray(mn)).cuda(), mw, mh, est, ref)
        trk.close()
        assert r["status"] == 0
        return r


def test_refpose_contract(cuda_lib):
    SC.refpose(GpuBackend())


def test_lowres_model_contract(cuda_lib):
    SC.lowres_model(GpuBackend())
