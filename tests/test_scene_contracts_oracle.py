"""The CPU restatement against the reference's room-scene contracts
(tests/scene_contracts.py): ICP with the model's reference pose and with
models rendered at 640x480, 320x240 and 160x120."""
import pytest

import scene_contracts as SC


class OracleBackend:
    def __init__(self, orc):
        self.o = orc
        self.K = orc.intr(*SC.K640)

    def volume(self, prm):
        o, K = self.o, self.K
        vol = o.Volume(o.tsdf_params(**prm))

        class V:
            def integrate(self, depth, pose):
                vol.integrate(depth, pose, K, 640, 480, prm["min_depth"], prm["max_depth"])

            def raycast(self, pose, Kr, w, h):
                r = vol.raycast(pose, o.intr(*Kr), w, h)
                return r["vertices"], r["normals"]

        return V()

    def track(self, live, mv, mn, mw, mh, est, ref, iters=(10, 5, 4), dist=0.1, angle=30.0):
        o = self.o
        pyr = o.frame_pyramid_from_depth(live, self.K)
        prm = o.icp_params(iters=iters, dist=dist, angle=angle, fold_threads=0)
        return o.icp_track(prm, self.K, pyr, mv, mn, est, ref).as_dict()


@pytest.fixture(scope="module")
def backend(orc):
    return OracleBackend(orc)


def test_refpose_contract(backend):
    SC.refpose(backend)


def test_lowres_model_contract(backend):
    SC.lowres_model(backend)
