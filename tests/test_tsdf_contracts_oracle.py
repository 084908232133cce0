"""The CPU restatement against the reference's TSDF contracts
(tests/tsdf_contracts.py): min-depth band and fold, fusion bias and weights,
raycast accuracy."""
import numpy as np
import pytest

import tsdf_contracts as TC


class OracleBackend:
    def __init__(self, orc):
        self.o = orc

    def volume(self, prm, color=False):
        o = self.o

        class V:
            def __init__(self):
                self.set_params(prm)

            def set_params(self, p):
                # TSDFVolume::setParams (src/tsdf/TSDFVolume.cpp:127-146): any change clears
                if getattr(self, "prm", None) != p:
                    self.prm = dict(p)
                    self.vol = o.Volume(o.tsdf_params(**p), color=color)

            def integrate(self, depth, rgb, pose, K, W, H, lo, hi):
                self.vol.integrate(depth, pose, o.intr(*K), W, H, lo, hi, rgb=rgb)

            def arrays(self):
                return self.vol.tsdf, self.vol.weight, self.vol.color

            def raycast(self, pose, K, W, H, colors=False):
                r = self.vol.raycast(pose, o.intr(*K), W, H, colors=colors)
                return (r["vertices"], r["normals"], r["colors"]) if colors else (r["vertices"], r["normals"])

            def load(self, t, w, c=None):
                self.vol.tsdf[:] = t
                self.vol.weight[:] = w
                if c is not None:
                    self.vol.color[:] = c

            def mesh(self):
                return self.vol.extract_mesh()

        return V()


@pytest.fixture(scope="module")
def backend(orc):
    return OracleBackend(orc)


def test_min_depth_contract(backend):
    TC.min_depth_gates(backend)


def test_fusion_bias_contract(backend):
    TC.fusion_bias(backend)


def test_raycast_accuracy_contract(backend):
    TC.raycast_accuracy(backend)


def test_subvoxel_thin_feature_contract(backend):
    TC.subvoxel_thin_feature(backend)

def test_raycast_negative_origin_contract(backend):
    TC.raycast_negative_origin(backend)
