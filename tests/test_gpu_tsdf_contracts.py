"""The CUDA volume against the reference's TSDF contracts
(tests/tsdf_contracts.py): min-depth band and fold (with colour), far and
non-finite depths, a band change clearing the volume; fusion bias and
weights of a fused plane; raycast accuracy from the front, behind and at
45 degrees."""
import pytest

import tsdf_contracts as TC

pytestmark = pytest.mark.gpu


class GpuBackend:
    def volume(self, prm, color=False):
        from azu_gb300 import api

        def vp(p):
            return api.volume_params(p["resolution"], p["voxel_size"], p["truncation"], p["max_weight"],
                                     p["origin"], p["min_depth"], p["max_depth"], color=color)

        g = api.TSDFVolume(vp(prm))

        class V:
            def integrate(self, depth, rgb, pose, K, W, H, lo, hi):
                g.integrate(depth, pose, K, W, H, lo, hi, rgb=rgb)

            def arrays(self):
                if color:
                    return g.download(color=True)
                t, w = g.download()
                return t, w, None

            def raycast(self, pose, K, W, H, colors=False):
                r = g.raycast(pose, K, W, H, colors=colors)
                return (r["vertices"], r["normals"], r["colors"]) if colors else (r["vertices"], r["normals"])

            def load(self, t, w, c=None):
                g.upload(t, w, c)

            def mesh(self):
                return api.MarchingCubes().extract(g)

            def set_params(self, p):
                g.set_params(vp(p))

        return V()


def test_min_depth_contract(cuda_lib):
    TC.min_depth_gates(GpuBackend())


def test_fusion_bias_contract(cuda_lib):
    TC.fusion_bias(GpuBackend())


def test_raycast_accuracy_contract(cuda_lib):
    TC.raycast_accuracy(GpuBackend())


def test_subvoxel_thin_feature_contract(cuda_lib):
    TC.subvoxel_thin_feature(GpuBackend())

def test_raycast_negative_origin_contract(cuda_lib, orc):
    from test_tsdf_contracts_oracle import OracleBackend
    import numpy as np
    g = TC.raycast_negative_origin(GpuBackend())
    o = TC.raycast_negative_origin(OracleBackend(orc))
    for u, w in zip(g, o):
        assert np.array_equal(np.asarray(u).view(np.uint8), np.asarray(w).view(np.uint8))
