"""azu_gb300 — GB300 (sm_103a) backend of Azu's KinectFusion hot path.

The product is libazu_gb300.so (CUDA kernels behind the C ABI of
include/azu_gpu.h). This package builds it in-tree, binds it with ctypes and
mirrors the reference's Preprocessor / ICPTracker / TSDFVolume /
MarchingCubes interfaces on top (azu_gb300.api). There is no CPU fallback:
without the built library every call raises.
"""
from . import _abi  # noqa: F401

__all__ = ["_abi", "build", "synth", "api"]
