"""Python mirror of the reference's GPU-twin interfaces over the C ABI.

  TSDFVolume     tsdf::TSDFVolume        (include/tsdf/TSDFVolume.h:69-190)
  ICPTracker     tracking::ICPTracker    (include/tracking/ICPTracker.h:80-126)
  Preprocessor   sensor::Preprocessor    (include/sensor/Preprocessor.h:23-113)
  MarchingCubes  meshing::MarchingCubes  (include/meshing/MarchingCubes.h:35-62)
  Pipeline       PipelineController's per-frame GPU body, lockstep

Device buffers are torch CUDA tensors (plumbing only); every handle runs on
the torch stream current at construction, so torch copies and library
kernels are ordered on one stream. Poses are (4, 4) row-major float32.
"""
from __future__ import annotations

import ctypes as C
import sys

import numpy as np

from . import _abi
from ._abi import check

FP = C.POINTER(C.c_float)


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("azu_gb300 needs a CUDA device (sm_103a); there is no CPU fallback")
    return torch


def _pose(p) -> C.Array:
    a = np.ascontiguousarray(np.asarray(p, np.float32).reshape(16))
    return (C.c_float * 16)(*a.tolist())


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


_lib_stream = None


def lib_stream():
    """The torch stream every handle of this module enqueues on (never the legacy
    default stream, whose NULL handle would make the library create a private one)."""
    global _lib_stream
    if _lib_stream is None:
        _lib_stream = _torch().cuda.Stream()
    return _lib_stream


def _stream_handle():
    return C.c_void_p(lib_stream().cuda_stream)


def _ready():
    """Inputs written on the caller's torch stream are complete before library work."""
    _torch().cuda.current_stream().synchronize()


def _done():
    lib_stream().synchronize()


def _finalize(obj):
    """Garbage-collected handles are destroyed, except during interpreter
    shutdown, when the CUDA runtime may already be torn down (the process exit
    releases the device memory)."""
    if sys.is_finalizing():
        return
    try:
        obj.close()
    except Exception:
        pass


def volume_params(resolution, voxel_size, truncation, max_weight=64.0, origin=(0, 0, 0), min_depth=0.3,
                  max_depth=2.5, format=_abi.AZU_TSDF_FP32, color=False) -> _abi.VolumeParams:
    return _abi.VolumeParams(int(resolution), float(voxel_size), float(truncation), float(max_weight),
                             (C.c_float * 3)(*[float(v) for v in origin]), float(min_depth), float(max_depth),
                             int(format), int(bool(color)))


def tracker_params(iters=(10, 5, 4), dist=0.1, angle=30.0, min_depth=0.3, max_depth=2.5, fx=525.0, fy=525.0,
                   cx=319.5, cy=239.5, precision=0) -> _abi.TrackerParams:
    return _abi.TrackerParams((C.c_int * 3)(*iters), float(dist), float(angle), float(min_depth),
                              float(max_depth), float(fx), float(fy), float(cx), float(cy), int(precision))


def result_dict(r: _abi.IcpResult) -> dict:
    return dict(pose=np.array(r.pose, np.float32).reshape(4, 4), error=r.error, inliers=r.inliers,
                converged=bool(r.converged), tracking_ok=bool(r.tracking_ok), final_step=r.final_step,
                information=np.array(r.information, np.float32).reshape(6, 6),
                valid_live_points=r.valid_live_points, valid_model_points=r.valid_model_points,
                projected_points=r.projected_points, dist_filtered=r.dist_filtered,
                angle_filtered=r.angle_filtered, iterations=list(r.iterations), status=r.status)


class TSDFVolume:
    def __init__(self, params: _abi.VolumeParams, device: int = 0):
        self.lib = _abi.load()
        self.device = device
        self.h = C.c_void_p()
        check(self.lib.azu_volume_create(device, C.byref(params), _stream_handle(), C.byref(self.h)),
              "azu_volume_create")
        self.params = params

    @classmethod
    def borrowed(cls, handle, params: _abi.VolumeParams, device: int = 0):
        """A view of a volume owned by another object (pipeline, batch)."""
        v = cls.__new__(cls)
        v.lib = _abi.load()
        v.device = device
        v.h = handle if isinstance(handle, C.c_void_p) else C.c_void_p(handle)
        v.params = params
        v._borrowed = True
        return v

    def close(self):
        if self.h and not getattr(self, "_borrowed", False):
            self.lib.azu_volume_destroy(self.h)
        self.h = C.c_void_p()

    def __del__(self):
        _finalize(self)

    @property
    def n(self):
        return self.params.resolution ** 3

    def reset(self):
        check(self.lib.azu_volume_reset(self.h), "reset")

    def set_params(self, p):
        check(self.lib.azu_volume_set_params(self.h, C.byref(p)), "set_params")
        self.params = p

    def voxels_changed(self):
        """After writing voxels through the device pointer: recompute the free-space flags."""
        check(self.lib.azu_volume_voxels_changed(self.h), "voxels_changed")

    def set_free_space_skipping(self, on: bool):
        check(self.lib.azu_volume_set_free_space_skipping(self.h, int(bool(on))), "set_free_space_skipping")

    def integrate_gpu(self, d_depth, pose, K, W, H, min_depth, max_depth, d_rgb=None):
        _ready()
        check(self.lib.azu_volume_integrate(self.h, _ptr(d_depth), _ptr(d_rgb), _pose(pose), *map(float, K), W, H,
                                            float(min_depth), float(max_depth)), "integrate")

    def integrate(self, depth_m: np.ndarray, pose, K, W, H, min_depth, max_depth, rgb=None):
        d = np.ascontiguousarray(depth_m, np.float32)
        c = None if rgb is None else np.ascontiguousarray(rgb, np.uint8)
        check(self.lib.azu_volume_integrate_host(self.h, d.ctypes.data_as(C.c_void_p),
                                                 None if c is None else c.ctypes.data_as(C.c_void_p), _pose(pose),
                                                 *map(float, K), W, H, float(min_depth), float(max_depth)),
              "integrate_host")

    def raycast_gpu(self, pose, K, W, H, colors=False):
        torch = _torch()
        v = torch.empty((H, W, 3), dtype=torch.float32, device="cuda")
        n = torch.empty((H, W, 3), dtype=torch.float32, device="cuda")
        c = torch.empty((H, W, 3), dtype=torch.uint8, device="cuda") if colors else None
        _ready()
        check(self.lib.azu_volume_raycast(self.h, _pose(pose), *map(float, K), W, H, _ptr(v), _ptr(n), _ptr(c)),
              "raycast")
        return v, n, c

    def raycast(self, pose, K, W, H, colors=False):
        v, n, c = self.raycast_gpu(pose, K, W, H, colors)
        _done()
        out = dict(vertices=v.cpu().numpy(), normals=n.cpu().numpy())
        if colors:
            out["colors"] = c.cpu().numpy()
        return out

    def raycast_many(self, poses, K, W, H):
        """Model images at several poses in one launch (device tensors [n, H, W, 3])."""
        torch = _torch()
        P = np.ascontiguousarray(np.asarray(poses, np.float32).reshape(-1, 16))
        n = P.shape[0]
        v = torch.empty((n, H, W, 3), dtype=torch.float32, device="cuda")
        nrm = torch.empty((n, H, W, 3), dtype=torch.float32, device="cuda")
        _ready()
        check(self.lib.azu_volume_raycast_many(self.h, P.ctypes.data_as(_abi.fp), n, *map(float, K), W, H, _ptr(v),
                                               _ptr(nrm)), "raycast_many")
        _done()
        return v, nrm

    def point_cloud(self):
        """extractGlobalPointCloud: (N, 3) float32 world points, (N, 3) uint8 colours."""
        n = C.c_int64(0)
        check(self.lib.azu_volume_point_cloud(self.h, None, None, 0, C.byref(n)), "point_cloud")
        pts = np.empty((max(n.value, 1), 3), np.float32)
        col = np.empty((max(n.value, 1), 3), np.uint8)
        check(self.lib.azu_volume_point_cloud(self.h, pts.ctypes.data_as(C.c_void_p), col.ctypes.data_as(C.c_void_p),
                                              n.value, C.byref(n)), "point_cloud")
        return pts[:n.value], col[:n.value]

    # ---- differentiation form -------------------------------------------
    def render_depth(self, pose, K, W, H) -> np.ndarray:
        torch = _torch()
        d = torch.empty((H, W), dtype=torch.float32, device="cuda")
        _ready()
        check(self.lib.azu_volume_render_depth(self.h, _pose(pose), *map(float, K), W, H, _ptr(d)), "render_depth")
        _done()
        return d.cpu().numpy()

    def depth_backward(self, pose, K, W, H, depth_obs, huber_delta=0.01, grad_tsdf=False, jacobian=False):
        """Huber depth loss, dL/dxi (right se(3) perturbation), Gauss-Newton
        terms, and optionally dL/dtsdf and the per-pixel dD/dxi."""
        torch = _torch()
        obs = torch.from_numpy(np.ascontiguousarray(depth_obs, np.float32)).cuda()
        depth = torch.empty((H, W), dtype=torch.float32, device="cuda")
        jac = torch.empty((H, W, 6), dtype=torch.float32, device="cuda") if jacobian else None
        n = self.params.resolution ** 3
        g = torch.zeros(n, dtype=torch.float32, device="cuda") if grad_tsdf else None
        sums = (C.c_double * 35)()
        over = C.c_uint(0)
        _ready()
        check(self.lib.azu_volume_depth_backward(self.h, _pose(pose), *map(float, K), W, H, _ptr(obs),
                                                 float(huber_delta), _ptr(depth), _ptr(jac), _ptr(g), sums,
                                                 C.byref(over)), "depth_backward")
        _done()
        s = np.array(sums[:], np.float64)
        out = dict(loss=s[0], grad_xi=s[1:7], jtj=s[7:28], jtr=s[28:34], n_valid=int(s[34]),
                   depth=depth.cpu().numpy(), chain_overflow=over.value)
        if jacobian:
            out["jacobian"] = jac.cpu().numpy()
        if grad_tsdf:
            out["grad_tsdf"] = g.cpu().numpy()
        return out

    def refine_pose(self, pose, K, W, H, depth_obs, huber_delta=0.01, max_iterations=20):
        torch = _torch()
        obs = torch.from_numpy(np.ascontiguousarray(depth_obs, np.float32)).cuda()
        out = (C.c_float * 16)()
        trace = (C.c_double * (max_iterations + 1))()
        its = C.c_int(0)
        _ready()
        check(self.lib.azu_volume_refine_pose(self.h, _pose(pose), *map(float, K), W, H, _ptr(obs),
                                              float(huber_delta), int(max_iterations), out, trace, C.byref(its)),
              "refine_pose")
        _done()
        return np.array(out[:], np.float32).reshape(4, 4), np.array(trace[:its.value + 1]), its.value

    def stats(self) -> dict:
        s = _abi.VolumeStats()
        check(self.lib.azu_volume_get_stats(self.h, C.byref(s)), "stats")
        return dict(integrated_frames=s.integrated_frames, observed_voxels=s.observed_voxels,
                    last_voxels_updated=s.last_voxels_updated, last_color_updates=s.last_color_updates)

    def download(self, color=False):
        t = np.empty(self.n, np.float32)
        w = np.empty(self.n, np.float32)
        c = np.empty(3 * self.n, np.float32) if color else None
        check(self.lib.azu_volume_download(self.h, t.ctypes.data_as(C.c_void_p), w.ctypes.data_as(C.c_void_p),
                                           None if c is None else c.ctypes.data_as(C.c_void_p)), "download")
        return (t, w, c) if color else (t, w)

    def upload(self, tsdf, weight, color=None):
        t = np.ascontiguousarray(tsdf, np.float32)
        w = np.ascontiguousarray(weight, np.float32)
        c = None if color is None else np.ascontiguousarray(color, np.float32)
        check(self.lib.azu_volume_upload(self.h, t.ctypes.data_as(C.c_void_p), w.ctypes.data_as(C.c_void_p),
                                         None if c is None else c.ctypes.data_as(C.c_void_p)), "upload")


class ICPTracker:
    def __init__(self, params: _abi.TrackerParams, device: int = 0):
        self.lib = _abi.load()
        self.h = C.c_void_p()
        check(self.lib.azu_tracker_create(device, C.byref(params), _stream_handle(), C.byref(self.h)),
              "azu_tracker_create")
        self.params = params

    def close(self):
        if self.h:
            self.lib.azu_tracker_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        _finalize(self)

    def prepare_live(self, d_depth, W, H):
        _ready()
        check(self.lib.azu_tracker_prepare_live(self.h, _ptr(d_depth), W, H), "prepare_live")

    def load_live(self, level, d_v, d_n, W, H):
        _ready()
        check(self.lib.azu_tracker_load_live(self.h, level, _ptr(d_v), _ptr(d_n), W, H), "load_live")

    def track_prepared(self, W, H, d_mv, d_mn, MW, MH, estimate, ref_pose) -> dict:
        _ready()
        r = _abi.IcpResult()
        check(self.lib.azu_tracker_track_prepared(self.h, W, H, _ptr(d_mv), _ptr(d_mn), MW, MH, _pose(estimate),
                                                  _pose(ref_pose), C.byref(r)), "track_prepared")
        return result_dict(r)

    def track_many(self, W, H, d_mv, d_mn, MW, MH, estimates, ref_poses=None, params=None) -> list:
        """One solve per candidate k against model image k (d_mv/d_mn hold them back to back)."""
        E = np.ascontiguousarray(np.asarray(estimates, np.float32).reshape(-1, 16))
        n = E.shape[0]
        R = None if ref_poses is None else np.ascontiguousarray(np.asarray(ref_poses, np.float32).reshape(-1, 16))
        out = (_abi.IcpResult * n)()
        _ready()
        check(self.lib.azu_tracker_track_many(self.h, W, H, _ptr(d_mv), _ptr(d_mn), MW, MH, n,
                                              E.ctypes.data_as(_abi.fp),
                                              None if R is None else R.ctypes.data_as(_abi.fp),
                                              None if params is None else C.byref(params), out), "track_many")
        return [result_dict(out[k]) for k in range(n)]

    def build_system(self, level, d_mv, d_mn, MW, MH, pose, ref_pose) -> dict:
        _ready()
        A = (C.c_float * 36)()
        b = (C.c_float * 6)()
        res = C.c_float()
        cnt = (C.c_int * 6)()
        check(self.lib.azu_tracker_build_system(self.h, level, _ptr(d_mv), _ptr(d_mn), MW, MH, _pose(pose),
                                                _pose(ref_pose), A, b, C.byref(res), cnt), "build_system")
        c = list(cnt)
        return dict(A=np.array(A, np.float32).reshape(6, 6), b=np.array(b, np.float32), residual=res.value,
                    inliers=c[0], valid_live=c[1], valid_model=c[2], projected=c[3], dist_filtered=c[4],
                    angle_filtered=c[5])

    def live_maps(self, level, W, H):
        """(depth, vertices, normals) of a pyramid level as host arrays."""
        v, n, d = C.c_void_p(), C.c_void_p(), C.c_void_p()
        check(self.lib.azu_tracker_live_maps(self.h, level, C.byref(v), C.byref(n), C.byref(d)), "live_maps")
        w, h = W >> level, H >> level
        return (device_to_host(d.value, (h, w), np.float32), device_to_host(v.value, (h, w, 3), np.float32),
                device_to_host(n.value, (h, w, 3), np.float32))


class _DevArray:
    """A raw device pointer exposed through __cuda_array_interface__."""

    def __init__(self, ptr, shape, dtype):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": np.dtype(dtype).str,
                                         "data": (int(ptr), False), "version": 3}


def device_to_host(ptr: int, shape, dtype) -> np.ndarray:
    torch = _torch()
    _done()
    torch.cuda.synchronize()
    return torch.as_tensor(_DevArray(ptr, shape, dtype), device="cuda").cpu().numpy().copy()


class Preprocessor:
    def __init__(self, mode=_abi.AZU_PRE_FULL, device: int = 0):
        self.lib = _abi.load()
        self.h = C.c_void_p()
        check(self.lib.azu_preprocessor_create(device, int(mode), _stream_handle(), C.byref(self.h)),
              "azu_preprocessor_create")

    def close(self):
        if self.h:
            self.lib.azu_preprocessor_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        _finalize(self)

    def reset(self):
        check(self.lib.azu_preprocessor_reset(self.h), "reset")

    def reset_temporal(self):
        check(self.lib.azu_preprocessor_reset_temporal(self.h), "reset_temporal")

    def process(self, depth_raw: np.ndarray, rgb: np.ndarray, min_depth, max_depth):
        """RawFrame in place semantics: returns processed (depth, rgb) copies."""
        d = np.ascontiguousarray(depth_raw, np.uint16).copy()
        c = np.ascontiguousarray(rgb, np.uint8).copy()
        check(self.lib.azu_preprocessor_process(self.h, d.ctypes.data_as(C.c_void_p), c.ctypes.data_as(C.c_void_p),
                                                float(min_depth), float(max_depth)), "process")
        return d, c

    def device_outputs(self, W=640, H=480):
        """(depth_m, depth_raw, luma, rgb) of the last frame as host arrays."""
        L = self.lib
        return (device_to_host(L.azu_preprocessor_depth_meters(self.h), (H, W), np.float32),
                device_to_host(L.azu_preprocessor_depth_raw(self.h), (H, W), np.uint16),
                device_to_host(L.azu_preprocessor_luma(self.h), (H, W), np.float32),
                device_to_host(L.azu_preprocessor_rgb(self.h), (H, W, 3), np.uint8))


class MarchingCubes:
    def __init__(self, device: int = 0, max_triangles: int = 2_000_000, stream: int | None = None):
        self.lib = _abi.load()
        self.h = C.c_void_p()
        st = C.c_void_p(stream) if stream is not None else _stream_handle()
        check(self.lib.azu_mesher_create(device, st, C.byref(self.h)), "azu_mesher_create")
        self.set_max_triangles(max_triangles)

    def extract_counts(self, vol_handle) -> dict:
        """extractGPU without the host copy: counts only, mesh stays on the device."""
        info = _abi.MeshInfo()
        check(self.lib.azu_mesher_extract(self.h, vol_handle, C.byref(info)), "extract")
        return dict(n_vertices=info.n_vertices, n_indices=info.n_indices, truncated=bool(info.truncated),
                    launches=info.launches)

    def close(self):
        if self.h:
            self.lib.azu_mesher_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        _finalize(self)

    def set_max_triangles(self, n):
        check(self.lib.azu_mesher_set_max_triangles(self.h, C.c_int64(int(n))), "set_max_triangles")

    def extract(self, vol: TSDFVolume) -> dict:
        info = _abi.MeshInfo()
        check(self.lib.azu_mesher_extract(self.h, vol.h, C.byref(info)), "extract")
        nv, ni = info.n_vertices, info.n_indices
        pos = np.empty((max(nv, 1), 3), np.float32)
        nrm = np.empty((max(nv, 1), 3), np.float32)
        col = np.empty((max(nv, 1), 3), np.uint8)
        idx = np.empty(max(ni, 1), np.uint32)
        check(self.lib.azu_mesher_copy_out(self.h, pos.ctypes.data_as(C.c_void_p), nrm.ctypes.data_as(C.c_void_p),
                                           col.ctypes.data_as(C.c_void_p), idx.ctypes.data_as(C.c_void_p)),
              "copy_out")
        return dict(positions=pos[:nv], normals=nrm[:nv], colors=col[:nv], indices=idx[:ni],
                    truncated=bool(info.truncated))


def pipeline_params(volume: _abi.VolumeParams, tracker: _abi.TrackerParams, preprocess_mode=_abi.AZU_PRE_FULL,
                    min_depth=0.3, max_depth=2.5, input_is_mm=False, use_graph=True, width=0,
                    height=0) -> _abi.PipelineParams:
    return _abi.PipelineParams(volume, tracker, int(preprocess_mode), float(min_depth), float(max_depth),
                               int(bool(input_is_mm)), int(bool(use_graph)), int(width), int(height))


class Pipeline:
    def __init__(self, params: _abi.PipelineParams, device: int = 0):
        self.lib = _abi.load()
        self.h = C.c_void_p()
        check(self.lib.azu_pipeline_create(device, C.byref(params), C.byref(self.h)), "azu_pipeline_create")

    def close(self):
        if self.h:
            self.lib.azu_pipeline_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        _finalize(self)

    @staticmethod
    def _frame(r: _abi.FrameResult) -> dict:
        return dict(pose=np.array(r.pose, np.float32).reshape(4, 4), icp=result_dict(r.icp), quality=r.quality,
                    integrated=bool(r.integrated), frame_index=r.frame_index)

    def reset(self):
        """Empty volume, first-frame state (PipelineController's reset)."""
        check(self.lib.azu_pipeline_reset(self.h), "azu_pipeline_reset")

    def process_frame(self, depth: np.ndarray, rgb: np.ndarray | None = None) -> dict:
        """One frame from host buffers (H2D, whole frame on the device, D2H)."""
        r = _abi.FrameResult()
        d = np.ascontiguousarray(depth, np.uint16)
        c = None if rgb is None else np.ascontiguousarray(rgb, np.uint8)
        check(self.lib.azu_pipeline_process_frame(self.h, d.ctypes.data_as(C.c_void_p),
                                                  None if c is None else c.ctypes.data_as(C.c_void_p),
                                                  C.byref(r)), "process_frame")
        return self._frame(r)

    def process_frame_packed(self, h_packed_ptr: int) -> dict:
        """One frame from a packed host slot (depth | RGB) with one host-to-device copy."""
        r = _abi.FrameResult()
        check(self.lib.azu_pipeline_process_frame_packed(self.h, C.c_void_p(h_packed_ptr), C.byref(r)),
              "process_frame_packed")
        return self._frame(r)

    def process_frame_device(self, d_depth_ptr: int, d_rgb_ptr: int | None = None, sync: bool = False):
        """One frame from device buffers; only enqueued unless sync."""
        r = _abi.FrameResult() if sync else None
        check(self.lib.azu_pipeline_process_frame_device(self.h, C.c_void_p(d_depth_ptr),
                                                         None if d_rgb_ptr is None else C.c_void_p(d_rgb_ptr),
                                                         C.byref(r) if sync else None), "process_frame_device")
        return self._frame(r) if sync else None

    def last_result(self) -> dict:
        r = _abi.FrameResult()
        check(self.lib.azu_pipeline_last_result(self.h, C.byref(r)), "last_result")
        return self._frame(r)

    @property
    def stream(self) -> int:
        return self.lib.azu_pipeline_stream(self.h)

    def set_profiling(self, on: bool):
        check(self.lib.azu_pipeline_set_profiling(self.h, int(bool(on))), "set_profiling")

    def stage_times(self):
        ms = (C.c_double * 5)()
        n = C.c_int()
        check(self.lib.azu_pipeline_stage_times(self.h, ms, C.byref(n)), "stage_times")
        return dict(zip(("input", "frame", "track", "integrate", "raycast"), list(ms))), n.value

    def volume_stats(self) -> dict:
        s = _abi.VolumeStats()
        check(self.lib.azu_volume_get_stats(self.lib.azu_pipeline_volume(self.h), C.byref(s)), "stats")
        return dict(observed_voxels=s.observed_voxels, total_voxels_updated=s.total_voxels_updated,
                    last_voxels_updated=s.last_voxels_updated)

    def volume_handle(self):
        return C.c_void_p(self.lib.azu_pipeline_volume(self.h))


class Batch:
    """Many independent scenes on millimetre depth (the batching form): one
    frame per step for every scene given a depth image."""

    def __init__(self, scenes, device: int = 0):
        self.lib = _abi.load()
        self.device = device
        self.n = len(scenes)
        arr = (_abi.BatchScene * self.n)()
        self.params = []
        for i, sc in enumerate(scenes):
            v = sc.volume
            vp = volume_params(v["resolution"], v["voxel_size"], v["truncation"], v["max_weight"], v["origin"],
                               sc.min_depth, sc.max_depth, 0)
            tp = tracker_params(min_depth=sc.min_depth, max_depth=sc.max_depth, fx=sc.fx, fy=sc.fy, cx=sc.cx,
                                cy=sc.cy)
            arr[i] = _abi.BatchScene(vp, tp, int(sc.width), int(sc.height), float(sc.min_depth),
                                     float(sc.max_depth))
            self.params.append(vp)
        self.h = C.c_void_p()
        check(self.lib.azu_batch_create(device, self.n, arr, C.byref(self.h)), "azu_batch_create")

    def close(self):
        if self.h:
            self.lib.azu_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        _finalize(self)

    def process(self, depth_mm, on_device=False, results=True):
        """depth_mm: per scene a uint16 array (host) / device pointer, or None."""
        ptrs = (C.c_void_p * self.n)()
        keep = []
        for i, d in enumerate(depth_mm):
            if d is None:
                ptrs[i] = None
            elif on_device:
                ptrs[i] = int(d)
            else:
                a = np.ascontiguousarray(d, np.uint16)
                keep.append(a)
                ptrs[i] = a.ctypes.data_as(C.c_void_p).value
        res = (_abi.FrameResult * self.n)() if results else None
        check(self.lib.azu_batch_process(self.h, ptrs, int(bool(on_device)), res), "azu_batch_process")
        if not results:
            return None
        return [Pipeline._frame(res[i]) if depth_mm[i] is not None else None for i in range(self.n)]

    def autotune(self):
        a, b = C.c_float(0), C.c_float(0)
        check(self.lib.azu_batch_autotune(self.h, C.byref(a), C.byref(b)), "azu_batch_autotune")
        return a.value, b.value

    def shapes(self):
        """(integrate warps per block, integrate x-parts per row, raycast tile w, h)."""
        w, parts, rw, rh = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        check(self.lib.azu_batch_get_shapes(self.h, C.byref(w), C.byref(parts), C.byref(rw), C.byref(rh)),
              "get_shapes")
        return w.value, parts.value, rw.value, rh.value

    def set_shapes(self, int_warps, int_parts, ray_w, ray_h):
        check(self.lib.azu_batch_set_shapes(self.h, int(int_warps), int(int_parts), int(ray_w), int(ray_h)),
              "set_shapes")

    def volume(self, i) -> TSDFVolume:
        return TSDFVolume.borrowed(self.lib.azu_batch_volume(self.h, i), self.params[i], self.device)

    def synchronize(self):
        check(self.lib.azu_batch_synchronize(self.h), "synchronize")

    @property
    def stream(self):
        return self.lib.azu_batch_stream(self.h)


def _mesh_args(mesh):
    pos = np.ascontiguousarray(mesh["positions"], np.float32).reshape(-1, 3)
    nrm = mesh.get("normals")
    nrm = None if nrm is None or len(nrm) == 0 else np.ascontiguousarray(nrm, np.float32).reshape(-1, 3)
    col = mesh.get("colors")
    col = None if col is None or len(col) == 0 else np.ascontiguousarray(col, np.uint8).reshape(-1)
    idx = np.ascontiguousarray(mesh["indices"], np.uint32).reshape(-1)
    keep = (pos, nrm, col, idx)
    args = (pos.ctypes.data_as(C.c_void_p), len(pos),
            None if nrm is None else nrm.ctypes.data_as(C.c_void_p), 0 if nrm is None else len(nrm),
            None if col is None else col.ctypes.data_as(C.c_void_p), 0 if col is None else col.size,
            idx.ctypes.data_as(C.c_void_p), idx.size)
    return keep, args


def write_ply(path: str, mesh: dict, binary: bool = True):
    """PLYExporter (binary little endian or ASCII) of a mesh dict (positions,
    normals, colors, indices)."""
    keep, args = _mesh_args(mesh)
    check(_abi.load().azu_mesh_write_ply(str(path).encode(), int(bool(binary)), *args), "write_ply")


def write_glb(path: str, mesh: dict):
    """GLBExporter of a mesh dict."""
    keep, args = _mesh_args(mesh)
    check(_abi.load().azu_mesh_write_glb(str(path).encode(), *args), "write_glb")


class Recording:
    """A fakenect recording directory (INDEX.txt + PGM depth / PPM RGB), paired
    like the sensor pairs live frames."""

    def __init__(self, path: str):
        self.lib = _abi.load()
        self.h = C.c_void_p()
        check(self.lib.azu_recording_open(str(path).encode(), C.byref(self.h)), "azu_recording_open")

    def close(self):
        if self.h:
            self.lib.azu_recording_close(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        _finalize(self)

    def __len__(self):
        return self.lib.azu_recording_frame_count(self.h)

    def info(self, k):
        d, r, v = C.c_uint32(), C.c_uint32(), C.c_int()
        check(self.lib.azu_recording_frame_info(self.h, k, C.byref(d), C.byref(r), C.byref(v)), "frame_info")
        return d.value, (r.value if v.value else None)

    def read(self, k):
        depth = np.empty((480, 640), np.uint16)
        rgb = np.empty((480, 640, 3), np.uint8)
        v = C.c_int()
        check(self.lib.azu_recording_read(self.h, k, depth.ctypes.data_as(C.c_void_p), rgb.ctypes.data_as(C.c_void_p),
                                          C.byref(v)), "recording_read")
        return depth, rgb, bool(v.value)


class Ingest:
    """Read-ahead of a recording into pinned slots (depth | RGB per slot)."""

    def __init__(self, rec: Recording, slots=4, first=0, count=None):
        self.lib = _abi.load()
        self.rec = rec
        self.h = C.c_void_p()
        n = len(rec) - first if count is None else count
        check(self.lib.azu_ingest_create(rec.h, int(slots), int(first), int(n), C.byref(self.h)), "ingest_create")

    def close(self):
        if self.h:
            self.lib.azu_ingest_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        _finalize(self)

    def next(self):
        """(slot pointer, frame index, rgb_valid), or None at the end."""
        slot, k, v = C.c_void_p(), C.c_int(), C.c_int()
        rc = self.lib.azu_ingest_next(self.h, C.byref(slot), C.byref(k), C.byref(v))
        if rc == 1:
            return None
        check(rc, "ingest_next")
        return slot.value, k.value, bool(v.value)

    def release(self):
        check(self.lib.azu_ingest_release(self.h), "ingest_release")
