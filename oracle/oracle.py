"""Oracle (test infrastructure only): ctypes binding of oracle/_build/liborc.so,
the CPU restatement of Azu's KinectFusion hot path. Imported by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg only, to compare results
against and to time the CPU path.

Arrays are numpy; poses are row-major (4, 4) float32 world-from-camera.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liborc.so")


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


class TsdfParams(C.Structure):
    _fields_ = [("res", C.c_int), ("voxel_size", C.c_float), ("truncation", C.c_float),
                ("max_weight", C.c_float), ("origin", C.c_float * 3),
                ("min_depth", C.c_float), ("max_depth", C.c_float)]


class Intr(C.Structure):
    _fields_ = [("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float)]


class IcpParams(C.Structure):
    _fields_ = [("max_iterations", C.c_int * 3), ("dist_threshold", C.c_float),
                ("angle_threshold", C.c_float), ("fold_threads", C.c_int)]


class IcpResult(C.Structure):
    _fields_ = [("pose", C.c_float * 16), ("error", C.c_float), ("inliers", C.c_int),
                ("converged", C.c_int), ("tracking_ok", C.c_int), ("final_step", C.c_float),
                ("information", C.c_float * 36), ("valid_live_points", C.c_int),
                ("valid_model_points", C.c_int), ("projected_points", C.c_int),
                ("dist_filtered", C.c_int), ("angle_filtered", C.c_int), ("iterations", C.c_int * 3)]

    def as_dict(self):
        return dict(pose=np.array(self.pose, np.float32).reshape(4, 4), error=self.error,
                    inliers=self.inliers, converged=bool(self.converged),
                    tracking_ok=bool(self.tracking_ok), final_step=self.final_step,
                    information=np.array(self.information, np.float32).reshape(6, 6),
                    valid_live_points=self.valid_live_points,
                    valid_model_points=self.valid_model_points,
                    projected_points=self.projected_points, dist_filtered=self.dist_filtered,
                    angle_filtered=self.angle_filtered, iterations=list(self.iterations))


class MeshInfo(C.Structure):
    _fields_ = [("n_vertices", C.c_int64), ("n_indices", C.c_int64), ("truncated", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB_PATH)
    return _lib


def _p(a, t=C.c_float):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(t))


def _pose(p):
    return np.ascontiguousarray(np.asarray(p, np.float32).reshape(16))


def tsdf_params(res=None, voxel_size=0.01, truncation=0.03, max_weight=128.0, origin=(0, 0, 0), min_depth=0.3,
                max_depth=5.0, resolution=None, format=0):
    res = resolution if res is None else res
    return TsdfParams(int(res), float(voxel_size), float(truncation), float(max_weight),
                      (C.c_float * 3)(*[float(v) for v in origin]), float(min_depth), float(max_depth))


def intr(fx, fy, cx, cy):
    return Intr(float(fx), float(fy), float(cx), float(cy))


def set_threads(n: int):
    lib().orc_set_threads(int(n))


def get_threads() -> int:
    return lib().orc_get_threads()


class Volume:
    """Host volume: separate tsdf / weight (/ colour) arrays, z-major like the reference."""

    def __init__(self, p: TsdfParams, color: bool = False):
        self.p = p
        n = p.res ** 3
        self.tsdf = np.empty(n, np.float32)
        self.weight = np.empty(n, np.float32)
        self.color = np.empty(3 * n, np.float32) if color else None
        self.reset()

    def reset(self):
        lib().orc_tsdf_reset(C.byref(self.p), _p(self.tsdf), _p(self.weight), _p(self.color))

    def integrate(self, depth_m, pose, K, W, H, min_depth, max_depth, rgb=None):
        st = np.zeros(9, np.int64)
        depth_m = np.ascontiguousarray(depth_m, np.float32)
        rgbp = None if rgb is None else np.ascontiguousarray(rgb, np.uint8)
        lib().orc_tsdf_integrate(C.byref(self.p), _p(self.tsdf), _p(self.weight), _p(self.color),
                                 _p(depth_m), _p(rgbp, C.c_uint8), _p(_pose(pose)), K, int(W), int(H),
                                 C.c_float(min_depth), C.c_float(max_depth), _p(st, C.c_int64))
        return dict(newly_observed=int(st[0]), voxels_updated=int(st[1]), color_updates=int(st[2]),
                    aabb=[int(v) for v in st[3:9]])

    def raycast(self, pose, K, W, H, colors=False):
        v = np.zeros((H * W * 3), np.float32)
        n = np.zeros((H * W * 3), np.float32)
        c = np.zeros((H * W * 3), np.uint8) if colors else None
        s = C.c_int64(0)
        lib().orc_tsdf_raycast(C.byref(self.p), _p(self.tsdf), _p(self.weight), _p(self.color),
                               _p(_pose(pose)), K, int(W), int(H), _p(v), _p(n), _p(c, C.c_uint8),
                               C.byref(s))
        out = dict(vertices=v.reshape(H, W, 3), normals=n.reshape(H, W, 3), samples=s.value)
        if colors:
            out["colors"] = c.reshape(H, W, 3)
        return out

    def point_cloud(self):
        L = lib()
        L.orc_point_cloud.restype = C.c_int64
        n = L.orc_point_cloud(C.byref(self.p), _p(self.tsdf), _p(self.weight), _p(self.color), None, None)
        pts = np.zeros((max(n, 1), 3), np.float32)
        col = np.zeros((max(n, 1), 3), np.uint8)
        L.orc_point_cloud(C.byref(self.p), _p(self.tsdf), _p(self.weight), _p(self.color), _p(pts),
                          _p(col, C.c_uint8))
        return pts[:n], col[:n]

    def extract_mesh(self, max_triangles=2_000_000):
        info = MeshInfo()
        lib().orc_mc_extract(C.byref(self.p), _p(self.tsdf), _p(self.weight), _p(self.color),
                             C.c_int64(max_triangles), C.byref(info), None, None, None, None)
        nv, ni = info.n_vertices, info.n_indices
        pos = np.zeros(3 * max(nv, 1), np.float32)
        nrm = np.zeros(3 * max(nv, 1), np.float32)
        col = np.zeros(3 * max(nv, 1), np.uint8)
        idx = np.zeros(max(ni, 1), np.uint32)
        lib().orc_mc_extract(C.byref(self.p), _p(self.tsdf), _p(self.weight), _p(self.color),
                             C.c_int64(max_triangles), C.byref(info), _p(pos), _p(nrm),
                             _p(col, C.c_uint8), _p(idx, C.c_uint32))
        return dict(positions=pos[:3 * nv].reshape(-1, 3), normals=nrm[:3 * nv].reshape(-1, 3),
                    colors=col[:3 * nv].reshape(-1, 3), indices=idx[:ni],
                    truncated=bool(info.truncated))


def build_frame_raw(raw, K, min_depth, max_depth):
    H, W = raw.shape
    raw = np.ascontiguousarray(raw, np.uint16)
    d = np.zeros(W * H, np.float32)
    v = np.zeros(W * H * 3, np.float32)
    n = np.zeros(W * H * 3, np.float32)
    lib().orc_build_frame(_p(raw, C.c_uint16), W, H, K, C.c_float(min_depth), C.c_float(max_depth),
                          _p(d), _p(v), _p(n))
    return d.reshape(H, W), v.reshape(H, W, 3)


def vertices_from_depth(depth_m, K):
    H, W = depth_m.shape
    d = np.ascontiguousarray(depth_m, np.float32)
    v = np.zeros(W * H * 3, np.float32)
    lib().orc_vertices_from_depth(_p(d), W, H, K, _p(v))
    return v.reshape(H, W, 3)


def compute_normals(depth_m, vertices):
    H, W = depth_m.shape
    n = np.zeros(W * H * 3, np.float32)
    lib().orc_compute_normals(_p(np.ascontiguousarray(depth_m, np.float32)),
                              _p(np.ascontiguousarray(vertices, np.float32)), W, H, _p(n))
    return n.reshape(H, W, 3)


def downsample(depth_m, vertices, normals):
    H, W = depth_m.shape
    h, w = H // 2, W // 2
    d = np.zeros(w * h, np.float32)
    v = np.zeros(w * h * 3, np.float32)
    n = np.zeros(w * h * 3, np.float32)
    lib().orc_downsample(_p(np.ascontiguousarray(depth_m, np.float32)),
                         _p(np.ascontiguousarray(vertices, np.float32)),
                         _p(np.ascontiguousarray(normals, np.float32)), W, H, _p(d), _p(v), _p(n))
    return d.reshape(h, w), v.reshape(h, w, 3), n.reshape(h, w, 3)


def frame_pyramid_from_depth(depth_m, K):
    """Level 0 from metres (vertices + normals), then two jump-guarded halvings."""
    v0 = vertices_from_depth(depth_m, K)
    n0 = compute_normals(depth_m, v0)
    levels = [(np.ascontiguousarray(depth_m, np.float32), v0, n0)]
    for _ in range(2):
        levels.append(downsample(*levels[-1]))
    return levels


def icp_params(iters=(10, 5, 4), dist=0.1, angle=30.0, fold_threads=1):
    return IcpParams((C.c_int * 3)(*iters), float(dist), float(angle), int(fold_threads))


def icp_build_system(prm, K, live_v, live_n, model_v, model_n, pose, ref_pose):
    H, W = live_v.shape[:2]
    MH, MW = model_v.shape[:2]
    A = np.zeros(36, np.float32)
    b = np.zeros(6, np.float32)
    r = C.c_float(0)
    counts = np.zeros(6, np.int32)
    ok = lib().orc_icp_build_system(
        C.byref(prm), K, _p(np.ascontiguousarray(live_v, np.float32)),
        _p(np.ascontiguousarray(live_n, np.float32)), W, H,
        _p(np.ascontiguousarray(model_v, np.float32)), _p(np.ascontiguousarray(model_n, np.float32)),
        MW, MH, _p(_pose(pose)), _p(_pose(ref_pose)), _p(A), _p(b), C.byref(r), _p(counts, C.c_int))
    return dict(ok=bool(ok), A=A.reshape(6, 6), b=b, residual=r.value,
                inliers=int(counts[0]), valid_live=int(counts[1]), valid_model=int(counts[2]),
                projected=int(counts[3]), dist_filtered=int(counts[4]), angle_filtered=int(counts[5]))


def icp_build_system_f64(prm, K, live_v, live_n, model_v, model_n, pose, ref_pose):
    """The same association with the per-pixel float terms summed in double."""
    H, W = live_v.shape[:2]
    MH, MW = model_v.shape[:2]
    A = np.zeros(36, np.float64)
    b = np.zeros(6, np.float64)
    counts = np.zeros(6, np.int32)
    lib().orc_icp_build_system_f64(
        C.byref(prm), K, _p(np.ascontiguousarray(live_v, np.float32)),
        _p(np.ascontiguousarray(live_n, np.float32)), W, H,
        _p(np.ascontiguousarray(model_v, np.float32)), _p(np.ascontiguousarray(model_n, np.float32)),
        MW, MH, _p(_pose(pose)), _p(_pose(ref_pose)), _p(A, C.c_double), _p(b, C.c_double),
        _p(counts, C.c_int))
    return dict(A=A.reshape(6, 6), b=b, inliers=int(counts[0]))


def icp_track(prm, K, levels, model_v, model_n, estimate, ref_pose):
    """levels: [(depth, vertices, normals)] x 3 as from frame_pyramid_from_depth."""
    H, W = levels[0][1].shape[:2]
    MH, MW = model_v.shape[:2]
    keep = [np.ascontiguousarray(lv[1], np.float32) for lv in levels] + \
           [np.ascontiguousarray(lv[2], np.float32) for lv in levels]
    PV = (C.POINTER(C.c_float) * 3)(*[_p(a) for a in keep[:3]])
    PN = (C.POINTER(C.c_float) * 3)(*[_p(a) for a in keep[3:]])
    res = IcpResult()
    lib().orc_icp_track(C.byref(prm), K, PV, PN, W, H,
                        _p(np.ascontiguousarray(model_v, np.float32)),
                        _p(np.ascontiguousarray(model_n, np.float32)), MW, MH,
                        _p(_pose(estimate)), _p(_pose(ref_pose)), C.byref(res))
    return res


def classify_tracking(res: IcpResult, prev_pose) -> int:
    return lib().orc_classify_tracking(C.byref(res), _p(_pose(prev_pose)))


class Preprocessor:
    """SignalConditioner CPU path on 640x480 frames (EMA state kept here)."""

    def __init__(self, minimal=False):
        self.minimal = minimal
        self.ema = np.zeros(640 * 480, np.float32)

    def reset_temporal(self):
        self.ema[:] = 0

    def process(self, depth_raw, rgb, min_depth, max_depth):
        d = np.ascontiguousarray(depth_raw, np.uint16).copy()
        c = np.ascontiguousarray(rgb, np.uint8).copy()
        luma = np.zeros(640 * 480, np.float32)
        lib().orc_preprocess(_p(d, C.c_uint16), _p(c, C.c_uint8), _p(self.ema), _p(luma),
                             C.c_float(min_depth), C.c_float(max_depth), int(self.minimal))
        return d.reshape(480, 640), c.reshape(480, 640, 3), luma.reshape(480, 640)


def pre_stage(name, depth, *args):
    d = np.ascontiguousarray(depth, np.uint16).copy()
    f = getattr(lib(), "orc_pre_" + name)
    conv = [_p(a) if isinstance(a, np.ndarray) else C.c_float(a) for a in args]
    f(_p(d, C.c_uint16), *conv)
    return d


def raw_to_meters(raw):
    lib().orc_raw_to_meters.restype = C.c_float
    return lib().orc_raw_to_meters(C.c_uint16(int(raw)))


def cpu_depth_meters(raw, lo, hi):
    lib().orc_cpu_depth_meters.restype = C.c_float
    return lib().orc_cpu_depth_meters(C.c_uint16(int(raw)), C.c_float(lo), C.c_float(hi))


def meters_to_raw(m, lo, hi):
    lib().orc_meters_to_raw.restype = C.c_uint16
    return lib().orc_meters_to_raw(C.c_float(m), C.c_float(lo), C.c_float(hi))


def predict(cur, last):
    out = np.zeros(16, np.float32)
    lib().orc_predict(_p(_pose(cur)), _p(_pose(last)), _p(out))
    return out.reshape(4, 4)


class Lockstep:
    """The CPU pipeline in lockstep, as the reference's offline replay drives its
    tracking and integration workers (src/app/PipelineController.cpp:1003-1406,
    1624-1905): frame 0 at identity; constant-velocity prediction; ICP against
    the last raycast model (ref = model pose); a Failed grade retries from the
    previous pose; Good frames are integrated and the model is raycast at the
    new pose; Poor frames move the pose only; Failed keeps it.

    depth is uint16 mm (input_is_mm) or Kinect raw codes (preprocessed with rgb).
    Stage wall times (s) accumulate in self.times.
    """

    def __init__(self, vol: dict, K=(525.0, 525.0, 319.5, 239.5), W=640, H=480, min_depth=0.3, max_depth=2.5,
                 icp=None, input_is_mm=True, minimal=False, fold_threads=1):
        import time
        self._clock = time.perf_counter
        prm = dict(vol)
        prm.pop("format", None)
        self.vol = Volume(tsdf_params(**prm, min_depth=min_depth, max_depth=max_depth))
        self.K = intr(*K)
        self.W, self.H = W, H
        self.lo, self.hi = min_depth, max_depth
        self.icp = icp or icp_params(fold_threads=fold_threads)
        self.input_is_mm = input_is_mm
        self.pre = None if input_is_mm else Preprocessor(minimal=minimal)
        self.cur = np.eye(4, dtype=np.float32)
        self.last = np.eye(4, dtype=np.float32)
        self.model = None
        self.model_pose = np.eye(4, dtype=np.float32)
        self.frames = 0
        self.times = dict(preprocess=0.0, frame=0.0, track=0.0, integrate=0.0, raycast=0.0)

    def depth_meters(self, depth, rgb=None):
        if self.input_is_mm:
            m = depth.astype(np.float32) * np.float32(0.001)
            return np.where(np.isfinite(m) & (m >= np.float32(self.lo)) & (m <= np.float32(self.hi)), m,
                            np.float32(0)).astype(np.float32)
        d, _, _ = self.pre.process(depth, rgb, self.lo, self.hi)
        return build_frame_raw(d, self.K, self.lo, self.hi)[0]

    def process(self, depth, rgb=None) -> dict:
        t0 = self._clock()
        dm = self.depth_meters(depth, rgb)
        t1 = self._clock()
        levels = frame_pyramid_from_depth(dm, self.K)
        t2 = self._clock()
        quality, res = -1, None
        if self.frames == 0:
            self.cur = np.eye(4, dtype=np.float32)
            gate = True
        else:
            prev = self.cur.copy()
            pred = predict(self.cur, self.last)
            self.last = self.cur.copy()
            mv, mn = self.model
            res = icp_track(self.icp, self.K, levels, mv, mn, pred, self.model_pose)
            if classify_tracking(res, prev) == 2:
                res = icp_track(self.icp, self.K, levels, mv, mn, prev, self.model_pose)
            quality = classify_tracking(res, prev)
            if quality != 2:
                self.cur = np.array(res.pose, np.float32).reshape(4, 4)
            gate = quality == 0
        t3 = self._clock()
        if gate:
            self.vol.integrate(dm, self.cur, self.K, self.W, self.H, self.lo, self.hi)
        t4 = self._clock()
        if gate:
            r = self.vol.raycast(self.cur, self.K, self.W, self.H)
            self.model = (r["vertices"], r["normals"])
            self.model_pose = self.cur.copy()
        t5 = self._clock()
        for k, a, b in (("preprocess", t0, t1), ("frame", t1, t2), ("track", t2, t3), ("integrate", t3, t4),
                        ("raycast", t4, t5)):
            self.times[k] += b - a
        self.frames += 1
        return dict(pose=self.cur.copy(), quality=quality, integrated=bool(gate),
                    icp=None if res is None else res.as_dict())


class PrecisionVolume(Volume):
    """FP16-storage emulation (half_storage 1: half RN; 2: half plus the 9-bit
    residual of the FP16R format; 0/False: FP32), plus the FP64 running average
    of the same updates in `tsdf64`."""

    def __init__(self, p: TsdfParams, half_storage, fp64: bool = True):
        super().__init__(p)
        self.half = int(half_storage)
        self.tsdf64 = np.ones(p.res ** 3, np.float64) if fp64 else None

    def integrate(self, depth_m, pose, K, W, H, min_depth, max_depth, rgb=None):
        depth_m = np.ascontiguousarray(depth_m, np.float32)
        lib().orc_tsdf_integrate_prec(C.byref(self.p), _p(self.tsdf), _p(self.weight), _p(self.tsdf64, C.c_double),
                                      _p(depth_m), _p(_pose(pose)), K, int(W), int(H), C.c_float(min_depth),
                                      C.c_float(max_depth), int(self.half))


def depth_adjoint_f(prm, tsdf, weight, pose, K, W, H, depth_obs=None, huber_delta=0.01, grad_tsdf=False,
                    jac=False):
    """Depth render + Huber loss + adjoint on the reference's float march, the
    adjoint evaluated in double (differentiation form; test infrastructure)."""
    loss = C.c_double(0.0)
    g = np.zeros(6, np.float64)
    gv = np.zeros(tsdf.size, np.float64) if grad_tsdf else None
    d = np.zeros(W * H, np.float64)
    J = np.zeros(W * H * 6, np.float64) if jac else None
    nv = C.c_int(0)
    obs = None if depth_obs is None else np.ascontiguousarray(depth_obs, np.float32)
    lib().orc_depth_adjoint_f(C.byref(prm), _p(np.ascontiguousarray(tsdf, np.float32)),
                              _p(np.ascontiguousarray(weight, np.float32)), _p(_pose(pose)), K, int(W), int(H),
                              _p(obs), C.c_double(huber_delta), C.byref(loss), _p(g, C.c_double),
                              _p(gv, C.c_double), _p(d, C.c_double), _p(J, C.c_double), C.byref(nv))
    return dict(loss=loss.value, grad_xi=g, grad_tsdf=gv, depth=d.reshape(H, W),
                jac=None if J is None else J.reshape(H, W, 6), n_valid=nv.value)


def depth_loss_d(prm, tsdf64, weight, pose, xi, K, W, H, depth_obs=None, huber_delta=0.01, grads=False,
                 grad_tsdf=False, jac=False):
    """The same in double at pose * Exp(xi): the finite-difference reference."""
    loss = C.c_double(0.0)
    g = np.zeros(6, np.float64) if grads else None
    gv = np.zeros(tsdf64.size, np.float64) if grad_tsdf else None
    d = np.zeros(W * H, np.float64)
    J = np.zeros(W * H * 6, np.float64) if jac else None
    nv = C.c_int(0)
    obs = None if depth_obs is None else np.ascontiguousarray(depth_obs, np.float32)
    P = np.ascontiguousarray(np.asarray(pose, np.float64).reshape(16))
    x = np.ascontiguousarray(np.asarray(xi, np.float64).reshape(6))
    lib().orc_depth_loss_d(C.byref(prm), _p(np.ascontiguousarray(tsdf64, np.float64), C.c_double),
                           _p(np.ascontiguousarray(weight, np.float32)), _p(P, C.c_double), _p(x, C.c_double), K,
                           int(W), int(H), _p(obs), C.c_double(huber_delta), C.byref(loss), _p(g, C.c_double),
                           _p(gv, C.c_double), _p(d, C.c_double), _p(J, C.c_double), C.byref(nv))
    return dict(loss=loss.value, grad_xi=g, grad_tsdf=gv, depth=d.reshape(H, W),
                jac=None if J is None else J.reshape(H, W, 6), n_valid=nv.value)
