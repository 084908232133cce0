"""Oracle (test infrastructure only): ctypes binding of oracle/_ref/libazu_ref.so,
the reference's OWN hot-path sources (TSDFVolume, ICPTracker, FrameData,
MarchingCubes, SignalConditioner) compiled unmodified against the project's
Eigen-API shim by oracle/ref.mk. Used by tests/ to pin the CPU restatement
(oracle.py) to the reference's code, bit for bit where the reference is
deterministic. It exists only where the reference checkout does (it is built
from the reference's sources in place); callers skip when it is absent.

Same conventions as oracle.py: numpy arrays, row-major (4, 4) float32 poses,
float3 maps, separate tsdf / weight (/ colour) arrays.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libazu_ref.so")
REF_ENV = "AZU_REFERENCE_DIR"


def reference_dir() -> str | None:
    """The reference checkout to build from: $AZU_REFERENCE_DIR, else the one
    next to this build (absent on machines that only run the built library)."""
    d = os.environ.get(REF_ENV) or os.path.join(os.path.sep, "root", "reference")
    return d if os.path.isfile(os.path.join(d, "src", "tsdf", "TSDFVolume.cpp")) else None


def build(force: bool = False) -> str | None:
    """Builds libazu_ref.so when the reference checkout is present; returns
    its path, or None when neither the library nor the sources exist."""
    ref = reference_dir()
    if ref is not None and (force or not os.path.exists(LIB_PATH) or _stale(ref)):
        subprocess.run(["make", "-s", "-j8", "-C", HERE, "-f", "ref.mk", "REF=" + ref], check=True)
    return LIB_PATH if os.path.exists(LIB_PATH) else None


def _stale(ref: str) -> bool:
    t = os.path.getmtime(LIB_PATH)
    mine = [os.path.join(HERE, f) for f in ("ref_capi.cpp", "ref.mk", "orc_linalg.h", "orc_math.h")]
    for root, _, files in os.walk(os.path.join(HERE, "eigen_shim")):
        mine += [os.path.join(root, f) for f in files]
    return any(os.path.getmtime(f) > t for f in mine)


def available() -> bool:
    try:
        return build() is not None
    except (OSError, subprocess.CalledProcessError):
        return False


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build()
        if path is None:
            raise RuntimeError("the reference build (oracle/_ref) is not available here")
        _lib = C.CDLL(path)
        _lib.ref_volume_create.restype = C.c_void_p
        _lib.ref_conditioner_create.restype = C.c_void_p
        _lib.ref_volume_point_cloud.restype = C.c_int64
        for f in ("ref_volume_destroy", "ref_volume_set_params", "ref_volume_load", "ref_volume_store", "ref_volume_integrate",
                  "ref_volume_raycast", "ref_volume_point_cloud", "ref_volume_mesh", "ref_conditioner_destroy",
                  "ref_conditioner_process"):
            getattr(_lib, f).argtypes = None
    return _lib


_p = O._p
_pose = O._pose


def set_threads(n: int):
    lib().ref_set_threads(int(n))


class Volume:
    """tsdf::TSDFVolume of the reference, with the restatement's array view."""

    def __init__(self, p: O.TsdfParams):
        self.p = p
        self.h = C.c_void_p(lib().ref_volume_create(C.byref(p)))
        n = p.res ** 3
        self.n = n

    def close(self):
        if self.h:
            lib().ref_volume_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, p: O.TsdfParams):
        lib().ref_volume_set_params(self.h, C.byref(p))
        self.p = p
        self.n = p.res ** 3

    def load(self, tsdf, weight, color=None):
        lib().ref_volume_load(self.h, _p(np.ascontiguousarray(tsdf, np.float32)),
                              _p(np.ascontiguousarray(weight, np.float32)),
                              None if color is None else _p(np.ascontiguousarray(color, np.float32)))

    def arrays(self, color=False):
        t = np.empty(self.n, np.float32)
        w = np.empty(self.n, np.float32)
        c = np.empty(3 * self.n, np.float32) if color else None
        lib().ref_volume_store(self.h, _p(t), _p(w), _p(c))
        return (t, w, c) if color else (t, w)

    def integrate(self, depth_m, pose, K, W, H, min_depth, max_depth, rgb=None):
        nobs = C.c_int64(0)
        d = np.ascontiguousarray(depth_m, np.float32)
        r = None if rgb is None else np.ascontiguousarray(rgb, np.uint8)
        lib().ref_volume_integrate(self.h, _p(d), _p(r, C.c_uint8), _p(_pose(pose)), K, int(W), int(H),
                                   C.c_float(min_depth), C.c_float(max_depth), C.byref(nobs))
        return dict(newly_observed=int(nobs.value))

    def raycast(self, pose, K, W, H, colors=False):
        v = np.zeros(H * W * 3, np.float32)
        n = np.zeros(H * W * 3, np.float32)
        c = np.zeros(H * W * 3, np.uint8) if colors else None
        lib().ref_volume_raycast(self.h, _p(_pose(pose)), K, int(W), int(H), _p(v), _p(n), _p(c, C.c_uint8))
        out = dict(vertices=v.reshape(H, W, 3), normals=n.reshape(H, W, 3))
        if colors:
            out["colors"] = c.reshape(H, W, 3)
        return out

    def mesh(self, max_triangles=2_000_000):
        info = O.MeshInfo()
        lib().ref_volume_mesh(self.h, C.c_int64(max_triangles), C.byref(info), None, None, None, None)
        nv, ni = info.n_vertices, info.n_indices
        pos = np.empty(3 * nv, np.float32)
        nrm = np.empty(3 * nv, np.float32)
        col = np.empty(3 * nv, np.uint8)
        idx = np.empty(ni, np.uint32)
        lib().ref_volume_mesh(self.h, C.c_int64(max_triangles), C.byref(info), _p(pos), _p(nrm),
                              _p(col, C.c_uint8), _p(idx, C.c_uint32))
        return dict(positions=pos.reshape(-1, 3), normals=nrm.reshape(-1, 3), colors=col.reshape(-1, 3),
                    indices=idx, truncated=bool(info.truncated))

    def point_cloud(self):
        n = lib().ref_volume_point_cloud(self.h, None, None)
        pts = np.empty(3 * n, np.float32)
        cols = np.empty(3 * n, np.uint8)
        lib().ref_volume_point_cloud(self.h, _p(pts), _p(cols, C.c_uint8))
        return pts.reshape(-1, 3), cols.reshape(-1, 3)


def build_frame(raw, K, min_depth, max_depth):
    """sensor::buildFrameData on 640x480 raw codes: (depth_m, vertices, normals)."""
    raw = np.ascontiguousarray(raw, np.uint16)
    d = np.empty(640 * 480, np.float32)
    v = np.empty(640 * 480 * 3, np.float32)
    n = np.empty(640 * 480 * 3, np.float32)
    lib().ref_build_frame(_p(raw, C.c_uint16), K, C.c_float(min_depth), C.c_float(max_depth), _p(d), _p(v), _p(n))
    return d.reshape(480, 640), v.reshape(480, 640, 3), n.reshape(480, 640, 3)


def frame_pyramid(depth_m, vertices, K):
    """computeNormals + buildFramePyramid from level-0 depth and vertices:
    [(depth, vertices, normals)] for 640x480, 320x240, 160x120."""
    tot = 640 * 480 + 320 * 240 + 160 * 120
    d = np.empty(tot, np.float32)
    v = np.empty(3 * tot, np.float32)
    n = np.empty(3 * tot, np.float32)
    lib().ref_frame_pyramid(_p(np.ascontiguousarray(depth_m, np.float32)),
                            _p(np.ascontiguousarray(vertices, np.float32)), K, _p(d), _p(v), _p(n))
    out, off = [], 0
    for w, h in ((640, 480), (320, 240), (160, 120)):
        m = w * h
        out.append((d[off:off + m].reshape(h, w), v[3 * off:3 * (off + m)].reshape(h, w, 3),
                    n[3 * off:3 * (off + m)].reshape(h, w, 3)))
        off += m
    return out


def icp_build_system(prm, K, live_v, live_n, W, H, model_v, model_n, MW, MH, pose, ref_pose):
    A = np.zeros(36, np.float32)
    b = np.zeros(6, np.float32)
    r = C.c_float(0)
    cnt = np.zeros(6, np.int32)
    ok = lib().ref_icp_build_system(C.byref(prm), K, _p(np.ascontiguousarray(live_v, np.float32)),
                                    _p(np.ascontiguousarray(live_n, np.float32)), int(W), int(H),
                                    _p(np.ascontiguousarray(model_v, np.float32)),
                                    _p(np.ascontiguousarray(model_n, np.float32)), int(MW), int(MH),
                                    _p(_pose(pose)), _p(_pose(ref_pose)), _p(A), _p(b), C.byref(r),
                                    _p(cnt, C.c_int))
    return dict(ok=bool(ok), A=A.reshape(6, 6), b=b, residual=r.value, counts=cnt)


def icp_track(prm, K, pyramid, model_v, model_n, MW, MH, estimate, ref_pose, W=640, H=480):
    """ICPTracker::track; pyramid = [(vertices, normals)] per level."""
    keep = [(np.ascontiguousarray(v, np.float32), np.ascontiguousarray(n, np.float32)) for v, n in pyramid]
    lv = (C.POINTER(C.c_float) * 3)(*[_p(v) for v, _ in keep])
    ln = (C.POINTER(C.c_float) * 3)(*[_p(n) for _, n in keep])
    out = O.IcpResult()
    lib().ref_icp_track(C.byref(prm), K, lv, ln, int(W), int(H), _p(np.ascontiguousarray(model_v, np.float32)),
                        _p(np.ascontiguousarray(model_n, np.float32)), int(MW), int(MH), _p(_pose(estimate)),
                        _p(_pose(ref_pose)), C.byref(out))
    return out


def classify_tracking(result: O.IcpResult, prev_pose) -> int:
    return lib().ref_classify_tracking(C.byref(result), _p(_pose(prev_pose)))


class Conditioner:
    """sensor::SignalConditioner (CPU) of the reference: process() in place."""

    def __init__(self, minimal=False):
        self.h = C.c_void_p(lib().ref_conditioner_create(int(bool(minimal))))

    def process(self, depth, rgb, min_depth, max_depth):
        d = np.ascontiguousarray(depth, np.uint16).copy()
        c = np.ascontiguousarray(rgb, np.uint8).copy()
        lib().ref_conditioner_process(self.h, _p(d, C.c_uint16), _p(c, C.c_uint8), C.c_float(min_depth),
                                      C.c_float(max_depth))
        return d, c

    def close(self):
        if self.h:
            lib().ref_conditioner_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _mesh_args(positions, indices, normals, colors):
    pos = np.ascontiguousarray(positions, np.float32)
    idx = np.ascontiguousarray(indices, np.uint32)
    nrm = None if normals is None else np.ascontiguousarray(normals, np.float32)
    col = None if colors is None else np.ascontiguousarray(colors, np.uint8)
    keep = (pos, idx, nrm, col)
    args = [_p(pos), None if nrm is None else _p(nrm), None if col is None else col.ctypes.data_as(C.c_void_p),
            C.c_int64(len(pos)), idx.ctypes.data_as(C.c_void_p), C.c_int64(len(idx))]
    return keep, args


def export_ply(path, positions, indices, normals=None, colors=None, binary=True) -> bool:
    """PLYExporter::writeBinary / writeASCII of the reference."""
    keep, args = _mesh_args(positions, indices, normals, colors)
    f = lib().ref_export_ply
    f.restype = C.c_int
    return bool(f(*args, str(path).encode(), int(binary)))


def export_glb(path, positions, indices, normals=None, colors=None) -> bool:
    """GLBExporter::write of the reference."""
    keep, args = _mesh_args(positions, indices, normals, colors)
    f = lib().ref_export_glb
    f.restype = C.c_int
    return bool(f(*args, str(path).encode()))


def sensor_pairing(events):
    """KinectSensor's depth-led pairing of (kind, ticks) samples, kind 'd' or
    'r' (other kinds are skipped). Returns [(depth ticks, rgb ticks or None)]
    in publication order."""
    ev = [(0 if k == "d" else 1, int(t) % (1 << 32)) for k, t in events if k in ("d", "r")]
    kinds = np.array([e[0] for e in ev], np.int32)
    ticks = np.array([e[1] for e in ev], np.uint32)
    cap = max(1, len(ev))
    d = np.zeros(cap, np.int64)
    r = np.zeros(cap, np.int64)
    f = lib().ref_sensor_pairing
    f.restype = C.c_int
    n = f(kinds.ctypes.data_as(C.c_void_p), ticks.ctypes.data_as(C.c_void_p), len(ev), d.ctypes.data_as(C.c_void_p),
          r.ctypes.data_as(C.c_void_p), cap)
    return [(int(d[k]), None if r[k] < 0 else int(r[k])) for k in range(min(n, cap))]
