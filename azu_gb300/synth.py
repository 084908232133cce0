"""Seeded synthetic KinectFusion sequences (the benchmark and parity inputs).

Five configurations of depth-only 640x480 sequences rendered from an analytic
scene by libazu_synth.so, with Gaussian noise sigma = 0.0012 z^2 m, millimetre
quantisation and 2 % zero dropout, all from a seed:

  scene      sphere r 0.25 m at (0, 0, 1.5); 0.3 m box rotated 30 deg about y
             at (0.4, -0.1, 1.7); floor plane y = -0.35 (camera axes: y down)
  c1 small   30 frames, yaw 1 deg per frame about the vertical axis through the
             scene centre S = (0, 0, 1.5); 256^3 fp32 over a 2 m cube; trunc 3 vox
  c2 full    300 frames, full 360 deg orbit (1.2 deg per frame), plus 40 seeded
             spheres r in [2, 10] cm inside a 1.6 m cube about S; 512^3 fp32, 2 m
  c3 fp16    the c2 sequence, 1024^3 FP16R tsdf (half + 9-bit residual) + weight
             over a 4 m cube
  c4 batch   16 independent scenes, volumes 128/192/256/384^3, 320x240 or
             640x480, 50-200 frames
  c5 diff    512^3 built from 100 c2 frames; a perturbed render-and-compare pose

The camera orbits S at 1.5 m and always looks at S; the first camera is the
world frame (its pose is the identity), as in the reference pipeline. Volumes
are cubes centred on S. Max weight 64. Depth band [0.3, 2.5] m (the reference
pipeline's default hyperparameters).
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass, field

import numpy as np

from . import _abi

FX, FY, CX, CY = 525.0, 525.0, 319.5, 239.5
W, H = 640, 480
SCENE_CENTER = (0.0, 0.0, 1.5)
ORBIT_RADIUS = 1.5
MIN_DEPTH, MAX_DEPTH = 0.3, 2.5
GREY = 128


class _Sphere(C.Structure):
    _fields_ = [("center", C.c_double * 3), ("radius", C.c_double)]


class _Scene(C.Structure):
    _fields_ = [("n_spheres", C.c_int), ("spheres", C.POINTER(_Sphere)), ("box_center", C.c_double * 3),
                ("box_half", C.c_double), ("box_yaw_deg", C.c_double), ("floor_y", C.c_double),
                ("has_floor", C.c_int)]


class _Noise(C.Structure):
    _fields_ = [("sigma_a", C.c_double), ("dropout", C.c_double), ("seed", C.c_uint64),
                ("frame", C.c_uint64), ("max_range", C.c_double)]


_synth = None


def _lib():
    global _synth
    if _synth is None:
        if not os.path.exists(_abi.SYNTH_PATH):
            from . import build as _b
            _b.build()
        _synth = C.CDLL(_abi.SYNTH_PATH)
        _synth.azu_synth_render.restype = C.c_int
    return _synth


@dataclass
class Scene:
    spheres: list = field(default_factory=list)  # [(cx, cy, cz, r)]
    box_center: tuple = (0.4, -0.1, 1.7)
    box_half: float = 0.15
    box_yaw_deg: float = 30.0
    floor_y: float = -0.35


def base_scene() -> Scene:
    return Scene(spheres=[(0.0, 0.0, 1.5, 0.25)])


def random_spheres(seed: int, n: int = 40, cube: float = 1.6, rmin=0.02, rmax=0.10, keep_clear=1.15):
    """n spheres with uniform centres in a cube of side `cube` about the scene
    centre; a sphere reaching past `keep_clear` m from the orbit axis is redrawn,
    so no surface comes nearer than ~0.35 m to the orbiting camera."""
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n:
        c = np.array(SCENE_CENTER) + rng.uniform(-cube / 2, cube / 2, 3)
        r = rng.uniform(rmin, rmax)
        if math.hypot(c[0] - SCENE_CENTER[0], c[2] - SCENE_CENTER[2]) + r > keep_clear:
            continue
        out.append((float(c[0]), float(c[1]), float(c[2]), float(r)))
    return out


def orbit_pose(theta_rad: float, radius: float = ORBIT_RADIUS, center=SCENE_CENTER) -> np.ndarray:
    """World-from-camera pose on a circle about the vertical axis through
    `center`, looking at it; theta = 0 is the camera at center - (0, 0, radius)
    with the identity rotation."""
    c, s = math.cos(theta_rad), math.sin(theta_rad)
    P = np.eye(4)
    P[:3, :3] = np.array([[c, 0.0, -s], [0.0, 1.0, 0.0], [s, 0.0, c]])
    P[:3, 3] = np.array(center) + radius * np.array([s, 0.0, -c])
    return P


def render(scene: Scene, pose: np.ndarray, seed: int, frame: int, w=W, h=H, fx=FX, fy=FY, cx=CX, cy=CY,
           sigma_a=0.0012, dropout=0.02, max_range=10.0) -> np.ndarray:
    """uint16 depth in millimetres (0 = no measurement)."""
    sph = (_Sphere * max(1, len(scene.spheres)))()
    for i, (x, y, z, r) in enumerate(scene.spheres):
        sph[i].center[:] = [x, y, z]
        sph[i].radius = r
    sc = _Scene(len(scene.spheres), sph, (C.c_double * 3)(*scene.box_center), scene.box_half,
                scene.box_yaw_deg, scene.floor_y, 1)
    nz = _Noise(sigma_a, dropout, seed & 0xFFFFFFFFFFFFFFFF, frame, max_range)
    P = np.ascontiguousarray(pose, np.float64).reshape(16)
    out = np.zeros((h, w), np.uint16)
    rc = _lib().azu_synth_render(C.byref(sc), P.ctypes.data_as(C.POINTER(C.c_double)), C.c_double(fx),
                                 C.c_double(fy), C.c_double(cx), C.c_double(cy), w, h, C.byref(nz),
                                 out.ctypes.data_as(C.POINTER(C.c_uint16)))
    if rc != 0:
        raise RuntimeError("azu_synth_render failed")
    return out


@dataclass
class Sequence:
    name: str
    depth_mm: np.ndarray        # (N, H, W) uint16
    poses: np.ndarray           # (N, 4, 4) float32 ground truth, world = first camera
    volume: dict                # resolution, voxel_size, truncation, max_weight, origin, format
    width: int = W
    height: int = H
    fx: float = FX
    fy: float = FY
    cx: float = CX
    cy: float = CY
    min_depth: float = MIN_DEPTH
    max_depth: float = MAX_DEPTH


def _volume(res, side, fmt=0, center=SCENE_CENTER, max_weight=64.0):
    vs = side / res
    return dict(resolution=res, voxel_size=vs, truncation=3.0 * vs, max_weight=max_weight,
                origin=[center[0] - side / 2, center[1] - side / 2, center[2] - side / 2], format=fmt)


def sequence(name: str, seed: int = 1234, frames: int | None = None) -> Sequence:
    if name == "c1":
        scene, n, step, vol = base_scene(), 30, 1.0, _volume(256, 2.0)
    elif name in ("c2", "c3", "c5"):
        scene = base_scene()
        scene.spheres += random_spheres(seed + 1)
        n, step = 300, 360.0 / 300
        vol = _volume(1024, 4.0, fmt=2) if name == "c3" else _volume(512, 2.0)
        if name == "c5":
            n = 100
    else:
        raise ValueError(name)
    if frames is not None:
        n = min(n, frames)
    poses = np.stack([orbit_pose(math.radians(step * k)) for k in range(n)])
    world0 = np.linalg.inv(poses[0])
    depth = np.stack([render(scene, poses[k], seed, k) for k in range(n)])
    rel = np.stack([world0 @ p for p in poses]).astype(np.float32)
    return Sequence(name, depth, rel, vol)


def batch_scenes(seed: int = 99, n_scenes: int = 16, frames_scale: float = 1.0):
    """c4: independent scenes of uneven volume, image size and length."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_scenes):
        res = int(rng.choice([128, 192, 256, 384]))
        small = bool(rng.integers(0, 2))
        w, h = (320, 240) if small else (640, 480)
        n = max(2, int(int(rng.integers(50, 201)) * frames_scale))
        scene = base_scene()
        scene.spheres += random_spheres(seed * 100 + i, n=int(rng.integers(5, 41)))
        step = float(rng.uniform(0.5, 1.5))
        s = w / 640.0
        fx, fy, cx, cy = FX * s, FY * s, (CX + 0.5) * s - 0.5, (CY + 0.5) * s - 0.5
        poses = np.stack([orbit_pose(math.radians(step * k)) for k in range(n)])
        world0 = np.linalg.inv(poses[0])
        depth = np.stack([render(scene, poses[k], seed + i, k, w=w, h=h, fx=fx, fy=fy, cx=cx, cy=cy)
                          for k in range(n)])
        rel = np.stack([world0 @ p for p in poses]).astype(np.float32)
        out.append(Sequence(f"c4_{i}", depth, rel, _volume(res, 2.0), w, h, fx, fy, cx, cy))
    return out


# ---- depth domains -----------------------------------------------------------
KCURVE_A = np.float32(-0.0030711016)
KCURVE_B = np.float32(3.3309495161)


def mm_to_meters(depth_mm: np.ndarray) -> np.ndarray:
    """depth_m = float(mm) * 0.001f (0 stays 0)."""
    return depth_mm.astype(np.float32) * np.float32(0.001)


def encode_raw(depth_mm: np.ndarray, min_depth=MIN_DEPTH, max_depth=MAX_DEPTH) -> np.ndarray:
    """Kinect raw codes of mm depth via the reference's band-rejecting encoder
    (cpuDepthMetersToRaw, include/sensor/DepthValidity.h:100-109), float32
    arithmetic, std::lround rounding."""
    return encode_raw_m(mm_to_meters(depth_mm), min_depth, max_depth)


def encode_raw_m(m: np.ndarray, min_depth=MIN_DEPTH, max_depth=MAX_DEPTH) -> np.ndarray:
    """The same encoder from depth in metres (0 or out of band -> code 0)."""
    m = np.asarray(m, np.float32)
    lo, hi = np.float32(min_depth), np.float32(max_depth)
    ok = np.isfinite(m) & (m >= lo) & (m <= hi)
    with np.errstate(divide="ignore", invalid="ignore"):
        raw = (np.float32(1.0) / m - KCURVE_B) / KCURVE_A
    r64 = raw.astype(np.float64)
    code = np.where(r64 >= 0, np.floor(r64 + 0.5), -np.floor(-r64 + 0.5))
    ok &= np.isfinite(raw) & (code >= 1) & (code <= 2046)
    return np.where(ok, code, 0).astype(np.uint16)


def grey_rgb(w=W, h=H) -> np.ndarray:
    return np.full((h, w, 3), GREY, np.uint8)


def room_depth(pose, w=W, h=H, fx=FX, fy=FY, cx=CX, cy=CY) -> np.ndarray:
    """Depth in metres (0 = miss) of the room scene of the reference's contract
    tests (a room interior with a box and a sphere, sphere-traced), for the
    parity tests of those contracts."""
    P = np.ascontiguousarray(np.asarray(pose, np.float32).reshape(16))
    out = np.zeros((h, w), np.float32)
    lib = _lib()
    lib.azu_synth_room_depth.argtypes = [C.POINTER(C.c_float), C.c_float, C.c_float, C.c_float, C.c_float, C.c_int,
                                         C.c_int, C.POINTER(C.c_float)]
    rc = lib.azu_synth_room_depth(P.ctypes.data_as(C.POINTER(C.c_float)), fx, fy, cx, cy, w, h,
                                  out.ctypes.data_as(C.POINTER(C.c_float)))
    if rc != 0:
        raise RuntimeError("azu_synth_room_depth failed")
    return out


def axis_angle_pose(axis_angle, t) -> np.ndarray:
    """World-from-camera pose from a rotation vector (rad) and a translation,
    float32 (the contract tests' makePose)."""
    a = np.asarray(axis_angle, np.float64)
    T = np.eye(4)
    ang = float(np.linalg.norm(a))
    if ang > 0:
        k = a / ang
        Kx = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
        T[:3, :3] = np.eye(3) + math.sin(ang) * Kx + (1 - math.cos(ang)) * Kx @ Kx
    T[:3, 3] = t
    return T.astype(np.float32)
