"""Known-answer fixtures of the reference's CPU contract tests, rebuilt from
their definitions (expected values are the contracts' hand-derived numbers).

Each builder returns plain numpy data, so the same fixture drives the oracle
(CPU tests) and the CUDA backend (gpu tests).
"""
from __future__ import annotations

import math

import numpy as np

W0, H0 = 640, 480
FX, FY, CX, CY = 525.0, 525.0, 319.5, 239.5

# ---- tests/tsdf_raycast_contract.cpp:70-152 ---------------------------------
RC_RES, RC_VS, RC_TRUNC, RC_ORIGIN_XY = 32, 0.04, 0.025, -0.64
RC_MIN, RC_MAX = 0.12, 0.90
RC_IMG, RC_F, RC_C = 8, 4.0, 3.0
WALL_Z, WALL_HIT_Z = 0.38, 0.38
SLAB_A, SLAB_B, SLAB_TAU = 0.39, 0.41, 0.02
SLAB_FRONT_Z = 0.36 + 0.04 * (1.0 / 1.5)


def _clamp1(v):
    return np.float32(-1.0) if v < -1.0 else (np.float32(1.0) if v > 1.0 else np.float32(v))


def wall_field(z):
    z = np.float32(z)
    return _clamp1((np.float32(WALL_Z) - z) / np.float32(RC_VS))


def slab_field(z):
    z = np.float32(z)
    a, b = np.float32(SLAB_A), np.float32(SLAB_B)
    inside = a <= z <= b
    sdf = -min(z - a, b - z) if inside else (a - z if z < a else z - b)
    return _clamp1(np.float32(sdf) / np.float32(SLAB_TAU))


def layer_color(k):
    return (31 + 7 * (k % 29), 200 - k, 17 + 3 * (k % 11))


def raycast_volume(field):
    """res^3 lattice with tsdf = field(z * vs), weight 4, per-layer colour."""
    n = RC_RES
    tsdf = np.empty((n, n, n), np.float32)
    col = np.empty((n, n, n, 3), np.float32)
    for z in range(n):
        tsdf[z] = field(np.float32(RC_VS) * np.float32(z))
        c = layer_color(z)
        col[z] = [np.float32(c[0]) / np.float32(255), np.float32(c[1]) / np.float32(255),
                  np.float32(c[2]) / np.float32(255)]
    weight = np.full((n, n, n), 4.0, np.float32)
    return tsdf.reshape(-1), weight.reshape(-1), col.reshape(-1)


def raycast_params(min_depth=RC_MIN, max_depth=RC_MAX):
    return dict(resolution=RC_RES, voxel_size=RC_VS, truncation=RC_TRUNC, max_weight=128.0,
                origin=(RC_ORIGIN_XY, RC_ORIGIN_XY, 0.0), min_depth=min_depth, max_depth=max_depth)


# ---- tests/tsdf_integration_race_contract.cpp:251-323 -----------------------
HF_VS, HF_TRUNC, HF_RES = 0.01, 0.03, 64
HF_FRAMES = [(0.5015, 200, 100, 40), (0.5065, 60, 180, 250)]


def hand_fold_frames():
    """Two 4x4 frames: one valid pixel on the optical axis (cx = cy = 2)."""
    out = []
    for D, R, G, B in HF_FRAMES:
        depth = np.zeros((4, 4), np.float32)
        depth[2, 2] = np.float32(D)
        rgb = np.empty((4, 4, 3), np.uint8)
        rgb[...] = (R, G, B)
        out.append((depth, rgb))
    return out


def hand_fold_expected(k):
    """Double fold of axis voxel k over both frames (max weight 128)."""
    tsdf, w, r = 1.0, 0.0, 128.0 / 255.0
    for D, R, _, _ in HF_FRAMES:
        sdf = float(np.float32(D)) - float(np.float32(k) * np.float32(HF_VS))
        if sdf < -HF_TRUNC:
            continue
        tn = min(1.0, sdf / HF_TRUNC)
        tsdf = (tsdf * w + tn) / (w + 1.0)
        if abs(sdf) < 0.5 * HF_TRUNC:
            r = (r * w + R / 255.0) / (w + 1.0)
        w = min(w + 1.0, 128.0)
    return tsdf, w, r


# ---- tests/tsdf_integration_race_contract.cpp:130-175 (wall scenario A) ----
def wall_scene():
    W, H = 40, 30
    depth = np.full((H, W), 0.5, np.float32)
    rgb = np.empty((H, W, 3), np.uint8)
    for y in range(H):
        for x in range(W):
            rgb[y, x] = ((x * 7 + y * 3) & 0xFF, (x * 5 + y * 11 + 40) & 0xFF, (x * 13 + y * 2 + 90) & 0xFF)
    p0 = np.eye(4, dtype=np.float32)
    p1 = np.eye(4, dtype=np.float32)
    p1[0, 3] = 0.02
    params = dict(resolution=48, voxel_size=0.02, truncation=0.05, max_weight=128.0,
                  origin=(-0.48, -0.48, 0.05), min_depth=0.3, max_depth=5.0)
    K = (300.0, 300.0, 19.5, 14.5)
    return params, K, W, H, depth, rgb, [p0, p1]


# ---- tests/icp_weighting_contract.cpp:107-152 --------------------------------
def icp_weighting_fixture():
    """Live level-0 and model maps with 10 inliers (err 0.01) and one outlier
    (err 0.08). Expected: t_z = -0.12 / 11.25, error = 0.0038 / 11."""
    lv = np.zeros((H0, W0, 3), np.float32)
    ln = np.zeros((H0, W0, 3), np.float32)
    mv = np.zeros((H0, W0, 3), np.float32)
    mn = np.zeros((H0, W0, 3), np.float32)

    def put(px, py, err):
        z = np.float32(1.0)
        vx = (np.float32(px) - np.float32(CX)) / np.float32(FX) * z
        vy = (np.float32(py) - np.float32(CY)) / np.float32(FY) * z
        lv[py, px] = (vx, vy, z)
        ln[py, px] = (0, 0, 1)
        mv[py, px] = (vx, vy, z - np.float32(err))
        mn[py, px] = (0, 0, 1)

    for k in range(5):
        put(319 - k, 239 - k, 0.01)
        put(320 + k, 240 + k, 0.01)
    put(320, 239, 0.08)
    return lv, ln, mv, mn


ICP_TZ = -0.12 / 11.25
ICP_ERR = 0.0038 / 11.0

# ---- tests/depth_ema_determinism_contract.cpp:84-92 ---------------------------
EMA_WALL1, EMA_WALL2, EMA_CENTRE = 500, 548, 586
EMA_CX, EMA_CY = 320, 240
EMA_EXPECT_WALL, EMA_EXPECT_CENTRE = 534, 575


def ema_frame(wall, centre):
    d = np.full((H0, W0), wall, np.uint16)
    d[EMA_CY, EMA_CX] = centre
    return d


# ---- meshing ------------------------------------------------------------------
def sphere_volume(res=24, vs=0.05, radius=0.37, trunc=0.15, center=None):
    """Signed-distance sphere on a lattice (outside positive), weight 1."""
    c = center if center is not None else (res - 1) * vs / 2.0
    g = np.arange(res, dtype=np.float64) * vs
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    sdf = np.sqrt((x - c) ** 2 + (y - c) ** 2 + (z - c) ** 2) - radius
    tsdf = np.clip(sdf / trunc, -1, 1).astype(np.float32).reshape(-1)
    return tsdf, np.ones_like(tsdf), dict(resolution=res, voxel_size=vs, truncation=trunc, max_weight=64.0,
                                          origin=(0.0, 0.0, 0.0), min_depth=0.3, max_depth=5.0)


def crossing_mask(ci):
    edges = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7)]
    m = 0
    for e, (a, b) in enumerate(edges):
        if ((ci >> a) & 1) != ((ci >> b) & 1):
            m |= 1 << e
    return m


def signed_volume(pos, idx):
    t = idx.reshape(-1, 3)
    a, b, c = pos[t[:, 0]].astype(np.float64), pos[t[:, 1]].astype(np.float64), pos[t[:, 2]].astype(np.float64)
    return float(np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6.0)


def fnv1a(*arrays) -> int:
    h = 0xcbf29ce484222325
    for a in arrays:
        for byte in np.ascontiguousarray(a).view(np.uint8).tobytes():
            h ^= byte
            h = (h * 0x100000001b3) & 0xFFFFFFFFFFFFFFFF
    return h


def rel_pose_error(a, b):
    """(rotation angle rad, translation m) of a^-1 b."""
    d = np.linalg.inv(np.asarray(a, np.float64)) @ np.asarray(b, np.float64)
    c = max(-1.0, min(1.0, (np.trace(d[:3, :3]) - 1.0) * 0.5))
    return math.acos(c), float(np.linalg.norm(d[:3, 3]))


# ---- tests/icp_numeric_policy_contract.cpp:97-140, 226-239 (fixture plumbing) --
# One correspondence = a live level-0 pixel (vertex, normal) and the model pixel
# its vertex projects onto at identity poses; float32 arithmetic in the
# contract's order.
def _f(x):
    return np.float32(x)


def back_project(px, py, z):
    z = _f(z)
    return np.array([(_f(px) - _f(CX)) / _f(FX) * z, (_f(py) - _f(CY)) / _f(FY) * z, z], np.float32)


def projected_pixel(v):
    inv_z = _f(1.0) / _f(v[2])
    mx = int(math.floor(_f(_f(_f(FX) * _f(v[0])) * inv_z + _f(CX)) + _f(0.5)))
    my = int(math.floor(_f(_f(_f(FY) * _f(v[1])) * inv_z + _f(CY)) + _f(0.5)))
    return mx, my


def make_corr(px, py, z, n, axis, offset):
    lv = back_project(px, py, z)
    mv = lv.copy()
    mv[axis] = lv[axis] - _f(offset)
    n = np.asarray(n, np.float32)
    mpx, mpy = projected_pixel(lv)
    return dict(lp=(px, py), mp=(mpx, mpy), lv=lv, ln=n.copy(), mv=mv, mn=n.copy())


def corr_maps(cs):
    """Live level-0 vertex/normal maps and model vertex/normal maps (640x480)."""
    lv = np.zeros((H0, W0, 3), np.float32)
    ln = np.zeros((H0, W0, 3), np.float32)
    mv = np.zeros((H0, W0, 3), np.float32)
    mn = np.zeros((H0, W0, 3), np.float32)
    for c in cs:
        (px, py), (mx, my) = c["lp"], c["mp"]
        lv[py, px], ln[py, px] = c["lv"], c["ln"]
        mv[my, mx], mn[my, mx] = c["mv"], c["mn"]
    return lv, ln, mv, mn


def grid_fixture(x0, x1, y0, y1, z, offset, n=(0.0, 0.0, 1.0)):
    return [make_corr(x, y, z, n, 2, offset) for y in range(y0, y1 + 1) for x in range(x0, x1 + 1)]


# :315-325 two point-symmetric rows, opposite 1 m residuals (rotation cap)
def rotation_leak_fixture(per_row):
    x0 = 320 - per_row // 2
    cs = [make_corr(x0 + i, 450, 2.0, (0, 0, 1), 2, 1.0) for i in range(per_row)]
    cs += [make_corr(x0 + i, 29, 2.0, (0, 0, 1), 2, -1.0) for i in range(per_row)]
    return cs


# :455-461 escalation: six symmetric pairs at 0.01 and one outlier at 0.08
def escalation_fixture():
    cs = []
    for k in range(6):
        cs.append(make_corr(319 - k, 239 - k, 1.0, (0, 0, 1), 2, 0.01))
        cs.append(make_corr(320 + k, 240 + k, 1.0, (0, 0, 1), 2, 0.01))
    cs.append(make_corr(320, 239, 1.0, (0, 0, 1), 2, 0.08))
    return cs


# :476-494 well-conditioned three walls (no escalation)
def three_wall_fixture():
    cs = []
    for x in range(314, 326):
        cs.append(make_corr(x, 150, 1.0, (0, 0, 1), 2, 0.01))
        cs.append(make_corr(x, 329, 1.0, (0, 0, 1), 2, 0.01))
    depths = (1.0, 1.5, 2.0, 2.5)
    for x in range(300, 340):
        for y in range(200, 240):
            cs.append(make_corr(x, y, depths[(x + y) & 3], (1, 0, 0), 0, 0.0))
        for y in range(240, 280):
            cs.append(make_corr(x, y, depths[(2 * x + y) & 3], (0, 1, 0), 0, 0.0))
    return cs


# :541-552 ten clean +z pairs, plus one pixel (340, 260) with a chosen model normal
def model_normal_fixture(extra_normal=None):
    cs = []
    for k in range(5):
        cs.append(make_corr(319 - k, 239 - k, 1.0, (0, 0, 1), 2, 0.01))
        cs.append(make_corr(320 + k, 240 + k, 1.0, (0, 0, 1), 2, 0.01))
    if extra_normal is not None:
        c = make_corr(340, 260, 1.0, (0, 0, 1), 2, 0.01)
        c["mn"] = np.asarray(extra_normal, np.float32)
        cs.append(c)
    return cs


# :637-651 a tangent wall (model normals (1,0,0)) with a chosen live normal
def live_normal_fixture(live_n, offset=0.01, dist_offset=0.0):
    cs = []
    for k in range(5):
        for i in range(2):
            px, py = (320 + k, 240 + k) if i else (319 - k, 239 - k)
            c = make_corr(px, py, 1.0, (1, 0, 0), 0, offset)
            c["ln"] = np.asarray(live_n, np.float32)
            if dist_offset:
                c["mv"][2] = _f(c["mv"][2] + _f(dist_offset))
            cs.append(c)
    return cs


# :731-742 live normals (1,0,0) against model normals (0,0,1): |dot| = 0
def orthogonal_fixture():
    cs = []
    for k in range(5):
        for i in range(2):
            px, py = (320 + k, 240 + k) if i else (319 - k, 239 - k)
            c = make_corr(px, py, 1.0, (0, 0, 1), 2, 0.01)
            c["ln"] = np.array([1, 0, 0], np.float32)
            cs.append(c)
    return cs


# :781-806 a reflected, non-orthonormal estimate and a zero residual
REFLECTED_ESTIMATE = np.diag([-2.0, 1.0, 2.0, 1.0]).astype(np.float32)


def reflection_fixture():
    v_ref = np.array([0, 0, 2], np.float32)
    mp = projected_pixel(v_ref)
    return [dict(lp=(300 + i, 200), mp=mp, lv=np.array([0, 0, 1], np.float32), ln=np.array([0, 0, 1], np.float32),
                 mv=v_ref.copy(), mn=np.array([0, 0, 1], np.float32)) for i in range(12)]


ICP_TOL_MATCH = 1e-7     # the contract's kTolMatch
ICP_HUBER_K = 0.02
ICP_ROW_VY = (450.0 - CY) * 2.0 / FY


# ---- export and sensor-pairing fixtures (pinned to the reference's own writers
# and KinectSensor pairing by tests/golden/make_golden.py) ------------------------
def export_meshes(orc):
    """Meshes for the PLY/GLB writers: the oracle's sphere mesh with normals and
    colours; the same positions and indices alone; and an unwelded copy
    (every vertex twice) with a zero normal, a -0 coordinate and a saturated
    colour, which exercises the GLB writer's welding and normal fallback."""
    t, w, prm = sphere_volume()
    o = orc.Volume(orc.tsdf_params(**prm))
    o.tsdf[:] = t
    o.weight[:] = w
    m = o.extract_mesh()
    full = dict(positions=m["positions"], normals=m["normals"], colors=m["colors"], indices=m["indices"])
    bare = dict(positions=m["positions"], normals=None, colors=None, indices=m["indices"])
    n = len(m["positions"])
    pos = np.concatenate([m["positions"], m["positions"]]).astype(np.float32)
    nrm = np.concatenate([m["normals"], m["normals"]]).astype(np.float32)
    col = np.concatenate([m["colors"], m["colors"]]).astype(np.uint8)
    idx = np.concatenate([m["indices"], m["indices"] + n]).astype(np.uint32)
    col[0] = (0, 10, 255)
    nrm[int(idx[5])] = 0.0
    pos[int(idx[7]), 1] = -0.0
    dup = dict(positions=pos, normals=nrm, colors=col, indices=idx)
    return {"sphere": full, "sphere_bare": bare, "sphere_unwelded": dup}


PAIR_MS = 60000  # 60 MHz device ticks per millisecond (KinectSensor.h:85)


def pairing_events(name):
    """(kind, 60 MHz ticks) sample sequences for the depth-led pairing:
    'hand'     the hand-derived sequence of tests/test_ingest.py (skew limit
               edges, a late RGB, RGB ahead of depth, a counter wrap)
    'jitter'   depth and RGB samples at 30 Hz with seeded phase jitter,
               dropped samples and reordering across streams, through a wrap
               of the 32-bit counter"""
    ms = PAIR_MS
    if name == "hand":
        wrap_r = (1 << 32) - 3 * ms
        ev = [("r", 0.0), ("d", 5.0), ("d", 38.0), ("r", 40.0), ("r", 60.0), ("d", 100.0), ("d", 133.0),
              ("r", 140.0), ("r", 200.0), ("d", 170.0), ("d", 205.0), ("d", 300.0), ("r", wrap_r),
              ("d", 2 * ms)]
        return [(k, int(t * ms) % (1 << 32) if isinstance(t, float) else int(t) % (1 << 32)) for k, t in ev]
    rng = np.random.default_rng(77)
    t0 = (1 << 32) - 60 * 33 * ms  # the counter wraps about 60 frames in
    ev = []
    for i in range(150):
        td = t0 + int((33.37 * i + rng.normal(0, 1.5)) * ms)
        tr = t0 + int((33.37 * i + 9.0 + rng.normal(0, 6.0)) * ms)
        if rng.random() > 0.06:
            ev.append(("d", td % (1 << 32), td))
        if rng.random() > 0.1:
            ev.append(("r", tr % (1 << 32), tr + int(rng.normal(0, 4.0) * ms)))  # delivered out of order
    ev.sort(key=lambda e: e[2])
    return [(k, t) for k, t, _ in ev]
