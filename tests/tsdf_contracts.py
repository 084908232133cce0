"""Scenarios of the reference's TSDF contracts with their own expectations,
written against a backend so the CPU restatement and the CUDA path run the
same checks:

  tests/tsdf_integration_min_depth_contract.cpp   A-D: the per-pixel depth
      band (0.50125 m rejected at min 0.60, accepted at 0.10 and 0.50, the
      fold's surface voxel tsdf 0.05 and colour, free space tsdf 1), far and
      non-finite depths rejected, a band change clears the volume
  tests/fusion_bias_contract.cpp:95-135   a slanted plane fused 10 times meshes
      with |mean signed error| < 0.5 mm and p95 < 2 mm; after 1, 3 and 70
      frames every observed voxel has weight min(N, max_weight)
  tests/raycast_accuracy_contract.cpp:84-121   the fused plane seen from the
      front: >= 90 % hits, all within 1 mm, normals facing the camera; from
      behind: no hit; at 45 deg: > 1000 hits, <= 0.1 % off by > 2 mm

backend.volume(params, color=False) -> vol with vol.integrate(depth, rgb, pose,
K, W, H, min_d, max_d), vol.arrays() -> (tsdf, weight, color | None),
vol.raycast(pose, K, W, H) -> (vertices, normals), vol.mesh() -> dict,
vol.set_params(params).
"""
import math

import numpy as np

EMPTY_TSDF, EMPTY_WEIGHT = 1.0, 0.0
EMPTY_COLOR = np.float32(128.0) / np.float32(255.0)
I4 = np.eye(4, dtype=np.float32)
FX, FY, CX, CY = 525.0, 525.0, 319.5, 239.5

# ---- tsdf_integration_min_depth_contract.cpp:60-101 -----------------------------
MD_PARAMS = dict(resolution=64, voxel_size=0.01, truncation=0.025, max_weight=128.0, origin=(-0.32, -0.32, 0.0),
                 min_depth=0.3, max_depth=5.0)
MD_DEPTH = 0.50125
MD_K = (500.0, 500.0, 2.0, 2.0)
MD_RGB = (200, 100, 40)


def md_frame(value):
    d = np.zeros((4, 4), np.float32)
    d[2, 2] = np.float32(value)
    rgb = np.empty((4, 4, 3), np.uint8)
    rgb[...] = MD_RGB
    return d, rgb


def _integrate_once(vol, lo, hi, value):
    d, rgb = md_frame(value)
    vol.integrate(d, rgb, I4, MD_K, 4, 4, lo, hi)


def _voxel(arr, x, y, z, res=64):
    return int((z * res + y) * res + x)


def _all_empty(vol):
    t, w, c = vol.arrays()
    return bool(np.all(t == EMPTY_TSDF) and np.all(w == EMPTY_WEIGHT) and (c is None or np.all(c == EMPTY_COLOR)))


def min_depth_gates(backend):
    # A: the band is per pixel
    rej = backend.volume(MD_PARAMS, color=True)
    _integrate_once(rej, 0.60, 3.0, MD_DEPTH)
    assert _all_empty(rej)
    acc = backend.volume(MD_PARAMS, color=True)
    _integrate_once(acc, 0.10, 3.0, MD_DEPTH)
    assert (acc.arrays()[1] > 0).sum() > 0
    # B: the accepted fold, identical at min 0.10 and 0.50
    tight = backend.volume(MD_PARAMS, color=True)
    _integrate_once(tight, 0.50, 3.0, MD_DEPTH)
    want = (MD_DEPTH - 0.50) / 0.025
    arrays = []
    for vol in (acc, tight):
        t, w, c = vol.arrays()
        s50, f47 = _voxel(t, 32, 32, 50), _voxel(t, 32, 32, 47)
        assert w[s50] == 1.0 and abs(float(t[s50]) - want) < 1e-5, (t[s50], want)
        for ch, byte in enumerate(MD_RGB):
            assert abs(float(c[3 * s50 + ch]) - byte / 255.0 / (1.0 + 1e-6)) < 1e-6
            assert min(255, max(0, round(float(c[3 * s50 + ch]) * 255.0))) == byte
        assert w[f47] == 1.0 and t[f47] == 1.0
        assert np.all(c[3 * f47:3 * f47 + 3] == EMPTY_COLOR)
        arrays.append((t, w, c))
    for a, b in zip(arrays[0], arrays[1]):
        assert np.array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))
    # C: far and non-finite depths
    for value, lo, hi in ((MD_DEPTH, 0.1, 0.40), (float("nan"), 0.1, 3.0), (float("inf"), 0.1, 3.0),
                          (-float("inf"), 0.1, 3.0)):
        vol = backend.volume(MD_PARAMS, color=True)
        _integrate_once(vol, lo, hi, value)
        assert _all_empty(vol), value
    inside = backend.volume(MD_PARAMS, color=True)
    _integrate_once(inside, 0.1, 0.51, MD_DEPTH)
    assert (inside.arrays()[1] > 0).sum() > 0
    # D: a depth-band change of the volume parameters clears the volume
    vol = backend.volume(dict(MD_PARAMS, min_depth=0.55, max_depth=2.25), color=True)
    _integrate_once(vol, 0.1, 3.0, MD_DEPTH)
    assert (vol.arrays()[1] > 0).sum() > 0
    vol.set_params(dict(MD_PARAMS, min_depth=0.55, max_depth=2.75))
    assert _all_empty(vol)


# ---- fusion_bias_contract.cpp / raycast_accuracy_contract.cpp: the slanted plane ---
SLOPE, Z0 = 0.2, 1.0
PLANE_PARAMS = dict(resolution=256, voxel_size=0.01, truncation=0.03, max_weight=64.0, origin=(-1.28, -1.28, 0.0),
                    min_depth=0.3, max_depth=3.0)


def plane_depth(accuracy_form=False):
    """The plane's Z-depth per pixel: fusion_bias_contract.cpp:58-66 takes
    a = (u - CX) / FX in float, raycast_accuracy_contract.cpp:98-101 the
    slope product in double."""
    du = np.arange(640, dtype=np.float32) - np.float32(CX)
    if accuracy_form:
        row = (Z0 / (1.0 - SLOPE * du.astype(np.float64) / np.float64(np.float32(FX)))).astype(np.float32)
    else:
        a = (du / np.float32(FX)).astype(np.float64)
        row = (Z0 / (1.0 - SLOPE * a)).astype(np.float32)
    return np.ascontiguousarray(np.broadcast_to(row, (480, 640)))


def plane_distance(p):
    p = np.asarray(p, np.float64)
    return (SLOPE * p[:, 0] - p[:, 2] + Z0) / math.sqrt(1.0 + SLOPE * SLOPE)


def fusion_bias(backend):
    depth = plane_depth()
    K = (FX, FY, CX, CY)
    vol = backend.volume(PLANE_PARAMS)
    for _ in range(10):
        vol.integrate(depth, None, I4, K, 640, 480, 0.3, 3.0)
    m = vol.mesh()
    assert len(m["positions"]) > 10000
    d = plane_distance(m["positions"])
    assert abs(d.mean()) < 0.5e-3, d.mean()
    assert np.sort(np.abs(d))[len(d) * 95 // 100] < 2.0e-3
    for n in (1, 3, 70):
        v = backend.volume(PLANE_PARAMS)
        for _ in range(n):
            v.integrate(depth, None, I4, K, 640, 480, 0.3, 3.0)
        w = v.arrays()[1]
        obs = w[w != 0]
        assert obs.size > 0 and np.all(obs == min(float(n), 64.0)), n


def _look_from(eye, forward):
    z = np.asarray(forward, np.float64)
    z = z / np.linalg.norm(z)
    x = np.cross([0.0, 1.0, 0.0], z)
    x = x / np.linalg.norm(x)
    y = np.cross(z, x)
    T = np.eye(4)
    T[:3, 0], T[:3, 1], T[:3, 2], T[:3, 3] = x, y, z, eye
    return T.astype(np.float32)


def raycast_accuracy(backend):
    depth = plane_depth(accuracy_form=True)
    K = (FX, FY, CX, CY)
    vol = backend.volume(dict(PLANE_PARAMS, max_weight=128.0))
    for _ in range(5):
        vol.integrate(depth, None, I4, K, 640, 480, 0.3, 3.0)
    n_plane = np.array([SLOPE, 0.0, -1.0], np.float32)
    n_plane /= np.linalg.norm(n_plane)

    def cast(pose):
        v, n = vol.raycast(pose, K, 640, 480)
        v, n = v.reshape(-1, 3), n.reshape(-1, 3)
        hit = np.any(v != 0, axis=1)
        d = np.abs(plane_distance(v[hit]))
        return hit.sum(), (d > 1e-3).sum(), (d > 2e-3).sum(), (~((n[hit] @ n_plane) > 0.99)).sum()

    hits, off1, _, bad_n = cast(I4)
    assert hits >= 640 * 480 * 90 // 100 and off1 == 0 and bad_n == 0, (hits, off1, bad_n)
    assert cast(_look_from((0.0, 0.0, 2.0), (0, 0, -1)))[0] == 0
    eye = np.array([-1.0, 0.0, 0.0])
    hits, _, off2, _ = cast(_look_from(eye, np.array([0.0, 0.0, 1.0]) - eye))
    assert hits > 1000 and off2 <= hits // 1000, (hits, off2)


# ---- tsdf_subvoxel_thin_feature_contract.cpp:53-159 ------------------------------
SV_RES, SV_VS, SV_TAU = 32, np.float32(0.04), np.float32(0.02)
SV_NEAR, SV_FAR = 0.12, 0.90


def sv_params(lo=SV_NEAR, hi=SV_FAR):
    return dict(resolution=SV_RES, voxel_size=0.04, truncation=0.025, max_weight=128.0, origin=(-0.64, -0.64, 0.0),
                min_depth=lo, max_depth=hi)


def _signed_dist(z, slabs):
    best_in, best_out, inside = np.float32(0), np.float32(np.inf), False
    for a, b in slabs:
        a, b = np.float32(a), np.float32(b)
        if a <= z <= b:
            inside = True
            best_in = max(best_in, min(z - a, b - z))
        else:
            best_out = min(best_out, a - z if z < a else z - b)
    return -best_in if inside else best_out


def sv_lattice(slabs):
    return np.array([max(np.float32(-1), min(np.float32(1), np.float32(_signed_dist(np.float32(k) * SV_VS, slabs))
                                             / SV_TAU)) for k in range(SV_RES)], np.float32)


def sv_oracle_zero(f):
    for k in range(1, SV_RES):
        prev, cur = f[k - 1], f[k]
        if cur < 0:
            if prev <= 0:
                return np.float32(k - 1) * SV_VS
            return np.float32(np.float32(k - 1) * SV_VS + SV_VS * prev / (prev - cur))
    return float("nan")


def sv_layer(z):
    return 31 + 7 * (z % 29), 200 - z, 17 + 3 * (z % 11)


def sv_cast(backend, slabs, lo, hi):
    f = sv_lattice(slabs)
    n = SV_RES ** 3
    t = np.repeat(f, SV_RES * SV_RES).astype(np.float32)
    col = np.empty((SV_RES, SV_RES * SV_RES, 3), np.float32)
    for z in range(SV_RES):
        col[z] = [np.float32(c) / np.float32(255) for c in sv_layer(z)]
    vol = backend.volume(sv_params(lo, hi), color=True)
    vol.load(t, np.ones(n, np.float32), col.reshape(-1))
    v, nrm, c = vol.raycast(I4, (1.0, 1.0, 0.0, 0.0), 1, 1, colors=True)
    return v.reshape(3), nrm.reshape(3), c.reshape(3)


def _hit(h, want_z, layer):
    v, n, c = h
    assert not (np.all(v == 0) and np.all(n == 0) and np.all(c == 0)), "expected a hit"
    assert abs(float(v[2]) - want_z) < 1e-5 and abs(float(v[0])) < 1e-5 and abs(float(v[1])) < 1e-5, (v, want_z)
    assert tuple(int(x) for x in c) == sv_layer(layer), (c, layer)


def _miss(h):
    v, n, c = h
    assert np.all(v == 0) and np.all(n == 0) and np.all(c == 0), v


def subvoxel_thin_feature(backend):
    # A: near bound
    slabs = [(0.19, 0.21)]
    want = sv_oracle_zero(sv_lattice(slabs))
    assert abs(want - 0.18666667) < 1e-6
    h = sv_cast(backend, slabs, SV_NEAR, SV_FAR)
    _hit(h, want, 4)
    assert abs(float(h[1][2]) + 1) < 1e-4 and abs(float(h[1][0])) < 1e-4 and abs(float(h[1][1])) < 1e-4
    _miss(sv_cast(backend, slabs, 0.20, SV_FAR))
    _miss(sv_cast(backend, slabs, 0.22, SV_FAR))
    # B: sub-voxel precision
    for a, b in ((0.19, 0.21), (0.39, 0.41), (0.395, 0.405)):
        want = sv_oracle_zero(sv_lattice([(a, b)]))
        assert not math.isnan(want)
        h = sv_cast(backend, [(a, b)], SV_NEAR, SV_FAR)
        _hit(h, want, int(math.floor(want / SV_VS)))
        frac = float(h[0][2]) / float(SV_VS) - math.floor(float(h[0][2]) / float(SV_VS))
        assert 1e-3 < frac < 1 - 1e-3
    # C: first hit wins
    want = sv_oracle_zero(sv_lattice([(0.39, 0.41), (0.47, 0.49)]))
    second = sv_oracle_zero(sv_lattice([(0.47, 0.49)]))
    assert abs(second - 0.46666667) < 1e-6 and abs(want - 0.38666667) < 1e-6
    h = sv_cast(backend, [(0.39, 0.41), (0.47, 0.49)], SV_NEAR, SV_FAR)
    _hit(h, want, 9)
    assert abs(float(h[0][2]) - second) > 1e-3
    # D: far bound
    want = sv_oracle_zero(sv_lattice([(0.91, 0.93)]))
    assert abs(want - 0.90666667) < 1e-6
    _miss(sv_cast(backend, [(0.91, 0.93)], SV_NEAR, 0.90))
    _hit(sv_cast(backend, [(0.91, 0.93)], SV_NEAR, 0.95), want, 22)
    # E: phase sweep
    hits = 0
    for d in (0.0, 0.005, 0.0075, 0.015, 0.02, 0.025):
        slabs = [(np.float32(0.19) + np.float32(d), np.float32(0.21) + np.float32(d))]
        want = sv_oracle_zero(sv_lattice(slabs))
        h = sv_cast(backend, slabs, SV_NEAR, SV_FAR)
        if math.isnan(want):
            _miss(h)
            continue
        hits += 1
        _hit(h, want, int(math.floor(want / SV_VS)))
    assert hits == 3


# ---- coordinate_rounding_contract.cpp:268-300: raycast through a negative origin --
def raycast_negative_origin(backend):
    prm = dict(resolution=8, voxel_size=0.25, truncation=0.25, max_weight=128.0, origin=(-1.0, -1.0, -1.0),
               min_depth=0.3, max_depth=5.0)
    x = np.arange(8)
    t = np.broadcast_to(np.where(x % 2 == 1, 0.4, -0.4).astype(np.float32), (8, 8, 8)).reshape(-1)
    vol = backend.volume(prm, color=True)
    vol.load(np.ascontiguousarray(t), np.full(512, 5.0, np.float32))
    a = vol.raycast(I4, (200.0, 200.0, 7.5, 7.5), 16, 16, colors=True)
    b = vol.raycast(I4, (200.0, 200.0, 7.5, 7.5), 16, 16, colors=True)
    assert np.all(np.isfinite(a[0])) and np.all(np.isfinite(a[1]))
    for u, w in zip(a, b):
        assert np.array_equal(np.asarray(u).view(np.uint8), np.asarray(w).view(np.uint8))
    return a
