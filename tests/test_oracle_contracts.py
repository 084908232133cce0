"""Pins the oracle (CPU restatement) to the reference's own known-answer tests.

Each test rebuilds a fixture of a reference contract test and checks the
contract's hand-derived numbers against the oracle. Runs without a GPU.
"""
import math

import numpy as np
import pytest

import fixtures as F


# ---- depth domain: tests/depth_domain_contract.cpp:140-205 -------------------
def test_depth_domain_default_band(orc):
    acc = [r for r in range(0, 65536) if orc.cpu_depth_meters(r, 0.3, 2.5) != 0.0]
    assert len(acc) == 954 and acc[0] == 1 and acc[-1] == 954
    for r in (0, 2047, 2048, 65535):
        assert orc.raw_to_meters(r) == 0.0
        assert math.copysign(1.0, orc.raw_to_meters(r)) > 0
    for r in (1, 100, 500, 954):
        m = 1.0 / (r * -0.0030711016 + 3.3309495161)
        assert abs(orc.cpu_depth_meters(r, 0.3, 2.5) - m) < 1e-6
    assert orc.cpu_depth_meters(955, 0.3, 2.5) == 0.0
    # band-rejecting encoder: never a wall clamp
    assert orc.meters_to_raw(0.29, 0.3, 2.5) == 0
    assert orc.meters_to_raw(2.6, 0.3, 2.5) == 0
    assert orc.meters_to_raw(float("nan"), 0.3, 2.5) == 0


def test_encoder_round_trip(orc):
    # every accepted raw code encodes back to itself
    for r in range(1, 955):
        m = orc.cpu_depth_meters(r, 0.3, 2.5)
        assert orc.meters_to_raw(m, 0.3, 2.5) == r


# ---- temporal EMA: tests/depth_ema_determinism_contract.cpp:220-266 -----------
def test_ema_hand_derived_literals(orc):
    orc.set_threads(1)
    ema = np.zeros(640 * 480, np.float32)
    f1 = orc.pre_stage("ema", F.ema_frame(F.EMA_WALL1, F.EMA_WALL2), ema, 0.3, 2.5)
    f2 = orc.pre_stage("ema", F.ema_frame(F.EMA_WALL2, F.EMA_CENTRE), ema, 0.3, 2.5)
    orc.set_threads(8)
    f2 = f2.reshape(480, 640)
    assert f2[F.EMA_CY, F.EMA_CX + 40] == F.EMA_EXPECT_WALL
    assert f2[F.EMA_CY, F.EMA_CX] == F.EMA_EXPECT_CENTRE
    assert f1.max() > 0


# ---- TSDF integration: tests/tsdf_integration_race_contract.cpp:251-323 ------
def test_integration_hand_fold(orc):
    p = orc.tsdf_params(F.HF_RES, F.HF_VS, F.HF_TRUNC, 128.0, (-0.32, -0.32, 0.0))
    vol = orc.Volume(p, color=True)
    K = orc.intr(500.0, 500.0, 2.0, 2.0)
    for depth, rgb in F.hand_fold_frames():
        vol.integrate(depth, np.eye(4), K, 4, 4, 0.1, 3.0, rgb=rgb)
    t = vol.tsdf.reshape(64, 64, 64)
    w = vol.weight.reshape(64, 64, 64)
    c = vol.color.reshape(64, 64, 64, 3)
    checked = 0
    for k in range(1, 64):
        et, ew, er = F.hand_fold_expected(k)
        assert w[k, 32, 32] == np.float32(ew)
        assert abs(t[k, 32, 32] - et) < 2e-5
        assert abs(c[k, 32, 32, 0] - er) < 2e-6
        checked += ew == 2.0 and abs(et) < 0.5
    assert checked >= 2
    assert w[50, 32, 32] == 2.0
    assert abs(c[50, 32, 32, 0] - (200 / 255 + 60 / 255) / 2) < 2e-6
    assert w[54, 32, 32] == 0.0
    assert w[50, 32, 33] == 0.0


def test_integration_thread_count_equivalence(orc):
    params, K, W, H, depth, rgb, poses = F.wall_scene()
    outs = []
    for threads in (1, 2, 4):
        orc.set_threads(threads)
        p = orc.tsdf_params(**params)
        vol = orc.Volume(p, color=True)
        for pose in poses:
            vol.integrate(depth, pose, orc.intr(*K), W, H, 0.1, 3.0, rgb=rgb)
        mesh = vol.extract_mesh()
        outs.append((vol.tsdf.copy(), vol.weight.copy(), vol.color.copy(), mesh))
    orc.set_threads(8)
    assert (outs[0][1] > 0).sum() > 0 and len(outs[0][3]["indices"]) > 0
    for o in outs[1:]:
        for a, b in zip(o[:3], outs[0][:3]):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
        for key in ("positions", "normals", "colors", "indices"):
            assert np.array_equal(o[3][key], outs[0][3][key])


# ---- raycast: tests/tsdf_raycast_contract.cpp:193-300 -------------------------
def _rc_volume(orc, field, min_depth=F.RC_MIN, max_depth=F.RC_MAX):
    p = orc.tsdf_params(**F.raycast_params(min_depth, max_depth))
    vol = orc.Volume(p, color=True)
    t, w, c = F.raycast_volume(field)
    vol.tsdf[:] = t
    vol.weight[:] = w
    vol.color[:] = c
    return vol


def _cast(vol, orc):
    return vol.raycast(np.eye(4), orc.intr(F.RC_F, F.RC_F, F.RC_C, F.RC_C), F.RC_IMG, F.RC_IMG, colors=True)


def test_raycast_planar_hit(orc):
    r = _cast(_rc_volume(orc, F.wall_field), orc)
    v, n, c = r["vertices"][3, 3], r["normals"][3, 3], r["colors"][3, 3]
    assert abs(v[0]) <= 1e-5 and abs(v[1]) <= 1e-5 and abs(v[2] - F.WALL_HIT_Z) <= 1e-5
    assert abs(n[2] + 1.0) <= 1e-5 and abs(np.linalg.norm(n) - 1.0) <= 1e-5
    assert tuple(c) == F.layer_color(int(math.floor(F.WALL_HIT_Z / F.RC_VS)))


def test_raycast_zdepth_band(orc):
    r = _cast(_rc_volume(orc, F.wall_field, max_depth=0.42), orc)
    v = r["vertices"][3, 7]
    assert abs(v[2] - F.WALL_HIT_Z) <= 1e-5 and abs(v[0] - F.WALL_HIT_Z) <= 1e-5


def test_raycast_band_gate(orc):
    r = _cast(_rc_volume(orc, F.wall_field, max_depth=0.30), orc)
    assert not r["vertices"][3, 3].any() and not r["normals"][3, 3].any() and not r["colors"][3, 3].any()


def test_raycast_slab_front_face(orc):
    r = _cast(_rc_volume(orc, F.slab_field), orc)
    v = r["vertices"][3, 3]
    assert abs(v[2] - F.SLAB_FRONT_Z) <= 1e-5
    # a ray that starts inside the material reports no surface
    r2 = _cast(_rc_volume(orc, F.slab_field, min_depth=0.395, max_depth=F.RC_MAX), orc)
    assert not r2["vertices"][3, 3].any()


def test_raycast_nonfinite_layer_is_not_a_hit(orc):
    vol = _rc_volume(orc, F.wall_field)
    t = vol.tsdf.reshape(32, 32, 32)
    t[9] = np.nan  # the layer in front of the crossing
    r = _cast(vol, orc)
    assert not r["vertices"][3, 3].any()


# ---- ICP weighting: tests/icp_weighting_contract.cpp:83-209 -------------------
def test_icp_canonical_weighting(orc):
    lv, ln, mv, mn = F.icp_weighting_fixture()
    zeros = [np.zeros((480 >> l, 640 >> l, 3), np.float32) for l in (1, 2)]
    levels = [(None, lv, ln), (None, zeros[0], zeros[0]), (None, zeros[1], zeros[1])]
    prm = orc.icp_params(iters=(1, 0, 0), fold_threads=1)
    r = orc.icp_track(prm, orc.intr(F.FX, F.FY, F.CX, F.CY), levels, mv, mn, np.eye(4), np.eye(4)).as_dict()
    assert r["valid_live_points"] == 11 and r["valid_model_points"] == 11 and r["projected_points"] == 11
    assert r["inliers"] == 11 and r["dist_filtered"] == 0 and r["angle_filtered"] == 0
    assert abs(r["pose"][2, 3] - F.ICP_TZ) <= 5e-6
    assert abs(r["error"] - F.ICP_ERR) <= 5e-6
    assert abs(r["pose"][0, 3]) <= 5e-6 and abs(r["pose"][1, 3]) <= 5e-6


def test_icp_nonfinite_correspondence_rejected(orc):
    lv, ln, mv, mn = F.icp_weighting_fixture()
    zeros = [np.zeros((480 >> l, 640 >> l, 3), np.float32) for l in (1, 2)]
    prm = orc.icp_params(iters=(1, 0, 0), fold_threads=1)
    K = orc.intr(F.FX, F.FY, F.CX, F.CY)
    clean = orc.icp_track(prm, K, [(None, lv, ln), (None, zeros[0], zeros[0]), (None, zeros[1], zeros[1])],
                          mv, mn, np.eye(4), np.eye(4)).as_dict()
    mv2 = mv.copy()
    lv2, ln2 = lv.copy(), ln.copy()
    z = np.float32(1.0)
    vx = (np.float32(300) - np.float32(F.CX)) / np.float32(F.FX) * z
    vy = (np.float32(220) - np.float32(F.CY)) / np.float32(F.FY) * z
    lv2[220, 300] = (vx, vy, z)
    ln2[220, 300] = (0, 0, 1)
    mv2[220, 300] = (vx, vy, np.nan)
    mn2 = mn.copy()
    mn2[220, 300] = (0, 0, 1)
    dirty = orc.icp_track(prm, K, [(None, lv2, ln2), (None, zeros[0], zeros[0]), (None, zeros[1], zeros[1])],
                          mv2, mn2, np.eye(4), np.eye(4)).as_dict()
    assert np.array_equal(clean["pose"], dirty["pose"]) and clean["error"] == dirty["error"]


# ---- pyramid jump guard: tests/icp_weighting_contract.cpp:362-379 ------------
def test_pyramid_keeps_nearest_across_jump(orc):
    d = np.zeros((8, 8), np.float32)
    d[0:2, 0:2] = [[1.0, 1.0], [1.0, 2.0]]       # a 1 m jump inside one 2x2 block
    d[0:2, 2:4] = [[1.0, 1.01], [1.02, 1.03]]    # within the guard: averaged
    v = orc.vertices_from_depth(d, orc.intr(10, 10, 3.5, 3.5))
    n = np.zeros_like(v)
    n[..., 2] = 1.0
    dd, vv, nn = orc.downsample(d, v, n)
    assert dd[0, 0] == np.float32(1.0) and np.array_equal(vv[0, 0], v[0, 0])
    assert abs(dd[0, 1] - np.float32((1.0 + 1.01 + 1.02 + 1.03) / 4)) < 1e-6


# ---- marching cubes: tests/marching_cubes_table_contract.cpp, mesh_welding, winding
def test_mc_table_rows_use_crossing_edges():
    import os
    import re
    here = os.path.dirname(os.path.abspath(__file__))
    text = open(os.path.join(here, "..", "oracle", "orc_mc_tables.h")).read()
    rows = [int(v, 16) for v in re.findall(r"0x([0-9a-f]{16})ull", text)]
    assert len(rows) == 256
    for ci, row in enumerate(rows):
        edges = []
        k = 0
        while ((row >> (4 * k)) & 0xF) != 0xF:
            edges.append((row >> (4 * k)) & 0xF)
            k += 1
        assert len(edges) % 3 == 0
        m = F.crossing_mask(ci)
        assert all((m >> e) & 1 for e in edges)
        assert (len(edges) == 0) == (m == 0)
    # repaired rows of the reference's edge table
    assert (F.crossing_mask(213), F.crossing_mask(214), F.crossing_mask(215)) == (0x83f, 0xb35, 0xa3c)
    product = open(os.path.join(here, "..", "azu_gb300", "csrc", "mc_tables.h")).read()
    assert [int(v, 16) for v in re.findall(r"0x([0-9a-f]{16})ull", product)] == rows


def test_mc_sphere_weld_and_winding(orc):
    t, w, prm = F.sphere_volume()
    vol = orc.Volume(orc.tsdf_params(**prm))
    vol.tsdf[:] = t
    vol.weight[:] = w
    m = vol.extract_mesh()
    pos, idx = m["positions"], m["indices"]
    assert len(idx) > 0 and len(idx) % 3 == 0
    # welded vertex count == number of distinct referenced vertices (exact-edge weld)
    assert len(np.unique(idx)) == len(pos)
    # closed manifold: every undirected edge shared by exactly two triangles
    tri = idx.reshape(-1, 3)
    e = np.sort(np.concatenate([tri[:, [0, 1]], tri[:, [1, 2]], tri[:, [2, 0]]]), axis=1)
    _, counts = np.unique(e, axis=0, return_counts=True)
    assert (counts == 2).all()
    # outward winding: positive signed volume close to the sphere's
    vol_mesh = F.signed_volume(pos, idx)
    assert vol_mesh > 0 and abs(vol_mesh - 4 / 3 * math.pi * 0.37 ** 3) / vol_mesh < 0.05
    assert not m["truncated"]


def test_mc_truncation_at_triangle_boundary(orc):
    t, w, prm = F.sphere_volume()
    vol = orc.Volume(orc.tsdf_params(**prm))
    vol.tsdf[:] = t
    vol.weight[:] = w
    full = vol.extract_mesh()
    cap = len(full["indices"]) // 3 - 7
    part = vol.extract_mesh(max_triangles=cap)
    assert part["truncated"] and len(part["indices"]) == 3 * cap
    assert np.array_equal(part["indices"], full["indices"][:3 * cap])
    exact = vol.extract_mesh(max_triangles=len(full["indices"]) // 3)
    assert not exact["truncated"]
