"""GPU parity of the TSDF volume (integrate, raycast) against the oracle, through
the C ABI. Integer and byte results bit-exact; float results bit-exact too,
because the kernels evaluate the reference's float expressions in its order."""
import numpy as np
import pytest

import fixtures as F

pytestmark = pytest.mark.gpu


def _gpu_volume(prm, color=False, fmt=0):
    from azu_gb300 import api
    p = api.volume_params(prm["resolution"], prm["voxel_size"], prm["truncation"], prm["max_weight"],
                          prm["origin"], prm.get("min_depth", 0.3), prm.get("max_depth", 5.0), fmt, color)
    return api.TSDFVolume(p)


def _orc_volume(orc, prm, color=False):
    return orc.Volume(orc.tsdf_params(**prm), color=color)


def test_integration_hand_fold_gpu(cuda_lib, orc):
    prm = dict(resolution=F.HF_RES, voxel_size=F.HF_VS, truncation=F.HF_TRUNC, max_weight=128.0,
               origin=(-0.32, -0.32, 0.0))
    g = _gpu_volume(prm, color=True)
    o = _orc_volume(orc, prm, color=True)
    for depth, rgb in F.hand_fold_frames():
        g.integrate(depth, np.eye(4), (500.0, 500.0, 2.0, 2.0), 4, 4, 0.1, 3.0, rgb=rgb)
        o.integrate(depth, np.eye(4), orc.intr(500.0, 500.0, 2.0, 2.0), 4, 4, 0.1, 3.0, rgb=rgb)
    t, w, c = g.download(color=True)
    assert np.array_equal(t.view(np.uint32), o.tsdf.view(np.uint32))
    assert np.array_equal(w, o.weight)
    assert np.array_equal(c.view(np.uint32), o.color.view(np.uint32))
    tt, ww = t.reshape(64, 64, 64), w.reshape(64, 64, 64)
    assert ww[50, 32, 32] == 2.0 and ww[54, 32, 32] == 0.0
    et, _, _ = F.hand_fold_expected(50)
    assert abs(tt[50, 32, 32] - et) < 2e-5


def test_integration_wall_scene_gpu(cuda_lib, orc):
    params, K, W, H, depth, rgb, poses = F.wall_scene()
    g = _gpu_volume(params, color=True)
    o = _orc_volume(orc, params, color=True)
    for pose in poses:
        g.integrate(depth, pose, K, W, H, 0.1, 3.0, rgb=rgb)
        st = o.integrate(depth, pose, orc.intr(*K), W, H, 0.1, 3.0, rgb=rgb)
        gs = g.stats()
        assert gs["last_voxels_updated"] == st["voxels_updated"]
        assert gs["last_color_updates"] == st["color_updates"]
    t, w, c = g.download(color=True)
    assert np.array_equal(t.view(np.uint32), o.tsdf.view(np.uint32))
    assert np.array_equal(w, o.weight)
    assert np.array_equal(c.view(np.uint32), o.color.view(np.uint32))


@pytest.fixture(scope="module")
def c1_seq():
    from azu_gb300 import synth
    return synth.sequence("c1", frames=12)


def test_integration_sequence_bit_exact(cuda_lib, orc, c1_seq):
    from azu_gb300 import synth
    s = c1_seq
    prm = dict(s.volume, min_depth=s.min_depth, max_depth=s.max_depth)
    prm.pop("format")
    g = _gpu_volume(prm)
    o = _orc_volume(orc, prm)
    K = (s.fx, s.fy, s.cx, s.cy)
    observed = 0
    for k in range(len(s.poses)):
        dm = synth.mm_to_meters(s.depth_mm[k])
        g.integrate(dm, s.poses[k], K, s.width, s.height, s.min_depth, s.max_depth)
        st = o.integrate(dm, s.poses[k], orc.intr(*K), s.width, s.height, s.min_depth, s.max_depth)
        observed += st["newly_observed"]
        gs = g.stats()
        assert gs["last_voxels_updated"] == st["voxels_updated"], k
    assert g.stats()["observed_voxels"] == observed
    t, w = g.download()
    assert np.array_equal(w, o.weight)
    assert np.array_equal(t.view(np.uint32), o.tsdf.view(np.uint32))


def test_raycast_sequence_bit_exact(cuda_lib, orc, c1_seq):
    from azu_gb300 import synth
    s = c1_seq
    prm = dict(s.volume, min_depth=s.min_depth, max_depth=s.max_depth)
    prm.pop("format")
    g = _gpu_volume(prm)
    o = _orc_volume(orc, prm)
    K = (s.fx, s.fy, s.cx, s.cy)
    for k in range(6):
        dm = synth.mm_to_meters(s.depth_mm[k])
        o.integrate(dm, s.poses[k], orc.intr(*K), s.width, s.height, s.min_depth, s.max_depth)
    g.upload(o.tsdf, o.weight)
    for k in (5, 9):
        rg = g.raycast(s.poses[k], K, s.width, s.height, colors=True)
        ro = o.raycast(s.poses[k], orc.intr(*K), s.width, s.height, colors=True)
        hits = (ro["vertices"] != 0).any(-1).sum()
        assert hits > 10000
        assert np.array_equal(rg["vertices"].view(np.uint32), ro["vertices"].view(np.uint32))
        assert np.array_equal(rg["normals"].view(np.uint32), ro["normals"].view(np.uint32))
        assert np.array_equal(rg["colors"], ro["colors"])


def _rc(cuda_lib, field, min_depth=F.RC_MIN, max_depth=F.RC_MAX):
    g = _gpu_volume(F.raycast_params(min_depth, max_depth), color=True)
    t, w, c = F.raycast_volume(field)
    g.upload(t, w, c)
    return g.raycast(np.eye(4), (F.RC_F, F.RC_F, F.RC_C, F.RC_C), F.RC_IMG, F.RC_IMG, colors=True)


def test_raycast_contract_fixtures_gpu(cuda_lib):
    import math
    r = _rc(cuda_lib, F.wall_field)
    v, n, c = r["vertices"][3, 3], r["normals"][3, 3], r["colors"][3, 3]
    assert abs(v[2] - F.WALL_HIT_Z) <= 1e-5 and abs(v[0]) <= 1e-5 and abs(n[2] + 1) <= 1e-5
    assert tuple(c) == F.layer_color(int(math.floor(F.WALL_HIT_Z / F.RC_VS)))
    r = _rc(cuda_lib, F.wall_field, max_depth=0.42)
    assert abs(r["vertices"][3, 7][2] - F.WALL_HIT_Z) <= 1e-5
    r = _rc(cuda_lib, F.wall_field, max_depth=0.30)
    assert not r["vertices"][3, 3].any() and not r["colors"][3, 3].any()
    r = _rc(cuda_lib, F.slab_field)
    assert abs(r["vertices"][3, 3][2] - F.SLAB_FRONT_Z) <= 1e-5
    r = _rc(cuda_lib, F.slab_field, min_depth=0.395)
    assert not r["vertices"][3, 3].any()


def test_reset_and_set_params(cuda_lib):
    from azu_gb300 import api
    g = _gpu_volume(dict(resolution=16, voxel_size=0.1, truncation=0.3, max_weight=64.0, origin=(0, 0, 0)))
    t = np.zeros(16 ** 3, np.float32)
    w = np.ones(16 ** 3, np.float32)
    g.upload(t, w)
    g.reset()
    t2, w2 = g.download()
    assert (t2 == 1.0).all() and (w2 == 0.0).all()
    g.set_params(api.volume_params(24, 0.1, 0.3, 64.0, (0, 0, 0)))
    t3, w3 = g.download()
    assert t3.size == 24 ** 3 and (t3 == 1.0).all() and (w3 == 0.0).all()


def test_invalid_arguments_rejected(cuda_lib):
    import ctypes as C
    from azu_gb300 import _abi, api
    lib = _abi.load()
    h = C.c_void_p()
    bad = api.volume_params(1, 0.1, 0.3)
    assert lib.azu_volume_create(0, C.byref(bad), None, C.byref(h)) == _abi.AZU_E_INVALID
    bad = api.volume_params(16, -0.1, 0.3)
    assert lib.azu_volume_create(0, C.byref(bad), None, C.byref(h)) == _abi.AZU_E_INVALID
    assert b"voxel_size" in lib.azu_last_error()


def test_free_space_skipping_is_exact(cuda_lib, orc, c1_seq):
    """Bricks maintained by integration (not rebuilt): raycasts with and without
    skipping are bit-identical, and equal the oracle's."""
    from azu_gb300 import synth
    s = c1_seq
    prm = dict(s.volume, min_depth=s.min_depth, max_depth=s.max_depth)
    prm.pop("format")
    g = _gpu_volume(prm)
    o = _orc_volume(orc, prm)
    K = (s.fx, s.fy, s.cx, s.cy)
    for k in range(8):
        dm = synth.mm_to_meters(s.depth_mm[k])
        g.integrate(dm, s.poses[k], K, s.width, s.height, s.min_depth, s.max_depth)
        o.integrate(dm, s.poses[k], orc.intr(*K), s.width, s.height, s.min_depth, s.max_depth)
    for k in (7, 11):
        on = g.raycast(s.poses[k], K, s.width, s.height)
        g.lib.azu_volume_set_free_space_skipping(g.h, 0)
        off = g.raycast(s.poses[k], K, s.width, s.height)
        g.lib.azu_volume_set_free_space_skipping(g.h, 1)
        ro = o.raycast(s.poses[k], orc.intr(*K), s.width, s.height)
        for key in ("vertices", "normals"):
            assert np.array_equal(on[key].view(np.uint32), off[key].view(np.uint32))
            assert np.array_equal(on[key].view(np.uint32), ro[key].view(np.uint32))


@pytest.mark.gpu
def test_ray_start_map_near_and_inside_surfaces(cuda_lib, orc, c1_seq):
    """The ray start map skips far steps only below every brick that is not
    free: cameras moved towards and into the fused surfaces (bricks across the
    camera plane bound every tile), turned away from them, and looking along
    them give the same images with skipping on and off, and the oracle's."""
    from azu_gb300 import synth
    s = c1_seq
    prm = dict(s.volume, min_depth=s.min_depth, max_depth=s.max_depth)
    prm.pop("format")
    g = _gpu_volume(prm)
    o = _orc_volume(orc, prm)
    K = (s.fx, s.fy, s.cx, s.cy)
    for k in range(8):
        dm = synth.mm_to_meters(s.depth_mm[k])
        g.integrate(dm, s.poses[k], K, s.width, s.height, s.min_depth, s.max_depth)
        o.integrate(dm, s.poses[k], orc.intr(*K), s.width, s.height, s.min_depth, s.max_depth)
    base = np.asarray(s.poses[7], np.float32)
    fwd = base[:3, 2]
    poses = []
    for d in (0.6, 1.0, 1.15, 1.25):  # towards the scene centre, 1.5 m ahead: up to inside the sphere's band
        p = base.copy()
        p[:3, 3] += np.float32(d) * fwd
        poses.append(p)
    turn = base.copy()  # looking away from the scene
    turn[:3, 0] *= -1
    turn[:3, 2] *= -1
    poses.append(turn)
    c, sn = np.float32(np.cos(1.3)), np.float32(np.sin(1.3))
    side = base.copy()  # yawed 75 degrees: along the fused surfaces
    side[:3, :3] = base[:3, :3] @ np.array([[c, 0, sn], [0, 1, 0], [-sn, 0, c]], np.float32)
    poses.append(side)
    for i, p in enumerate(poses):
        on = g.raycast(p, K, s.width, s.height)
        g.lib.azu_volume_set_free_space_skipping(g.h, 0)
        off = g.raycast(p, K, s.width, s.height)
        g.lib.azu_volume_set_free_space_skipping(g.h, 1)
        ro = o.raycast(p, orc.intr(*K), s.width, s.height)
        for key in ("vertices", "normals"):
            assert np.array_equal(on[key].view(np.uint32), off[key].view(np.uint32)), (i, key)
            assert np.array_equal(on[key].view(np.uint32), ro[key].view(np.uint32)), (i, key)


def test_voxels_written_through_the_device_pointer(cuda_lib, orc, c1_seq):
    """Voxels written through azu_volume_device_voxels (here: a fused volume's
    array copied into a fresh volume by the driver API) take effect in the
    raycast and the marching cubes once azu_volume_voxels_changed has
    recomputed the free-space flags, and with skipping off before that: the
    same images and mesh as the source volume."""
    import ctypes as C
    import torch
    from azu_gb300 import api, synth
    s = c1_seq
    prm = dict(s.volume, min_depth=s.min_depth, max_depth=s.max_depth)
    prm.pop("format")
    src = _gpu_volume(prm)
    K = (s.fx, s.fy, s.cx, s.cy)
    for k in range(6):
        src.integrate(synth.mm_to_meters(s.depth_mm[k]), s.poses[k], K, s.width, s.height, s.min_depth,
                      s.max_depth)
    dst = _gpu_volume(prm)  # fresh: every brick flagged free
    torch.cuda.synchronize()
    drv = C.CDLL("libcuda.so.1")
    drv.cuMemcpyDtoD_v2.argtypes = [C.c_uint64, C.c_uint64, C.c_size_t]
    ps = src.lib.azu_volume_device_voxels(src.h)
    pd = dst.lib.azu_volume_device_voxels(dst.h)
    assert drv.cuMemcpyDtoD_v2(pd, ps, src.n * 8) == 0
    torch.cuda.synchronize()
    pose = s.poses[5]
    want = src.raycast(pose, K, s.width, s.height)
    dst.set_free_space_skipping(False)
    off = dst.raycast(pose, K, s.width, s.height)
    mc = api.MarchingCubes()
    m_off = mc.extract(dst)
    dst.set_free_space_skipping(True)
    dst.voxels_changed()
    on = dst.raycast(pose, K, s.width, s.height)
    m_src = mc.extract(src)
    m_on = mc.extract(dst)
    for key in ("vertices", "normals"):
        assert np.array_equal(off[key].view(np.uint32), want[key].view(np.uint32))
        assert np.array_equal(on[key].view(np.uint32), want[key].view(np.uint32))
    assert len(m_src["positions"]) > 0
    for key, val in m_src.items():
        if isinstance(val, np.ndarray):
            assert np.array_equal(val, m_off[key]) and np.array_equal(val, m_on[key]), key
