"""GPU parity of the depth preprocessor and the marching-cubes mesher against
the oracle: processed raw codes, RGB, guidance luma and band-gated metres are
bit-exact; meshes (positions, normals, colours, welded indices, truncation)
are bit-exact."""
import numpy as np
import pytest

import fixtures as F

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def raw_frames():
    from azu_gb300 import synth
    s = synth.sequence("c1", frames=4)
    return [synth.encode_raw(d) for d in s.depth_mm]


def _textured_rgb(seed=3):
    rng = np.random.default_rng(seed)
    base = rng.integers(0, 256, (480 // 8, 640 // 8, 3), dtype=np.uint8)
    img = np.kron(base, np.ones((8, 8, 1), np.uint8))
    return np.clip(img.astype(int) + rng.integers(-6, 7, img.shape), 0, 255).astype(np.uint8)


@pytest.mark.parametrize("mode", [0, 1])
def test_preprocess_sequence_bit_exact_grey(cuda_lib, orc, raw_frames, mode):
    from azu_gb300 import api, synth
    g = api.Preprocessor(mode)
    o = orc.Preprocessor(minimal=bool(mode))
    rgb = synth.grey_rgb()
    for raw in raw_frames:
        gd, gc = g.process(raw, rgb, 0.3, 2.5)
        od, oc, ol = o.process(raw, rgb, 0.3, 2.5)
        assert np.array_equal(gd, od)
        assert np.array_equal(gc, oc)
        dm, draw, luma, _ = g.device_outputs()
        assert np.array_equal(draw, od)
        assert np.array_equal(luma.view(np.uint32), ol.view(np.uint32))
        om, _ = orc.build_frame_raw(od, orc.intr(525, 525, 319.5, 239.5), 0.3, 2.5)
        assert np.array_equal(dm.view(np.uint32), om.view(np.uint32))


def test_preprocess_textured_rgb(cuda_lib, orc, raw_frames):
    """Non-constant guidance: the RGB chain stays bit-exact; the luma weight uses
    expf, so a raw code may move by at most 1 and only rarely."""
    from azu_gb300 import api
    g = api.Preprocessor(0)
    o = orc.Preprocessor()
    rgb = _textured_rgb()
    flips = 0
    for raw in raw_frames[:3]:
        gd, gc = g.process(raw, rgb, 0.3, 2.5)
        od, oc, ol = o.process(raw, rgb, 0.3, 2.5)
        assert np.array_equal(gc, oc)
        _, _, luma, _ = g.device_outputs()
        assert np.array_equal(luma.view(np.uint32), ol.view(np.uint32))
        assert np.array_equal(gd == 0, od == 0)
        d = np.abs(gd.astype(int) - od.astype(int))
        assert d.max() <= 1
        flips += int((d > 0).sum())
    assert flips <= 1e-3 * 3 * gd.size, flips


def test_preprocess_stage_contracts_gpu(cuda_lib, orc):
    """The EMA literals of tests/depth_ema_determinism_contract.cpp through the
    whole GPU chain in minimal mode is not possible (EMA runs only in full mode),
    so run full mode on frames where median, fill and guided filter are the
    identity (constant walls) and check the hand-derived outputs."""
    from azu_gb300 import api, synth
    g = api.Preprocessor(0)
    rgb = synth.grey_rgb()
    wall1 = np.full((480, 640), F.EMA_WALL1, np.uint16)
    wall2 = np.full((480, 640), F.EMA_WALL2, np.uint16)
    g.process(wall1, rgb, 0.3, 2.5)
    d2, _ = g.process(wall2, rgb, 0.3, 2.5)
    assert (d2 == F.EMA_EXPECT_WALL).all()


def _vol_from(prm, t, w, color=None):
    from azu_gb300 import api
    g = api.TSDFVolume(api.volume_params(prm["resolution"], prm["voxel_size"], prm["truncation"],
                                         prm["max_weight"], prm["origin"], color=color is not None))
    g.upload(t, w, color)
    return g


def _mesh_equal(a, b):
    assert a["truncated"] == b["truncated"]
    assert np.array_equal(a["indices"], b["indices"])
    assert np.array_equal(a["positions"].view(np.uint32), b["positions"].view(np.uint32))
    assert np.array_equal(a["normals"].view(np.uint32), b["normals"].view(np.uint32))
    assert np.array_equal(a["colors"], b["colors"])


def test_mesh_sphere_bit_exact(cuda_lib, orc):
    from azu_gb300 import api
    t, w, prm = F.sphere_volume()
    o = orc.Volume(orc.tsdf_params(**prm))
    o.tsdf[:] = t
    o.weight[:] = w
    om = o.extract_mesh()
    gm = api.MarchingCubes().extract(_vol_from(prm, t, w))
    _mesh_equal(gm, om)
    assert len(np.unique(gm["indices"])) == len(gm["positions"])
    assert F.signed_volume(gm["positions"], gm["indices"]) > 0


def test_mesh_truncation_gpu(cuda_lib, orc):
    from azu_gb300 import api
    t, w, prm = F.sphere_volume()
    o = orc.Volume(orc.tsdf_params(**prm))
    o.tsdf[:] = t
    o.weight[:] = w
    full = o.extract_mesh()
    cap = len(full["indices"]) // 3 - 7
    mc = api.MarchingCubes(max_triangles=cap)
    g = _vol_from(prm, t, w)
    _mesh_equal(mc.extract(g), o.extract_mesh(max_triangles=cap))
    mc.set_max_triangles(0)
    m0 = mc.extract(g)
    assert m0["truncated"] and len(m0["indices"]) == 0


def test_mesh_colored_wall_scene(cuda_lib, orc):
    from azu_gb300 import api
    params, K, W, H, depth, rgb, poses = F.wall_scene()
    o = orc.Volume(orc.tsdf_params(**params), color=True)
    for pose in poses:
        o.integrate(depth, pose, orc.intr(*K), W, H, 0.1, 3.0, rgb=rgb)
    gm = api.MarchingCubes().extract(_vol_from(params, o.tsdf, o.weight, o.color))
    om = o.extract_mesh()
    assert len(om["indices"]) > 0
    _mesh_equal(gm, om)


def test_mesh_fused_sequence(cuda_lib, orc):
    from azu_gb300 import api, synth
    s = synth.sequence("c1", frames=6)
    prm = dict(s.volume)
    prm.pop("format")
    o = orc.Volume(orc.tsdf_params(**prm, min_depth=s.min_depth, max_depth=s.max_depth))
    for k in range(6):
        o.integrate(synth.mm_to_meters(s.depth_mm[k]), s.poses[k], orc.intr(s.fx, s.fy, s.cx, s.cy), 640, 480,
                    s.min_depth, s.max_depth)
    # non-finite and unobserved corners must be refused like the CPU path does
    o.tsdf[1000:1010] = np.nan
    gm = api.MarchingCubes().extract(_vol_from(prm, o.tsdf, o.weight))
    om = o.extract_mesh()
    assert len(om["indices"]) > 30000
    _mesh_equal(gm, om)


def test_mesh_ragged_tiles_and_cap(cuda_lib, orc):
    """A resolution that fills no classify tile evenly, an off-centre sphere
    touching the volume's faces, and a cap that falls inside a 256-cube block."""
    from azu_gb300 import api
    t, w, prm = F.sphere_volume(res=77, vs=0.02, radius=0.55, trunc=0.06, center=0.5)
    w = w.copy()
    w[::97] = 0.0  # scattered unobserved voxels
    o = orc.Volume(orc.tsdf_params(**prm))
    o.tsdf[:] = t
    o.weight[:] = w
    full = o.extract_mesh()
    assert len(full["indices"]) // 3 > 10000
    g = _vol_from(prm, t, w)
    _mesh_equal(api.MarchingCubes().extract(g), full)
    cap = len(full["indices"]) // 3 // 2 + 3
    _mesh_equal(api.MarchingCubes(max_triangles=cap).extract(g), o.extract_mesh(max_triangles=cap))


def test_mesh_noise_volume_regrows_candidate_list(cuda_lib, orc):
    """Random signs make nearly every cube a candidate: more than the first
    candidate list holds, so the extraction grows it and runs again."""
    from azu_gb300 import api
    rng = np.random.default_rng(11)
    res = 48
    t = rng.uniform(-1, 1, res ** 3).astype(np.float32)
    w = (rng.uniform(0, 1, res ** 3) > 0.1).astype(np.float32)
    prm = dict(resolution=res, voxel_size=0.01, truncation=0.03, max_weight=64.0, origin=(0.1, -0.2, 0.3),
               min_depth=0.3, max_depth=5.0)
    o = orc.Volume(orc.tsdf_params(**prm))
    o.tsdf[:] = t
    o.weight[:] = w
    om = o.extract_mesh()
    assert len(om["indices"]) // 3 > 100000
    mc = api.MarchingCubes()
    g = _vol_from(prm, t, w)
    _mesh_equal(mc.extract(g), om)
    _mesh_equal(mc.extract(g), om)  # the grown list is reused
