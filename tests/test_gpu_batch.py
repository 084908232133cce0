"""Batching form on the GPU: independent scenes of uneven volume, image size and
length advanced together (integration and raycasting of all scenes in one
launch per stage, one CUDA graph per step) give every scene exactly the
result of its own single pipeline: poses and the final volume bit for bit,
also after the autotuner has changed the launch shapes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _params(sc):
    from azu_gb300 import api
    v = sc.volume
    vp = api.volume_params(v["resolution"], v["voxel_size"], v["truncation"], v["max_weight"], v["origin"],
                           sc.min_depth, sc.max_depth, 0)
    tp = api.tracker_params(min_depth=sc.min_depth, max_depth=sc.max_depth, fx=sc.fx, fy=sc.fy, cx=sc.cx,
                            cy=sc.cy)
    return vp, tp


@pytest.fixture(scope="module")
def scenes():
    from azu_gb300 import synth
    sc = synth.batch_scenes(seed=7, n_scenes=5, frames_scale=0.08)
    assert len({s.width for s in sc}) == 2 and len({s.volume["resolution"] for s in sc}) >= 2
    assert len({len(s.depth_mm) for s in sc}) >= 2
    return sc


def _single(sc):
    from azu_gb300 import api
    vp, tp = _params(sc)
    pl = api.Pipeline(api.pipeline_params(vp, tp, 0, sc.min_depth, sc.max_depth, input_is_mm=True,
                                          use_graph=True, width=sc.width, height=sc.height))
    poses = [pl.process_frame(d)["pose"] for d in sc.depth_mm]
    t, w = api.TSDFVolume.borrowed(pl.volume_handle(), vp).download()
    pl.close()
    return poses, t, w


def test_batch_equals_single_pipelines(cuda_lib, scenes):
    from azu_gb300 import api
    ref = [_single(sc) for sc in scenes]
    b = api.Batch(scenes)
    n = max(len(sc.depth_mm) for sc in scenes)
    poses = [[] for _ in scenes]
    for k in range(n):
        depth = [sc.depth_mm[k] if k < len(sc.depth_mm) else None for sc in scenes]
        res = b.process(depth)
        for i, r in enumerate(res):
            if r is not None:
                poses[i].append(r["pose"])
        if k == 1:
            b.autotune()
    for i, sc in enumerate(scenes):
        assert len(poses[i]) == len(ref[i][0])
        for a, c in zip(poses[i], ref[i][0]):
            assert np.array_equal(a.view(np.uint32), c.view(np.uint32)), (i, sc.name)
        t, w = b.volume(i).download()
        assert np.array_equal(w, ref[i][2]), i
        assert np.array_equal(t.view(np.uint32), ref[i][1].view(np.uint32)), i
    iw, parts, rw, rh = b.shapes()
    assert iw in (1, 2, 4) and parts in (1, 2, 4) and rw * rh <= 256
    b.close()


def test_batch_rejects_bad_scenes(cuda_lib, scenes):
    import ctypes as C
    from azu_gb300 import _abi
    lib = _abi.load()
    h = C.c_void_p()
    assert lib.azu_batch_create(0, 0, None, C.byref(h)) == _abi.AZU_E_INVALID


def test_c4_scene_set_equals_single_pipelines(cuda_lib):
    """The batching form's own scene set (16 scenes, volumes 128^3..384^3,
    320x240 and 640x480 frames), each cut to its first frames: one batch step
    per frame index gives every scene its single pipeline's poses and volume."""
    from azu_gb300 import api, synth
    scenes = synth.batch_scenes(n_scenes=16, frames_scale=0.04)
    assert len({s.volume["resolution"] for s in scenes}) >= 3 and len({s.width for s in scenes}) == 2
    ref = [_single(sc) for sc in scenes]
    b = api.Batch(scenes)
    n = max(len(sc.depth_mm) for sc in scenes)
    poses = [[] for _ in scenes]
    for k in range(n):
        res = b.process([sc.depth_mm[k] if k < len(sc.depth_mm) else None for sc in scenes])
        for i, r in enumerate(res):
            if r is not None:
                poses[i].append(r["pose"])
    for i in range(len(scenes)):
        assert len(poses[i]) == len(ref[i][0])
        for a, c in zip(poses[i], ref[i][0]):
            assert np.array_equal(a.view(np.uint32), c.view(np.uint32)), i
        t, w = b.volume(i).download()
        assert np.array_equal(w, ref[i][2]), i
        assert np.array_equal(t.view(np.uint32), ref[i][1].view(np.uint32)), i
    b.close()
