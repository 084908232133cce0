"""Sensor-side ingest: fakenect recordings (INDEX.txt, PGM depth, PPM RGB)
parsed and paired by the rules of the reference's sensor (depth-led, nearest
RGB within 17 ms of the 60 MHz counter, counter wrap), payloads read exactly;
on a GPU, frames through the pinned read-ahead ring and the single-copy input
give the pipeline the results of the plain host input and of the lockstep
oracle."""
import os

import numpy as np
import pytest

MS = 60000  # ticks per millisecond


def _write(dir_, name, header, payload):
    with open(os.path.join(dir_, name), "wb") as f:
        f.write(header)
        f.write(payload)


def _recording(tmp, events, seed=0):
    """events: (type, ms or ticks) in capture order; returns the directory."""
    rng = np.random.default_rng(seed)
    lines = []
    payloads = {}
    for k, (t, ms) in enumerate(events):
        ticks = int(ms * MS) % (1 << 32) if isinstance(ms, float) else int(ms) % (1 << 32)
        name = f"{t}-{1000.0 + k:.6f}-{ticks}-{k}.{'pgm' if t == 'd' else 'ppm' if t == 'r' else 'dump'}"
        lines.append(name)
        if t == "d":
            p = rng.integers(0, 2048, (480, 640), dtype=np.uint16)
            _write(tmp, name, b"P5 640 480 65535\n", p.astype("<u2").tobytes())
        elif t == "r":
            p = rng.integers(0, 256, (480, 640, 3), dtype=np.uint8)
            _write(tmp, name, b"P6 640 480 255\n", p.tobytes())
        else:
            p = np.array([0, 819, 0], np.int16)
            _write(tmp, name, b"", p.tobytes())
        payloads[k] = p
    with open(os.path.join(tmp, "INDEX.txt"), "w") as f:
        f.write("\n".join(lines) + "\n")
    return payloads


def _lib_ready():
    from azu_gb300 import _abi
    if not os.path.exists(_abi.LIB_PATH):
        pytest.skip("library not built")


def test_pairing_follows_the_sensor_rules(tmp_path):
    _lib_ready()
    from azu_gb300 import api
    wrap_r = (1 << 32) - 3 * MS
    events = [("r", 0.0), ("d", 5.0), ("d", 38.0), ("r", 40.0), ("r", 60.0), ("d", 100.0), ("d", 133.0),
              ("r", 140.0), ("r", 200.0), ("d", 170.0), ("a", 175.0), ("d", 205.0), ("d", 300.0),
              ("r", wrap_r), ("d", 2 * MS)]
    payloads = _recording(str(tmp_path), events)
    rec = api.Recording(tmp_path)
    ticks = {k: (int(ms * MS) % (1 << 32) if isinstance(ms, float) else int(ms)) for k, (_, ms) in enumerate(events)}
    # (depth entry, rgb entry or None), hand-derived from the rules
    expect = [(1, 0), (2, 3), (5, None), (6, 7), (9, None), (11, 8), (12, None), (14, 13)]
    assert len(rec) == len(expect)
    for k, (d, r) in enumerate(expect):
        assert rec.info(k) == (ticks[d], None if r is None else ticks[r]), k
    depth, rgb, ok = rec.read(3)
    assert ok and np.array_equal(depth, payloads[6]) and np.array_equal(rgb, payloads[7])
    depth, rgb, ok = rec.read(2)
    assert not ok and np.array_equal(depth, payloads[5]) and not rgb.any()
    rec.close()


@pytest.mark.parametrize("name", ["hand", "jitter"])
def test_pairing_equals_the_reference_sensor(tmp_path, name):
    """The same depth / RGB samples fed to the reference's KinectSensor
    (onDepth / onRgb through its test seam, src/sensor/KinectSensor.cpp)
    published these frames (tests/golden, made by
    tests/golden/make_golden.py): the recording pairs them identically, in
    the same order."""
    _lib_ready()
    import fixtures as F
    from golden_check import golden
    from azu_gb300 import api
    g = golden()
    events = F.pairing_events(name)
    _recording(str(tmp_path), events)
    rec = api.Recording(tmp_path)
    want_d, want_r = g[f"pairing/{name}/depth"], g[f"pairing/{name}/rgb"]
    got = [rec.info(k) for k in range(len(rec))]
    rec.close()
    assert len(got) == len(want_d)
    for k, (d, r) in enumerate(got):
        assert d == want_d[k] and (-1 if r is None else r) == want_r[k], k


def test_missing_index_is_an_error(tmp_path):
    _lib_ready()
    from azu_gb300 import api, _abi
    with pytest.raises(_abi.AzuError):
        api.Recording(tmp_path / "nope")


@pytest.mark.gpu
def test_ring_and_single_copy_input_match_host_input(cuda_lib, orc, tmp_path):
    """Frames through the recording ingest (pinned read-ahead ring, one
    host-to-device copy of depth | RGB per frame) give the pipeline the poses of
    the plain host input bit for bit, and the grades, fusion decisions and poses
    (within 5e-4) of the lockstep oracle fed the same raw codes and RGB."""
    import fixtures as F
    from azu_gb300 import api, synth
    s = synth.sequence("c1", frames=8)
    raw = [synth.encode_raw(d, s.min_depth, s.max_depth) for d in s.depth_mm]
    rgb = synth.grey_rgb()
    lines = []
    for k, r in enumerate(raw):
        dn, rn = f"d-{k:.3f}-{k * 33 * MS + 60}-0.pgm", f"r-{k:.3f}-{k * 33 * MS}-0.ppm"
        _write(str(tmp_path), rn, b"P6 640 480 255\n", rgb.tobytes())
        _write(str(tmp_path), dn, b"P5 640 480 65535\n", r.astype("<u2").tobytes())
        lines += [rn, dn]
    (tmp_path / "INDEX.txt").write_text("\n".join(lines) + "\n")
    v = s.volume
    vp = api.volume_params(v["resolution"], v["voxel_size"], v["truncation"], v["max_weight"], v["origin"],
                           s.min_depth, s.max_depth)
    tp = api.tracker_params(min_depth=s.min_depth, max_depth=s.max_depth)
    a = api.Pipeline(api.pipeline_params(vp, tp, 0, s.min_depth, s.max_depth, False, True))
    b = api.Pipeline(api.pipeline_params(vp, tp, 0, s.min_depth, s.max_depth, False, True))
    rec = api.Recording(tmp_path)
    assert len(rec) == len(raw)
    ing = api.Ingest(rec, slots=3)
    L = orc.Lockstep(s.volume, input_is_mm=False, min_depth=s.min_depth, max_depth=s.max_depth, fold_threads=0)
    for k in range(len(raw)):
        got = ing.next()
        assert got is not None and got[1] == k and got[2]
        ra = a.process_frame_packed(got[0])
        ing.release()
        rb = b.process_frame(raw[k], rgb)
        assert np.array_equal(ra["pose"].view(np.uint32), rb["pose"].view(np.uint32)), k
        o = L.process(raw[k], rgb)
        assert (ra["quality"], ra["integrated"]) == (o["quality"], o["integrated"]), k
        rot, trans = F.rel_pose_error(ra["pose"], o["pose"])
        assert rot <= 5e-4 and trans <= 5e-4, (k, rot, trans)
    assert ing.next() is None
    ing.close()
    rec.close()
    a.close()
    b.close()
