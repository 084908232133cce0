"""Mesh export (PLY binary/ASCII and GLB) from the CUDA library's host code
against a plain restatement of the reference's writers: PLY byte for byte,
GLB's binary chunk byte for byte and its glTF JSON by content; invalid meshes
create no file. CPU only."""
import json

import numpy as np
import pytest

import fixtures as F


def _mesh(orc):
    t, w, prm = F.sphere_volume()
    o = orc.Volume(orc.tsdf_params(**prm))
    o.tsdf[:] = t
    o.weight[:] = w
    m = o.extract_mesh()
    assert len(m["indices"]) > 300
    return m


def _lib_ready():
    from azu_gb300 import _abi
    import os
    if not os.path.exists(_abi.LIB_PATH):
        pytest.skip("library not built")


@pytest.mark.parametrize("binary", [True, False])
def test_ply_bytes(orc, tmp_path, binary):
    _lib_ready()
    import export_ref
    from azu_gb300 import api
    m = _mesh(orc)
    p = tmp_path / "m.ply"
    api.write_ply(p, m, binary)
    ref = export_ref.ply_bytes(m["positions"], m["normals"], m["colors"].reshape(-1), m["indices"], binary)
    assert p.read_bytes() == ref
    # without normals and colours
    api.write_ply(p, dict(positions=m["positions"], indices=m["indices"]), binary)
    assert p.read_bytes() == export_ref.ply_bytes(m["positions"], None, None, m["indices"], binary)


def test_glb_chunks(orc, tmp_path):
    _lib_ready()
    import export_ref
    from azu_gb300 import api
    m = _mesh(orc)
    # an unwelded copy (duplicated vertices), a zero normal and a -0 coordinate
    pos = np.concatenate([m["positions"], m["positions"]]).copy()
    nrm = np.concatenate([m["normals"], m["normals"]]).copy()
    col = np.concatenate([m["colors"], m["colors"]]).copy()
    col[0] = (0, 10, 255)
    n = len(m["positions"])
    idx = np.concatenate([m["indices"], m["indices"] + n]).astype(np.uint32)
    nrm[int(idx[5])] = 0.0
    p = tmp_path / "m.glb"
    api.write_glb(p, dict(positions=pos, normals=nrm, colors=col, indices=idx))
    g = export_ref.read_glb(p.read_bytes())
    assert g["magic"] == b"glTF" and g["version"] == 2 and g["length"] == len(p.read_bytes())
    assert g["json_type"] == b"JSON" and g["bin_type"] == b"BIN\x00"
    b, nv = export_ref.glb_bin(pos, nrm, col.reshape(-1), idx)
    assert g["bin"] == b
    assert nv <= n
    doc = json.loads(g["json"])
    prim = doc["meshes"][0]["primitives"][0]
    acc = doc["accessors"]
    assert acc[prim["attributes"]["POSITION"]]["count"] == nv
    assert acc[prim["indices"]]["count"] == len(idx)
    pg = np.asarray(pos, np.float32) * np.array([1, -1, -1], np.float32)
    assert acc[prim["attributes"]["POSITION"]]["min"] == [float(v) for v in pg.min(0)]
    assert doc["materials"][0]["pbrMetallicRoughness"]["baseColorFactor"] == [1.0, 1.0, 1.0, 1.0]
    assert doc["buffers"][0]["byteLength"] == len(b)


def test_invalid_mesh_creates_no_file(orc, tmp_path):
    _lib_ready()
    from azu_gb300 import api, _abi
    m = _mesh(orc)
    bad = [dict(positions=m["positions"], indices=m["indices"][:-1]),
           dict(positions=m["positions"], indices=np.append(m["indices"][:-3], [0, 1, len(m["positions"])])),
           dict(positions=m["positions"], normals=m["normals"][:-1], indices=m["indices"]),
           dict(positions=np.where(np.arange(len(m["positions"]))[:, None] == 3, np.nan, m["positions"]),
                indices=m["indices"])]
    for k, mesh in enumerate(bad):
        for fn in (lambda p: api.write_ply(p, mesh), lambda p: api.write_glb(p, mesh)):
            p = tmp_path / f"bad{k}.out"
            with pytest.raises(_abi.AzuError):
                fn(p)
            assert not p.exists()
