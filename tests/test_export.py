"""Mesh export (PLY binary/ASCII and GLB) from the CUDA library's host code.

  reference   the files the reference's own PLYExporter / GLBExporter write
              for the tests/fixtures.py export meshes (tests/golden, made by
              tests/golden/make_golden.py): every file byte for byte
  restatement a plain restatement of the writers (oracle/export_ref.py): PLY
              byte for byte, GLB's binary chunk byte for byte and its glTF
              JSON by content
  invalid meshes create no file. CPU only."""
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
    # a white base colour is the glTF default, left out as the reference leaves it out
    assert "baseColorFactor" not in doc["materials"][0]["pbrMetallicRoughness"]
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


@pytest.mark.parametrize("name", ["sphere", "sphere_bare", "sphere_unwelded"])
def test_files_equal_the_reference_writers(orc, tmp_path, name):
    """PLYExporter::writeBinary / writeASCII and GLBExporter::write of the
    reference (src/export/PLYExporter.cpp, GLBExporter.cpp) wrote these files
    for the same meshes: ours are the same bytes."""
    _lib_ready()
    import hashlib
    import struct
    from golden_check import golden
    from azu_gb300 import api
    g = golden()
    m = F.export_meshes(orc)[name]
    md = {k: v for k, v in m.items() if v is not None}
    for binary, tag in ((True, "ply_binary"), (False, "ply_ascii")):
        p = tmp_path / f"{tag}.ply"
        api.write_ply(p, md, binary)
        data = p.read_bytes()
        sha, size = g[f"export/{name}/{tag}"]
        assert len(data) == int(size) and hashlib.sha256(data).hexdigest() == sha, tag
    p = tmp_path / "m.glb"
    api.write_glb(p, md)
    data = p.read_bytes()
    size, bin_sha = g[f"export/{name}/glb"]
    jlen = struct.unpack_from("<I", data, 12)[0]
    blen = struct.unpack_from("<I", data, 20 + jlen)[0]
    assert data[20:20 + jlen] == g[f"export/{name}/glb_json"].tobytes()
    assert hashlib.sha256(data[28 + jlen:28 + jlen + blen]).hexdigest() == bin_sha
    assert len(data) == int(size)
