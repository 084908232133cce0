"""Oracle (test infrastructure only): a plain restatement of the reference's
mesh exporters for byte comparison.

  ply_bytes  src/export/PLYExporter.cpp:94-152 (header, records), binary little
             endian and ASCII ("%.9g" floats)
  glb_bin    src/export/GLBExporter.cpp:136-272 (weld by exact position in
             index order, glTF axes (x, -y, -z), normals unit length or the
             fallback (0, -0, -1), sRGB bytes -> linear RGBA floats per
             include/export/ColorConversion.h, 4-byte padded sections)
  validate   include/meshing/MeshData.h:49-95
"""
import math
import struct

import numpy as np


def validate(pos, nrm, col, idx):
    nv = len(pos)
    if nv == 0:
        return False
    if len(idx) == 0 or len(idx) % 3:
        return False
    if np.any(np.asarray(idx, np.int64) >= nv):
        return False
    if not np.all(np.isfinite(pos)):
        return False
    if nrm is not None and len(nrm) not in (0, nv):
        return False
    if nrm is not None and not np.all(np.isfinite(nrm)):
        return False
    if col is not None and len(col) not in (0, 3 * nv):
        return False
    return True


def ply_bytes(pos, nrm, col, idx, binary=True):
    nv, nf = len(pos), len(idx) // 3
    has_n = nrm is not None and len(nrm) == nv
    has_c = col is not None and len(col) == 3 * nv
    h = "ply\nformat " + ("binary_little_endian" if binary else "ascii") + " 1.0\n"
    h += "comment KinectFusionQt export\n" + f"element vertex {nv}\n"
    h += "property float x\nproperty float y\nproperty float z\n"
    if has_n:
        h += "property float nx\nproperty float ny\nproperty float nz\n"
    if has_c:
        h += "property uchar red\nproperty uchar green\nproperty uchar blue\n"
    h += f"element face {nf}\nproperty list uchar int vertex_indices\nend_header\n"
    out = bytearray(h.encode())
    pos = np.asarray(pos, np.float32).reshape(-1, 3)
    if binary:
        cols = [pos.view(np.uint8).reshape(nv, 12)]
        if has_n:
            cols.append(np.asarray(nrm, np.float32).reshape(-1, 3).view(np.uint8).reshape(nv, 12))
        if has_c:
            cols.append(np.asarray(col, np.uint8).reshape(nv, 3))
        out += np.concatenate(cols, axis=1).tobytes()
        f = np.zeros((nf, 13), np.uint8)
        f[:, 0] = 3
        f[:, 1:] = np.asarray(idx, np.uint32).astype("<u4").reshape(nf, 3).view(np.uint8).reshape(nf, 12)
        out += f.tobytes()
    else:
        lines = []
        for i in range(nv):
            fields = ["%.9g" % float(v) for v in pos[i]]
            if has_n:
                fields += ["%.9g" % float(v) for v in np.asarray(nrm, np.float32).reshape(-1, 3)[i]]
            if has_c:
                fields += [str(int(v)) for v in np.asarray(col, np.uint8).reshape(-1, 3)[i]]
            lines.append(" ".join(fields))
        tri = np.asarray(idx, np.uint32).reshape(-1, 3)
        lines += ["3 %d %d %d" % tuple(int(v) for v in t) for t in tri]
        out += ("\n".join(lines) + "\n").encode()
    return bytes(out)


def _srgb_linear(c8):
    s = float(np.float32(c8) / np.float32(255.0))
    return np.float32(s / 12.92 if s <= 0.04045 else math.pow((s + 0.055) / 1.055, 2.4))


def glb_bin(pos, nrm, col, idx):
    pos = np.asarray(pos, np.float32).reshape(-1, 3)
    nv_in = len(pos)
    in_n = nrm is not None and len(nrm) == nv_in
    in_c = col is not None and len(col) == 3 * nv_in
    nrm = None if not in_n else np.asarray(nrm, np.float32).reshape(-1, 3)
    col = None if not in_c else np.asarray(col, np.uint8).reshape(-1, 3)
    key_of = {}
    P, N, Cc, I = [], [], [], []
    for o in np.asarray(idx, np.uint32):
        k = tuple(float(v) + 0.0 for v in pos[o])  # + 0.0 folds -0 into +0, as == does
        if k in key_of:
            I.append(key_of[k])
            continue
        key_of[k] = len(P)
        P.append(pos[o])
        if in_n:
            N.append(nrm[o])
        if in_c:
            Cc.append(col[o])
        I.append(key_of[k])
    buf = bytearray()

    def pad():
        while len(buf) % 4:
            buf.append(0)

    Pg = np.array(P, np.float32) * np.array([1, -1, -1], np.float32)
    buf += Pg.astype("<f4").tobytes()
    pad()
    if in_n:
        out = []
        for n in N:
            n = np.asarray(n, np.float32)
            ln = np.float32(np.sqrt(np.float32(n[0] * n[0]) + np.float32(np.float32(n[1] * n[1]) + np.float32(n[2] * n[2]))))
            if not np.isfinite(ln) or ln < np.float32(1e-6):
                out.append(np.array([0.0, -0.0, -1.0], np.float32))
            else:
                out.append(np.array([n[0] / ln, -n[1] / ln, -n[2] / ln], np.float32))
        buf += np.array(out, np.float32).astype("<f4").tobytes()
        pad()
    if in_c:
        rows = [[_srgb_linear(c[0]), _srgb_linear(c[1]), _srgb_linear(c[2]), np.float32(1.0)] for c in Cc]
        buf += np.array(rows, np.float32).astype("<f4").tobytes()
        pad()
    buf += np.array(I, np.uint32).astype("<u4").tobytes()
    pad()
    return bytes(buf), len(P)


def read_glb(data):
    magic, version, length = struct.unpack_from("<4sII", data, 0)
    jlen, jtype = struct.unpack_from("<I4s", data, 12)
    js = data[20:20 + jlen]
    blen, btype = struct.unpack_from("<I4s", data, 20 + jlen)
    b = data[28 + jlen:28 + jlen + blen]
    return dict(magic=magic, version=version, length=length, json=js, json_type=jtype, bin=b, bin_type=btype)
