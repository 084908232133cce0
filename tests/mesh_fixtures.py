"""Fixture volumes of the reference's marching-cubes contracts, rebuilt from
their definitions:

  tests/marching_cubes_frontier_contract.cpp   R1-R6: a stale negative tsdf
      in an unobserved corner, a sphere with an unobserved frontier, an
      unsupported crossing edge, cancelled normals, non-finite tsdf values, a
      degenerate isolated corner and its control, one-sided normals at the
      border, and the determinism sphere
  tests/mesh_welding_contract.cpp   a sphere whose welded vertices must equal
      the distinct crossing edges, an exactly-zero shared corner, and the
      determinism sphere

Each builder returns (params, tsdf, weight, colour) as float32 arrays, z-major;
the same arrays go to the reference build (golden outputs, make_golden.py),
the CPU restatement and the CUDA mesher. welded_edge_count() restates the
welding contract's distinct-edge oracle (:95-140).
"""
import numpy as np

F = np.float32
EMPTY_TSDF, EMPTY_WEIGHT = F(1.0), F(0.0)
EMPTY_COLOR = F(128.0) / F(255.0)


def params(res, vs, trunc):
    """makeParams of both contracts: max weight 8, origin 0."""
    return dict(resolution=res, voxel_size=float(F(vs)), truncation=float(F(trunc)), max_weight=8.0,
                origin=(0.0, 0.0, 0.0), min_depth=0.3, max_depth=5.0)


def _grid(res, vs):
    i = np.arange(res, dtype=np.float32) * F(vs)
    z, y, x = np.meshgrid(i, i, i, indexing="ij")
    return x, y, z


def _dist(res, vs):
    """|voxelToWorld - centre| with the centre 0.5 (R - 1) vs on every axis."""
    c = F(F(0.5) * F(res - 1)) * F(vs)
    x, y, z = _grid(res, vs)
    dx, dy, dz = x - c, y - c, z - c
    return np.sqrt(dx * dx + (dy * dy + dz * dz)).astype(np.float32)


def _color(res, rgb):
    c = np.empty((res ** 3, 3), np.float32)
    c[:] = [F(v) / F(255.0) for v in rgb]
    return c.reshape(-1)


def _clamp1(a):
    return np.clip(a, F(-1), F(1)).astype(np.float32)


def _fill_outside(res, value=0.5, ramp_x=0.0, rgb=(10, 20, 30)):
    x = np.broadcast_to(np.arange(res, dtype=np.float32), (res, res, res))
    t = (F(value) + F(ramp_x) * x).astype(np.float32).reshape(-1)
    return t, np.full(res ** 3, 8.0, np.float32), _color(res, rgb)


def _stamp(t, w, res, x, y, z, tsdf, weight):
    i = (z * res + y) * res + x
    t[i], w[i] = F(tsdf), F(weight)


def stale_corner():
    p = params(8, 0.05, 0.15)
    t, w, c = _fill_outside(8, 0.5, 0.02)
    _stamp(t, w, 8, 2, 2, 2, -0.6, 8.0)
    _stamp(t, w, 8, 3, 3, 3, -0.8, 0.0)
    return p, t, w, c


def _shell_sphere(res, vs, rad, rgb):
    p = params(res, vs, 3 * F(vs))
    s = _dist(res, vs) - F(rad)
    inside = s <= F(1.2) * F(vs)
    t = np.where(inside, _clamp1(s / F(p["truncation"])), EMPTY_TSDF).astype(np.float32).reshape(-1)
    w = np.where(inside, F(8.0), EMPTY_WEIGHT).astype(np.float32).reshape(-1)
    c = _color(res, rgb) if rgb else np.full(3 * res ** 3, EMPTY_COLOR, np.float32)
    return p, t, w, c


def frontier_sphere():
    return _shell_sphere(32, 0.03, 0.30, (200, 100, 50))


def _plane_x(res, vs, plane_vox, rgb):
    p = params(res, vs, 3 * F(vs))
    x, _, _ = _grid(res, vs)
    t = _clamp1((x - F(plane_vox) * F(vs)) / F(p["truncation"])).reshape(-1)
    return p, t, np.full(res ** 3, 8.0, np.float32), _color(res, rgb)


def unsupported_edge():
    p, t, w, c = _plane_x(12, 0.05, 2.5, (70, 70, 70))
    _stamp(t, w, 12, 3, 3, 3, -0.9, 0.0)
    return p, t, w, c


def cancelled_normal():
    p = params(16, 0.05, 3 * F(0.05))
    pat = np.array([-0.9, -0.5, 0.5, -0.9], np.float32)
    t = np.broadcast_to(pat[np.arange(16) % 4], (16, 16, 16)).astype(np.float32).reshape(-1)
    return p, np.ascontiguousarray(t), np.full(16 ** 3, 8.0, np.float32), _color(16, (30, 60, 90))


def non_finite_tsdf():
    res, vs = 24, 0.04
    p = params(res, vs, 3 * F(vs))
    t = _clamp1((_dist(res, vs) - F(0.30)) / F(p["truncation"])).reshape(-1).copy()
    w = np.full(res ** 3, 8.0, np.float32)
    for z in range(8, 16):
        for y in range(8, 16):
            for x in range(8, 16):
                k = (x + y + z) % 3
                _stamp(t, w, res, x, y, z, np.nan if k == 0 else (np.inf if k == 1 else -np.inf), 8.0)
    return p, t, w, _color(res, (11, 22, 33))


def degenerate_corner(control=False):
    p = params(10, 0.05, 0.15)
    t, w, c = _fill_outside(10, 0.5)
    _stamp(t, w, 10, 5, 5, 5, -0.6, 8.0)
    if control:
        _stamp(t, w, 10, 6, 5, 5, 0.9, 8.0)
    return p, t, w, c


def border_one_sided():
    return _plane_x(20, 0.05, 9.5, (90, 90, 90))


def frontier_determinism():
    return _shell_sphere(24, 0.04, 0.25, None)


def weld_sphere():
    res, vs = 28, 0.03
    p = params(res, vs, 3 * F(vs))
    t = _clamp1((_dist(res, vs) - F(0.30)) / F(p["truncation"])).reshape(-1)
    return p, t, np.full(res ** 3, 8.0, np.float32), _color(res, (120, 160, 200))


def weld_zero_corner():
    res, c0 = 10, 5
    p = params(res, 0.05, 3 * F(0.05))
    z, y, x = np.meshgrid(np.arange(res), np.arange(res), np.arange(res), indexing="ij")
    block = (x <= c0) & (y <= c0) & (z <= c0)
    t = np.where(block, F(-0.5), F(0.5) + F(0.01) * x.astype(np.float32)).astype(np.float32).reshape(-1)
    t[(c0 * res + c0) * res + c0] = F(0.0)
    return p, t, np.full(res ** 3, 8.0, np.float32), _color(res, (40, 80, 120))


def weld_determinism():
    res, vs = 22, 0.04
    p = params(res, vs, 3 * F(vs))
    t = _clamp1((_dist(res, vs) - F(0.25)) / F(p["truncation"])).reshape(-1)
    return p, t, np.full(res ** 3, 8.0, np.float32), _color(res, (7, 14, 21))


FIXTURES = {
    "stale_corner": stale_corner, "frontier_sphere": frontier_sphere, "unsupported_edge": unsupported_edge,
    "cancelled_normal": cancelled_normal, "non_finite_tsdf": non_finite_tsdf,
    "degenerate_corner": degenerate_corner, "degenerate_corner_control": lambda: degenerate_corner(True),
    "border_one_sided": border_one_sided, "frontier_determinism": frontier_determinism,
    "weld_sphere": weld_sphere, "weld_zero_corner": weld_zero_corner, "weld_determinism": weld_determinism,
}

_CORNERS = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
_EDGES = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7)]


def welded_edge_count(prm, t, w, tri_table):
    """Distinct canonical crossing edges of every emitted triangle
    (mesh_welding_contract.cpp:95-140): the vertex count a correct weld gives."""
    res = prm["resolution"]
    T = t.reshape(res, res, res)
    Wt = w.reshape(res, res, res)
    sup = (Wt > F(1e-3)) & np.isfinite(T)
    val = np.where(sup, T, EMPTY_TSDF)
    keys = set()
    for z in range(res - 1):
        for y in range(res - 1):
            for x in range(res - 1):
                v = [val[z + o[2], y + o[1], x + o[0]] for o in _CORNERS]
                ok = [sup[z + o[2], y + o[1], x + o[0]] for o in _CORNERS]
                cfg = sum(1 << i for i in range(8) if v[i] < 0)
                if cfg in (0, 255):
                    continue
                row = tri_table[cfg]
                for k in range(0, len(row), 3):
                    tri = row[k:k + 3]
                    if not all(ok[_EDGES[e][0]] and ok[_EDGES[e][1]] for e in tri):
                        continue
                    for e in tri:
                        a, b = _CORNERS[_EDGES[e][0]], _CORNERS[_EDGES[e][1]]
                        pa = (x + a[0], y + a[1], z + a[2])
                        pb = (x + b[0], y + b[1], z + b[2])
                        axis = 0 if pa[0] != pb[0] else (1 if pa[1] != pb[1] else 2)
                        keys.add((min(pa, pb), axis))
    return len(keys)


def tri_table():
    """The triangle table rows (edge ids per row), from the oracle's packed copy."""
    import os
    import re
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "orc_mc_tables.h")
    words = [int(w, 16) for w in re.findall(r"0x([0-9a-f]{16})ull", open(path).read())[:256]]
    rows = []
    for wd in words:
        row = []
        for k in range(16):
            e = (wd >> (4 * k)) & 0xF
            if e == 0xF:
                break
            row.append(e)
        rows.append(row)
    return rows
