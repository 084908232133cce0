"""Generates tests/golden/reference_outputs.npz: the outputs of the reference's
OWN code on the contract fixtures, for the GPU tests to compare against on a
machine without the reference.

The reference's hot-path sources are built unmodified against the project's
Eigen-API shim (oracle/ref.mk -> oracle/_ref/libazu_ref.so, binding
oracle/refimpl.py), so this script runs only where the reference checkout is.
It drives the same scenario code the tests use, through recording backends:

  icp/<scenario>/<k>    ICPTracker::track of the k-th call of each scenario of
                        tests/icp_policy.py (pose, error, counts, flags)
  tsdf/<scenario>/<k>   sha256 of the k-th array/raycast/mesh output of each
                        scenario of tests/tsdf_contracts.py
  scene/<scenario>/<k>  ICPTracker::track of the k-th call of the room-scene
                        scenarios of tests/scene_contracts.py
  mesh/<fixture>/...    MarchingCubes::extract of every fixture volume of
                        tests/mesh_fixtures.py (positions, normals, colours,
                        indices, truncated)
  export/<mesh>/...     PLYExporter::writeBinary / writeASCII (sha256 and size
                        of the file) and GLBExporter::write (the JSON chunk,
                        the BIN chunk's sha256, the file size) of the
                        tests/fixtures.py export meshes
  pairing/<seq>/...     KinectSensor's depth-led pairing of the tests/fixtures.py
                        sample sequences (depth ticks, RGB ticks or -1)

Run: python tests/golden/make_golden.py   (from the repository root)
"""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")]

import fixtures as F  # noqa: E402
import icp_policy  # noqa: E402
import mesh_fixtures  # noqa: E402
import oracle as O  # noqa: E402
import refimpl as R  # noqa: E402
import scene_contracts  # noqa: E402
import tsdf_contracts  # noqa: E402

OUT = os.path.join(ROOT, "tests", "golden", "reference_outputs.npz")


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def result_arrays(prefix, r, store):
    store[prefix + "/pose"] = np.array(r.pose, np.float32).reshape(4, 4)
    store[prefix + "/scalars"] = np.array([r.error, r.final_step], np.float32)
    store[prefix + "/ints"] = np.array([r.inliers, r.converged, r.tracking_ok, r.valid_live_points,
                                        r.valid_model_points, r.projected_points, r.dist_filtered,
                                        r.angle_filtered], np.int64)


def as_dict(r):
    d = r.as_dict()
    d["status"] = 0
    return d


def record_icp(store):
    K = O.intr(F.FX, F.FY, F.CX, F.CY)
    for scen in icp_policy.SCENARIOS:
        calls = []

        def run(cs, iters=(1, 0, 0), dist=0.1, angle=30.0, estimate=icp_policy.I4):
            lv, ln, mv, mn = F.corr_maps(cs)
            z1 = np.zeros((240, 320, 3), np.float32)
            z2 = np.zeros((120, 160, 3), np.float32)
            prm = O.icp_params(iters=iters, dist=dist, angle=angle, fold_threads=1)
            r = R.icp_track(prm, K, [(lv, ln), (z1, z1), (z2, z2)], mv, mn, 640, 480, estimate, icp_policy.I4)
            calls.append(r)
            return as_dict(r)

        scen(run)  # the reference must satisfy the contract's own expectations too
        for k, r in enumerate(calls):
            result_arrays(f"icp/{scen.__name__}/{k}", r, store)


class RefTsdfBackend:
    """tests/tsdf_contracts.py backend over the reference's TSDFVolume, recording digests."""

    def __init__(self, rec):
        self.rec = rec

    def volume(self, prm, color=False):
        rec = self.rec

        def tp(p):
            return O.tsdf_params(**p)

        vol = R.Volume(tp(prm))

        class V:
            def integrate(self, depth, rgb, pose, K, W, H, lo, hi):
                vol.integrate(depth, pose, O.intr(*K), W, H, lo, hi, rgb=rgb)

            def arrays(self):
                out = vol.arrays(color=True)
                rec.append(digest(*out) if color else digest(out[0], out[1]))
                return out if color else (out[0], out[1], None)

            def raycast(self, pose, K, W, H, colors=False):
                r = vol.raycast(pose, O.intr(*K), W, H, colors=colors)
                out = (r["vertices"], r["normals"], r["colors"]) if colors else (r["vertices"], r["normals"])
                rec.append(digest(*out))
                return out

            def mesh(self):
                m = vol.mesh()
                rec.append(digest(m["positions"], m["normals"], m["colors"], m["indices"]))
                return m

            def load(self, t, w, c=None):
                vol.load(t, w, c)

            def set_params(self, p):
                vol.set_params(tp(p))

        return V()


def record_tsdf(store):
    for scen in (tsdf_contracts.min_depth_gates, tsdf_contracts.fusion_bias, tsdf_contracts.raycast_accuracy,
                 tsdf_contracts.subvoxel_thin_feature, tsdf_contracts.raycast_negative_origin):
        rec = []
        scen(RefTsdfBackend(rec))
        store[f"tsdf/{scen.__name__}"] = np.array(rec)


class RefSceneBackend:
    def __init__(self, calls):
        self.calls = calls
        self.K = O.intr(*scene_contracts.K640)

    def volume(self, prm):
        vol = R.Volume(O.tsdf_params(**prm))
        K = self.K

        class V:
            def integrate(self, depth, pose):
                vol.integrate(depth, pose, K, 640, 480, prm["min_depth"], prm["max_depth"])

            def raycast(self, pose, Kr, w, h):
                r = vol.raycast(pose, O.intr(*Kr), w, h)
                return r["vertices"], r["normals"]

        return V()

    def track(self, live, mv, mn, mw, mh, est, ref, iters=(10, 5, 4), dist=0.1, angle=30.0):
        v0 = O.vertices_from_depth(live, self.K)
        pyr = R.frame_pyramid(live, v0, self.K)
        prm = O.icp_params(iters=iters, dist=dist, angle=angle, fold_threads=1)
        r = R.icp_track(prm, self.K, [(lv[1], lv[2]) for lv in pyr], mv, mn, mw, mh, est, ref)
        self.calls.append(r)
        return as_dict(r)


def record_scene(store):
    for scen in (scene_contracts.refpose, scene_contracts.lowres_model):
        calls = []
        scen(RefSceneBackend(calls))
        for k, r in enumerate(calls):
            result_arrays(f"scene/{scen.__name__}/{k}", r, store)


def record_meshes(store):
    for name, build in mesh_fixtures.FIXTURES.items():
        prm, t, w, c = build()
        vol = R.Volume(O.tsdf_params(**prm))
        vol.load(t, w, c)
        m = vol.mesh()
        for k in ("positions", "normals", "colors", "indices"):
            store[f"mesh/{name}/{k}"] = m[k]
        store[f"mesh/{name}/truncated"] = np.array(m["truncated"])


def _sha_file(path):
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


def record_exports(store):
    import struct
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        for name, m in F.export_meshes(O).items():
            for binary, tag in ((True, "ply_binary"), (False, "ply_ascii")):
                p = os.path.join(d, f"{name}.{tag}.ply")
                assert R.export_ply(p, m["positions"], m["indices"], m["normals"], m["colors"], binary)
                store[f"export/{name}/{tag}"] = np.array([_sha_file(p), str(os.path.getsize(p))])
            p = os.path.join(d, f"{name}.glb")
            assert R.export_glb(p, m["positions"], m["indices"], m["normals"], m["colors"])
            data = open(p, "rb").read()
            jlen = struct.unpack_from("<I", data, 12)[0]
            blen = struct.unpack_from("<I", data, 20 + jlen)[0]
            store[f"export/{name}/glb"] = np.array([str(len(data)),
                                                    hashlib.sha256(data[28 + jlen:28 + jlen + blen]).hexdigest()])
            store[f"export/{name}/glb_json"] = np.frombuffer(data[20:20 + jlen], np.uint8)


def record_pairing(store):
    for name in ("hand", "jitter"):
        pairs = R.sensor_pairing(F.pairing_events(name))
        store[f"pairing/{name}/depth"] = np.array([d for d, _ in pairs], np.int64)
        store[f"pairing/{name}/rgb"] = np.array([-1 if r is None else r for _, r in pairs], np.int64)


def main():
    if not R.available():
        raise SystemExit("the reference build is not available (oracle/_ref needs the reference checkout)")
    R.set_threads(1)
    store = {}
    record_icp(store)
    record_tsdf(store)
    record_scene(store)
    record_meshes(store)
    record_exports(store)
    record_pairing(store)
    np.savez_compressed(OUT, **store)
    print(f"wrote {OUT}: {len(store)} arrays, {os.path.getsize(OUT) / 1e3:.0f} kB")


if __name__ == "__main__":
    main()
