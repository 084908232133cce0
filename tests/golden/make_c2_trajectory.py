"""Generates tests/golden/c2_orbit_oracle.npz: the lockstep oracle's poses and
grades over the whole 300-frame c2 orbit (raw codes + grey RGB, the benchmark
workload), the reference algorithm's own trajectory for the GPU test to be
held to (the CPU pipeline takes minutes; the GPU test reads this instead).

Run: python tests/golden/make_c2_trajectory.py   (from the repository root)
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]

import oracle as O  # noqa: E402
from azu_gb300 import synth  # noqa: E402

OUT = os.path.join(ROOT, "tests", "golden", "c2_orbit_oracle.npz")


def main():
    s = synth.sequence("c2")
    L = O.Lockstep(s.volume, input_is_mm=False, fold_threads=0)
    rgb = synth.grey_rgb()
    poses, quality, integrated = [], [], []
    for k in range(len(s.poses)):
        o = L.process(synth.encode_raw(s.depth_mm[k]), rgb)
        poses.append(np.asarray(o["pose"], np.float32))
        quality.append(o["quality"])
        integrated.append(o["integrated"])
    np.savez_compressed(OUT, poses=np.stack(poses), quality=np.array(quality, np.int32),
                        integrated=np.array(integrated, np.int32))
    print("wrote", OUT)


if __name__ == "__main__":
    main()
