"""The closed form of the running float sum (azu_gb300/csrc/fstep.cuh) that
the integration uses in place of the reference's sequential coordinate
stepping (src/tsdf/TSDFVolume.cpp:284-285, c += R_wc.col(0) * vs per voxel)
returns the bits of the sequential chain: checked on the host, compiled from
the same header, over random and edge-case starts, steps and lengths —
metre-scale rows, rows through zero, rounding ties, power-of-two steps, steps
below half an ulp, zero and subnormal values."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_closed_form_equals_sequential_chain(tmp_path):
    exe = str(tmp_path / "fstep_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe,
                    os.path.join(ROOT, "tests", "native", "fstep_check.cpp")], check=True)
    out = subprocess.run([exe, "100000"], capture_output=True, text=True)
    bad, checked = map(int, out.stdout.split()[-2:])
    assert out.returncode == 0 and bad == 0, out.stdout[-2000:]
    assert checked > 30_000_000
