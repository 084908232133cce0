"""The C-ABI library builds for sm_103a, loads, and exports every function
include/azu_gpu.h declares (no GPU calls)."""
import ctypes
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib_path():
    from azu_gb300 import _abi, build
    build.build()
    return _abi.LIB_PATH


def test_library_loads(lib_path):
    lib = ctypes.CDLL(lib_path)
    lib.azu_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.azu_version()


def test_exports_every_declared_symbol(lib_path):
    from azu_gb300 import _abi
    declared = _abi.header_symbols(os.path.join(ROOT, "include", "azu_gpu.h"))
    assert len(declared) > 40
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    lib = ctypes.CDLL(lib_path)
    for s in declared:
        assert getattr(lib, s) is not None
    # every declared function has a ctypes signature in the Python binding
    assert not [s for s in declared if s not in _abi.SIGNATURES]


def test_only_sm103a_code_is_built(lib_path):
    from azu_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_no_device_returns_a_status_not_a_crash(lib_path):
    """Without a GPU every entry point returns an error code."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from azu_gb300 import _abi, api
    lib = _abi.load()
    h = ctypes.c_void_p()
    p = api.volume_params(16, 0.1, 0.3)
    rc = lib.azu_volume_create(0, ctypes.byref(p), None, ctypes.byref(h))
    assert rc in (_abi.AZU_E_INVALID, _abi.AZU_E_CUDA, _abi.AZU_E_UNSUPPORTED)
    assert lib.azu_last_error()
    assert lib.azu_volume_reset(None) == _abi.AZU_E_INVALID
    assert lib.azu_tracker_prepare_live(None, None, 640, 480) == _abi.AZU_E_INVALID


def test_synth_encoder_matches_oracle(orc):
    import numpy as np
    from azu_gb300 import synth
    mm = np.arange(0, 65536, dtype=np.uint16).reshape(256, 256)
    raw = synth.encode_raw(mm, 0.3, 2.5)
    for v in list(range(0, 3000, 7)) + [299, 300, 301, 2499, 2500, 2501, 65535]:
        assert raw.reshape(-1)[v] == orc.meters_to_raw(float(np.float32(v) * np.float32(0.001)), 0.3, 2.5), v


def test_synth_sequences_are_seeded():
    import numpy as np
    from azu_gb300 import synth
    a = synth.sequence("c1", frames=2)
    b = synth.sequence("c1", frames=2)
    assert np.array_equal(a.depth_mm, b.depth_mm)
    assert np.allclose(a.poses[0], np.eye(4))
    v = a.depth_mm[0]
    assert 0.3 < (v > 0).mean() < 0.9


def test_header_compiles_as_c_and_cxx_and_links(lib_path, tmp_path):
    """A C program and a C++ program including include/azu_gpu.h link against the
    library (the reference-side adapters are C++)."""
    src = tmp_path / "use.c"
    src.write_text('#include "azu_gpu.h"\n#include <stdio.h>\n'
                   'int main(void) { azu_volume* v = 0; azu_volume_params p = {0};\n'
                   '  int rc = azu_volume_create(0, &p, 0, &v);\n'
                   '  printf("%s %d\\n", azu_version(), rc == AZU_E_INVALID); return 0; }\n')
    inc = os.path.join(ROOT, "include")
    libdir = os.path.dirname(lib_path)
    for cc, extra in (("gcc", ["-std=c99"]), ("g++", ["-std=c++17", "-x", "c++"])):
        exe = tmp_path / ("use_" + cc.replace("+", "x"))
        subprocess.run([cc] + extra + ["-Wall", "-Werror", "-I", inc, str(src), "-L", libdir, "-lazu_gb300",
                                        "-Wl,-rpath," + libdir, "-o", str(exe)], check=True)
        out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
        assert "sm_103a" in out and out.strip().endswith("1")
