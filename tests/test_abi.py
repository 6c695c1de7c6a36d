"""The C-ABI library loads and exports every symbol include/slam_gb300.h
declares; argument validation happens before any CUDA call (no GPU needed)."""
import ctypes
import os
import re

from conftest import ROOT


def header_functions():
    text = open(os.path.join(ROOT, "include", "slam_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(odo_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_reference_surface():
    fns = header_functions()
    for name in ["odo_create", "odo_destroy", "odo_init_icp_depth", "odo_init_icp_maps", "odo_init_icp_model",
                 "odo_init_rgb", "odo_init_rgb_model", "odo_init_first_rgb", "odo_get_incremental_transformation",
                 "odo_get_covariance", "odo_get_stats"]:
        assert name in fns


def test_library_exports_every_declared_symbol(built):
    from slam_gb300 import _native
    lib = ctypes.CDLL(_native.lib_path())
    missing = [f for f in header_functions() if not hasattr(lib, f)]
    assert not missing, missing


def test_python_signatures_cover_header(built):
    from slam_gb300 import _native
    declared = {s[0] for s in _native.SIGNATURES}
    assert set(header_functions()) <= declared


def test_argument_validation_without_gpu(built):
    from slam_gb300 import _native
    L = _native.load()
    h = ctypes.c_void_p()
    # sizes are checked before the CUDA runtime is touched
    assert L.odo_create(0, 480, 319.5, 239.5, 525.0, 525.0, 0.1, 0.34, ctypes.byref(h)) == 1
    assert L.odo_create(640, 480, 319.5, 239.5, 0.0, 525.0, 0.1, 0.34, ctypes.byref(h)) == 1
    assert L.odo_create(640, 480, 319.5, 239.5, 525.0, 525.0, 0.1, 0.34, None) == 1
    assert L.odo_destroy(None) == 1
    assert L.odo_get_stats(None, None) == 1
    assert L.odo_status_string(0) == b"ok"
    assert L.odo_status_string(5) == b"device-side wait timed out"
