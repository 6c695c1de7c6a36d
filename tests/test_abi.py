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


def test_noalloc_extent_checks_without_gpu(built):
    """The allocation-free entry point refuses oversized images and maps
    whose 3 x rows x pitch reaches 4 GiB (its kernels use 32-bit byte
    offsets) before any CUDA call: the map pointers here are never read."""
    from slam_gb300 import _native
    L = _native.load()
    fake = ctypes.c_void_p(256)
    f = lambda n, v=0.0: (ctypes.c_float * n)(*([v] * n))
    out = lambda n: (ctypes.c_float * n)()

    def call(pitch, cols, rows):
        return L.odo_icp_step_noalloc(fake, fake, fake, fake, pitch, cols, rows, f(4, 1.0), 0.1, 0.34, f(9), f(3),
                                      f(9), f(3), None, out(36), out(6), out(2))
    ODO_ERR_ARG, ODO_ERR_SIZE = 1, 6
    assert call(640 * 4 - 4, 640, 480) == ODO_ERR_ARG             # pitch below one row
    assert call(2048 * 4, 2048, 1024) == ODO_ERR_SIZE              # more than ODO_NOALLOC_MAX_PIXELS
    assert call(1 << 31, 640, 480) == ODO_ERR_SIZE                 # 3 x 480 x 2 GiB >= 4 GiB
    assert call((1 << 32) // (3 * 480) + 4, 640, 480) == ODO_ERR_SIZE


def test_default_thresholds_match_reference_expression():
    """ODO_DEFAULT_ANGLE_THRESH is sin(20.f * 3.14159254f / 180.f) rounded to
    float, as the reference evaluates its default (src/odom/RGBDOdometryef.h:36),
    bit for bit; the Python side uses the same value."""
    import re
    import numpy as np
    from slam_gb300 import DEFAULT_ANGLE_THRESH, DEFAULT_DIST_THRESH
    hdr = open(os.path.join(ROOT, "include", "slam_gb300.h")).read()
    ang = float(re.search(r"#define ODO_DEFAULT_ANGLE_THRESH ([0-9.]+)f", hdr).group(1))
    dist = float(re.search(r"#define ODO_DEFAULT_DIST_THRESH ([0-9.]+)f", hdr).group(1))
    x = np.float32(np.float32(20.0) * np.float32(3.14159254)) / np.float32(180.0)
    assert np.float32(ang) == np.float32(np.sin(np.float64(x))) == np.float32(DEFAULT_ANGLE_THRESH)
    assert np.float32(dist) == np.float32(0.10) == np.float32(DEFAULT_DIST_THRESH)
