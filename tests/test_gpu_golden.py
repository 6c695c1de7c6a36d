"""The CUDA library on the golden fixtures recorded from the REFERENCE's own
kernels (tests/golden/ref_golden_*.npz): every per-frame map, pyramid, image,
association and photometric correspondence must be identical to the
reference's bit for bit (float maps on valid pixels), sums within 2e-5."""
import glob
import os

import numpy as np
import pytest

from conftest import ROOT
from gpu_helpers import dev, dev_u16, new_gpu_odo, rel_close

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "ref_golden_*.npz")))


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def same_map(ours, ref):
    r = ref.reshape(3, -1)
    o = ours.reshape(3, -1)
    if not np.array_equal(np.isnan(o[0]), np.isnan(r[0])):
        return False
    ok = ~np.isnan(r[0])
    return np.array_equal(bits(o[:, ok]), bits(r[:, ok]))


def same_float(ours, ref):
    return np.array_equal(np.isnan(ours), np.isnan(ref)) and np.array_equal(bits(ours[~np.isnan(ref)]),
                                                                            bits(ref[~np.isnan(ref)]))


@pytest.fixture(scope="module", params=GOLDEN, ids=lambda p: os.path.basename(p)[11:-4])
def run(request, gpu):
    from slam_gb300 import synth
    g = dict(np.load(request.param))
    cam = synth.Camera(int(g["width"]), int(g["height"]), float(g["fx"]), float(g["fy"]), float(g["cx"]),
                       float(g["cy"]))
    odo = new_gpu_odo(cam)
    odo.initFirstRGB(dev(g["in_prev_rgba"]))
    odo.initICPModel(dev(g["in_model_vert"]), dev(g["in_model_norm"]), 20.0, g["T1"].astype(np.float32))
    odo.initRGBModel(dev(g["in_model_rgba"]))
    odo.initICP(dev_u16(g["in_depth"]), 20.0)
    odo.initRGB(dev(g["in_rgba"]))
    odo.debug_derivatives()
    return g, odo


def test_maps_and_pyramids_bit_exact(run):
    g, odo = run
    for l in range(3):
        assert np.array_equal(odo.download(0, l), g[f"depth_{l}"]), ("depth", l)
        assert same_map(odo.download(1, l), g[f"vmap_curr_{l}"]), ("vmap_curr", l)
        assert same_map(odo.download(2, l), g[f"nmap_curr_{l}"]), ("nmap_curr", l)
        assert same_map(odo.download(3, l), g[f"vmap_prev_{l}"]), ("vmap_prev", l)
        assert same_map(odo.download(4, l), g[f"nmap_prev_{l}"]), ("nmap_prev", l)
        assert same_float(odo.download(5, l), g[f"lastDepth_{l}"]), ("lastDepth", l)
        assert same_float(odo.download(6, l), g[f"nextDepth_{l}"]), ("nextDepth", l)
        assert np.array_equal(odo.download(7, l), g[f"lastImage_{l}"]), ("lastImage", l)
        assert np.array_equal(odo.download(8, l), g[f"nextImage_{l}"]), ("nextImage", l)
        assert np.array_equal(odo.download(9, l), g[f"lastnextImage_{l}"]), ("lastNextImage", l)
        assert np.array_equal(odo.download(10, l), g[f"dIdx_{l}"]), ("dIdx", l)
        assert np.array_equal(odo.download(11, l), g[f"dIdy_{l}"]), ("dIdy", l)


@pytest.mark.parametrize("level", [0, 1, 2])
def test_association_and_correspondences_bit_exact(run, level):
    from oracle.ref_runner import DATATERM
    g, odo = run
    p = g["icp_pose"]
    out, assoc = odo.debug_icp_step(level, p[0:9], p[9:12], p[12:21], p[21:24])
    found = g[f"icp_found_{level}"] == 1
    assert np.array_equal(assoc >= 0, found)
    vp = odo.download(3, level)
    idx = assoc[found]
    gathered = np.stack([vp[c].reshape(-1)[idx] for c in range(3)], axis=-1)
    assert np.array_equal(bits(gathered), bits(g[f"icp_d_{level}"][found]))
    ok, err = rel_close(out, g[f"icp_sum_{level}"], 2e-5)
    assert ok, err
    cnt, sig = odo.debug_rgb_residual(level, g[f"rgb_krk_{level}"], g[f"rgb_kt_{level}"])
    h, w = g[f"nextImage_{level}"].shape
    ref = g[f"rgb_dataterm_{level}"].view(DATATERM).reshape(h, w)
    corr = odo.download(12, level)
    valid = ref["valid"] == 1
    assert np.array_equal(corr[..., 3] == 1, valid)
    assert np.array_equal(corr[..., 0][valid], ref["zero_x"][valid])
    assert np.array_equal(corr[..., 1][valid], ref["zero_y"][valid])
    assert np.array_equal(corr[..., 2][valid].astype(np.float32), ref["diff"][valid])
    assert (cnt, sig) == (int(g[f"rgb_count_{level}"]), int(g[f"rgb_sigma_{level}"]))
    out = odo.debug_rgb_step(level, float(g[f"rgb_step_sigma_{level}"]))
    ok, err = rel_close(out, g[f"rgb_sum_{level}"], 2e-5)
    assert ok, err


def test_so3_reduction(run):
    g, odo = run
    m = g["so3_mats"]
    out = odo.debug_so3_step(m[0], m[1], m[2])
    ok, err = rel_close(out, g["so3_sum"], 2e-5)
    assert ok, err
    assert out[10] == g["so3_sum"][10]
