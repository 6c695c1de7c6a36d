"""Pins the CPU oracle against golden fixtures recorded from the REFERENCE's own
kernels (tests/golden/make_ref_golden.py ran src/odom/utils.cu and
src/odom/reduce.cu, compiled unmodified, on a GB300).  CPU only.

Each oracle stage runs on the reference's inputs for that stage.  Integer and
index outputs must match except on pixels the oracle flags as rounding ties
(the reference divides with --prec-div=false); float maps match to a few ulp;
sums to 2e-5 relative (summation order differs)."""
import glob
import os

import numpy as np
import pytest

from conftest import ANGLE_THRESH, DIST_THRESH, ROOT

GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "ref_golden_*.npz")))


def level_intr(g, l):
    d = np.float32(1 << l)
    return tuple(float(np.float32(g[k]) / d) for k in ("fx", "fy", "cx", "cy"))


def planar(a):
    h3, w = a.shape
    return a.reshape(3, h3 // 3, w)


def close_map(ours, ref, rtol, atol=0.0):
    assert np.array_equal(np.isnan(ours[0]), np.isnan(ref[0]))
    ok = ~np.isnan(ref[0])
    return np.allclose(ours[:, ok], ref[:, ok], rtol=rtol, atol=atol)


def rel_close(a, b, rtol):
    return np.abs(np.asarray(a) - np.asarray(b)).max() <= rtol * max(np.abs(b).max(), 1e-30)


@pytest.fixture(scope="module", params=GOLDEN, ids=lambda p: os.path.basename(p)[11:-4])
def g(request):
    return dict(np.load(request.param))


@pytest.fixture(scope="module")
def orc(built):
    from oracle import oracle
    return oracle


def test_golden_fixtures_present():
    assert len(GOLDEN) >= 2


def test_depth_vertex_normal_maps(g, orc):
    k = orc.Kernels(32)
    for l in range(3):
        if l > 0:
            d = orc.pyr_down_depth(g[f"depth_{l - 1}"])
            diff = np.abs(d.astype(np.int32) - g[f"depth_{l}"].astype(np.int32))
            assert diff.max() <= 1 and (diff > 0).mean() < 2e-3, (l, int((diff > 0).sum()))
        fx, fy, cx, cy = level_intr(g, l)
        v = k.create_vmap(g[f"depth_{l}"], fx, fy, cx, cy, 20.0)
        assert close_map(v, planar(g[f"vmap_curr_{l}"]), rtol=2.4e-6), l
        n = k.create_nmap(planar(g[f"vmap_curr_{l}"]))
        assert close_map(n, planar(g[f"nmap_curr_{l}"]), rtol=0, atol=2e-6), l


def test_model_maps(g, orc):
    k = orc.Kernels(32)
    vm, nm = k.copy_maps(g["in_model_vert"], g["in_model_norm"])
    raw = [(vm, nm)]
    for l in (1, 2):
        raw.append((k.resize_map(raw[-1][0], False), k.resize_map(raw[-1][1], True)))
    T1 = g["T1"].astype(np.float32)
    for l in range(3):
        v, n = k.transform_maps(raw[l][0], raw[l][1], T1[:3, :3], T1[:3, 3])
        assert close_map(v, planar(g[f"vmap_prev_{l}"]), rtol=1e-6, atol=1e-6), l
        assert close_map(n, planar(g[f"nmap_prev_{l}"]), rtol=1e-6, atol=1e-6), l


def test_photometric_pyramids_and_derivatives(g, orc):
    k = orc.Kernels(32)
    d0 = k.vertices_to_depth(g["in_model_vert"])
    ref0 = g["lastDepth_0"]
    assert np.array_equal(np.isnan(d0), np.isnan(ref0)) and np.array_equal(d0[~np.isnan(d0)], ref0[~np.isnan(d0)])
    for name, src in (("last", "in_model_rgba"), ("next", "in_rgba"), ("lastnext", "in_prev_rgba")):
        img, tie = orc.bgr_to_intensity(g[src], with_tie=True)
        mism = img != g[f"{name}Image_0"]
        assert np.all(tie[mism] != 0), (name, int((mism & (tie == 0)).sum()))
        for l in (1, 2):
            img, tie = orc.pyr_down_uchar_gauss(g[f"{name}Image_{l - 1}"], with_tie=True)
            mism = img != g[f"{name}Image_{l}"]
            assert np.all(tie[mism] != 0), (name, l, int((mism & (tie == 0)).sum()))
    for l in (1, 2):
        d = k.pyr_down_gauss_f(g[f"lastDepth_{l - 1}"])
        r = g[f"lastDepth_{l}"]
        assert np.array_equal(np.isnan(d), np.isnan(r))
        assert np.allclose(d[~np.isnan(r)], r[~np.isnan(r)], rtol=2.5e-7, atol=0)
    for l in range(3):
        dx, dy, tie = orc.derivatives(g[f"nextImage_{l}"], with_tie=True)
        mism = (dx != g[f"dIdx_{l}"]) | (dy != g[f"dIdy_{l}"])
        assert np.all(tie[mism] != 0), (l, int((mism & (tie == 0)).sum()))


@pytest.mark.parametrize("level", [0, 1, 2])
def test_icp_association(g, orc, level):
    k = orc.Kernels(32)
    fx, fy, cx, cy = level_intr(g, level)
    p = g["icp_pose"]
    out, assoc, tie = k.icp_step(p[0:9], p[9:12], planar(g[f"vmap_curr_{level}"]), planar(g[f"nmap_curr_{level}"]),
                                 p[12:21], p[21:24], fx, fy, cx, cy, planar(g[f"vmap_prev_{level}"]),
                                 planar(g[f"nmap_prev_{level}"]), DIST_THRESH, ANGLE_THRESH)
    found = g[f"icp_found_{level}"] == 1
    mism = (assoc >= 0) != found
    assert np.all(tie[mism] != 0), int((mism & (tie == 0)).sum())
    # gathered model vertex of every correspondence
    vp = planar(g[f"vmap_prev_{level}"])
    both = (assoc >= 0) & found
    idx = assoc[both]
    gathered = np.stack([vp[c].reshape(-1)[idx] for c in range(3)], axis=-1)
    assert np.array_equal(gathered, g[f"icp_d_{level}"][both])
    if not mism.any():
        assert rel_close(out, g[f"icp_sum_{level}"], 2e-5)


@pytest.mark.parametrize("level", [0, 1, 2])
def test_photometric_residual_and_reduction(g, orc, level):
    from oracle.oracle import DATATERM_DTYPE
    from oracle.ref_runner import DATATERM
    k = orc.Kernels(32)
    fx, fy, cx, cy = level_intr(g, level)
    minScale = float(np.float32([5, 3, 1][level] ** 2 / 0.125 ** 2))
    corres, (cnt, sig), tie = k.rgb_residual(minScale, g[f"dIdx_{level}"], g[f"dIdy_{level}"],
                                             g[f"lastDepth_{level}"], g[f"nextDepth_{level}"],
                                             g[f"lastImage_{level}"], g[f"nextImage_{level}"], 0.07,
                                             g[f"rgb_kt_{level}"], g[f"rgb_krk_{level}"])
    h, w = g[f"nextImage_{level}"].shape
    ref = g[f"rgb_dataterm_{level}"].view(DATATERM).reshape(h, w)
    valid = ref["valid"] == 1
    mism = ((corres["valid"] == 1) != valid) | (valid & ((corres["zero_x"] != ref["zero_x"]) |
                                                         (corres["zero_y"] != ref["zero_y"]) |
                                                         (corres["diff"] != ref["diff"])))
    assert np.all(tie[mism] != 0), int((mism & (tie == 0)).sum())
    if not mism.any():
        assert (cnt, sig) == (int(g[f"rgb_count_{level}"]), int(g[f"rgb_sigma_{level}"]))
    # reduction over the reference's correspondences
    dt = np.zeros((h, w), DATATERM_DTYPE)
    for f in ("zero_x", "zero_y", "one_x", "one_y", "diff"):
        dt[f] = ref[f]
    dt["valid"] = ref["valid"]
    cloud = k.project_cloud(g[f"lastDepth_{level}"], fx, fy, cx, cy)
    out = k.rgb_step(dt, float(g[f"rgb_step_sigma_{level}"]), cloud, fx, fy, g[f"dIdx_{level}"], g[f"dIdy_{level}"])
    assert rel_close(out, g[f"rgb_sum_{level}"], 2e-5)


def test_so3_reduction(g, orc):
    m = g["so3_mats"]
    out = orc.Kernels(32).so3_step(g["lastnextImage_2"], g["nextImage_2"], m[0], m[1], m[2])
    assert rel_close(out, g["so3_sum"], 2e-5)
    assert out[10] == g["so3_sum"][10]
