"""Known-answer tests of the CPU oracle against values derived by hand from
the reference's formulas (src/odom/utils.cu, src/odom/reduce.cu,
src/odom/RGBDOdometryef.cpp), plus FP32/FP64 twin agreement.  CPU only."""
import math

import numpy as np
import pytest

from conftest import ANGLE_THRESH, DIST_THRESH

FX, FY, CX, CY = 525.0, 525.0, 319.5, 239.5


@pytest.fixture(scope="module")
def orc(built):
    from oracle import oracle
    return oracle


def test_pyr_down_depth_constant_and_edge(orc):
    # utils.cu:57-94: weights accepted only within 3*sigma_color = 90 mm of the centre
    d = np.full((16, 16), 1000, np.uint16)
    assert np.all(orc.pyr_down_depth(d) == 1000)
    d[:, 8:] = 2000  # a step edge larger than 90 mm is never blended
    out = orc.pyr_down_depth(d)
    assert np.all(out[:, :4] == 1000) and np.all(out[:, 4:] == 2000)
    d[:, 8:] = 1050  # within 90 mm: blended
    out = orc.pyr_down_depth(d)
    assert out[4, 3] > 1000 and out[4, 4] < 1050


def test_create_vmap_formula_and_invalid_x_plane(orc):
    k = orc.Kernels(32)
    d = np.zeros((4, 6), np.uint16)
    d[1, 2] = 1500
    d[2, 3] = 25000  # beyond the cutoff
    init = np.full((3, 4, 6), 7.0, np.float32)
    v = k.create_vmap(d, FX, FY, CX, CY, 20.0, init=init)
    z = np.float32(1500) / np.float32(1000)
    fxi = np.float32(1.0) / np.float32(FX)
    assert v[0, 1, 2] == np.float32(z * (np.float32(2) - np.float32(CX))) * fxi
    assert v[2, 1, 2] == z
    assert np.isnan(v[0, 0, 0]) and np.isnan(v[0, 2, 3])
    # y/z planes of invalid pixels keep stale contents (utils.cu:130)
    assert v[1, 0, 0] == 7.0 and v[2, 2, 3] == 7.0


def test_create_nmap_plane(orc):
    k = orc.Kernels(32)
    d = np.full((8, 8), 2000, np.uint16)
    v = k.create_vmap(d, FX, FY, CX, CY, 20.0)
    n = k.create_nmap(v)
    assert np.allclose(n[:, :7, :7].reshape(3, -1).T, [0, 0, 1], atol=1e-6)
    assert np.all(np.isnan(n[0, 7, :])) and np.all(np.isnan(n[0, :, 7]))


def test_intensity_weights_are_swapped_rgba(orc):
    # utils.cu:560: 0.114 * byte0 + 0.299 * byte1 + 0.587 * byte2 on RGBA input
    px = np.array([[[255, 0, 0, 255], [0, 255, 0, 255], [0, 0, 255, 255], [100, 100, 100, 255]]], np.uint8)
    assert list(orc.bgr_to_intensity(px)[0]) == [29, 76, 149, 100]


def test_uchar_gauss_constant_and_zero(orc):
    assert np.all(orc.pyr_down_uchar_gauss(np.full((12, 12), 100, np.uint8)) == 100)
    assert np.all(orc.pyr_down_uchar_gauss(np.zeros((12, 12), np.uint8)) == 0)  # 0/0 -> 0


def test_derivatives_ramp(orc):
    img = np.tile((np.arange(16) * 10).astype(np.uint8), (8, 1))
    dx, dy = orc.derivatives(img)
    # interior: (0.52201 + 0.79451 + 0.52201) * (I(x+1) - I(x-1)) = 36.77 -> 36
    assert np.all(dx[1:-1, 1:-1] == 36) and np.all(dy[1:-1, 1:-1] == 0)


def test_resize_nan_propagation(orc):
    k = orc.Kernels(32)
    m = np.ones((3, 4, 4), np.float32)
    m[0, 0, 0] = np.nan
    out = k.resize_map(m, normalize=False)
    assert np.isnan(out[0, 0, 0]) and out[0, 1, 1] == 1.0
    outn = k.resize_map(m, normalize=True)
    assert abs(outn[0, 1, 1] - 1 / math.sqrt(3)) < 1e-6


def test_icp_identity_plane(orc):
    k = orc.Kernels(32)
    d = np.full((24, 32), 2000, np.uint16)
    v = k.create_vmap(d, FX / 8, FY / 8, CX / 8, CY / 8, 20.0)
    n = k.create_nmap(v)
    I = np.eye(3, dtype=np.float32)
    z = np.zeros(3, np.float32)
    out, assoc, tie = k.icp_step(I, z, v, n, I, z, FX / 8, FY / 8, CX / 8, CY / 8, v, n, DIST_THRESH, ANGLE_THRESH)
    valid = ~np.isnan(n[0])
    idx = np.arange(24 * 32).reshape(24, 32)
    assert np.all(assoc[valid] == idx[valid]) and np.all(assoc[~valid] == -1)
    assert out[28] == valid.sum()  # inliers
    assert out[27] == 0.0  # residual: s == d
    # JtJ upper triangle order aa..ag, bb..: cc (n_z^2) is entry 13
    assert abs(out[13] - valid.sum()) < 1e-3


def test_rgb_residual_identity_has_zero_diff(orc):
    k = orc.Kernels(32)
    rng = np.random.default_rng(0)
    img = rng.integers(1, 255, size=(30, 40)).astype(np.uint8)
    depth = np.full((30, 40), 1.5, np.float32)
    dx, dy = orc.derivatives(img)
    krk = np.eye(3, dtype=np.float32)
    corres, (cnt, sig), tie = k.rgb_residual(0.0, dx, dy, depth, depth, img, img, 0.07, np.zeros(3), krk)
    assert cnt > 0 and sig == 0
    v = corres[corres["valid"] == 1]
    assert np.all(v["zero_x"] == v["one_x"]) and np.all(v["zero_y"] == v["one_y"])
    # window/gate rules: j0 < cols - 5 and i < rows - 1 (reduce.cu:782)
    assert not np.any(corres["valid"][:, 35:]) and not np.any(corres["valid"][29, :])


def test_ldlt_matches_numpy_and_pseudo_inverse(orc):
    rng = np.random.default_rng(1)
    M = rng.normal(size=(6, 6))
    A = M @ M.T + 6 * np.eye(6)
    b = rng.normal(size=6)
    assert np.allclose(orc.ldlt_solve6(A, b), np.linalg.solve(A, b), rtol=1e-12, atol=1e-12)
    Z = np.zeros((6, 6))
    assert np.all(orc.ldlt_solve6(Z, b) == 0)  # zero pivots -> 0 (pseudo-inverse of D)


def test_rodrigues(orc):
    from slam_gb300.synth import rotvec_to_R
    w = np.array([0.01, -0.02, 0.03])
    assert np.allclose(orc.rodrigues(w), rotvec_to_R(w), atol=1e-15)
    assert np.all(orc.rodrigues(np.zeros(3)) == np.eye(3))


def _track(orc, pair, prec, **kw):
    cam = pair["cam"]
    o = orc.Odometry(cam.width, cam.height, cam.cx, cam.cy, cam.fx, cam.fy, DIST_THRESH, ANGLE_THRESH, prec=prec)
    T1 = pair["T1"]
    o.initFirstRGB(pair["prev_rgba"])
    o.initICPModel(pair["model_vert"], pair["model_norm"], 20.0, T1)
    o.initRGBModel(pair["model_rgba"])
    o.initICP(pair["depth"], 20.0)
    o.initRGB(pair["rgba"])
    t, R = o.getIncrementalTransformation(T1[:3, 3], T1[:3, :3], **kw)
    return t.astype(np.float64), R.astype(np.float64), o


def test_fp32_and_fp64_twins_agree(orc):
    from slam_gb300 import synth
    pair = synth.make_pair(5, cam=synth.Camera().scaled(320, 240))
    t32, R32, _ = _track(orc, pair, 32)
    t64, R64, _ = _track(orc, pair, 64)
    rot, tr = synth.pose_error(synth.pose(R32, t32), synth.pose(R64, t64))
    assert rot < 1e-4 and tr < 1e-4


def test_icp_only_recovers_noise_free_motion(orc):
    from slam_gb300 import synth
    cam = synth.Camera().scaled(320, 240)
    rng = np.random.default_rng(11)
    scene = synth.make_room(11)
    T1 = synth.room_camera(rng)
    T2 = T1 @ synth.random_motion(rng, 2.0, 0.02)
    model = synth.render(scene, T1, cam, depth=False, model=True)
    live = synth.render(scene, T2, cam, noise_k=0.0, dropout=0.0)
    pair = {"cam": cam, "T1": T1, "model_vert": model["vert"], "model_norm": model["norm"],
            "model_rgba": model["rgba"], "depth": live["depth"], "rgba": live["rgba"], "prev_rgba": model["rgba"]}
    t, R, o = _track(orc, pair, 64, rgbOnly=False, icpWeight=100.0, pyramid=True, fastOdom=False, so3=False)
    rot, tr = synth.pose_error(synth.pose(R, t), T2)
    assert rot < 1e-4 and tr < 2e-4  # limited by mm depth quantisation
    assert o.iterations() == [0, 10, 5, 4]
