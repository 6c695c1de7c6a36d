"""GPU parity: every kernel of the tracking path against the CPU oracle on the
same inputs, and whole tracking calls against the oracle's host loop.

Integer and index outputs must be identical; a mismatch is accepted only on a
pixel the oracle flags as a rounding tie (a quotient or threshold within a few
ulp of the decision boundary, where the GPU's --prec-div=false division may
round the other way).  Floating-point maps and sums are compared with the
tolerances written in each test.  Poses: 1e-5 rad / 1e-5 m."""
import numpy as np
import pytest

from conftest import ANGLE_THRESH, DIST_THRESH
from gpu_helpers import (POSE_TOL_M, POSE_TOL_RAD, OracleRuns, check_pose, corr_to_dataterm, dev, frame_runs,
                         gpu_images, intr, load_frame, new_gpu_odo, new_oracle_odo, pose_diff, rel_close, set_images,
                         track)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def orc(built):
    from oracle import oracle
    return oracle


@pytest.fixture(scope="module", params=[(640, 480), (90, 66), (80, 60)], ids=["640x480", "90x66", "80x60"])
def pair640(gpu, request):
    """The per-kernel parity pair: 640x480 (the reference's configuration)
    and two small sizes whose coarsest level is a few hundred pixels."""
    from slam_gb300 import synth
    w, h = request.param
    return synth.make_pair(3, cam=synth.Camera().scaled(w, h))


@pytest.fixture(scope="module")
def loaded(pair640):
    odo = new_gpu_odo(pair640["cam"])
    load_frame(odo, pair640)
    odo.debug_derivatives()
    return odo


def _nan_mask_equal(a, b):
    return np.array_equal(np.isnan(a), np.isnan(b))


def test_depth_pyramid(loaded, orc):
    for l in (1, 2):
        src = loaded.download(0, l - 1)
        got = loaded.download(0, l)
        exp = orc.pyr_down_depth(src)
        diff = np.abs(got.astype(np.int32) - exp.astype(np.int32))
        # sum/wall is exact in FP32; the approximate division may truncate an
        # exact-integer quotient one lower
        assert diff.max() <= 1 and (diff > 0).mean() < 1e-3, (l, diff.max(), (diff > 0).sum())


def test_vertex_and_normal_maps(loaded, orc, pair640):
    k = orc.Kernels(32)
    cam = pair640["cam"]
    for l in range(3):
        fx, fy, cx, cy = intr(cam, l)
        depth = loaded.download(0, l)
        v = loaded.download(1, l)
        n = loaded.download(2, l)
        ve = k.create_vmap(depth, fx, fy, cx, cy, 20.0)
        assert _nan_mask_equal(v[0], ve[0]), l
        ok = ~np.isnan(ve[0])
        assert np.allclose(v[:, ok], ve[:, ok], rtol=3e-7 * 8, atol=0), l
        ne = k.create_nmap(v)  # the oracle's normals from the GPU's vertices
        assert _nan_mask_equal(n[0], ne[0]), l
        ok = ~np.isnan(ne[0])
        assert np.abs(n[:, ok] - ne[:, ok]).max() < 2e-6, l  # rsqrtf approximation


def test_model_maps(loaded, orc, pair640):
    k = orc.Kernels(32)
    T1 = pair640["T1"].astype(np.float32)
    vm, nm = k.copy_maps(pair640["model_vert"], pair640["model_norm"])
    raw = [(vm, nm)]
    for l in (1, 2):
        raw.append((k.resize_map(raw[-1][0], False), k.resize_map(raw[-1][1], True)))
    for l in range(3):
        ve, ne = k.transform_maps(raw[l][0], raw[l][1], T1[:3, :3], T1[:3, 3])
        v = loaded.download(3, l)
        n = loaded.download(4, l)
        assert _nan_mask_equal(v[0], ve[0]) and _nan_mask_equal(n[0], ne[0]), l
        ok = ~np.isnan(ve[0])
        assert np.allclose(v[:, ok], ve[:, ok], rtol=1e-6, atol=1e-6), l
        ok = ~np.isnan(ne[0])
        assert np.allclose(n[:, ok], ne[:, ok], rtol=1e-6, atol=1e-6), l


def test_photometric_pyramids(loaded, orc, pair640):
    k = orc.Kernels(32)
    # level 0: depth from the model vertices (cut at 6 m), intensity from RGBA
    assert np.array_equal(np.isnan(loaded.download(5, 0)), np.isnan(k.vertices_to_depth(pair640["model_vert"])))
    got = loaded.download(7, 0)
    exp, tie = orc.bgr_to_intensity(pair640["model_rgba"], with_tie=True)
    mism = got != exp
    assert np.all(tie[mism] != 0), int((mism & (tie == 0)).sum())
    for which_d, which_i in ((5, 7), (6, 8)):
        for l in (1, 2):
            dsrc = loaded.download(which_d, l - 1)
            dgot = loaded.download(which_d, l)
            dexp = k.pyr_down_gauss_f(dsrc)
            assert _nan_mask_equal(dgot, dexp), (which_d, l)
            ok = ~np.isnan(dexp)
            assert np.allclose(dgot[ok], dexp[ok], rtol=2.5e-7, atol=0), (which_d, l)
            igot = loaded.download(which_i, l)
            iexp, tie = orc.pyr_down_uchar_gauss(loaded.download(which_i, l - 1), with_tie=True)
            mism = igot != iexp
            assert np.all(tie[mism] != 0), (which_i, l, int((mism & (tie == 0)).sum()))


def test_derivative_images(loaded, orc):
    for l in range(3):
        img = loaded.download(8, l)
        dx, dy, tie = orc.derivatives(img, with_tie=True)
        gx, gy = loaded.download(10, l), loaded.download(11, l)
        mism = (gx != dx) | (gy != dy)
        assert np.all(tie[mism] != 0), (l, int((mism & (tie == 0)).sum()))


def _poses(pair, perturb):
    from slam_gb300 import synth
    T1 = pair["T1"]
    Tc = T1 @ synth.random_motion(np.random.default_rng(perturb), 1.0, 0.01)
    Rc, tc = Tc[:3, :3].astype(np.float32), Tc[:3, 3].astype(np.float32)
    Rp, tp = T1[:3, :3].astype(np.float32), T1[:3, 3].astype(np.float32)
    Rpi = np.linalg.inv(Rp.astype(np.float64)).astype(np.float32)
    return Rc, tc, Rpi, tp


@pytest.mark.parametrize("level", [0, 1, 2])
def test_icp_association_and_sums(loaded, orc, pair640, level):
    k = orc.Kernels(32)
    cam = pair640["cam"]
    fx, fy, cx, cy = intr(cam, level)
    vc, nc, vp, np_ = (loaded.download(w, level) for w in (1, 2, 3, 4))
    for perturb in (1, 2):
        Rc, tc, Rpi, tp = _poses(pair640, perturb)
        out_g, assoc_g = loaded.debug_icp_step(level, Rc, tc, Rpi, tp)
        out_e, assoc_e, tie = k.icp_step(Rc, tc, vc, nc, Rpi, tp, fx, fy, cx, cy, vp, np_, DIST_THRESH,
                                         ANGLE_THRESH)
        mism = assoc_g != assoc_e
        assert np.all(tie[mism] != 0), (level, int(mism.sum()), int((mism & (tie == 0)).sum()))
        assert (assoc_e >= 0).sum() > 0.02 * assoc_e.size
        if not mism.any():
            ok, err = rel_close(out_g, out_e, 2e-5)
            assert ok, (level, err)
            assert out_g[28] == out_e[28]


@pytest.mark.parametrize("level", [0, 1, 2])
def test_rgb_residual_and_step(loaded, orc, pair640, level):
    from slam_gb300 import synth
    from slam_gb300.odometry import RGBDOdometry
    k = orc.Kernels(32)
    cam = pair640["cam"]
    fx, fy, cx, cy = intr(cam, level)
    # warp of a small motion, as getIncrementalTransformation builds it
    T = synth.random_motion(np.random.default_rng(7), 1.0, 0.01)
    K = np.array([[fx, 0, cx], [0, fy, cy], [0, 0, 1.0]])
    krk = (K @ T[:3, :3] @ np.linalg.inv(K)).astype(np.float32)
    kt = (K @ T[:3, 3]).astype(np.float32)
    minScale = float(np.float32([5, 3, 1][level] ** 2 / 0.125 ** 2))
    cnt_g, sig_g = loaded.debug_rgb_residual(level, krk, kt)
    corr_g = loaded.download(12, level)
    dIdx, dIdy = loaded.download(10, level), loaded.download(11, level)
    ld, nd = loaded.download(5, level), loaded.download(6, level)
    li, ni = loaded.download(7, level), loaded.download(8, level)
    corres_e, (cnt_e, sig_e), tie = k.rgb_residual(minScale, dIdx, dIdy, ld, nd, li, ni, 0.07, kt, krk)
    valid_g = corr_g[..., 3] == 1
    valid_e = corres_e["valid"] == 1
    mism = (valid_g != valid_e) | (valid_e & ((corr_g[..., 0] != corres_e["zero_x"]) |
                                              (corr_g[..., 1] != corres_e["zero_y"]) |
                                              (corr_g[..., 2] != corres_e["diff"].astype(np.int16))))
    assert np.all(tie[mism] != 0), (level, int(mism.sum()), int((mism & (tie == 0)).sum()))
    assert valid_e.sum() > 0.01 * valid_e.size
    if not mism.any():
        assert (cnt_g, sig_g) == (cnt_e, sig_e)
    # photometric reduction on the GPU's correspondences
    sigma = float(np.float32(np.sqrt(cnt_g)))
    out_g = loaded.debug_rgb_step(level, sigma)
    cloud = k.project_cloud(ld, fx, fy, cx, cy)
    out_e = k.rgb_step(corr_to_dataterm(corr_g), sigma, cloud, fx, fy, dIdx, dIdy)
    ok, err = rel_close(out_g, out_e, 2e-5)
    assert ok, (level, err)
    assert out_g[28] == out_e[28] == valid_g.sum()


def test_so3_step(loaded, orc, pair640):
    from slam_gb300 import synth
    cam = pair640["cam"]
    fx, fy, cx, cy = intr(cam, 2)
    K = np.array([[fx, 0, cx], [0, fy, cy], [0, 0, 1.0]])
    R = synth.rotvec_to_R([0.004, -0.006, 0.002])
    H = (K @ R @ np.linalg.inv(K)).astype(np.float32)
    kinv = np.linalg.inv(K).astype(np.float32)
    krlr = (K @ R).astype(np.float32)
    out_g = loaded.debug_so3_step(H, kinv, krlr)
    out_e = orc.Kernels(32).so3_step(loaded.download(9, 2), loaded.download(8, 2), H, kinv, krlr)
    ok, err = rel_close(out_g, out_e, 2e-5)
    assert ok, err
    assert out_g[10] == out_e[10]


FLAGS = [
    dict(),
    dict(so3=False),
    dict(icpWeight=100.0, so3=False),
    dict(rgbOnly=True, so3=False),
    dict(fastOdom=True),
    dict(pyramid=False, so3=False),
]


@pytest.mark.parametrize("seed", [3, 8])
@pytest.mark.parametrize("flags", FLAGS, ids=lambda f: ",".join(f"{k}={v}" for k, v in f.items()) or "default")
def test_tracking_matches_oracle(gpu, orc, seed, flags):
    from slam_gb300 import synth
    pair = synth.make_pair(seed)
    g = new_gpu_odo(pair["cam"])
    load_frame(g, pair)
    images = gpu_images(g)
    tg, Rg = track(g, pair, **flags)
    ref = frame_runs(pair, flags, images=images)
    to, Ro, o = ref.main
    label = "tracking seed %d %s" % (seed, ",".join(f"{k}={v}" for k, v in flags.items()) or "default")
    _, _, flat = check_pose(label, tg, Rg, to, Ro, ref.tolerance)
    assert ref.iterations_ok(g.iterations()), (g.iterations(), o.iterations())
    st = o.stats
    assert ref.count_ok("lastICPCount", g.lastICPCount, flat)
    assert ref.count_ok("lastRGBCount", g.lastRGBCount, flat)
    ok, err = ref.jtj_ok(g.lastA, flat)
    assert ok, err


def test_modes_and_determinism(gpu, pair640):
    from slam_gb300 import MODE_GRAPH, MODE_PERSISTENT, MODE_STREAM
    res = {}
    for mode in (MODE_GRAPH, MODE_STREAM, MODE_PERSISTENT, MODE_GRAPH):
        g = new_gpu_odo(pair640["cam"])
        g.set_mode(mode)
        load_frame(g, pair640)
        res.setdefault(mode, []).append(track(g, pair640))
    (tg, Rg), (tg2, Rg2) = res[MODE_GRAPH]
    assert np.array_equal(tg, tg2) and np.array_equal(Rg, Rg2)  # run-to-run identical
    ts, Rs = res[MODE_STREAM][0]
    assert np.array_equal(tg, ts) and np.array_equal(Rg, Rs)  # same kernels, same sums
    tp, Rp = res[MODE_PERSISTENT][0]
    # same grid and pass bodies, same summation order: identical bits
    assert np.array_equal(tg, tp) and np.array_equal(Rg, Rp)


def test_compensated_precision_close(gpu, pair640):
    from slam_gb300 import PREC_COMPENSATED
    g = new_gpu_odo(pair640["cam"])
    load_frame(g, pair640)
    t0, R0 = track(g, pair640)
    g2 = new_gpu_odo(pair640["cam"])
    g2.set_precision(PREC_COMPENSATED)
    load_frame(g2, pair640)
    t1, R1 = track(g2, pair640)
    rot, tr = pose_diff(t0, R0, t1, R1)
    assert rot < 1e-5 and tr < 1e-5


def test_sequence_with_image_swap(gpu, orc):
    """Three consecutive frames: lastNextImage/nextImage swap after each SO3
    call (src/odom/RGBDOdometryef.cpp:585-591)."""
    from slam_gb300 import synth
    cam = synth.Camera().scaled(320, 240)
    scene = synth.make_room(21)
    rng = np.random.default_rng(21)
    T = [synth.room_camera(rng)]
    for _ in range(3):
        T.append(T[-1] @ synth.random_motion(rng, 1.5, 0.03))
    g = new_gpu_odo(cam)
    o = new_oracle_odo(cam)
    first = synth.render(scene, T[0], cam, noise_seed=100)
    g.initFirstRGB(dev(first["rgba"]))
    o.initFirstRGB(first["rgba"])
    start = (T[0][:3, 3].astype(np.float32), T[0][:3, :3].astype(np.float32))
    for k in range(1, 4):
        model = synth.render(scene, T[k - 1], cam, depth=False, model=True)
        live = synth.render(scene, T[k], cam, noise_seed=100 + k)
        pair = {"cam": cam, "T1": T[k - 1], "model_vert": model["vert"], "model_norm": model["norm"],
                "model_rgba": model["rgba"], "depth": live["depth"], "rgba": live["rgba"]}
        load_frame(g, pair, first=False)
        load_frame(o, pair, first=False)
        images = gpu_images(g)  # includes the swapped lastNextImage
        set_images(o, images)
        pg = g.getIncrementalTransformation(start[0], start[1])
        po = o.getIncrementalTransformation(start[0], start[1])

        def load(h, pair=pair, images=images):
            load_frame(h, pair, first=False)
            set_images(h, images)
        ref = OracleRuns(cam, load, start, {})
        assert ref.iterations_ok(g.iterations()), (k, g.iterations(), o.iterations())
        check_pose("sequence frame %d" % k, np.float64(pg[0]), np.float64(pg[1]), np.float64(po[0]),
                   np.float64(po[1]), ref.tolerance)
        start = (np.float32(po[0]), np.float32(po[1]))  # continue both from the oracle's pose


@pytest.mark.parametrize("size", [(90, 66), (80, 60), (320, 240)])
def test_small_and_odd_sizes(gpu, orc, size):
    from slam_gb300 import synth
    w, h = size
    pair = synth.make_pair(4, cam=synth.Camera().scaled(w, h))
    g = new_gpu_odo(pair["cam"])
    load_frame(g, pair)
    images = gpu_images(g)
    tg, Rg = track(g, pair)
    ref = frame_runs(pair, {}, images=images)
    to, Ro, o = ref.main
    assert ref.iterations_ok(g.iterations()), (size, g.iterations(), o.iterations())
    check_pose("size %dx%d" % size, tg, Rg, to, Ro, ref.tolerance)


def test_tiny_image_runs(gpu):
    """16x16 (level 2 is 4x4): nothing to track, but no error and a finite pose."""
    from slam_gb300 import synth
    pair = synth.make_pair(4, cam=synth.Camera().scaled(16, 16))
    g = new_gpu_odo(pair["cam"])
    load_frame(g, pair)
    t, R = track(g, pair)
    assert np.all(np.isfinite(t)) and np.all(np.isfinite(R))


def test_empty_and_invalid_inputs(gpu, orc, pair640):
    """All-zero depth and all-hole model maps: no valid term at all; the
    pseudo-inverse solve leaves the pose unchanged, as in the oracle."""
    p = dict(pair640)
    p["depth"] = np.zeros_like(p["depth"])
    p["model_vert"] = np.zeros_like(p["model_vert"])
    g = new_gpu_odo(p["cam"])
    load_frame(g, p)
    tg, Rg = track(g, p)
    o = new_oracle_odo(p["cam"])
    load_frame(o, p)
    to, Ro = track(o, p)
    assert np.all(np.isfinite(tg)) and np.all(np.isfinite(Rg))
    rot, tr = pose_diff(tg, Rg, to, Ro)
    assert rot <= POSE_TOL_RAD and tr <= POSE_TOL_M
    assert g.lastICPCount == 0


def test_errors_are_returned_not_fatal(gpu):
    import torch
    from slam_gb300 import OdometryError, synth
    g = new_gpu_odo(synth.Camera().scaled(64, 48))
    with pytest.raises(OdometryError) as e:
        g.initICP(torch.zeros((48, 16), dtype=torch.int16, device="cuda").view(torch.uint16), 20.0)
    assert e.value.status == 1
    with pytest.raises(TypeError):
        g.initRGB(torch.zeros((48, 64, 4), dtype=torch.float32, device="cuda"))


def test_smoke_entry(gpu):
    """The build entry point's smoke check (160x120 pair, GPU vs oracle)."""
    import importlib.util
    import os
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("graft_entry", os.path.join(root, "__graft_entry__.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.smoke()
