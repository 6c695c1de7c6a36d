"""Loop-closure verification through the batched tracker (odo_batch_verify,
slam_gb300/verify.py): the Ferns relocalisation check (80x60, ICP only, no
pyramid; src/lc/Ferns.cpp:253-279) and the model-to-model check (ICP + RGB,
pyramid, covariance gate; src/apps/elastic_fusion_file.cpp:462-498), with the
live side of every candidate given as RGBA32F maps.

Each candidate's pose is bit-identical to the single-pair call with
initICP(verts, norms); it is within the oracle's tolerance of the oracle's
host loop; and the accept decision equals the one made from the oracle's
statistics and covariance.  Every batch mixes candidates that should pass
(the live view a small motion away) with ones that should not (the live view
of another room)."""
import numpy as np
import pytest

from gpu_helpers import OracleRuns, check_pose, dev, dev_u16, gpu_images, new_gpu_odo, report, set_images, track

pytestmark = pytest.mark.gpu


def candidates(n, cam, seed, wrong_every=4, max_deg=3.0, max_m=0.04):
    """n candidate pairs: model maps at T1, live maps at T2 = T1 * motion of
    the same room, except every `wrong_every`-th whose live maps come from
    another room."""
    from slam_gb300 import synth
    out = []
    for i in range(n):
        s = seed * 1000 + i
        p = synth.make_pair(s, cam=cam, max_deg=max_deg, max_m=max_m)
        scene = synth.make_room(s + (500 if i % wrong_every == wrong_every - 1 else 0))
        m = synth.render(scene, p["T2"], cam, depth=False, rgba=True, model=True)
        p["live_vert"], p["live_norm"], p["live_rgba"] = m["vert"], m["norm"], m["rgba"]
        out.append(p)
    return out


def load_maps(odo, p, rgb):
    cv = dev if hasattr(odo, "handle") else (lambda a: a)
    odo.initICPModel(cv(p["model_vert"]), cv(p["model_norm"]), 20.0, p["T1"].astype(np.float32))
    if rgb:
        odo.initRGBModel(cv(p["model_rgba"]))
    odo.initICP(cv(p["live_vert"]), cv(p["live_norm"]), 20.0)
    if rgb:
        odo.initRGB(cv(p["live_rgba"]))


def run_check(pairs, params, levels, tag):
    from slam_gb300 import verify
    from slam_gb300.batch import BatchOdometry, result_pose
    rgb = params["icpWeight"] < 100
    flags = dict(rgbOnly=params["rgbOnly"], icpWeight=params["icpWeight"], pyramid=levels == 3,
                 fastOdom=params["fastOdom"], so3=params["so3"])
    cands = [verify.Candidate(p["cam"], dev(p["model_vert"]), dev(p["model_norm"]), dev(p["model_rgba"]),
                              dev(p["live_vert"]), dev(p["live_norm"]), dev(p["live_rgba"]), p["T1"], levels=levels)
             for p in pairs]
    b = BatchOdometry(len(cands))
    res, cov, acc = verify.verify(b, cands, params)
    n_acc = 0
    for i, p in enumerate(pairs):
        T = result_pose(res[i])
        # the single-pair path on the same inputs: the same bits
        g = new_gpu_odo(p["cam"])
        load_maps(g, p, rgb)
        images = gpu_images(g) if rgb else None
        tg, Rg = track(g, p, **flags)
        assert np.array_equal(np.float32(T[:3, 3]), np.float32(tg)), (tag, i)
        assert np.array_equal(np.float32(T[:3, :3]), np.float32(Rg)), (tag, i)
        assert list(res[i].iterations) == g.iterations(), (tag, i)

        # the oracle's host loop
        def load(o, p=p, images=images):
            load_maps(o, p, rgb)
            if rgb:
                set_images(o, images)
        ref = OracleRuns(p["cam"], load, (p["T1"][:3, 3], p["T1"][:3, :3]), flags)
        to, Ro, o = ref.main
        _, _, flat = check_pose("%s candidate %d" % (tag, i), T[:3, 3], T[:3, :3], to, Ro, ref.tolerance)
        inv = np.linalg.inv(np.asarray(res[i].lastA, np.float64).reshape(6, 6))
        assert np.abs(cov[i] - inv).max() <= 1e-9 * np.abs(inv).max(), (tag, i)
        n_acc += int(acc[i])
        if not flat and ref.undetermined():
            continue  # no decision to compare on an input the algorithm does not determine
        assert ref.iterations_ok(res[i].iterations), (tag, i)
        st = o.stats
        co = o.getCovariance()
        cov_ok = all(not (co[k, k] > params["max_covariance"]) for k in range(6)) \
            if params["max_covariance"] > 0 else True
        acc_o = (cov_ok and st["lastICPCount"] > params["min_icp_count"]
                 and st["lastICPError"] < params["max_icp_error"])
        assert bool(acc[i]) == acc_o, (tag, i, res[i].lastICPError, res[i].lastICPCount, st["lastICPError"],
                                       st["lastICPCount"])
    report("%s: %d candidates, %d accepted (the oracle's decisions identical)" % (tag, len(pairs), n_acc))
    return acc


def test_ferns_relocalisation_check(gpu):
    from slam_gb300 import synth, verify
    cam = synth.Camera().scaled(80, 60)
    pairs = candidates(16, cam, seed=3)
    acc = run_check(pairs, verify.ferns_params(), levels=1, tag="ferns 80x60")
    assert acc.any() and not acc.all()


def test_model_to_model_check(gpu):
    from slam_gb300 import synth, verify
    cam = synth.Camera().scaled(320, 240)
    pairs = candidates(8, cam, seed=5)
    # icpCountThresh scaled to the 320x240 image (40000 is for 640x480)
    params = verify.model_to_model_params(icp_count_thresh=10000)
    acc = run_check(pairs, params, levels=3, tag="model-to-model 320x240")
    assert not acc.all()


def test_live_input_kinds_do_not_mix(gpu):
    """A call whose pairs mix depth and map live inputs is refused."""
    from slam_gb300 import OdometryError, synth, verify
    from slam_gb300.batch import BatchOdometry, FramePair
    cam = synth.Camera().scaled(160, 120)
    p = candidates(1, cam, seed=9)[0]
    c = verify.Candidate(cam, dev(p["model_vert"]), dev(p["model_norm"]), dev(p["model_rgba"]), dev(p["live_vert"]),
                         dev(p["live_norm"]), dev(p["live_rgba"]), p["T1"], levels=3)
    d = FramePair(cam, dev(p["model_vert"]), dev(p["model_norm"]), dev(p["model_rgba"]), dev_u16(p["depth"]),
                  dev(p["rgba"]), dev(p["prev_rgba"]), p["T1"])
    with pytest.raises(OdometryError) as e:
        verify.verify(BatchOdometry(2), [c, d], verify.ferns_params())
    assert e.value.status == 1
