"""Frame-to-model tracking over a 300-frame trajectory at 640x480 (the
reference's per-frame use, src/apps/elastic_fusion_file.cpp:359-376): a
smooth Catmull-Rom camera path at 30 fps (<= 1.5 deg / 3 cm per frame)
through a seeded room; each frame's model prediction is ray-cast from the
ground-truth scene at the current pose estimate, the live frame (noisy depth +
RGB) at the true pose.  Every frame is tracked by the GPU handle and by the
oracle's host loop from the same start pose (the GPU handle carries its
state -- the SO3 image swap -- from frame to frame; the oracle gets that
state with the GPU's reference-exact images); per-frame pose and JtJ (lastA)
are compared, and the max / p99 of both are reported.  JtJ is a function of
the pose the last iteration starts from: it is held to 1e-3 (summation
order), or to its spread under the oracle's perturbations, on every frame
whose pose is within the flat 1e-5 bound, and only
reported on frames where the reference algorithm itself leaves the pose
less determined (the pose is then checked against the oracle's measured
sensitivity)."""
import numpy as np
import pytest

from gpu_helpers import (GAP_LIMIT, POSE_TOL_M, POSE_TOL_RAD, OracleRuns, check_pose, dev, dev_u16, gpu_images,
                         new_gpu_odo, pose_diff, report, set_images)

pytestmark = pytest.mark.gpu

FRAMES = 300


def test_trajectory_frame_to_model_matches_oracle(gpu):
    from slam_gb300 import evaluate, synth
    seed = 17
    cam = synth.Camera()
    scene = synth.make_room(seed)
    T = synth.trajectory(seed, FRAMES)
    g = new_gpu_odo(cam)
    prev = synth.render(scene, T[0], cam, noise_seed=seed * 100003, depth=False, rgba=True)
    g.initFirstRGB(dev(prev["rgba"]))
    est = [T[0].astype(np.float32).astype(np.float64)]
    rot_err, tr_err, jtj_err, flat_frames, determined, tie_explained = [], [], [], [], [], []
    for k in range(1, FRAMES):
        start = est[-1].astype(np.float32)
        model = synth.render(scene, start.astype(np.float64), cam, depth=False, rgba=True, model=True)
        live = synth.render(scene, T[k], cam, noise_seed=seed * 100003 + k, depth=True, rgba=True)
        g.initICPModel(dev(model["vert"]), dev(model["norm"]), 20.0, start)
        g.initRGBModel(dev(model["rgba"]))
        g.initICP(dev_u16(live["depth"]), 20.0)
        g.initRGB(dev(live["rgba"]))
        images = gpu_images(g)
        tg, Rg = g.getIncrementalTransformation(start[:3, 3], start[:3, :3])
        tg, Rg = np.asarray(tg, np.float64), np.asarray(Rg, np.float64)

        def load(h, model=model, live=live, start=start, images=images):
            # a fresh handle with the GPU's images (lastNextImage included)
            # holds the oracle's state at this frame
            h.initICPModel(model["vert"], model["norm"], 20.0, start)
            h.initRGBModel(model["rgba"])
            h.initICP(live["depth"], 20.0)
            h.initRGB(live["rgba"])
            set_images(h, images)
        ref = OracleRuns(cam, load, (start[:3, 3], start[:3, :3]), {})
        to, Ro, o = ref.main
        rot, tr = pose_diff(tg, Rg, to, Ro)
        flat = rot <= POSE_TOL_RAD and tr <= POSE_TOL_M
        assert g.iterations() == o.iterations() or ref.iterations_ok(g.iterations()), \
            (k, g.iterations(), o.iterations())
        if not flat:
            check_pose("trajectory frame %d" % k, tg, Rg, to, Ro, ref.tolerance)
        A_g = np.asarray(g.lastA, np.float64).reshape(6, 6)
        A_o = o.stats["lastA"]
        jtj = float(np.abs(A_g - A_o).max() / np.abs(A_o).max())
        if flat:
            ok, _ = ref.jtj_ok(g.lastA, flat)
            assert ok, (k, jtj)
        rot_err.append(rot)
        tr_err.append(tr)
        jtj_err.append(jtj)
        flat_frames.append(flat)
        determined.append(ref.summation_gap() < GAP_LIMIT)
        tie_explained.append(determined[-1] and not flat and ref.matches_a_tie_run(tg, Rg))
        est.append(synth.pose(Ro, to))
        prev = live
    rot_err, tr_err, jtj_err, flat_frames, determined = (np.array(v) for v in (rot_err, tr_err, jtj_err, flat_frames,
                                                                                 determined))
    within = float(np.mean(flat_frames))
    jf = jtj_err[flat_frames] if flat_frames.any() else np.zeros(1)
    ate = evaluate.ate_rmse(np.array(T), np.array(est))
    rpe = evaluate.rpe(np.array(T), np.array(est), delta=1)
    report("trajectory %d frames 640x480: GPU vs oracle pose max %.2e rad %.2e m, p99 %.2e rad %.2e m, "
           "%.1f %% within the flat 1e-5; JtJ rel diff on those frames max %.2e p99 %.2e, on all frames max %.2e "
           "p99 %.2e; oracle chain vs ground truth ATE %.4f m RPE trans %.4f m rot %.4f deg"
           % (FRAMES, rot_err.max(), tr_err.max(), np.percentile(rot_err, 99), np.percentile(tr_err, 99),
              100 * within, jf.max(), np.percentile(jf, 99), jtj_err.max(), np.percentile(jtj_err, 99), ate,
              rpe["trans_rmse"], np.degrees(rpe["rot_rmse"])))
    report("trajectory: on %d of %d frames the oracle's own pose moves by less than %.0e under another summation "
           "order and in FP64 (the reference algorithm determines the pose there); the GPU is within the flat 1e-5 "
           "on %d of them and within 1e-5 of an oracle run with some rounding ties decided the other way on %d of the "
           "others" % (determined.sum(), len(determined), GAP_LIMIT, (determined & flat_frames).sum(),
                       sum(tie_explained)))
