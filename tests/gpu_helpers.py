"""Shared helpers of the GPU parity tests."""
import numpy as np

from conftest import ANGLE_THRESH, DIST_THRESH, TOLERANCE_REPORT

# Pose tolerance against the oracle: 1e-5 rad / 1e-5 m, the bound the
# reference path is held to.  It is widened only for inputs on which the
# reference algorithm itself does not determine the pose to that precision:
# where the oracle's FP32 and FP64 runs differ by GAP_LIMIT or more.
POSE_TOL_RAD = 1e-5
POSE_TOL_M = 1e-5
GAP_LIMIT = 5e-6


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def dev_u16(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int16)).cuda().view(torch.uint16)


def new_gpu_odo(cam):
    from slam_gb300 import RGBDOdometry
    return RGBDOdometry(cam.width, cam.height, cam.cx, cam.cy, cam.fx, cam.fy, DIST_THRESH, ANGLE_THRESH)


def new_oracle_odo(cam, prec=32):
    from oracle import oracle
    return oracle.Odometry(cam.width, cam.height, cam.cx, cam.cy, cam.fx, cam.fy, DIST_THRESH, ANGLE_THRESH,
                           prec=prec)


def load_frame(odo, pair, first=True):
    """The reference call order (src/apps/elastic_fusion_file.cpp:359-374)."""
    is_gpu = hasattr(odo, "handle")
    cv = dev if is_gpu else (lambda a: a)
    cd = dev_u16 if is_gpu else (lambda a: a)
    if first:
        odo.initFirstRGB(cv(pair["prev_rgba"]))
    odo.initICPModel(cv(pair["model_vert"]), cv(pair["model_norm"]), 20.0, pair["T1"].astype(np.float32))
    odo.initRGBModel(cv(pair["model_rgba"]))
    odo.initICP(cd(pair["depth"]), 20.0)
    odo.initRGB(cv(pair["rgba"]))


def track(odo, pair, **kw):
    T1 = pair["T1"]
    args = dict(rgbOnly=False, icpWeight=10.0, pyramid=True, fastOdom=False, so3=True)
    args.update(kw)
    t, R = odo.getIncrementalTransformation(T1[:3, 3].astype(np.float32), T1[:3, :3].astype(np.float32), **args)
    return np.asarray(t, np.float64), np.asarray(R, np.float64)


def pose_diff(t1, R1, t2, R2):
    from slam_gb300 import synth
    return synth.pose_error(synth.pose(R1, t1), synth.pose(R2, t2))


def intr(cam, level):
    d = float(1 << level)
    return (float(np.float32(cam.fx) / np.float32(d)), float(np.float32(cam.fy) / np.float32(d)),
            float(np.float32(cam.cx) / np.float32(d)), float(np.float32(cam.cy) / np.float32(d)))


def corr_to_dataterm(corr):
    """GPU correspondence records (u0, v0, diff, valid) -> oracle DataTerm array."""
    from oracle.oracle import DATATERM_DTYPE
    h, w, _ = corr.shape
    out = np.zeros((h, w), DATATERM_DTYPE)
    out["zero_x"] = corr[..., 0]
    out["zero_y"] = corr[..., 1]
    yy, xx = np.mgrid[0:h, 0:w]
    out["one_x"] = xx
    out["one_y"] = yy
    out["diff"] = corr[..., 2].astype(np.float32)
    out["valid"] = corr[..., 3]
    return out


def rel_close(a, b, rtol):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = max(np.abs(b).max(), 1e-30)
    return np.abs(a - b).max() <= rtol * scale, float(np.abs(a - b).max() / scale)


def report(line):
    TOLERANCE_REPORT.append(line)
    print(line)


# The integer images of the photometric term (intensity pyramids, derivative
# images).  Their kernels make rounding decisions -- truncations of quotients
# and weighted sums -- that the reference takes with its approximate
# division; the CPU oracle takes them with IEEE arithmetic and differs on tie
# pixels.  Ours match the reference's kernels bit for bit
# (test_gpu_reference.py), so whole-tracking comparisons give the oracle's
# host loop these images from the GPU: what remains between the two is the
# tracking loop itself.
IMAGE_BUFFERS = (("lastImage", 7), ("nextImage", 8), ("lastNextImage", 9), ("dIdx", 10), ("dIdy", 11))


def gpu_images(g):
    """The reference-exact integer images of a loaded GPU handle (derivatives
    computed from its nextImage, as the tracking call does)."""
    g.debug_derivatives()
    return {(name, l): g.download(which, l) for name, which in IMAGE_BUFFERS for l in range(3)}


def pair_images(pair, first=True):
    """gpu_images of a frame pair loaded on a fresh GPU handle."""
    g = new_gpu_odo(pair["cam"])
    load_frame(g, pair, first)
    out = gpu_images(g)
    g.close()
    return out


def set_images(o, images):
    for (name, l), a in images.items():
        o.set_buffer(name, l, a)
    o.keep_derivatives(True)


def oracle_track(pair, flags, levels=0, iterations=(0, 0, 0), prec=32, first=True, images=None):
    """The oracle's host loop on one pair (with the batched tracker's per-pair
    schedule when levels > 0), on the GPU's integer images when given.
    Returns (t, R, oracle handle)."""
    o = new_oracle_odo(pair["cam"], prec)
    if levels:
        o.set_schedule(levels, iterations)
    load_frame(o, pair, first)
    if images is not None:
        set_images(o, images)
    t, R = track(o, pair, **flags)
    return t, R, o


def pose_tolerance(pair, t32, R32, o32, flags, levels=0, iterations=(0, 0, 0), first=True, images=None):
    """(tol_rad, tol_m, how): flat 1e-5 where the FP32 oracle and its FP64
    twin agree to GAP_LIMIT; otherwise twice the precision to which the
    reference algorithm determines the pose on this input -- the FP32/FP64
    gap or the size of the last Gauss-Newton increment (an iteration that has
    not converged leaves the pose undetermined to about one step), whichever
    is larger."""
    t64, R64, _ = oracle_track(pair, flags, levels, iterations, prec=64, first=first, images=images)
    gap = pose_diff(t32, R32, t64, R64)
    if gap[0] < GAP_LIMIT and gap[1] < GAP_LIMIT:
        return POSE_TOL_RAD, POSE_TOL_M, "flat (fp32/fp64 gap %.1e rad %.1e m)" % gap
    rot, tr = gap
    hist = o32.history()
    if len(hist):
        rot = max(rot, float(np.linalg.norm(hist[-1][6:9])))
        tr = max(tr, float(np.linalg.norm(hist[-1][3:6])))
    return (max(POSE_TOL_RAD, 2 * rot), max(POSE_TOL_M, 2 * tr),
            "widened (fp32/fp64 gap %.1e rad %.1e m, last step %.1e rad %.1e m)" % (gap[0], gap[1], rot, tr))


def check_pose(label, tg, Rg, to, Ro, tol_fn):
    """Asserts that the GPU pose is within tolerance of the oracle's and
    records the tolerance applied.  A pose within the flat 1e-5 bound passes
    as it is; otherwise tol_fn() -> (tol_rad, tol_m, how) gives the bound for
    this input (pose_tolerance)."""
    rot, tr = pose_diff(tg, Rg, to, Ro)
    if rot <= POSE_TOL_RAD and tr <= POSE_TOL_M:
        report("%s: pose diff %.2e rad %.2e m <= flat 1e-5" % (label, rot, tr))
        return rot, tr, True
    tol_r, tol_t, how = tol_fn()
    report("%s: pose diff %.2e rad %.2e m, tolerance %.2e rad %.2e m %s" % (label, rot, tr, tol_r, tol_t, how))
    assert rot <= tol_r and tr <= tol_t, (label, rot, tr, tol_r, tol_t, how)
    return rot, tr, False
