"""Shared helpers of the GPU parity tests."""
import numpy as np

from conftest import ANGLE_THRESH, DIST_THRESH


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
