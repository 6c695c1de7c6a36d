"""Loop-closure verification: the reference's two callers of the tracker
that check candidate alignments, over the batched tracker.

* Ferns::findFrame (src/lc/Ferns.cpp:237-307): a relocalisation candidate
  (the stored fern frame) is aligned to the current frame at 1/8 resolution
  (80x60 for 640x480): initICPModel(fern maps, fern pose), initICP(current
  maps), getIncrementalTransformation(rgbOnly false, icpWeight 100, pyramid
  false, fastOdom false, so3 false); accepted when lastICPError < 3e-4,
  lastICPCount > 2400 (1400 when tracking is lost) and the photometric check
  over the fern's sample points is below photoThresh.
* model-to-model (src/apps/elastic_fusion_file.cpp:450-498): the inactive
  model's prediction against the active one's: initICPModel(old maps),
  initRGBModel(old image), initICP(new maps), initRGB(new image),
  getIncrementalTransformation(false, 10, pyramid, fastOdom, false);
  accepted when every diagonal entry of getCovariance() is <= covThresh,
  lastICPCount > icpCountThresh and lastICPError < icpErrThresh
  (src/configs/ef_file.cfg:9-14: 5e-5, 1e-5, 40000).

All candidates of a call run in one batched call (odo_batch_verify); the live
side of every pair is given as camera-frame RGBA32F maps."""
import ctypes

import numpy as np

from . import _native
from .batch import FramePair


def ferns_params(lost=False, max_icp_error=3e-4):
    """Tracking flags and accept thresholds of Ferns::findFrame
    (src/lc/Ferns.cpp:262-279)."""
    return dict(rgbOnly=False, icpWeight=100.0, fastOdom=False, so3=False, max_icp_error=max_icp_error,
                min_icp_count=1400.0 if lost else 2400.0, max_covariance=0.0)


def model_to_model_params(cov_thresh=1e-5, icp_count_thresh=40000, icp_err_thresh=5e-5, fastOdom=False):
    """Tracking flags and accept thresholds of the model-to-model check
    (src/apps/elastic_fusion_file.cpp:472-498, defaults of
    src/configs/ef_file.cfg)."""
    return dict(rgbOnly=False, icpWeight=10.0, fastOdom=fastOdom, so3=False, max_icp_error=icp_err_thresh,
                min_icp_count=float(icp_count_thresh), max_covariance=cov_thresh)


class Candidate(FramePair):
    """One candidate pair: the model side (maps, RGBA, pose) and the live side
    as camera-frame RGBA32F maps (+ RGBA when the check uses the photometric
    term).  levels = 1 is the reference's pyramid = false."""

    def __init__(self, cam, model_vert, model_norm, model_rgba, live_vert, live_norm, live_rgba, pose, levels=3):
        super().__init__(cam, model_vert, model_norm, model_rgba, None,
                         live_rgba if live_rgba is not None else model_rgba, None, pose, levels=levels)
        self.live_vert, self.live_norm = live_vert, live_norm

    def desc(self):
        import torch
        from .odometry import _check_cuda_tensor
        d = _native.OdoPair()
        c = self.cam
        d.width, d.height = c.width, c.height
        d.fx, d.fy, d.cx, d.cy = c.fx, c.fy, c.cx, c.cy
        d.distThresh = d.angleThresh = d.depthCutoff = 0.0
        d.levels = self.levels
        for l in range(3):
            d.iterations[l] = self.iterations[l]
        d.model_pitch = _check_cuda_tensor(self.model_vert, torch.float32, (4,), "model_vert")
        if _check_cuda_tensor(self.model_norm, torch.float32, (4,), "model_norm") != d.model_pitch:
            raise ValueError("model maps must share a pitch")
        d.model_verts, d.model_norms = self.model_vert.data_ptr(), self.model_norm.data_ptr()
        d.model_rgba = self.model_rgba.data_ptr()
        d.model_rgba_pitch = _check_cuda_tensor(self.model_rgba, torch.uint8, (4,), "model_rgba")
        d.rgba = self.rgba.data_ptr()
        d.rgba_pitch = _check_cuda_tensor(self.rgba, torch.uint8, (4,), "live_rgba")
        d.live_pitch = _check_cuda_tensor(self.live_vert, torch.float32, (4,), "live_vert")
        if _check_cuda_tensor(self.live_norm, torch.float32, (4,), "live_norm") != d.live_pitch:
            raise ValueError("live maps must share a pitch")
        d.live_verts, d.live_norms = self.live_vert.data_ptr(), self.live_norm.data_ptr()
        for k in range(16):
            d.pose[k] = float(self.pose.reshape(16)[k])
        return d


def verify(batch, candidates, params):
    """One batched verification call.  Returns (results, covariances [n,6,6],
    accept mask)."""
    n = len(candidates)
    descs = (_native.OdoPair * n)()
    for i, c in enumerate(candidates):
        descs[i] = c.desc()
    vp = _native.OdoVerifyParams()
    vp.rgbOnly, vp.icpWeight = int(bool(params["rgbOnly"])), float(params["icpWeight"])
    vp.fastOdom, vp.so3 = int(bool(params["fastOdom"])), int(bool(params["so3"]))
    vp.max_icp_error, vp.min_icp_count = float(params["max_icp_error"]), float(params["min_icp_count"])
    vp.max_covariance = float(params["max_covariance"])
    res = (_native.OdoPairResult * n)()
    cov = np.zeros((n, 36), np.float64)
    acc = (ctypes.c_int * n)()
    batch._check(batch._L.odo_batch_verify(batch._h, descs, n, ctypes.byref(vp), res,
                                           cov.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), acc),
                 "odo_batch_verify")
    return res, cov.reshape(n, 6, 6), np.array(acc[:], bool)


def photometric_check(vert_small, img_small, est_pose, fern_pose, fern_rgb, points, cam, max_depth_mm):
    """Ferns::photometricCheck (src/lc/Ferns.cpp:309-356), on the host as in
    the reference: the mean absolute RGB difference between the current
    frame's small image at the fern's sample points and the fern's stored
    image at those points moved by fernPose^-1 estPose and projected (the
    projected coordinates truncated to int, as the reference's Vector2i
    does).  vert_small [h][w][4] float, img_small / fern_rgb [h][w][3] uint8,
    points [k][2] (x, y) sample pixels; cam = the small image's intrinsics.
    NaN when no sample point compares (the reference's 0 / 0)."""
    vert_small = np.asarray(vert_small, np.float32)
    h, w = vert_small.shape[:2]
    cx, cy = np.float32(cam.cx), np.float32(cam.cy)
    invfx, invfy = np.float32(1.0) / np.float32(cam.fx), np.float32(1.0) / np.float32(cam.fy)
    diff = (np.linalg.inv(np.asarray(fern_pose, np.float32).astype(np.float64)).astype(np.float32)
            @ np.asarray(est_pose, np.float32)).astype(np.float32)
    photo_sum, photo_count = np.float32(0.0), 0
    for x, y in np.asarray(points, np.int64):
        v = vert_small[y, x]
        if not (v[2] > 0 and int(np.float32(v[2]) * np.float32(1000.0)) < max_depth_mm):
            continue
        p = diff @ np.array([v[0], v[1], v[2], 1.0], np.float32)
        u = int(p[0] * (np.float32(1.0) / invfx) / p[2] + cx)
        r = int(p[1] * (np.float32(1.0) / invfy) / p[2] + cy)
        if 0 <= u < w and 0 <= r < h and (fern_rgb[r, u] > 0).any():
            photo_sum += np.float32(np.abs(fern_rgb[r, u].astype(np.int32) - img_small[y, x].astype(np.int32)).sum())
            photo_count += 1
    return float(photo_sum / np.float32(photo_count)) if photo_count else float("nan")
