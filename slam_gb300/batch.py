"""Batched tracking of many independent frame pairs (C ABI odo_batch_*).

Each pair does what initFirstRGB + initICPModel + initRGBModel + initICP +
initRGB + getIncrementalTransformation do on one RGBDOdometry handle; all
pairs run in one CUDA graph.  Inputs are CUDA tensors (see odometry.py)."""
import ctypes

import numpy as np

from . import _native
from .odometry import OdometryError, _check_cuda_tensor


class FramePair:
    """Device inputs of one pair; `pose` is the model pose = starting pose."""

    def __init__(self, cam, model_vert, model_norm, model_rgba, depth, rgba, prev_rgba, pose, levels=3,
                 iterations=(0, 0, 0)):
        self.cam, self.levels = cam, int(levels)
        self.iterations = tuple(int(i) for i in iterations)
        self.model_vert, self.model_norm, self.model_rgba = model_vert, model_norm, model_rgba
        self.depth, self.rgba, self.prev_rgba = depth, rgba, prev_rgba
        self.pose = np.asarray(pose, np.float32).reshape(4, 4)

    def desc(self):
        import torch
        d = _native.OdoPair()
        c = self.cam
        d.width, d.height = c.width, c.height
        d.fx, d.fy, d.cx, d.cy = c.fx, c.fy, c.cx, c.cy
        d.distThresh = d.angleThresh = d.depthCutoff = 0.0
        d.levels = self.levels
        for l in range(3):
            d.iterations[l] = self.iterations[l]
        d.model_pitch = _check_cuda_tensor(self.model_vert, torch.float32, (4,), "model_vert")
        d.model_verts, d.model_norms = self.model_vert.data_ptr(), self.model_norm.data_ptr()
        d.model_rgba = self.model_rgba.data_ptr()
        d.model_rgba_pitch = _check_cuda_tensor(self.model_rgba, torch.uint8, (4,), "model_rgba")
        d.depth = self.depth.data_ptr()
        d.depth_pitch = _check_cuda_tensor(self.depth, torch.uint16, (), "depth")
        d.rgba = self.rgba.data_ptr()
        d.rgba_pitch = _check_cuda_tensor(self.rgba, torch.uint8, (4,), "rgba")
        if self.prev_rgba is not None:
            d.prev_rgba = self.prev_rgba.data_ptr()
            d.prev_rgba_pitch = _check_cuda_tensor(self.prev_rgba, torch.uint8, (4,), "prev_rgba")
        for k in range(16):
            d.pose[k] = float(self.pose.reshape(16)[k])
        return d


class BatchOdometry:
    def __init__(self, max_pairs, stream=None):
        self._L = _native.load()
        h = ctypes.c_void_p()
        rc = self._L.odo_batch_create(int(max_pairs), ctypes.byref(h))
        if rc != 0:
            raise OdometryError(rc, "odo_batch_create failed")
        self._h = h
        self.max_pairs = int(max_pairs)
        if stream is None:
            import torch
            stream = torch.cuda.current_stream().cuda_stream
        self._check(self._L.odo_batch_set_stream(self._h, ctypes.c_void_p(stream)), "odo_batch_set_stream")

    def _check(self, rc, what):
        if rc != 0:
            raise OdometryError(rc, "%s: %s %s" % (what, self._L.odo_status_string(rc).decode(),
                                                   self._L.odo_batch_last_error(self._h).decode()))

    def close(self):
        if getattr(self, "_h", None):
            self._L.odo_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_launch(self, threads, pixels_per_thread):
        self._check(self._L.odo_batch_set_launch(self._h, int(threads), int(pixels_per_thread)), "set_launch")

    def _descs(self, pairs):
        arr = (_native.OdoPair * len(pairs))()
        for i, p in enumerate(pairs):
            arr[i] = p.desc()
        return arr

    def track(self, pairs, rgbOnly=False, icpWeight=10.0, fastOdom=False, so3=True, descs=None):
        descs = descs if descs is not None else self._descs(pairs)
        res = (_native.OdoPairResult * len(pairs))()
        self._check(self._L.odo_batch_track(self._h, descs, len(pairs), int(bool(rgbOnly)), float(icpWeight),
                                            int(bool(fastOdom)), int(bool(so3)), res), "odo_batch_track")
        return res

    def track_init(self, pairs, init, rgbOnly=False, icpWeight=10.0, fastOdom=False, descs=None):
        """Tracking from per-pair motion estimates: init is a CUDA float32
        tensor [n, 6] (translation m, rotation vector rad of the live camera
        in the model camera's frame); no SO3 stage."""
        import torch
        if not (isinstance(init, torch.Tensor) and init.is_cuda and init.dtype == torch.float32
                and init.is_contiguous() and tuple(init.shape) == (len(pairs), 6)):
            raise ValueError("init must be a contiguous CUDA float32 tensor [n, 6]")
        descs = descs if descs is not None else self._descs(pairs)
        res = (_native.OdoPairResult * len(pairs))()
        self._check(self._L.odo_batch_track_init(self._h, descs, len(pairs), ctypes.c_void_p(init.data_ptr()),
                                                 int(bool(rgbOnly)), float(icpWeight), int(bool(fastOdom)), res),
                    "odo_batch_track_init")
        return res

    def track_warm(self, net, pairs, levels=2, iterations=(4, 3, 0), residual_limit=0.0, max_disagree_deg=0.0,
                   rgbOnly=False, icpWeight=10.0, fastOdom=False, descs=None):
        """Learned warm start (odo_batch_track_warm): the network's proposal
        per pair, tracking with the short schedule, fall-back to the plain
        schedule where the residual or the disagreement test fails.  Returns
        (results, fallback mask)."""
        descs = descs if descs is not None else self._descs(pairs)
        n = len(descs)
        res = (_native.OdoPairResult * n)()
        fb = (ctypes.c_int * n)()
        wp = _native.OdoWarmParams()
        wp.levels = int(levels)
        for l in range(3):
            wp.iterations[l] = int(iterations[l])
        wp.residual_limit = float(residual_limit)
        wp.max_disagree = float(np.radians(max_disagree_deg))
        wp.rgbOnly, wp.icpWeight, wp.fastOdom = int(bool(rgbOnly)), float(icpWeight), int(bool(fastOdom))
        self._check(self._L.odo_batch_track_warm(self._h, net._h, descs, n, ctypes.byref(wp), res, fb),
                    "odo_batch_track_warm")
        return res, np.array(fb[:], bool)

    def time_iteration(self, level, reps=20):
        """Mean CUDA-event times (ms) over all pairs of the last track() call:
        association kernel, photometric/solve kernel, one whole iteration."""
        out = (ctypes.c_float * 3)()
        self._check(self._L.odo_batch_debug_time_iteration(self._h, int(level), int(reps), out), "time_iteration")
        return list(out)

    def autotune(self, pairs, rgbOnly=False, icpWeight=10.0, fastOdom=False, so3=True):
        descs = self._descs(pairs)
        res = (_native.OdoPairResult * len(pairs))()
        t, p, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
        self._check(self._L.odo_batch_autotune(self._h, descs, len(pairs), int(bool(rgbOnly)), float(icpWeight),
                                               int(bool(fastOdom)), int(bool(so3)), res, ctypes.byref(t),
                                               ctypes.byref(p), ctypes.byref(ms)), "odo_batch_autotune")
        return t.value, p.value, ms.value


def result_pose(r):
    return np.array(r.pose, np.float64).reshape(4, 4)
