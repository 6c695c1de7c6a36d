"""Python mirror of the reference's RGBDOdometryef class
(src/odom/RGBDOdometryef.h:28-131) over the C ABI (include/slam_gb300.h).

Frame inputs are CUDA tensors (torch is used only to hold device memory and
to name the stream):
  depth   uint16 [H, W]      (initICP, millimetres)
  verts   float32 [H, W, 4]  (initICP / initICPModel, RGBA32F camera frame)
  norms   float32 [H, W, 4]
  rgb     uint8  [H, W, 4]   (initRGB / initRGBModel / initFirstRGB, RGBA)
Row pitches are taken from the tensors' strides.  Errors raise OdometryError
carrying the C status; nothing falls back to a CPU path.
"""
import ctypes
import math

import numpy as np

from . import _native

MODE_GRAPH, MODE_STREAM, MODE_PERSISTENT = 0, 1, 2
PREC_FP32, PREC_COMPENSATED = 0, 1

# RGBDOdometryef default thresholds (src/odom/RGBDOdometryef.h:35-36), in float
DEFAULT_DIST_THRESH = float(np.float32(0.10))
DEFAULT_ANGLE_THRESH = float(np.float32(math.sin(float(np.float32(np.float32(20.0) * np.float32(3.14159254))
                                                       / np.float32(180.0)))))


class OdometryError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(msg)
        self.status = status


def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _check_cuda_tensor(t, dtype, shape_tail, name):
    import torch
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name}: expected a CUDA tensor")
    if t.dtype != dtype:
        raise TypeError(f"{name}: expected dtype {dtype}, got {t.dtype}")
    if tuple(t.shape[2:]) != tuple(shape_tail):
        raise ValueError(f"{name}: bad shape {tuple(t.shape)}")
    if t.stride(-1) != 1 or (t.dim() == 3 and t.stride(1) != t.shape[2]):
        raise ValueError(f"{name}: rows must be contiguous")
    return t.stride(0) * t.element_size()


class RGBDOdometry:
    """Same methods, arguments and statistics as RGBDOdometryef."""

    def __init__(self, width, height, cx, cy, fx, fy, distThresh=DEFAULT_DIST_THRESH,
                 angleThresh=DEFAULT_ANGLE_THRESH, stream=None):
        self._L = _native.load()
        self.width, self.height = int(width), int(height)
        h = ctypes.c_void_p()
        rc = self._L.odo_create(self.width, self.height, cx, cy, fx, fy, distThresh, angleThresh, ctypes.byref(h))
        if rc != 0:
            raise OdometryError(rc, "odo_create failed: %s" % self._L.odo_status_string(rc).decode())
        self._h = h
        if stream is None:
            import torch
            stream = torch.cuda.current_stream().cuda_stream
        self._check(self._L.odo_set_stream(self._h, ctypes.c_void_p(stream)), "odo_set_stream")
        self._stats = _native.OdoStats()

    # -- plumbing ---------------------------------------------------------
    def _check(self, rc, what):
        if rc != 0:
            msg = self._L.odo_last_error(self._h).decode() if getattr(self, "_h", None) else ""
            raise OdometryError(rc, "%s: %s %s" % (what, self._L.odo_status_string(rc).decode(), msg))

    def close(self):
        if getattr(self, "_h", None):
            self._L.odo_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_mode(self, mode):
        self._check(self._L.odo_set_mode(self._h, int(mode)), "odo_set_mode")

    def set_precision(self, prec):
        self._check(self._L.odo_set_precision(self._h, int(prec)), "odo_set_precision")

    # -- reference call surface -----------------------------------------
    def initICP(self, a, b=None, depthCutoff=20.0):
        """initICP(depth, depthCutoff) or initICP(verts, norms, depthCutoff)."""
        import torch
        if b is None or not isinstance(b, torch.Tensor):
            if b is not None:
                depthCutoff = b
            pitch = _check_cuda_tensor(a, torch.uint16, (), "depth")
            self._check(self._L.odo_init_icp_depth(self._h, a.data_ptr(), pitch, float(depthCutoff)), "initICP")
        else:
            pitch = _check_cuda_tensor(a, torch.float32, (4,), "verts")
            if _check_cuda_tensor(b, torch.float32, (4,), "norms") != pitch:
                raise ValueError("verts and norms must share a pitch")
            self._check(self._L.odo_init_icp_maps(self._h, a.data_ptr(), b.data_ptr(), pitch, float(depthCutoff)),
                        "initICP")

    def initICPRawDepth(self, raw_depth, maxD, depthCutoff=20.0):
        """The reference's depth pre-filter (depth_bilateral.frag) on raw u16
        depth, then initICP on the filtered image."""
        import torch
        pitch = _check_cuda_tensor(raw_depth, torch.uint16, (), "raw_depth")
        self._check(self._L.odo_init_icp_raw_depth(self._h, raw_depth.data_ptr(), pitch, float(maxD),
                                                   float(depthCutoff)), "initICPRawDepth")

    def initICPModel(self, verts, norms, depthCutoff, modelPose):
        import torch
        pitch = _check_cuda_tensor(verts, torch.float32, (4,), "verts")
        if _check_cuda_tensor(norms, torch.float32, (4,), "norms") != pitch:
            raise ValueError("verts and norms must share a pitch")
        pose = np.ascontiguousarray(np.asarray(modelPose, dtype=np.float32).reshape(4, 4))
        self._check(self._L.odo_init_icp_model(self._h, verts.data_ptr(), norms.data_ptr(), pitch,
                                               float(depthCutoff), _fptr(pose)), "initICPModel")

    def _rgb(self, fn, rgb, what):
        import torch
        pitch = _check_cuda_tensor(rgb, torch.uint8, (4,), "rgb")
        self._check(fn(self._h, rgb.data_ptr(), pitch), what)

    def initRGB(self, rgb):
        self._rgb(self._L.odo_init_rgb, rgb, "initRGB")

    def initRGBModel(self, rgb):
        self._rgb(self._L.odo_init_rgb_model, rgb, "initRGBModel")

    def initFirstRGB(self, rgb):
        self._rgb(self._L.odo_init_first_rgb, rgb, "initFirstRGB")

    def getIncrementalTransformation(self, trans, rot, rgbOnly=False, icpWeight=10.0, pyramid=True, fastOdom=False,
                                     so3=True):
        """trans (3,), rot (3,3) row-major: previous pose in, tracked pose out
        (returned as new float32 arrays)."""
        t = np.ascontiguousarray(np.asarray(trans, dtype=np.float32).reshape(3)).copy()
        R = np.ascontiguousarray(np.asarray(rot, dtype=np.float32).reshape(3, 3)).copy()
        self._check(self._L.odo_get_incremental_transformation(self._h, _fptr(t), _fptr(R), int(bool(rgbOnly)),
                                                               float(icpWeight), int(bool(pyramid)),
                                                               int(bool(fastOdom)), int(bool(so3))),
                    "getIncrementalTransformation")
        self._check(self._L.odo_get_stats(self._h, ctypes.byref(self._stats)), "odo_get_stats")
        return t, R

    def getCovariance(self):
        out = np.zeros(36, dtype=np.float64)
        self._check(self._L.odo_get_covariance(self._h, _dptr(out)), "getCovariance")
        return out.reshape(6, 6)

    def iterations(self):
        out = (ctypes.c_int * 4)()
        self._check(self._L.odo_get_iterations(self._h, out), "odo_get_iterations")
        return list(out)

    # statistics, as public members of RGBDOdometryef (src/odom/RGBDOdometryef.h:62-70)
    lastICPError = property(lambda s: s._stats.lastICPError)
    lastICPCount = property(lambda s: s._stats.lastICPCount)
    lastRGBError = property(lambda s: s._stats.lastRGBError)
    lastRGBCount = property(lambda s: s._stats.lastRGBCount)
    lastSO3Error = property(lambda s: s._stats.lastSO3Error)
    lastSO3Count = property(lambda s: s._stats.lastSO3Count)
    lastA = property(lambda s: np.array(s._stats.lastA, dtype=np.float64).reshape(6, 6))
    lastb = property(lambda s: np.array(s._stats.lastb, dtype=np.float64))

    # -- parity / debug access -------------------------------------------
    BUF_DTYPES = {0: np.uint16, 1: np.float32, 2: np.float32, 3: np.float32, 4: np.float32, 5: np.float32,
                  6: np.float32, 7: np.uint8, 8: np.uint8, 9: np.uint8, 10: np.int16, 11: np.int16, 12: np.int16}

    def _buf_shape(self, which, level):
        w, h = self.width >> level, self.height >> level
        if which in (1, 2, 3, 4):
            return (3, h, w)
        if which == 12:
            return (h, w, 8)  # int16 u0, v0, diff, valid, float z (2 slots), dIdx, dIdy
        return (h, w)

    def download(self, which, level):
        out = np.zeros(self._buf_shape(which, level), dtype=self.BUF_DTYPES[which])
        self._check(self._L.odo_debug_download(self._h, which, level, out.ctypes.data, out.nbytes), "download")
        return out

    def upload(self, which, level, arr):
        a = np.ascontiguousarray(arr, dtype=self.BUF_DTYPES[which]).reshape(self._buf_shape(which, level))
        self._check(self._L.odo_debug_upload(self._h, which, level, a.ctypes.data, a.nbytes), "upload")

    def debug_icp_step(self, level, Rcurr, tcurr, Rprev_inv, tprev, want_assoc=True):
        w, h = self.width >> level, self.height >> level
        f = lambda a, n: np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(n))
        Rc, tc, Ri, tp = f(Rcurr, 9), f(tcurr, 3), f(Rprev_inv, 9), f(tprev, 3)
        assoc = np.zeros(h * w, dtype=np.int32) if want_assoc else None
        out = np.zeros(29, dtype=np.float64)
        self._check(self._L.odo_debug_icp_step(self._h, level, _fptr(Rc), _fptr(tc), _fptr(Ri), _fptr(tp),
                                               assoc.ctypes.data if want_assoc else None, _dptr(out)),
                    "debug_icp_step")
        return out, (assoc.reshape(h, w) if want_assoc else None)

    def debug_icp_sums(self, level, Rcurr, tcurr, Rprev_inv, tprev):
        """The 29 ICP sums as a tracking iteration hands them to the solve
        (handle precision, tracker reduction order)."""
        f = lambda a, n: np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(n))
        Rc, tc, Ri, tp = f(Rcurr, 9), f(tcurr, 3), f(Rprev_inv, 9), f(tprev, 3)
        out = np.zeros(29, dtype=np.float64)
        self._check(self._L.odo_debug_icp_sums(self._h, level, _fptr(Rc), _fptr(tc), _fptr(Ri), _fptr(tp),
                                               _dptr(out)), "debug_icp_sums")
        return out

    def debug_rgb_sums(self, level, sigma):
        out = np.zeros(29, dtype=np.float64)
        self._check(self._L.odo_debug_rgb_sums(self._h, level, float(sigma), _dptr(out)), "debug_rgb_sums")
        return out

    def debug_rgb_residual(self, level, krkinv, kt):
        k = np.ascontiguousarray(np.asarray(krkinv, dtype=np.float32).reshape(9))
        t = np.ascontiguousarray(np.asarray(kt, dtype=np.float32).reshape(3))
        out = (ctypes.c_int32 * 2)()
        self._check(self._L.odo_debug_rgb_residual(self._h, level, _fptr(k), _fptr(t), out), "debug_rgb_residual")
        return int(out[0]), int(out[1])

    def debug_rgb_step(self, level, sigma):
        out = np.zeros(29, dtype=np.float64)
        self._check(self._L.odo_debug_rgb_step(self._h, level, float(sigma), _dptr(out)), "debug_rgb_step")
        return out

    def debug_so3_step(self, H, kinv, krlr):
        f = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(9))
        out = np.zeros(11, dtype=np.float64)
        self._check(self._L.odo_debug_so3_step(self._h, _fptr(f(H)), _fptr(f(kinv)), _fptr(f(krlr)), _dptr(out)),
                    "debug_so3_step")
        return out

    def time_iteration(self, level, reps=50):
        """Mean CUDA-event times (ms) of the association kernel, the
        photometric/solve kernel and one whole iteration at `level`."""
        out = (ctypes.c_float * 3)()
        self._check(self._L.odo_debug_time_iteration(self._h, level, int(reps), out), "time_iteration")
        return list(out)

    def profile(self, reset=True):
        """Device phase timers in microseconds per solve: (partial reduction,
        FP64 solve + pose update, residual finish, number of solves)."""
        out = np.zeros(8, np.float64)
        self._check(self._L.odo_debug_profile(self._h, _dptr(out), int(bool(reset))), "profile")
        n = max(out[3], 1.0)
        us = lambda k: out[k] / n / 1e3
        return {"reduce_us": us(0), "solve_us": us(1), "residual_finish_us": us(2), "solves": int(out[3]),
                "ldlt_us": us(4), "exp_compose_us": us(5), "pose_polar_us": us(6), "warp_us": us(7)}

    def history(self):
        """[n, 9] per-iteration record of the last tracking call: ICP inliers,
        photometric count, sigma, increment (v, omega)."""
        out = np.zeros((32, 9), np.float64)
        n = self._L.odo_debug_history(self._h, _dptr(out), 32)
        if n < 0:
            self._check(n, "history")
        return out[:n]

    def debug_derivatives(self):
        self._check(self._L.odo_debug_derivatives(self._h), "debug_derivatives")


def filter_depth(raw, maxD, out=None):
    """depth_bilateral.frag (src/gl/shaders/depth_bilateral.frag:30-76) on the
    GPU: raw u16 depth (mm, CUDA tensor [h][w]) -> filtered u16 depth, on the
    current torch stream."""
    import torch
    L = _native.load()
    pitch = _check_cuda_tensor(raw, torch.uint16, (), "raw")
    h, w = raw.shape
    out = torch.empty((h, w), dtype=torch.uint16, device=raw.device) if out is None else out
    opitch = _check_cuda_tensor(out, torch.uint16, (), "out")
    rc = L.odo_filter_depth(raw.data_ptr(), pitch, out.data_ptr(), opitch, w, h, float(maxD),
                            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    if rc != 0:
        raise OdometryError(rc, "odo_filter_depth failed")
    return out


def depth_metric(raw, maxD, out=None):
    """depth_metric.frag (src/gl/shaders/depth_metric.frag:28-40) on the GPU:
    raw u16 depth (mm) -> float metres, 0 outside [300 mm, maxD]."""
    import torch
    L = _native.load()
    pitch = _check_cuda_tensor(raw, torch.uint16, (), "raw")
    h, w = raw.shape
    out = torch.empty((h, w), dtype=torch.float32, device=raw.device) if out is None else out
    opitch = _check_cuda_tensor(out, torch.float32, (), "out")
    rc = L.odo_depth_metric(raw.data_ptr(), pitch, out.data_ptr(), opitch, w, h, float(maxD),
                            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    if rc != 0:
        raise OdometryError(rc, "odo_depth_metric failed")
    return out
