"""ctypes front end of the CPU oracle (oracle/odometry_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker; the product never imports it.

`prec` selects the FP32 restatement (32) or its FP64 twin (64).
"""
import ctypes
import math
import os

import numpy as np

from . import build as _build

_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        path = _build.build_oracle()
        _LIB = ctypes.CDLL(path)
    return _LIB


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class DataTerm(ctypes.Structure):
    _fields_ = [("zero_x", ctypes.c_int16), ("zero_y", ctypes.c_int16), ("one_x", ctypes.c_int16),
                ("one_y", ctypes.c_int16), ("diff", ctypes.c_float), ("valid", ctypes.c_int32)]


DATATERM_DTYPE = np.dtype([("zero_x", np.int16), ("zero_y", np.int16), ("one_x", np.int16), ("one_y", np.int16),
                           ("diff", np.float32), ("valid", np.int32)])


class Stats(ctypes.Structure):
    _fields_ = [("lastICPError", ctypes.c_float), ("lastICPCount", ctypes.c_float),
                ("lastRGBError", ctypes.c_float), ("lastRGBCount", ctypes.c_float),
                ("lastSO3Error", ctypes.c_float), ("lastSO3Count", ctypes.c_float),
                ("lastA", ctypes.c_double * 36), ("lastb", ctypes.c_double * 6)]


def set_threads(n):
    lib().orc_set_threads(int(n))


def get_threads():
    return lib().orc_get_threads()


# ---- integer-output kernels ----------------------------------------------
def pyr_down_depth(src):
    h, w = src.shape
    src = np.ascontiguousarray(src, dtype=np.uint16)
    dst = np.zeros((h // 2, w // 2), np.uint16)
    lib().orc_pyr_down_depth(_p(src), w, h, _p(dst))
    return dst


def bgr_to_intensity(rgba, with_tie=False):
    h, w, _ = rgba.shape
    rgba = np.ascontiguousarray(rgba, dtype=np.uint8)
    dst = np.zeros((h, w), np.uint8)
    tie = np.zeros((h, w), np.uint8) if with_tie else None
    lib().orc_bgr_to_intensity(_p(rgba), w, h, _p(dst), _p(tie))
    return (dst, tie) if with_tie else dst


def pyr_down_uchar_gauss(src, with_tie=False):
    h, w = src.shape
    src = np.ascontiguousarray(src, dtype=np.uint8)
    dst = np.zeros((h // 2, w // 2), np.uint8)
    tie = np.zeros((h // 2, w // 2), np.uint8) if with_tie else None
    lib().orc_pyr_down_uchar_gauss(_p(src), w, h, _p(dst), _p(tie))
    return (dst, tie) if with_tie else dst


def depth_bilateral(raw, maxD, with_tie=False):
    """depth_bilateral.frag (src/gl/shaders/depth_bilateral.frag:30-76) on a
    raw u16 depth image; (filtered, tie flags) when with_tie."""
    raw = np.ascontiguousarray(raw, np.uint16)
    h, w = raw.shape
    out = np.zeros((h, w), np.uint16)
    tie = np.zeros((h, w), np.uint8)
    lib().orc_depth_bilateral(_p(raw), w, h, ctypes.c_float(maxD), _p(out), _p(tie))
    return (out, tie) if with_tie else out


def depth_metric(raw, maxD):
    """depth_metric.frag (src/gl/shaders/depth_metric.frag:28-40): metres."""
    raw = np.ascontiguousarray(raw, np.uint16)
    h, w = raw.shape
    out = np.zeros((h, w), np.float32)
    lib().orc_depth_metric(_p(raw), w, h, ctypes.c_float(maxD), _p(out))
    return out


def model_predict(surfels, t_inv, cam, max_depth=20.0, conf_threshold=10.0, time=1, max_time=2 ** 30,
                  time_delta=2 ** 30):
    """IndexMap::combinedPredict (src/model/shaders/splat.vert, combo_splat.frag)
    on the CPU: (image u8 [h,w,4], vertex f32 [h,w,4], normal f32 [h,w,4], time u16 [h,w])."""
    s = np.ascontiguousarray(surfels, np.float32)
    t = np.ascontiguousarray(np.asarray(t_inv, np.float32).reshape(16))
    w, h = cam.width, cam.height
    image = np.zeros((h, w, 4), np.uint8)
    vertex = np.zeros((h, w, 4), np.float32)
    normal = np.zeros((h, w, 4), np.float32)
    tm = np.zeros((h, w), np.uint16)
    f = ctypes.c_float
    lib().orc_model_predict(_p(s), len(s), _p(t), w, h, f(cam.cx), f(cam.cy), f(cam.fx), f(cam.fy), f(max_depth),
                            f(conf_threshold), int(time), int(max_time), int(time_delta), _p(image), _p(vertex),
                            _p(normal), _p(tm))
    return image, vertex, normal, tm


def fill_in(pv, pn, pi, raw_depth, raw_rgba, cam, passthrough=False):
    """FillIn::vertex / normal / image (src/gl/shaders/fill_*.frag) on the CPU."""
    pv, pn = np.ascontiguousarray(pv, np.float32), np.ascontiguousarray(pn, np.float32)
    pi, rd = np.ascontiguousarray(pi, np.uint8), np.ascontiguousarray(raw_depth, np.uint16)
    rr = np.ascontiguousarray(raw_rgba, np.uint8)
    ov, on, oi = np.zeros_like(pv), np.zeros_like(pn), np.zeros_like(pi)
    f = ctypes.c_float
    lib().orc_fill_in(_p(pv), _p(pn), _p(pi), _p(rd), _p(rr), cam.width, cam.height, f(cam.cx), f(cam.cy),
                      f(cam.fx), f(cam.fy), int(bool(passthrough)), _p(ov), _p(on), _p(oi))
    return ov, on, oi


def derivatives(src, with_tie=False):
    h, w = src.shape
    src = np.ascontiguousarray(src, dtype=np.uint8)
    dx = np.zeros((h, w), np.int16)
    dy = np.zeros((h, w), np.int16)
    tie = np.zeros((h, w), np.uint8) if with_tie else None
    lib().orc_derivatives(_p(src), w, h, _p(dx), _p(dy), _p(tie))
    return (dx, dy, tie) if with_tie else (dx, dy)


# ---- precision-generic kernels ---------------------------------------------
class Kernels:
    def __init__(self, prec=32):
        self.prec = prec
        self.real = np.float32 if prec == 32 else np.float64
        self.ctype = ctypes.c_float if prec == 32 else ctypes.c_double
        self.pre = "orc32_" if prec == 32 else "orc64_"

    def f(self, name):
        return getattr(lib(), self.pre + name)

    def r(self, v):
        return self.ctype(v)

    def arr(self, a, n=None):
        a = np.ascontiguousarray(np.asarray(a, dtype=self.real))
        if n is not None:
            a = a.reshape(n)
        return a

    def create_vmap(self, depth, fx, fy, cx, cy, cutoff, init=None):
        h, w = depth.shape
        depth = np.ascontiguousarray(depth, dtype=np.uint16)
        vmap = np.zeros((3, h, w), self.real) if init is None else np.array(init, dtype=self.real)
        fxi = np.float32(1.0) / np.float32(fx) if self.prec == 32 else 1.0 / float(np.float32(fx))
        fyi = np.float32(1.0) / np.float32(fy) if self.prec == 32 else 1.0 / float(np.float32(fy))
        self.f("create_vmap")(_p(depth), w, h, self.r(fxi), self.r(fyi), self.r(cx), self.r(cy), self.r(cutoff),
                              _p(vmap))
        return vmap

    def create_nmap(self, vmap):
        _, h, w = vmap.shape
        vmap = self.arr(vmap)
        nmap = np.zeros_like(vmap)
        self.f("create_nmap")(_p(vmap), w, h, _p(nmap))
        return nmap

    def copy_maps(self, v4, n4):
        h, w, _ = v4.shape
        v4 = np.ascontiguousarray(v4, np.float32)
        n4 = np.ascontiguousarray(n4, np.float32)
        vm = np.zeros((3, h, w), self.real)
        nm = np.zeros((3, h, w), self.real)
        self.f("copy_maps")(_p(v4), _p(n4), w, h, _p(vm), _p(nm))
        return vm, nm

    def resize_map(self, m, normalize):
        _, h, w = m.shape
        m = self.arr(m)
        out = np.zeros((3, h // 2, w // 2), self.real)
        self.f("resize_map")(_p(m), w, h, _p(out), int(normalize))
        return out

    def transform_maps(self, vm, nm, R, t):
        _, h, w = vm.shape
        vm = self.arr(vm).copy()
        nm = self.arr(nm).copy()
        R = self.arr(R, 9)
        t = self.arr(t, 3)
        self.f("transform_maps")(_p(vm), _p(nm), w, h, _p(R), _p(t), _p(vm), _p(nm))
        return vm, nm

    def pyr_down_gauss_f(self, src):
        h, w = src.shape
        src = self.arr(src)
        dst = np.zeros((h // 2, w // 2), self.real)
        self.f("pyr_down_gauss_f")(_p(src), w, h, _p(dst))
        return dst

    def vertices_to_depth(self, v4, cutoff=6.0):
        h, w, _ = v4.shape
        v4 = np.ascontiguousarray(v4, np.float32)
        dst = np.zeros((h, w), self.real)
        self.f("vertices_to_depth")(_p(v4), w, h, self.r(cutoff), _p(dst))
        return dst

    def icp_step(self, Rcurr, tcurr, vmap_curr, nmap_curr, Rprev_inv, tprev, fx, fy, cx, cy, vmap_prev, nmap_prev,
                 distThres, angleThres, with_assoc=True):
        _, h, w = vmap_curr.shape
        out = np.zeros(29, np.float64)
        assoc = np.zeros((h, w), np.int32) if with_assoc else None
        tie = np.zeros((h, w), np.uint8) if with_assoc else None
        args = [self.arr(Rcurr, 9), self.arr(tcurr, 3), self.arr(vmap_curr), self.arr(nmap_curr),
                self.arr(Rprev_inv, 9), self.arr(tprev, 3)]
        vp, np_ = self.arr(vmap_prev), self.arr(nmap_prev)
        self.f("icp_step")(*[_p(a) for a in args], self.r(fx), self.r(fy), self.r(cx), self.r(cy), _p(vp), _p(np_),
                           self.r(distThres), self.r(angleThres), w, h, _p(out), _p(assoc), _p(tie))
        return out, assoc, tie

    def rgb_residual(self, minScale, dIdx, dIdy, lastDepth, nextDepth, lastImage, nextImage, maxDepthDelta, kt,
                     krkinv):
        h, w = nextImage.shape
        corres = np.zeros((h, w), DATATERM_DTYPE)
        tie = np.zeros((h, w), np.uint8)
        out2 = np.zeros(2, np.int32)
        ld, nd = self.arr(lastDepth), self.arr(nextDepth)
        self.f("rgb_residual")(self.r(minScale), _p(np.ascontiguousarray(dIdx, np.int16)),
                               _p(np.ascontiguousarray(dIdy, np.int16)), _p(ld), _p(nd),
                               _p(np.ascontiguousarray(lastImage, np.uint8)),
                               _p(np.ascontiguousarray(nextImage, np.uint8)), w, h, self.r(maxDepthDelta),
                               _p(self.arr(kt, 3)), _p(self.arr(krkinv, 9)), _p(corres), _p(out2), _p(tie))
        return corres, (int(out2[0]), int(out2[1])), tie

    def project_cloud(self, depth, fx, fy, cx, cy):
        h, w = depth.shape
        cloud = np.zeros((h, w, 3), self.real)
        inv_fx = np.float32(1.0) / np.float32(fx)
        inv_fy = np.float32(1.0) / np.float32(fy)
        self.f("project_cloud")(_p(self.arr(depth)), w, h, self.r(inv_fx), self.r(inv_fy), self.r(cx), self.r(cy),
                                _p(cloud))
        return cloud

    def rgb_step(self, corres, sigma, cloud, fx, fy, dIdx, dIdy, sobelScale=0.125):
        h, w = corres.shape
        out = np.zeros(29, np.float64)
        self.f("rgb_step")(_p(np.ascontiguousarray(corres)), self.r(sigma), _p(self.arr(cloud)), self.r(fx),
                           self.r(fy), _p(np.ascontiguousarray(dIdx, np.int16)),
                           _p(np.ascontiguousarray(dIdy, np.int16)), self.r(sobelScale), w, h, _p(out))
        return out

    def so3_step(self, lastImage, nextImage, H, kinv, krlr):
        h, w = nextImage.shape
        out = np.zeros(11, np.float64)
        self.f("so3_step")(_p(np.ascontiguousarray(lastImage, np.uint8)), _p(np.ascontiguousarray(nextImage, np.uint8)),
                           w, h, _p(self.arr(H, 9)), _p(self.arr(kinv, 9)), _p(self.arr(krlr, 9)), _p(out))
        return out


def set_flip_ties(prec, mode):
    """Decisions flagged as rounding ties are taken the other way in the
    per-pixel kernels of the given precision: mode 0 none, 1 all, 2 / 3 the
    two halves of a hash of the tied value."""
    Kernels(prec).f("set_flip_ties")(int(mode))


def set_reverse_sums(prec, mode):
    """Summation-order perturbations of every pairwise sum of the given
    precision: 0 / False none, 1 / True records in reverse order, 2 another
    tree (split at a third, leaves of at most 5 records)."""
    Kernels(prec).f("set_reverse_sums")(int(mode))


def ldlt_solve6(A, b):
    A = np.ascontiguousarray(A, np.float64).reshape(36)
    b = np.ascontiguousarray(b, np.float64).reshape(6)
    x = np.zeros(6, np.float64)
    lib().orc64_ldlt_solve6(_p(A), _p(b), _p(x))
    return x


def rodrigues(w):
    w = np.ascontiguousarray(w, np.float64).reshape(3)
    R = np.zeros(9, np.float64)
    lib().orc64_rodrigues(_p(w), _p(R))
    return R.reshape(3, 3)


class Odometry:
    """CPU restatement of RGBDOdometryef over host numpy arrays."""

    BUF = {"depth_tmp": 0, "vmap_curr": 1, "nmap_curr": 2, "vmap_prev": 3, "nmap_prev": 4, "lastDepth": 5,
           "nextDepth": 6, "lastImage": 7, "nextImage": 8, "lastNextImage": 9, "dIdx": 10, "dIdy": 11,
           "corres": 12, "cloud": 13}

    def __init__(self, width, height, cx, cy, fx, fy, distThresh, angleThresh, prec=32):
        self.k = Kernels(prec)
        self.prec = prec
        self.width, self.height = width, height
        L = lib()
        self._create = self.k.f("odo_create")
        self._create.restype = ctypes.c_void_p
        self._h = ctypes.c_void_p(self._create(width, height, ctypes.c_float(cx), ctypes.c_float(cy),
                                               ctypes.c_float(fx), ctypes.c_float(fy), ctypes.c_float(distThresh),
                                               ctypes.c_float(angleThresh)))
        self.k.f("odo_buffer").restype = ctypes.c_void_p
        self._stats = Stats()

    def close(self):
        if self._h:
            self.k.f("odo_destroy")(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def initICP(self, a, b=None, depthCutoff=20.0):
        if b is None or not isinstance(b, np.ndarray):
            if b is not None:
                depthCutoff = b
            d = np.ascontiguousarray(a, np.uint16)
            self.k.f("odo_init_icp_depth")(self._h, _p(d), ctypes.c_float(depthCutoff))
        else:
            v = np.ascontiguousarray(a, np.float32)
            n = np.ascontiguousarray(b, np.float32)
            self.k.f("odo_init_icp_maps")(self._h, _p(v), _p(n), ctypes.c_float(depthCutoff))

    def initICPModel(self, verts, norms, depthCutoff, pose):
        v = np.ascontiguousarray(verts, np.float32)
        n = np.ascontiguousarray(norms, np.float32)
        p = np.ascontiguousarray(np.asarray(pose, np.float32).reshape(16))
        self.k.f("odo_init_icp_model")(self._h, _p(v), _p(n), ctypes.c_float(depthCutoff), _p(p))

    def initRGB(self, rgba):
        self.k.f("odo_init_rgb")(self._h, _p(np.ascontiguousarray(rgba, np.uint8)))

    def initRGBModel(self, rgba):
        self.k.f("odo_init_rgb_model")(self._h, _p(np.ascontiguousarray(rgba, np.uint8)))

    def initFirstRGB(self, rgba):
        self.k.f("odo_init_first_rgb")(self._h, _p(np.ascontiguousarray(rgba, np.uint8)))

    def getIncrementalTransformation(self, trans, rot, rgbOnly=False, icpWeight=10.0, pyramid=True, fastOdom=False,
                                     so3=True):
        t = np.ascontiguousarray(np.asarray(trans, self.k.real).reshape(3)).copy()
        R = np.ascontiguousarray(np.asarray(rot, self.k.real).reshape(9)).copy()
        self.k.f("odo_track")(self._h, _p(t), _p(R), int(bool(rgbOnly)), ctypes.c_float(icpWeight),
                              int(bool(pyramid)), int(bool(fastOdom)), int(bool(so3)))
        self.k.f("odo_stats")(self._h, ctypes.byref(self._stats))
        return t, R.reshape(3, 3)

    def set_schedule(self, levels, iterations=(0, 0, 0)):
        """Iterate only the first `levels` pyramid levels, with iterations[l]
        in place of the reference's count where it is > 0 (levels <= 0: the
        reference's schedule) -- the batched tracker's per-pair schedule."""
        it = (ctypes.c_int * 3)(*[int(v) for v in iterations])
        self.k.f("odo_set_schedule")(self._h, int(levels), it)

    def getCovariance(self):
        out = np.zeros(36, np.float64)
        self.k.f("odo_covariance")(self._h, _p(out))
        return out.reshape(6, 6)

    def iterations(self):
        out = (ctypes.c_int * 4)()
        self.k.f("odo_iters")(self._h, out)
        return list(out)

    def history(self):
        out = np.zeros((32, 9), np.float64)
        n = self.k.f("odo_history")(self._h, _p(out), 32)
        return out[:n]

    @property
    def stats(self):
        s = self._stats
        return {"lastICPError": s.lastICPError, "lastICPCount": s.lastICPCount, "lastRGBError": s.lastRGBError,
                "lastRGBCount": s.lastRGBCount, "lastSO3Error": s.lastSO3Error, "lastSO3Count": s.lastSO3Count,
                "lastA": np.array(s.lastA).reshape(6, 6), "lastb": np.array(s.lastb)}

    def set_buffer(self, name, level, arr):
        """Overwrites one of the handle's buffers (same shapes and types as
        buffer())."""
        cur = self.buffer(name, level)
        a = np.ascontiguousarray(np.asarray(arr).astype(cur.dtype, copy=False).reshape(cur.shape))
        ptr = self.k.f("odo_buffer")(self._h, self.BUF[name], level)
        ctypes.memmove(ptr, a.ctypes.data, a.nbytes)

    def set_flip_decision(self, index):
        """The tracking loop takes its decision number `index` (SO3
        convergence / divergence tests, the rgbOnly early exit, in the order
        taken) the other way; -1: none."""
        self.k.f("odo_set_flip_decision")(self._h, int(index))

    def decision_margin(self):
        """(smallest relative margin of the last call's loop decisions, its
        index or -1)."""
        f = self.k.f("odo_decision_margin")
        f.restype = ctypes.c_double
        idx = ctypes.c_int()
        m = f(self._h, ctypes.byref(idx))
        return m, idx.value

    def keep_derivatives(self, keep=True):
        """Tracking calls use the derivative images set with set_buffer
        instead of computing them from nextImage."""
        self.k.f("odo_set_keep_derivatives")(self._h, int(bool(keep)))

    def buffer(self, name, level):
        which = self.BUF[name]
        ptr = self.k.f("odo_buffer")(self._h, which, level)
        w, h = self.width >> level, self.height >> level
        n = w * h
        r = self.k.real
        spec = {0: (np.uint16, (h, w)), 1: (r, (3, h, w)), 2: (r, (3, h, w)), 3: (r, (3, h, w)), 4: (r, (3, h, w)),
                5: (r, (h, w)), 6: (r, (h, w)), 7: (np.uint8, (h, w)), 8: (np.uint8, (h, w)),
                9: (np.uint8, (h, w)), 10: (np.int16, (h, w)), 11: (np.int16, (h, w)), 12: (DATATERM_DTYPE, (h, w)),
                13: (r, (h, w, 3))}[which]
        dt = np.dtype(spec[0])
        size = int(np.prod(spec[1])) * dt.itemsize
        buf = (ctypes.c_char * size).from_address(ptr)
        return np.frombuffer(buf, dtype=dt).reshape(spec[1]).copy()


# ---------------------------------------------------------------- warm-start network
def cnn_layout():
    w = (ctypes.c_size_t * 8)()
    b = (ctypes.c_size_t * 8)()
    t = ctypes.c_size_t()
    lib().cnn_layout(w, b, ctypes.byref(t))
    return list(w), list(b), t.value


def cnn_run(params, inputs_f16, labels, metric, rounding=True, want_grad=True):
    """Forward + loss (+ gradients) of the warm-start network on the CPU.
    params: FP32 parameter vector; inputs_f16: uint16 [B,120,160,8] (FP16
    bits); labels [B,6]; metric: 6x6 loss metric.  Returns (out [B,6], loss,
    grad or None)."""
    p = np.ascontiguousarray(params, np.float64)
    x = np.ascontiguousarray(inputs_f16, np.uint16)
    B = x.shape[0]
    lab = np.ascontiguousarray(labels, np.float64).reshape(B, 6)
    sc = np.ascontiguousarray(metric, np.float64).reshape(36)
    out = np.zeros((B, 6), np.float64)
    loss = ctypes.c_double()
    grad = np.zeros_like(p) if want_grad else None
    f = lib().cnn_oracle_run
    f.restype = ctypes.c_int
    f(_p(p), x.ctypes.data_as(ctypes.c_void_p), _p(lab), _p(sc), ctypes.c_int(B), ctypes.c_int(int(bool(rounding))),
      _p(out), ctypes.byref(loss), _p(grad) if want_grad else None)
    return out, loss.value, grad
