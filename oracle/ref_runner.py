"""Runs the reference's own kernels (oracle/_ref/ref_kernels.cubin, built by
oracle/build_ref.py) on the GPU through the CUDA driver API, sharing torch's
context and current stream.  TEST INFRASTRUCTURE ONLY: the bit-exact oracle
of the tests and of the golden fixtures.

Every method takes and returns dense CUDA tensors; buffers are sized exactly
for the kernels' index ranges.
"""
import ctypes
import os

import numpy as np

from . import build_ref

# exported names of the reference kernels (Itanium-mangled by nvcc)
K = {
    "pyrDown": "_Z18pyrDownGaussKernel9PtrStepSzItES0_f",
    "vmap": "_Z17computeVmapKernel9PtrStepSzItE7PtrStepIfEfffff",
    "nmap": "_Z17computeNmapKernelii7PtrStepIfES0_",
    "transform": "_Z18tranformMapsKernelii7PtrStepIfES0_5mat336float39PtrStepSzIfES0_",
    "copyMaps": "_Z14copyMapsKerneliiPKfS0_9PtrStepSzIfE7PtrStepIfE",
    "resizeV": "_Z15resizeMapKernelILb0EEviii7PtrStepIfES1_",
    "resizeN": "_Z15resizeMapKernelILb1EEviii7PtrStepIfES1_",
    "gaussF": "_Z19pyrDownKernelGaussF9PtrStepSzIfES0_Pf",
    "gaussU8": "_Z27pyrDownKernelIntensityGauss9PtrStepSzIhES0_Pf",
    "vertsToDepth": "_Z21verticesToDepthKernelPKf9PtrStepSzIfEf",
    "intensity": "_Z19bgr2IntensityKernel9PtrStepSzIhE",
    "deriv": "_Z11applyKernel9PtrStepSzIhE7PtrStepIsES2_",
    "cloud": "_Z19projectPointsKernel9PtrStepSzIfES_I6float3Effff",
}

# DataTerm (src/cuda/types.cuh:75-81): short2 zero, short2 one, float diff, bool valid
DATATERM = np.dtype({"names": ["zero_x", "zero_y", "one_x", "one_y", "diff", "valid"],
                     "formats": [np.int16, np.int16, np.int16, np.int16, np.float32, np.uint8],
                     "offsets": [0, 2, 4, 6, 8, 12], "itemsize": 16})

# computeDerivativeImages filter constants (src/odom/utils.cu:614-620)
SOBEL_X = [0.52201, 0.00000, -0.52201, 0.79451, -0.00000, -0.79451, 0.52201, 0.00000, -0.52201]
SOBEL_Y = [0.52201, 0.79451, 0.52201, 0.00000, 0.00000, 0.00000, -0.52201, -0.79451, -0.52201]
GAUSS = [1, 4, 6, 4, 1, 4, 16, 24, 16, 4, 6, 24, 36, 24, 6, 4, 16, 24, 16, 4, 1, 4, 6, 4, 1]


class PtrStepSz(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("step", ctypes.c_size_t), ("cols", ctypes.c_int), ("rows", ctypes.c_int)]


class PtrStep(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("step", ctypes.c_size_t)]


class Mat33(ctypes.Structure):
    _fields_ = [("m", ctypes.c_float * 9)]


class Float3(ctypes.Structure):
    _fields_ = [("v", ctypes.c_float * 3)]


def available():
    return build_ref.build_ref() is not None


class RefKernels:
    def __init__(self):
        import torch
        path = build_ref.build_ref()
        if path is None:
            raise FileNotFoundError("reference cubin not available")
        torch.cuda.init()
        torch.empty(1, device="cuda")  # make torch's primary context current
        self.torch = torch
        self.cu = ctypes.CDLL("libcuda.so.1")
        ctx = ctypes.c_void_p()
        self._ck(self.cu.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context")
        self.mod = ctypes.c_void_p()
        self._ck(self.cu.cuModuleLoad(ctypes.byref(self.mod), path.encode()), "cuModuleLoad")
        self.fn = {}
        for key, name in list(K.items()) + [(n, n) for n in ("shim_icp_pixels", "shim_rgb_residual",
                                                            "shim_rgb_step", "shim_so3_pixels", "shim_set_rgba",
                                                            "shim_warp_variants")]:
            f = ctypes.c_void_p()
            self._ck(self.cu.cuModuleGetFunction(ctypes.byref(f), self.mod, name.encode()), name)
            self.fn[key] = f
        self._set_const("gsobel_x3x3", SOBEL_X)
        self._set_const("gsobel_y3x3", SOBEL_Y)
        self.gauss = torch.tensor(GAUSS, dtype=torch.float32, device="cuda")

    def _ck(self, rc, what):
        if rc != 0:
            s = ctypes.c_char_p()
            self.cu.cuGetErrorString(rc, ctypes.byref(s))
            raise RuntimeError(f"{what}: CUDA driver error {rc} {s.value}")

    def _set_const(self, name, values):
        ptr = ctypes.c_uint64()
        size = ctypes.c_size_t()
        self._ck(self.cu.cuModuleGetGlobal_v2(ctypes.byref(ptr), ctypes.byref(size), self.mod, name.encode()), name)
        arr = np.asarray(values, np.float32)
        assert size.value == arr.nbytes
        self._ck(self.cu.cuMemcpyHtoD_v2(ptr, arr.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(arr.nbytes)), name)

    def _launch(self, key, grid, block, args):
        ptrs = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p) for a in args])
        stream = ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)
        gx, gy = grid
        bx, by = block
        self._ck(self.cu.cuLaunchKernel(self.fn[key], gx, gy, 1, bx, by, 1, 0, stream, ptrs, None), key)

    # ---- helpers ------------------------------------------------------
    @staticmethod
    def _pss(t, cols, rows):
        return PtrStepSz(t.data_ptr(), t.stride(0) * t.element_size(), cols, rows)

    @staticmethod
    def _ps(t):
        return PtrStep(t.data_ptr(), t.stride(0) * t.element_size())

    @staticmethod
    def _g2(cols, rows):
        return ((cols + 31) // 32, (rows + 7) // 8), (32, 8)

    def _empty(self, shape, dtype, fill=0):
        return self.torch.full(shape, fill, dtype=dtype, device="cuda")

    # ---- image kernels (src/odom/utils.cu) ------------------------------
    def pyr_down_depth(self, src):
        h, w = src.shape
        dst = self._empty((h // 2, w // 2), self.torch.int16).view(self.torch.uint16)
        g, b = self._g2(w // 2, h // 2)
        self._launch("pyrDown", g, b, [self._pss(src, w, h), self._pss(dst, w // 2, h // 2), ctypes.c_float(30.0)])
        return dst

    def vmap(self, depth, fx, fy, cx, cy, cutoff, fill=0.0):
        h, w = depth.shape
        vm = self._empty((3 * h, w), self.torch.float32, fill)
        g, b = self._g2(w, h)
        fxi = np.float32(1.0) / np.float32(fx)
        fyi = np.float32(1.0) / np.float32(fy)
        self._launch("vmap", g, b, [self._pss(depth, w, h), self._ps(vm), ctypes.c_float(fxi), ctypes.c_float(fyi),
                                    ctypes.c_float(cx), ctypes.c_float(cy), ctypes.c_float(cutoff)])
        return vm

    def nmap(self, vm):
        h3, w = vm.shape
        h = h3 // 3
        nm = self._empty((3 * h, w), self.torch.float32)
        g, b = self._g2(w, h)
        self._launch("nmap", g, b, [ctypes.c_int(h), ctypes.c_int(w), self._ps(vm), self._ps(nm)])
        return nm

    def copy_maps(self, v4, n4):
        h, w, _ = v4.shape
        vm = self._empty((3 * h, w), self.torch.float32)
        nm = self._empty((3 * h, w), self.torch.float32)
        g, b = self._g2(w, h)
        self._launch("copyMaps", g, b, [ctypes.c_int(h), ctypes.c_int(w), ctypes.c_void_p(v4.data_ptr()),
                                        ctypes.c_void_p(n4.data_ptr()), self._pss(vm, w, 3 * h), self._ps(nm)])
        return vm, nm

    def resize(self, m, normalize, fill=0.0):
        h3, w = m.shape
        sh = h3 // 3
        dh, dw = sh // 2, w // 2
        out = self._empty((3 * dh, dw), self.torch.float32, fill)
        g, b = self._g2(dw, dh)
        self._launch("resizeN" if normalize else "resizeV", g, b,
                     [ctypes.c_int(dh), ctypes.c_int(dw), ctypes.c_int(sh), self._ps(m), self._ps(out)])
        return out

    def transform(self, vm, nm, R, t):
        h3, w = vm.shape
        h = h3 // 3
        vm, nm = vm.clone(), nm.clone()
        g, b = self._g2(w, h)
        M = Mat33((ctypes.c_float * 9)(*np.asarray(R, np.float32).reshape(9)))
        T = Float3((ctypes.c_float * 3)(*np.asarray(t, np.float32).reshape(3)))
        self._launch("transform", g, b, [ctypes.c_int(h), ctypes.c_int(w), self._ps(vm), self._ps(nm), M, T,
                                         self._pss(vm, w, 3 * h), self._ps(nm)])
        return vm, nm

    def gauss_f(self, src):
        h, w = src.shape
        dst = self._empty((h // 2, w // 2), self.torch.float32)
        g, b = self._g2(w // 2, h // 2)
        self._launch("gaussF", g, b, [self._pss(src, w, h), self._pss(dst, w // 2, h // 2),
                                      ctypes.c_void_p(self.gauss.data_ptr())])
        return dst

    def gauss_u8(self, src):
        h, w = src.shape
        dst = self._empty((h // 2, w // 2), self.torch.uint8)
        g, b = self._g2(w // 2, h // 2)
        self._launch("gaussU8", g, b, [self._pss(src, w, h), self._pss(dst, w // 2, h // 2),
                                       ctypes.c_void_p(self.gauss.data_ptr())])
        return dst

    def verts_to_depth(self, v4, cutoff=6.0):
        h, w, _ = v4.shape
        dst = self._empty((h, w), self.torch.float32)
        g, b = self._g2(w, h)
        self._launch("vertsToDepth", g, b, [ctypes.c_void_p(v4.data_ptr()), self._pss(dst, w, h),
                                            ctypes.c_float(cutoff)])
        return dst

    def intensity(self, rgba):
        h, w, _ = rgba.shape
        dst = self._empty((h, w), self.torch.uint8)
        self._launch("shim_set_rgba", (1, 1), (1, 1), [ctypes.c_void_p(rgba.data_ptr()),
                                                       ctypes.c_uint64(rgba.stride(0))])
        g, b = self._g2(w, h)
        self._launch("intensity", g, b, [self._pss(dst, w, h)])
        return dst

    def derivatives(self, src):
        h, w = src.shape
        dx = self._empty((h, w), self.torch.int16)
        dy = self._empty((h, w), self.torch.int16)
        g, b = self._g2(w, h)
        self._launch("deriv", g, b, [self._pss(src, w, h), self._ps(dx), self._ps(dy)])
        return dx, dy

    def cloud(self, depth, fx, fy, cx, cy):
        h, w = depth.shape
        out = self._empty((h, w, 3), self.torch.float32)
        g, b = self._g2(w, h)
        self._launch("cloud", g, b, [self._pss(depth, w, h), PtrStepSz(out.data_ptr(), w * 12, w, h),
                                     ctypes.c_float(np.float32(1.0) / np.float32(fx)),
                                     ctypes.c_float(np.float32(1.0) / np.float32(fy)), ctypes.c_float(cx),
                                     ctypes.c_float(cy)])
        return out

    # ---- reduction functors, per pixel (src/odom/reduce.cu) ----------------
    def _grid1(self, n):
        return ((n + 255) // 256, 1), (256, 1)

    def icp_pixels(self, Rcurr, tcurr, Rprev_inv, tprev, vc, nc, vp, np_, fx, fy, cx, cy, dist, angle):
        h3, w = vc.shape
        h = h3 // 3
        n = h * w
        pose = self.torch.tensor(np.concatenate([np.asarray(Rcurr, np.float32).reshape(9),
                                                 np.asarray(tcurr, np.float32).reshape(3),
                                                 np.asarray(Rprev_inv, np.float32).reshape(9),
                                                 np.asarray(tprev, np.float32).reshape(3)]), device="cuda")
        found = self._empty((h, w), self.torch.int32)
        d = self._empty((h, w, 3), self.torch.float32)
        prod = self._empty((h, w, 29), self.torch.float32)
        g, b = self._grid1(n)
        f = lambda v: ctypes.c_float(v)
        self._launch("shim_icp_pixels", g, b, [ctypes.c_void_p(pose.data_ptr()), ctypes.c_void_p(vc.data_ptr()),
                                               ctypes.c_void_p(nc.data_ptr()), ctypes.c_void_p(vp.data_ptr()),
                                               ctypes.c_void_p(np_.data_ptr()), ctypes.c_uint64(w * 4),
                                               ctypes.c_int(w), ctypes.c_int(h), f(fx), f(fy), f(cx), f(cy), f(dist),
                                               f(angle), ctypes.c_void_p(found.data_ptr()),
                                               ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(prod.data_ptr())])
        return found, d, prod

    def rgb_residual(self, minScale, dIdx, dIdy, lastDepth, nextDepth, lastImage, nextImage, maxDelta, kt, krk):
        h, w = nextImage.shape
        n = h * w
        corres = self._empty((h, w, 16), self.torch.uint8)
        out = self._empty((h, w, 2), self.torch.int32)
        par = self.torch.tensor(np.concatenate([np.asarray(kt, np.float32).reshape(3),
                                                np.asarray(krk, np.float32).reshape(9)]), device="cuda")
        g, b = self._grid1(n)
        p = lambda t: ctypes.c_void_p(t.data_ptr())
        self._launch("shim_rgb_residual", g, b, [ctypes.c_float(minScale), p(dIdx), p(dIdy), ctypes.c_uint64(w * 2),
                                                 p(lastDepth), p(nextDepth), ctypes.c_uint64(w * 4), p(lastImage),
                                                 p(nextImage), ctypes.c_uint64(w), ctypes.c_int(w), ctypes.c_int(h),
                                                 ctypes.c_float(maxDelta), p(par), p(corres), p(out)])
        return corres, out

    def rgb_step(self, corres, sigma, cloud, fx, fy, dIdx, dIdy):
        h, w, _ = corres.shape
        prod = self._empty((h, w, 29), self.torch.float32)
        g, b = self._grid1(h * w)
        p = lambda t: ctypes.c_void_p(t.data_ptr())
        self._launch("shim_rgb_step", g, b, [p(corres), ctypes.c_float(sigma), p(cloud), ctypes.c_uint64(w * 12),
                                             ctypes.c_float(fx), ctypes.c_float(fy), p(dIdx), p(dIdy),
                                             ctypes.c_uint64(w * 2), ctypes.c_int(w), ctypes.c_int(h), p(prod)])
        return prod

    def so3_pixels(self, last, nxt, H, kinv, krlr):
        h, w = nxt.shape
        mats = self.torch.tensor(np.concatenate([np.asarray(m, np.float32).reshape(9) for m in (H, kinv, krlr)]),
                                 device="cuda")
        prod = self._empty((h, w, 11), self.torch.float32)
        g, b = self._grid1(h * w)
        p = lambda t: ctypes.c_void_p(t.data_ptr())
        self._launch("shim_so3_pixels", g, b, [p(last), p(nxt), ctypes.c_uint64(w), ctypes.c_int(w), ctypes.c_int(h),
                                               p(mats), p(prod)])
        return prod

    def warp_variants(self, nextDepth, kt, krk):
        """[h, w, 36, 2] int32: (u0, v0) for every evaluation order of the
        photometric warp (numerator order a, denominator order b -> a*6+b)."""
        h, w = nextDepth.shape
        par = self.torch.tensor(np.concatenate([np.asarray(kt, np.float32).reshape(3),
                                                np.asarray(krk, np.float32).reshape(9)]), device="cuda")
        out = self._empty((h, w, 36, 2), self.torch.int32)
        g, b = self._grid1(h * w)
        self._launch("shim_warp_variants", g, b, [ctypes.c_void_p(nextDepth.data_ptr()), ctypes.c_int(w),
                                                  ctypes.c_int(h), ctypes.c_void_p(par.data_ptr()),
                                                  ctypes.c_void_p(out.data_ptr())])
        return out
