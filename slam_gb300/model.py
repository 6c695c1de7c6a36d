"""Model prediction and fill-in on the GPU: the producers of the maps that
initICPModel / initRGBModel consume (C ABI odo_model_predict, odo_fill_in).

Surfels are the reference's Vertex records (src/model/shaders/surfels.glsl
and data.vert): [n][12] float32 -- position xyz + confidence, packed colour,
unused, initialisation time, last update time, normal xyz + radius."""
import ctypes

import numpy as np

from . import _native
from .odometry import OdometryError, _check_cuda_tensor


def encode_color(rgb):
    """encodeColor of src/model/shaders/color.glsl: (r << 16) + (g << 8) + b
    as a float, from u8 channels."""
    rgb = np.asarray(rgb, np.int64)
    return ((rgb[..., 0] << 16) + (rgb[..., 1] << 8) + rgb[..., 2]).astype(np.float32)


def surfel_radius(depth, norm_z, fx, fy):
    """getRadius of src/model/shaders/surfels.glsl:18-33 (FP32); the shader's
    cam holds 1/fx, 1/fy (src/model/shaders/data.vert:36)."""
    depth = np.asarray(depth, np.float32)
    cz, cw = np.float32(1.0) / np.float32(fx), np.float32(1.0) / np.float32(fy)
    mean_focal = np.float32(((np.float32(1.0) / np.abs(cz)) + (np.float32(1.0) / np.abs(cw))) / np.float32(2.0))
    radius = (depth / mean_focal) * np.float32(1.41421356237)
    radius_n = radius / np.abs(np.asarray(norm_z, np.float32))
    return np.minimum(np.float32(2.0) * radius, radius_n).astype(np.float32)


def surfels_from_view(vert, norm, rgba, pose, cam, conf=10.0, t_init=1, t_last=1, stride=1):
    """A surfel map from one camera-frame view (vertex / normal RGBA32F maps,
    RGBA colour) seen from `pose` (camera-to-world): one surfel per valid
    pixel (every `stride`-th), in world coordinates, radius from getRadius."""
    v = np.asarray(vert, np.float32)[::stride, ::stride].reshape(-1, 4)
    n = np.asarray(norm, np.float32)[::stride, ::stride].reshape(-1, 4)
    c = np.asarray(rgba)[::stride, ::stride].reshape(-1, 4)
    ok = (v[:, 2] > 0) & np.isfinite(n[:, 0])
    v, n, c = v[ok], n[ok], c[ok]
    T = np.asarray(pose, np.float64)
    pw = (v[:, :3].astype(np.float64) @ T[:3, :3].T + T[:3, 3]).astype(np.float32)
    nw = (n[:, :3].astype(np.float64) @ T[:3, :3].T).astype(np.float32)
    out = np.zeros((len(v), 12), np.float32)
    out[:, 0:3] = pw
    out[:, 3] = conf
    out[:, 4] = encode_color(c[:, :3])
    out[:, 6] = t_init
    out[:, 7] = t_last
    out[:, 8:11] = nw
    out[:, 11] = surfel_radius(v[:, 2], n[:, 2], cam.fx, cam.fy)
    return out


def predict_params(cam, max_depth=20.0, conf_threshold=10.0, time=1, max_time=2 ** 30, time_delta=2 ** 30):
    p = _native.OdoPredictParams()
    p.width, p.height = cam.width, cam.height
    p.cx, p.cy, p.fx, p.fy = cam.cx, cam.cy, cam.fx, cam.fy
    p.maxDepth, p.confThreshold = float(max_depth), float(conf_threshold)
    p.time, p.maxTime, p.timeDelta = int(time), int(max_time), int(time_delta)
    return p


def t_inv_of(pose):
    """The camera-from-world matrix as the prediction reads it (float32,
    row-major), inverted in FP64."""
    return np.linalg.inv(np.asarray(pose, np.float64)).astype(np.float32)


def predict(surfels, pose, params, scratch=None):
    """IndexMap::combinedPredict on the GPU.  surfels: CUDA float32 [n, 12].
    Returns CUDA tensors (image [h,w,4] u8, vertex [h,w,4] f32, normal
    [h,w,4] f32, time [h,w] u16)."""
    import torch
    L = _native.load()
    if not (isinstance(surfels, torch.Tensor) and surfels.is_cuda and surfels.dtype == torch.float32 and
            surfels.dim() == 2 and surfels.shape[1] == 12 and surfels.is_contiguous()):
        raise ValueError("surfels must be a contiguous CUDA float32 tensor [n, 12]")
    w, h = params.width, params.height
    dev = surfels.device
    need = L.odo_model_predict_scratch_bytes(w, h)
    if scratch is None or scratch.numel() * scratch.element_size() < need:
        scratch = torch.empty(need // 8, dtype=torch.int64, device=dev)
    image = torch.empty((h, w, 4), dtype=torch.uint8, device=dev)
    vertex = torch.empty((h, w, 4), dtype=torch.float32, device=dev)
    normal = torch.empty((h, w, 4), dtype=torch.float32, device=dev)
    time = torch.empty((h, w), dtype=torch.uint16, device=dev)
    ti = np.ascontiguousarray(t_inv_of(pose))
    rc = L.odo_model_predict(ctypes.c_void_p(surfels.data_ptr()), surfels.shape[0],
                             ti.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), ctypes.byref(params),
                             ctypes.c_void_p(scratch.data_ptr()), ctypes.c_void_p(image.data_ptr()), w * 4,
                             ctypes.c_void_p(vertex.data_ptr()), ctypes.c_void_p(normal.data_ptr()), w * 16,
                             ctypes.c_void_p(time.data_ptr()), w * 2,
                             ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    if rc != 0:
        raise OdometryError(rc, "odo_model_predict failed")
    return image, vertex, normal, time


def fill_in(pred_vertex, pred_normal, pred_image, raw_depth, raw_rgba, cam, passthrough=False):
    """FillIn::vertex / normal / image on the GPU (CUDA tensors as returned by
    predict(); raw_depth u16 [h,w] filtered depth in mm, raw_rgba u8 [h,w,4])."""
    import torch
    L = _native.load()
    h, w = raw_depth.shape
    mp = _check_cuda_tensor(pred_vertex, torch.float32, (4,), "pred_vertex")
    if _check_cuda_tensor(pred_normal, torch.float32, (4,), "pred_normal") != mp:
        raise ValueError("predicted maps must share a pitch")
    ip = _check_cuda_tensor(pred_image, torch.uint8, (4,), "pred_image")
    dp = _check_cuda_tensor(raw_depth, torch.uint16, (), "raw_depth")
    rp = _check_cuda_tensor(raw_rgba, torch.uint8, (4,), "raw_rgba")
    ov = torch.empty_like(pred_vertex)
    on = torch.empty_like(pred_normal)
    oi = torch.empty_like(pred_image)
    rc = L.odo_fill_in(ctypes.c_void_p(pred_vertex.data_ptr()), ctypes.c_void_p(pred_normal.data_ptr()), mp,
                       ctypes.c_void_p(pred_image.data_ptr()), ip, ctypes.c_void_p(raw_depth.data_ptr()), dp,
                       ctypes.c_void_p(raw_rgba.data_ptr()), rp, w, h, cam.cx, cam.cy, cam.fx, cam.fy,
                       int(bool(passthrough)), ctypes.c_void_p(ov.data_ptr()), ctypes.c_void_p(on.data_ptr()),
                       ov.stride(0) * 4, ctypes.c_void_p(oi.data_ptr()), oi.stride(0),
                       ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    if rc != 0:
        raise OdometryError(rc, "odo_fill_in failed")
    return ov, on, oi
