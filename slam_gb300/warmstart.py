"""Learned warm start of the tracker (C ABI odo_cnn_*; no counterpart in the
reference).

A BF16 CNN proposes the SE(3) motion of a frame pair from both frames'
160x120 depth and gray images; its forward and backward products run on the
library's tcgen05 GEMM.  Inputs are CUDA tensors: [B, 120, 160, 8] float16
(model depth m, model gray, live depth m, live gray, live - model gray, live
- model depth, valid-depth fractions of both frames); outputs [B, 6] float32
(translation m, rotation vector rad).
"""
import ctypes

import numpy as np

from . import _native
from .odometry import OdometryError

IN_H, IN_W, IN_C = 120, 160, 8
DEFAULT_LOSS_METRIC = np.diag([100.0, 100.0, 100.0, 36.0, 36.0, 36.0])


class WarmStartNet:
    def __init__(self, max_batch=256, seed=1, stream=None):
        self._L = _native.load()
        h = ctypes.c_void_p()
        rc = self._L.odo_cnn_create(int(max_batch), ctypes.byref(h))
        if rc != 0:
            raise OdometryError(rc, "odo_cnn_create failed (%s)" % self._L.odo_status_string(rc).decode())
        self._h = h
        self.max_batch = int(max_batch)
        if stream is None:
            import torch
            stream = torch.cuda.current_stream().cuda_stream
        self._check(self._L.odo_cnn_set_stream(self._h, ctypes.c_void_p(stream)), "odo_cnn_set_stream")
        if seed != 1:
            self._check(self._L.odo_cnn_init_params(self._h, ctypes.c_uint64(seed)), "odo_cnn_init_params")

    def _check(self, rc, what):
        if rc != 0:
            raise OdometryError(rc, "%s: %s %s" % (what, self._L.odo_status_string(rc).decode(),
                                                   self._L.odo_cnn_last_error(self._h).decode()))

    def close(self):
        if getattr(self, "_h", None):
            self._L.odo_cnn_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def param_count():
        return int(_native.load().odo_cnn_param_count())

    def get_params(self):
        p = np.zeros(self.param_count(), np.float32)
        self._check(self._L.odo_cnn_get_params(self._h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float))),
                    "odo_cnn_get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32).reshape(-1)
        if p.size != self.param_count():
            raise ValueError("expected %d parameters" % self.param_count())
        self._check(self._L.odo_cnn_set_params(self._h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float))),
                    "odo_cnn_set_params")

    def set_loss_metric(self, M):
        """Loss e^T M e (M symmetric 6x6; e = output - label)."""
        m = np.ascontiguousarray(M, np.float32).reshape(6, 6)
        m = np.ascontiguousarray(0.5 * (m + m.T), np.float32)
        self._check(self._L.odo_cnn_set_loss_metric(self._h, m.ctypes.data_as(ctypes.POINTER(ctypes.c_float))),
                    "odo_cnn_set_loss_metric")

    def _inp(self, x):
        import torch
        if not (isinstance(x, torch.Tensor) and x.is_cuda and x.dtype == torch.float16 and x.is_contiguous()
                and x.dim() == 4 and tuple(x.shape[1:]) == (IN_H, IN_W, IN_C)):
            raise ValueError("input must be a contiguous CUDA float16 tensor [B, 120, 160, 8]")
        if not 1 <= x.shape[0] <= self.max_batch:
            raise ValueError("batch must be in 1..%d" % self.max_batch)
        return x.shape[0]

    def pack(self, frame_pairs, out):
        """Network inputs of FramePairs (level-0 size (160 s) x (120 s)) into
        out[:len(frame_pairs)] (CUDA float16 [>= n, 120, 160, 8])."""
        import torch
        n = len(frame_pairs)
        if not (isinstance(out, torch.Tensor) and out.is_cuda and out.dtype == torch.float16 and out.is_contiguous()
                and out.dim() == 4 and tuple(out.shape[1:]) == (IN_H, IN_W, IN_C) and out.shape[0] >= n):
            raise ValueError("out must be a contiguous CUDA float16 tensor [>=n, 120, 160, 8]")
        arr = (_native.OdoPair * n)()
        for i, p in enumerate(frame_pairs):
            arr[i] = p.desc()
        self._check(self._L.odo_cnn_pack_input(self._h, arr, n, ctypes.c_void_p(out.data_ptr())),
                    "odo_cnn_pack_input")
        return out

    def propose(self, frame_pairs, out=None):
        """Motion proposals [n, 6] (CUDA float32) of FramePairs: packing and
        forward pass in chunks of max_batch (odo_cnn_propose)."""
        import torch
        n = len(frame_pairs)
        if out is None:
            out = torch.empty((n, 6), dtype=torch.float32, device="cuda")
        arr = (_native.OdoPair * n)()
        for i, p in enumerate(frame_pairs):
            arr[i] = p.desc()
        self._check(self._L.odo_cnn_propose(self._h, arr, n, ctypes.c_void_p(out.data_ptr())), "odo_cnn_propose")
        self._check(self._L.odo_cnn_wait(self._h), "odo_cnn_wait")
        return out

    def forward(self, x, out=None):
        import torch
        B = self._inp(x)
        if out is None:
            out = torch.empty((B, 6), dtype=torch.float32, device=x.device)
        self._check(self._L.odo_cnn_forward(self._h, ctypes.c_void_p(x.data_ptr()), B, ctypes.c_void_p(out.data_ptr())),
                    "odo_cnn_forward")
        return out

    def train_step(self, x, labels, lr, want_loss=True):
        B = self._inp(x)
        loss = ctypes.c_float()
        self._check(self._L.odo_cnn_train_step(self._h, ctypes.c_void_p(x.data_ptr()),
                                               ctypes.c_void_p(labels.data_ptr()), B, float(lr),
                                               ctypes.byref(loss) if want_loss else None), "odo_cnn_train_step")
        return loss.value if want_loss else None

    def gradients(self, x, labels):
        B = self._inp(x)
        g = np.zeros(self.param_count(), np.float32)
        loss = ctypes.c_float()
        self._check(self._L.odo_cnn_gradients(self._h, ctypes.c_void_p(x.data_ptr()),
                                              ctypes.c_void_p(labels.data_ptr()), B,
                                              g.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), ctypes.byref(loss)),
                    "odo_cnn_gradients")
        return g, loss.value


def debug_gemm(A, B, bn=128, layout=0):
    """C = A B^T on the library's tensor-core GEMM (A [M, K], B [N, K] bf16
    CUDA tensors, K a multiple of 8)."""
    import torch
    L = _native.load()
    M, K = A.shape
    N = B.shape[0]
    C = torch.empty((M, N), dtype=torch.float32, device=A.device)
    rc = L.odo_cnn_debug_gemm(ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(B.data_ptr()),
                              ctypes.c_void_p(C.data_ptr()), M, N, K, bn, layout,
                              ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    if rc != 0:
        raise OdometryError(rc, "odo_cnn_debug_gemm: %s" % L.odo_status_string(rc).decode())
    return C


# ---------------------------------------------------------------- SE(3) helpers
def motion_vec(T):
    """(translation, rotation vector) 6-vector of a 4x4 rigid motion."""
    from .synth import R_to_rotvec
    T = np.asarray(T, np.float64)
    return np.concatenate([T[:3, 3], R_to_rotvec(T[:3, :3])])


def vec_motion(v):
    from .synth import pose, rotvec_to_R
    v = np.asarray(v, np.float64)
    return pose(rotvec_to_R(v[3:]), v[:3])


# ---------------------------------------------------------------- GPU-rendered frame pairs
class PairSet:
    """n frame pairs of one resolution resident on the GPU, stacked:
    model prediction (vertices, normals, RGBA) at T1 and live frame (depth,
    RGBA) at T2 = T1 * motion."""

    def __init__(self, cam, T1, T2, model_vert, model_norm, model_rgba, depth, rgba):
        self.cam, self.T1, self.T2 = cam, T1, T2
        self.model_vert, self.model_norm, self.model_rgba = model_vert, model_norm, model_rgba
        self.depth, self.rgba = depth, rgba
        self.n = len(T1)

    def frame_pairs(self, idx=None, levels=3, iterations=(0, 0, 0)):
        from .batch import FramePair
        idx = range(self.n) if idx is None else idx
        return [FramePair(self.cam, self.model_vert[i], self.model_norm[i], self.model_rgba[i], self.depth[i],
                          self.rgba[i], self.model_rgba[i], self.T1[i], levels=levels, iterations=iterations)
                for i in idx]


def render_views(scenes, view_scene, poses, seeds, cam, depth=True, rgba=True, model=False, noise_k=0.0012,
                 dropout=0.05, min_mm=300, max_mm=5000):
    """Renders len(poses) views on the GPU (odo_synth_render); returns a dict
    of CUDA tensors 'depth' [n,h,w] uint16, 'rgba' [n,h,w,4] uint8 and, when
    model, 'vert' / 'norm' [n,h,w,4] float32."""
    import torch
    from .synth import Scene
    L = _native.load()
    n, h, w = len(poses), cam.height, cam.width
    sc = (Scene * len(scenes))(*scenes)
    vs = np.ascontiguousarray(view_scene, np.int32)
    ps = np.ascontiguousarray(np.asarray(poses, np.float32).reshape(n, 16))
    sd = np.ascontiguousarray(seeds, np.uint64)
    out = {}
    dev = torch.device("cuda")
    out["depth"] = torch.empty((n, h, w), dtype=torch.uint16, device=dev) if depth else None
    out["rgba"] = torch.empty((n, h, w, 4), dtype=torch.uint8, device=dev) if rgba else None
    out["vert"] = torch.empty((n, h, w, 4), dtype=torch.float32, device=dev) if model else None
    out["norm"] = torch.empty((n, h, w, 4), dtype=torch.float32, device=dev) if model else None
    ptr = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None
    rc = L.odo_synth_render(ctypes.cast(sc, ctypes.c_void_p), len(scenes),
                            vs.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                            ps.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                            sd.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), n, w, h, cam.fx, cam.fy, cam.cx,
                            cam.cy, noise_k, dropout, min_mm, max_mm, ptr(out["depth"]), ptr(out["rgba"]),
                            ptr(out["vert"]), ptr(out["norm"]), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    if rc != 0:
        raise OdometryError(rc, "odo_synth_render failed")
    return {k: v for k, v in out.items() if v is not None}


def make_room_pairs(seed, n, cam=None, max_deg=10.0, max_m=0.10, nscenes=64):
    """n seeded room pairs (6x4x3 m rooms, 20 spheres) rendered on the GPU:
    camera near the room centre, live frame at a random relative motion of at
    most max_deg / max_m."""
    from . import synth
    cam = cam or synth.Camera()
    rng = np.random.default_rng(seed)
    scenes = [synth.make_room(seed * 7919 + k, 20) for k in range(nscenes)]
    view_scene = rng.integers(0, nscenes, size=n)
    T1 = np.stack([synth.room_camera(rng) for _ in range(n)])
    T2 = np.stack([T1[i] @ synth.random_motion(rng, max_deg, max_m) for i in range(n)])
    seeds = rng.integers(1, 2 ** 62, size=n, dtype=np.uint64)
    m = render_views(scenes, view_scene, T1, seeds, cam, depth=False, rgba=True, model=True)
    lv = render_views(scenes, view_scene, T2, seeds + np.uint64(1), cam, depth=True, rgba=True, model=False)
    return PairSet(cam, T1, T2, m["vert"], m["norm"], m["rgba"], lv["depth"], lv["rgba"])


# ---------------------------------------------------------------- labelling, inputs, training
def track_plain(batch, pairset, idx, levels=3, iterations=(0, 0, 0)):
    """Plain tracking (SO3 + ICP + RGB, the reference schedule) of pairs idx."""
    return batch.track(pairset.frame_pairs(idx, levels=levels, iterations=iterations))


def label_pairs(batch, pairset, chunk=512, agree_deg=1.0, agree_m=0.02):
    """Labels = the plain tracker's relative motion T1^-1 T_icp per pair, and
    a mask of the pairs where the plain tracker converged (its result within
    agree_deg / agree_m of the rendering pose)."""
    from .batch import result_pose
    from .synth import pose_error
    labels = np.zeros((pairset.n, 6), np.float32)
    ok = np.zeros(pairset.n, bool)
    chunk = min(chunk, batch.max_pairs)
    for s in range(0, pairset.n, chunk):
        idx = list(range(s, min(pairset.n, s + chunk)))
        res = track_plain(batch, pairset, idx)
        for i, r in zip(idx, res):
            T = result_pose(r)
            labels[i] = motion_vec(np.linalg.inv(pairset.T1[i]) @ T)
            e = pose_error(T, pairset.T2[i])
            ok[i] = e[0] <= np.radians(agree_deg) and e[1] <= agree_m
    return labels, ok


def pack_inputs(net, pairset, out=None, chunk=None):
    """Network inputs [n,120,160,8] float16 of all pairs of a PairSet."""
    import torch
    if out is None:
        out = torch.empty((pairset.n, IN_H, IN_W, IN_C), dtype=torch.float16, device="cuda")
    chunk = chunk or net.max_batch
    fps = pairset.frame_pairs()
    for s in range(0, pairset.n, chunk):
        net.pack(fps[s:s + chunk], out[s:s + chunk])
    return out


# label of the horizontally mirrored pair (x -> -x in both cameras); the
# input channels are all mirror-invariant images
MIRROR_SIGN = (-1.0, 1.0, 1.0, 1.0, -1.0, -1.0)


def alignment_metric(pairset, sigma=0.01, npairs=64, stride=8):
    """Loss metric of the point-alignment error: e^T M e = mean squared
    displacement (in units of sigma) of the scene points p under the motion
    error e = (dt, dw): d = dt - [p]x dw, M = E[J^T J] / sigma^2 with
    J = [I, -[p]x], estimated from the model vertices of up to npairs pairs."""
    n = min(npairs, pairset.n)
    v = pairset.model_vert[:n, ::stride, ::stride, :].reshape(-1, 4).cpu().numpy().astype(np.float64)
    p = v[v[:, 3] > 0, :3]
    mp = p.mean(axis=0)
    X = np.array([[0, -mp[2], mp[1]], [mp[2], 0, -mp[0]], [-mp[1], mp[0], 0]])
    M = np.zeros((6, 6))
    M[:3, :3] = np.eye(3)
    M[:3, 3:] = -X
    M[3:, :3] = X
    M[3:, 3:] = np.mean((p * p).sum(axis=1)) * np.eye(3) - (p.T @ p) / len(p)
    return M / sigma ** 2


def train(net, inputs, labels, epochs=20, batch=256, lr=1e-3, lr_final=1e-4, seed=0, mirror=True, log=None):
    """Adam on shuffled mini-batches (the network's own CUDA kernels);
    cosine learning-rate decay from lr to lr_final; with `mirror`, half of
    every batch is mirrored horizontally (inputs flipped along x, labels
    MIRROR_SIGN).  Returns the last batch loss of every epoch."""
    import torch
    n = inputs.shape[0]
    g = torch.Generator(device="cpu").manual_seed(seed)
    steps = epochs * (n // batch)
    sign = torch.tensor(MIRROR_SIGN, dtype=torch.float32, device="cuda")
    hist, k = [], 0
    for ep in range(epochs):
        perm = torch.randperm(n, generator=g).cuda()
        tot = 0.0
        for s in range(0, n - batch + 1, batch):
            sel = perm[s:s + batch]
            x = inputs.index_select(0, sel)
            y = labels.index_select(0, sel)
            if mirror:
                h = batch // 2
                x = torch.cat([x[:h], x[h:].flip(2)])
                y = torch.cat([y[:h], y[h:] * sign])
            x, y = x.contiguous(), y.contiguous()
            cur = lr_final + 0.5 * (lr - lr_final) * (1 + np.cos(np.pi * k / max(1, steps)))
            want = (s + 2 * batch > n)
            l = net.train_step(x, y, cur, want_loss=want)
            k += 1
            if want:
                tot = l
        hist.append(tot)
        if log:
            log("epoch %d loss %.5f" % (ep, tot))
    return hist


def make_training_set(net, batch, seed, n, chunk=2048, max_deg=10.0, max_m=0.10, cam=None, agree_deg=0.5,
                      agree_m=0.02, log=None):
    """n seeded room pairs rendered on the GPU in chunks, labelled by the
    plain tracker and packed into network inputs; only the pairs where the
    plain tracker converged (within agree_deg / agree_m of the rendering pose)
    are kept.  Returns a dict: 'inputs' [m,120,160,8] float16 and 'labels'
    [m,6] float32 (CUDA), 'residuals' (plain tracker, kept pairs), 'kept'
    (fraction), 'metric' (alignment_metric of the first chunk)."""
    import torch
    from . import synth
    cam = cam or synth.Camera()
    xs, ys, res, kept, metric = [], [], [], 0, None
    for c, s in enumerate(range(0, n, chunk)):
        m = min(chunk, n - s)
        ps = make_room_pairs(seed * 1000003 + c, m, cam, max_deg, max_m)
        if metric is None:
            metric = alignment_metric(ps)
        lab, ok, err = _label_with_residual(batch, ps, agree_deg=agree_deg, agree_m=agree_m)
        X = pack_inputs(net, ps)
        sel = torch.from_numpy(np.nonzero(ok)[0]).cuda()
        xs.append(X.index_select(0, sel))
        ys.append(torch.from_numpy(lab[ok]).cuda())
        res.append(err[ok])
        kept += int(ok.sum())
        del ps, X
        if log:
            log("training chunk %d: %d pairs, %d kept" % (c, m, int(ok.sum())))
    return {"inputs": torch.cat(xs), "labels": torch.cat(ys), "residuals": np.concatenate(res),
            "kept": kept / max(n, 1), "metric": metric}


def _label_with_residual(batch, pairset, chunk=512, agree_deg=0.5, agree_m=0.02):
    from .batch import result_pose
    from .synth import pose_error
    labels = np.zeros((pairset.n, 6), np.float32)
    ok = np.zeros(pairset.n, bool)
    err = np.zeros(pairset.n, np.float32)
    chunk = min(chunk, batch.max_pairs)
    for s in range(0, pairset.n, chunk):
        idx = list(range(s, min(pairset.n, s + chunk)))
        res = track_plain(batch, pairset, idx)
        for i, r in zip(idx, res):
            T = result_pose(r)
            labels[i] = motion_vec(np.linalg.inv(pairset.T1[i]) @ T)
            e = pose_error(T, pairset.T2[i])
            ok[i] = e[0] <= np.radians(agree_deg) and e[1] <= agree_m
            err[i] = r.lastICPError
    return labels, ok, err


class WarmStartTracker:
    """Batched tracking started from the network's motion proposal, with a
    fallback to the plain tracker.

    Per batch: network inputs from the level-0 frames (block means to
    160x120), forward pass, tracking from pose * exp(proposal) with a short
    schedule (`levels`, `iterations`, no SO3 stage).  A pair falls back to the
    plain tracker (SO3 + the reference's 10/5/4 schedule) when its final ICP
    residual exceeds `residual_ratio` x the plain tracker's typical residual
    (`plain_residual`, the median over the training pairs) or when the refined
    pose differs from the proposal by more than `max_disagree_deg`."""

    def __init__(self, net, batch, plain_residual, levels=3, iterations=(2, 2, 2), residual_ratio=6.0,
                 max_disagree_deg=5.0, max_pairs=512):
        import torch
        self.net, self.batch = net, batch
        self.plain_residual = float(plain_residual)
        self.levels, self.iterations = int(levels), tuple(iterations)
        self.residual_ratio, self.max_disagree = float(residual_ratio), np.radians(max_disagree_deg)
        self.inputs = torch.empty((max_pairs, IN_H, IN_W, IN_C), dtype=torch.float16, device="cuda")
        self.props = torch.empty((max_pairs, 6), dtype=torch.float32, device="cuda")

    def track(self, frame_pairs):
        """Returns (results, fallback mask, proposals [n,6])."""
        from .batch import result_pose
        from .synth import pose_error
        n = len(frame_pairs)
        for s in range(0, n, self.net.max_batch):
            e = min(n, s + self.net.max_batch)
            self.net.pack(frame_pairs[s:e], self.inputs[s:e])
            self.net.forward(self.inputs[s:e], out=self.props[s:e])
        short = [_with_schedule(p, self.levels, self.iterations) for p in frame_pairs]
        res = list(self.batch.track_init(short, self.props[:n]))
        prop = self.props[:n].cpu().numpy().astype(np.float64)
        fb = np.zeros(n, bool)
        for i, r in enumerate(res):
            T0 = np.asarray(frame_pairs[i].pose, np.float64) @ vec_motion(prop[i])
            dis = pose_error(result_pose(r), T0)[0]
            fb[i] = (r.lastICPError > self.residual_ratio * self.plain_residual) or dis > self.max_disagree
        if fb.any():
            idx = np.nonzero(fb)[0]
            plain = self.batch.track([frame_pairs[i] for i in idx])
            for k, i in enumerate(idx):
                res[i] = plain[k]
        return res, fb, prop


def _with_schedule(p, levels, iterations):
    from .batch import FramePair
    return FramePair(p.cam, p.model_vert, p.model_norm, p.model_rgba, p.depth, p.rgba, p.prev_rgba, p.pose,
                     levels=levels, iterations=iterations)
