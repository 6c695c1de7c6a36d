"""Seeded synthetic RGB-D frames (stand-in for datasets, which are absent).

Wraps libslam_synth.so: box rooms (6x4x3 m, random spheres) and corridors
(2 m x 20 m, low texture, side clutter), ray-cast at a pinhole camera with a
Perlin solid texture, the depth noise model sigma = 0.0012 z^2 m, a dropout
fraction of zero pixels and the valid range 300-5000 mm.  Also renders the
noise-free model prediction (RGBA32F vertices/normals + RGBA) that the
reference gets from its GL map (src/gl/FillIn.cpp:22-42).
"""
import ctypes
import math

import numpy as np

from . import _native

MAX_SPH = 128


class Scene(ctypes.Structure):
    _fields_ = [("bmin", ctypes.c_float * 3), ("bmax", ctypes.c_float * 3), ("nsph", ctypes.c_int),
                ("sph", (ctypes.c_float * 4) * MAX_SPH), ("sph_col", (ctypes.c_float * 3) * MAX_SPH),
                ("wall_col", (ctypes.c_float * 3) * 6), ("tex_freq", ctypes.c_float), ("tex_amp", ctypes.c_float),
                ("tex_seed", ctypes.c_uint64), ("wall_taper", ctypes.c_float)]


def make_room(seed, nspheres=20):
    S = _native.load_synth()
    s = Scene()
    rc = S.synth_make_room(ctypes.c_uint64(seed), nspheres, ctypes.byref(s))
    if rc != 0:
        raise RuntimeError("synth_make_room failed (%d)" % rc)
    return s


def make_corridor(seed, nclutter=24):
    S = _native.load_synth()
    s = Scene()
    rc = S.synth_make_corridor(ctypes.c_uint64(seed), nclutter, ctypes.byref(s))
    if rc != 0:
        raise RuntimeError("synth_make_corridor failed (%d)" % rc)
    return s


class Camera:
    def __init__(self, width=640, height=480, fx=525.0, fy=525.0, cx=319.5, cy=239.5):
        self.width, self.height, self.fx, self.fy, self.cx, self.cy = width, height, fx, fy, cx, cy

    def scaled(self, width, height):
        s = width / self.width
        return Camera(width, height, self.fx * s, self.fy * s, (self.cx + 0.5) * s - 0.5, (self.cy + 0.5) * s - 0.5)


def render(scene, pose_wc, cam, noise_seed=0, noise_k=0.0012, dropout=0.05, min_mm=300, max_mm=5000,
           depth=True, rgba=True, model=False):
    """Returns a dict with 'depth' (uint16 HxW), 'rgba' (uint8 HxWx4) and,
    when model=True, 'vert'/'norm' (float32 HxWx4)."""
    S = _native.load_synth()
    h, w = cam.height, cam.width
    pose = np.ascontiguousarray(np.asarray(pose_wc, dtype=np.float32).reshape(4, 4))
    out = {}
    d = np.zeros((h, w), np.uint16) if depth else None
    c = np.zeros((h, w, 4), np.uint8) if rgba else None
    v = np.zeros((h, w, 4), np.float32) if model else None
    n = np.zeros((h, w, 4), np.float32) if model else None
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p) if a is not None else None
    S.synth_render.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                               ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_uint64, ctypes.c_float,
                               ctypes.c_float, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                               ctypes.c_void_p, ctypes.c_void_p]
    rc = S.synth_render(ctypes.byref(scene), pose.ctypes.data, w, h, cam.fx, cam.fy, cam.cx, cam.cy,
                        ctypes.c_uint64(noise_seed), noise_k, dropout, min_mm, max_mm, ptr(d), ptr(c), ptr(v), ptr(n))
    if rc != 0:
        raise RuntimeError("synth_render failed (%d)" % rc)
    if depth:
        out["depth"] = d
    if rgba:
        out["rgba"] = c
    if model:
        out["vert"] = v
        out["norm"] = n
    return out


# ---------------------------------------------------------------- poses
def rotvec_to_R(w):
    w = np.asarray(w, dtype=np.float64)
    th = np.linalg.norm(w)
    if th < 1e-15:
        return np.eye(3)
    k = w / th
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + math.sin(th) * K + (1 - math.cos(th)) * K @ K


def R_to_rotvec(R):
    """Rotation vector of R; atan2 form, accurate for tiny angles."""
    R = np.asarray(R, dtype=np.float64)
    w = 0.5 * np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]])
    s = np.linalg.norm(w)
    c = (np.trace(R) - 1) / 2
    th = math.atan2(s, c)
    if s < 1e-300:
        return np.zeros(3)
    return w / s * th


def pose(R, t):
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = t
    return T


def random_motion(rng, max_deg, max_m):
    """Relative pose: random-axis rotation <= max_deg, translation <= max_m."""
    axis = rng.normal(size=3)
    axis /= np.linalg.norm(axis)
    ang = math.radians(max_deg) * rng.uniform(0.0, 1.0)
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    return pose(rotvec_to_R(axis * ang), d * max_m * rng.uniform(0.0, 1.0))


def room_camera(rng):
    """A camera pose near the room centre looking at a random wall."""
    yaw = rng.uniform(0, 2 * math.pi)
    pitch = math.radians(rng.uniform(-10, 10))
    roll = math.radians(rng.uniform(-5, 5))
    Ry = rotvec_to_R([0, yaw, 0])
    Rx = rotvec_to_R([pitch, 0, 0])
    Rz = rotvec_to_R([0, 0, roll])
    t = rng.uniform(-0.3, 0.3, size=3)
    return pose(Ry @ Rx @ Rz, t)


def corridor_camera(rng):
    """A camera about 1.5 m above the corridor floor, looking along the
    corridor and pitched down 25-40 degrees so the floor plane fills most of
    the image."""
    yaw = math.radians(rng.uniform(-12, 12)) + (math.pi if rng.uniform() < 0.5 else 0.0)
    pitch = -math.radians(rng.uniform(25, 40))
    roll = math.radians(rng.uniform(-3, 3))
    R = rotvec_to_R([0, yaw, 0]) @ rotvec_to_R([pitch, 0, 0]) @ rotvec_to_R([0, 0, roll])
    t = np.array([rng.uniform(-0.4, 0.4), rng.uniform(-0.15, 0.15), rng.uniform(-5.0, 5.0)])
    return pose(R, t)


def make_corridor_pair(seed, cam=None, max_deg=3.0, max_m=0.05, nclutter=24, tex_amp=None, taper=0.0):
    """One frame pair of the precision study: a low-texture corridor seen
    from corridor_camera, live frame at a relative motion <= max_deg/max_m.
    taper != 0 tapers the side walls (x = +-(1 + taper z)): without clutter
    the translation along the corridor is then observed only through the
    walls' tilt, so the ICP normal equations' condition number grows as
    1 / taper^2 (about 1e9.5 at 1e-4, 1e8 at 1e-3, 1e6 at 3e-3 for these
    views); with taper 0 and no clutter that translation is unobservable."""
    cam = cam or Camera()
    rng = np.random.default_rng(seed + 0x5151)
    scene = make_corridor(seed, nclutter)
    scene.wall_taper = float(taper)
    if tex_amp is not None:
        scene.tex_amp = tex_amp
    T1 = corridor_camera(rng)
    T2 = T1 @ random_motion(rng, max_deg, max_m)
    model = render(scene, T1, cam, depth=False, rgba=True, model=True)
    live = render(scene, T2, cam, noise_seed=seed * 7919 + 1, depth=True, rgba=True, model=False)
    prev = render(scene, T1, cam, noise_seed=seed * 7919 + 2, depth=False, rgba=True, model=False)
    return {"cam": cam, "T1": T1, "T2": T2, "model_vert": model["vert"], "model_norm": model["norm"],
            "model_rgba": model["rgba"], "depth": live["depth"], "rgba": live["rgba"], "prev_rgba": prev["rgba"]}


def pose_error(T_est, T_gt):
    """(rotation error rad, translation error m)."""
    D = np.linalg.inv(T_gt) @ T_est
    return float(np.linalg.norm(R_to_rotvec(D[:3, :3]))), float(np.linalg.norm(T_est[:3, 3] - T_gt[:3, 3]))


def make_pair(seed, cam=None, max_deg=2.0, max_m=0.02, nspheres=20, scene=None):
    """One frame pair of the single-pair workload: the model prediction
    rendered noise-free at pose1 and the live frame (noisy depth + RGB) at
    pose2 = pose1 * motion."""
    cam = cam or Camera()
    rng = np.random.default_rng(seed)
    scene = scene if scene is not None else make_room(seed, nspheres)
    T1 = room_camera(rng)
    T2 = T1 @ random_motion(rng, max_deg, max_m)
    model = render(scene, T1, cam, depth=False, rgba=True, model=True)
    live = render(scene, T2, cam, noise_seed=seed * 7919 + 1, depth=True, rgba=True, model=False)
    prev = render(scene, T1, cam, noise_seed=seed * 7919 + 2, depth=False, rgba=True, model=False)
    return {"cam": cam, "T1": T1, "T2": T2, "model_vert": model["vert"], "model_norm": model["norm"],
            "model_rgba": model["rgba"], "depth": live["depth"], "rgba": live["rgba"], "prev_rgba": prev["rgba"]}


def _catmull_rom(P, n):
    """n samples along a uniform Catmull-Rom spline through control points P."""
    P = np.asarray(P, np.float64)
    segs = len(P) - 3
    out = []
    for i in range(n):
        u = i / (n - 1) * segs
        k = min(int(u), segs - 1)
        t = u - k
        p0, p1, p2, p3 = P[k], P[k + 1], P[k + 2], P[k + 3]
        out.append(0.5 * ((2 * p1) + (-p0 + p2) * t + (2 * p0 - 5 * p1 + 4 * p2 - p3) * t * t +
                          (-p0 + 3 * p1 - 3 * p2 + p3) * t ** 3))
    return np.array(out)


def trajectory(seed, n=300, max_deg=1.5, max_m=0.03):
    """A smooth camera path (30 fps) through the room: Catmull-Rom splines
    over position and (yaw, pitch, roll); rescaled so that no frame moves more
    than max_deg / max_m.  Returns a list of 4x4 camera-to-world poses."""
    rng = np.random.default_rng(seed)
    m = 8
    pos = rng.uniform([-0.6, -0.3, -0.6], [0.6, 0.3, 0.6], size=(m, 3))
    ang = np.cumsum(rng.uniform(-0.5, 0.5, size=(m, 3)) * np.array([1.0, 0.25, 0.1]), axis=0)
    ang[:, 0] += rng.uniform(0, 2 * math.pi)
    for _ in range(20):
        p = _catmull_rom(pos, n)
        a = _catmull_rom(ang, n)
        T = []
        for i in range(n):
            R = rotvec_to_R([0, a[i, 0], 0]) @ rotvec_to_R([a[i, 1], 0, 0]) @ rotvec_to_R([0, 0, a[i, 2]])
            T.append(pose(R, p[i]))
        dr = max(np.linalg.norm(R_to_rotvec(T[i][:3, :3].T @ T[i + 1][:3, :3])) for i in range(n - 1))
        dt = max(np.linalg.norm(T[i + 1][:3, 3] - T[i][:3, 3]) for i in range(n - 1))
        s = min(1.0, math.radians(max_deg) / max(dr, 1e-12), max_m / max(dt, 1e-12))
        if s >= 1.0:
            return T
        # shrink the excursion around the first control point
        pos = pos[0] + (pos - pos[0]) * s * 0.98
        ang = ang[0] + (ang - ang[0]) * s * 0.98
    return T


def trajectory_frame(scene, T, k, cam, seed=0):
    """Frame k of a trajectory as a frame-to-model pair: model prediction
    rendered noise-free at the ground-truth pose of frame k-1, live frame at
    frame k."""
    model = render(scene, T[k - 1], cam, depth=False, rgba=True, model=True)
    live = render(scene, T[k], cam, noise_seed=seed * 100003 + k, depth=True, rgba=True)
    return {"cam": cam, "T1": T[k - 1], "T2": T[k], "model_vert": model["vert"], "model_norm": model["norm"],
            "model_rgba": model["rgba"], "depth": live["depth"], "rgba": live["rgba"]}
