"""Generates golden fixtures from the REFERENCE's own kernels.

Runs on a machine with a GPU and oracle/_ref/ref_kernels.cubin (the
reference's src/odom/utils.cu + src/odom/reduce.cu compiled by
oracle/build_ref.py).  For a seeded synthetic frame pair it executes the
reference's per-frame pipeline kernel by kernel, in the order of
RGBDOdometryef (src/odom/RGBDOdometryef.cpp:118-265):
  initICPModel  copyMaps -> resizeVMap/NMap x2 -> tranformMaps
  initRGBModel  verticesToDepth -> pyrDownGaussF x2; imageBGRToIntensity -> pyrDownUcharGauss x2
  initICP       pyrDown x2 -> createVMap/createNMap per level
  initRGB       as initRGBModel with the live RGB (depth from the model vertices)
  initFirstRGB  intensity pyramid of the previous RGB
  derivatives   computeDerivativeImages of nextImage
and one evaluation of each reduction functor per level (ICP association,
photometric residual and reduction, SO3 at level 2) with fixed poses, saving
inputs and outputs to an .npz.

usage: python tests/golden/make_ref_golden.py OUT_DIR [WIDTHxHEIGHT ...]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

ANGLE = float(np.float32(np.sin(np.float32(np.float32(20.0) * np.float32(3.14159254)) / np.float32(180.0))))
DIST = float(np.float32(0.10))


def level_intr(cam, l):
    d = np.float32(1 << l)
    return tuple(float(np.float32(v) / d) for v in (cam.fx, cam.fy, cam.cx, cam.cy))


def make(width, height, seed, out_dir):
    import torch
    from oracle.ref_runner import RefKernels
    from slam_gb300 import synth

    ref = RefKernels()
    cam = synth.Camera().scaled(width, height)
    pair = synth.make_pair(seed, cam=cam)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    Tu16 = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.int16)).cuda().view(torch.uint16)

    def H(t):
        t = t.cpu()
        if t.dtype == torch.uint16:
            return t.view(torch.int16).numpy().view(np.uint16)
        return t.numpy()

    g = {"width": width, "height": height, "seed": seed, "fx": cam.fx, "fy": cam.fy, "cx": cam.cx, "cy": cam.cy,
         "T1": pair["T1"], "T2": pair["T2"]}
    for k in ("model_vert", "model_norm", "model_rgba", "depth", "rgba", "prev_rgba"):
        g["in_" + k] = pair[k]
    T1 = pair["T1"].astype(np.float32)
    # initICPModel
    vm, nm = ref.copy_maps(T(pair["model_vert"]), T(pair["model_norm"]))
    raw = [(vm, nm)]
    for l in (1, 2):
        raw.append((ref.resize(raw[-1][0], False), ref.resize(raw[-1][1], True)))
    for l in range(3):
        v, n = ref.transform(raw[l][0], raw[l][1], T1[:3, :3], T1[:3, 3])
        g[f"vmap_prev_{l}"], g[f"nmap_prev_{l}"] = H(v), H(n)
    # initRGBModel / initRGB / initFirstRGB
    vdepth = ref.verts_to_depth(T(pair["model_vert"]))
    for name, rgba in (("last", pair["model_rgba"]), ("next", pair["rgba"]), ("lastnext", pair["prev_rgba"])):
        img = ref.intensity(T(rgba))
        g[f"{name}Image_0"] = H(img)
        for l in (1, 2):
            img = ref.gauss_u8(img)
            g[f"{name}Image_{l}"] = H(img)
    for name in ("last", "next"):
        d = vdepth
        g[f"{name}Depth_0"] = H(d)
        for l in (1, 2):
            d = ref.gauss_f(d)
            g[f"{name}Depth_{l}"] = H(d)
    # initICP(depth)
    d = Tu16(pair["depth"])
    g["depth_0"] = pair["depth"]
    for l in range(3):
        if l > 0:
            d = ref.pyr_down_depth(d)
            g[f"depth_{l}"] = H(d)
        fx, fy, cx, cy = level_intr(cam, l)
        v = ref.vmap(d, fx, fy, cx, cy, 20.0)
        g[f"vmap_curr_{l}"], g[f"nmap_curr_{l}"] = H(v), H(ref.nmap(v))
    # derivatives of nextImage
    for l in range(3):
        dx, dy = ref.derivatives(T(g[f"nextImage_{l}"]))
        g[f"dIdx_{l}"], g[f"dIdy_{l}"] = H(dx), H(dy)
    # one evaluation of each functor per level
    rng = np.random.default_rng(seed + 1000)
    Tc = pair["T1"] @ synth.random_motion(rng, 1.0, 0.01)
    Rc, tc = Tc[:3, :3].astype(np.float32), Tc[:3, 3].astype(np.float32)
    Rpi = np.linalg.inv(T1[:3, :3].astype(np.float64)).astype(np.float32)
    g["icp_pose"] = np.concatenate([Rc.reshape(9), tc, Rpi.reshape(9), T1[:3, 3]]).astype(np.float32)
    Tm = synth.random_motion(rng, 1.0, 0.01)
    for l in range(3):
        fx, fy, cx, cy = level_intr(cam, l)
        h, w = g[f"nextImage_{l}"].shape
        found, dd, prod = ref.icp_pixels(Rc, tc, Rpi, T1[:3, 3], T(g[f"vmap_curr_{l}"]), T(g[f"nmap_curr_{l}"]),
                                         T(g[f"vmap_prev_{l}"]), T(g[f"nmap_prev_{l}"]), fx, fy, cx, cy, DIST, ANGLE)
        g[f"icp_found_{l}"] = H(found).astype(np.uint8)
        g[f"icp_d_{l}"] = H(dd)
        g[f"icp_sum_{l}"] = H(prod).reshape(-1, 29).astype(np.float64).sum(0)
        K = np.array([[fx, 0, cx], [0, fy, cy], [0, 0, 1.0]])
        krk = (K @ Tm[:3, :3] @ np.linalg.inv(K)).astype(np.float32)
        kt = (K @ Tm[:3, 3]).astype(np.float32)
        g[f"rgb_krk_{l}"], g[f"rgb_kt_{l}"] = krk, kt
        minScale = float(np.float32([5, 3, 1][l] ** 2 / 0.125 ** 2))
        dt, i2 = ref.rgb_residual(minScale, T(g[f"dIdx_{l}"]), T(g[f"dIdy_{l}"]), T(g[f"lastDepth_{l}"]),
                                  T(g[f"nextDepth_{l}"]), T(g[f"lastImage_{l}"]), T(g[f"nextImage_{l}"]), 0.07, kt,
                                  krk)
        g[f"rgb_dataterm_{l}"] = H(dt)
        i2 = H(i2)
        cnt = int(i2[..., 0].sum())
        g[f"rgb_count_{l}"] = cnt
        g[f"rgb_sigma_{l}"] = int(np.int32(np.uint32(int(i2[..., 1].astype(np.int64).sum()) & 0xffffffff)))
        sigma = float(np.float32(np.sqrt(cnt)))
        g[f"rgb_step_sigma_{l}"] = sigma
        cloud = ref.cloud(T(g[f"lastDepth_{l}"]), fx, fy, cx, cy)
        prod = ref.rgb_step(dt, sigma, cloud, fx, fy, T(g[f"dIdx_{l}"]), T(g[f"dIdy_{l}"]))
        g[f"rgb_sum_{l}"] = H(prod).reshape(-1, 29).astype(np.float64).sum(0)
    fx, fy, cx, cy = level_intr(cam, 2)
    K = np.array([[fx, 0, cx], [0, fy, cy], [0, 0, 1.0]])
    R = synth.rotvec_to_R([0.003, -0.004, 0.002])
    mats = [(K @ R @ np.linalg.inv(K)).astype(np.float32), np.linalg.inv(K).astype(np.float32),
            (K @ R).astype(np.float32)]
    g["so3_mats"] = np.stack(mats)
    prod = ref.so3_pixels(T(g["lastnextImage_2"]), T(g["nextImage_2"]), *mats)
    g["so3_sum"] = H(prod).reshape(-1, 11).astype(np.float64).sum(0)
    os.makedirs(out_dir, exist_ok=True)
    path = os.path.join(out_dir, f"ref_golden_{width}x{height}.npz")
    np.savez_compressed(path, **g)
    print("wrote", path)


if __name__ == "__main__":
    out = sys.argv[1] if len(sys.argv) > 1 else HERE
    sizes = sys.argv[2:] or ["80x60", "160x120"]
    for i, s in enumerate(sizes):
        w, h = map(int, s.split("x"))
        make(w, h, 100 + i, out)
