"""The precision study's corridor scenes on the CPU: the tapered-wall
corridor puts the condition number of the level-0 ICP normal equations
(FP64 oracle, at the true pose) in the 1e6-1e9 band that the ill-conditioned
workload asks for, and the ray caster's tapered walls have the plane
normals the taper implies."""
import numpy as np
import pytest

from slam_gb300 import synth


def icp_normal_equations(p, k64, dist, angle):
    from oracle import oracle
    cam = p["cam"]
    o = oracle.Odometry(cam.width, cam.height, cam.cx, cam.cy, cam.fx, cam.fy, dist, angle, prec=64)
    T1, T2 = p["T1"], p["T2"]
    o.initICPModel(p["model_vert"], p["model_norm"], 20.0, T1.astype(np.float32))
    o.initICP(p["depth"], 20.0)
    maps = [o.buffer(n, 0) for n in ("vmap_curr", "nmap_curr", "vmap_prev", "nmap_prev")]
    o.close()
    Rp, tp = T1[:3, :3].astype(np.float32), T1[:3, 3].astype(np.float32)
    Rpi = np.linalg.inv(Rp.astype(np.float64)).astype(np.float32)
    s, _, _ = k64.icp_step(T2[:3, :3].astype(np.float32), T2[:3, 3].astype(np.float32), maps[0], maps[1], Rpi, tp,
                           cam.fx, cam.fy, cam.cx, cam.cy, maps[2], maps[3], dist, angle, with_assoc=False)
    A = np.zeros((6, 6))
    k = 0
    for i in range(6):
        for j in range(i, 7):
            if j < 6:
                A[i, j] = A[j, i] = s[k]
            k += 1
    return A


@pytest.mark.parametrize("taper,band", [(2e-4, (1e8, 1e11)), (1e-3, (1e6, 1e9)), (4e-3, (1e5, 1e8))])
def test_tapered_corridor_condition_number(taper, band):
    from oracle import oracle
    from slam_gb300.odometry import DEFAULT_ANGLE_THRESH, DEFAULT_DIST_THRESH
    k64 = oracle.Kernels(64)
    cam = synth.Camera().scaled(320, 240)
    conds = []
    for seed in (70001, 70002, 70005):
        p = synth.make_corridor_pair(seed, cam=cam, nclutter=0, taper=taper)
        conds.append(np.linalg.cond(icp_normal_equations(p, k64, DEFAULT_DIST_THRESH, DEFAULT_ANGLE_THRESH)))
    assert band[0] <= np.median(conds) < band[1], conds


def test_straight_clutter_free_corridor_is_singular():
    from oracle import oracle
    from slam_gb300.odometry import DEFAULT_ANGLE_THRESH, DEFAULT_DIST_THRESH
    cam = synth.Camera().scaled(320, 240)
    p = synth.make_corridor_pair(70001, cam=cam, nclutter=0, taper=0.0)
    A = icp_normal_equations(p, oracle.Kernels(64), DEFAULT_DIST_THRESH, DEFAULT_ANGLE_THRESH)
    w = np.linalg.eigvalsh(A)
    assert w[0] < 1e-9 * w[-1]


def test_tapered_wall_normals():
    scene = synth.make_corridor(5, 0)
    scene.wall_taper = 0.05
    rng = np.random.default_rng(1)
    T = synth.corridor_camera(rng)
    cam = synth.Camera().scaled(160, 120)
    m = synth.render(scene, T, cam, depth=False, rgba=False, model=True)
    hit = m["vert"][..., 3] > 0
    nw = m["norm"][..., :3][hit] @ T[:3, :3].T      # camera -> world
    side = np.abs(nw[:, 0]) > 0.9
    assert side.any()
    inv = 1.0 / np.sqrt(1.0 + 0.05 ** 2)
    assert np.allclose(np.abs(nw[side, 0]), inv, atol=1e-5)
    assert np.allclose(nw[side, 2], 0.05 * inv, atol=1e-5)
