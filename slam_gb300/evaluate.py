"""Trajectory metrics of the TUM RGB-D benchmark, restated in Python 3 / numpy.

The reference evaluates its trajectories with the benchmark's Python 2
scripts (benchmark/evaluate_ate.py, benchmark/evaluate_rpe.py,
benchmark/associate.py).  This module computes the same quantities:

* absolute trajectory error (ATE): the estimated positions are aligned to the
  ground truth by the closed-form least-squares rotation and translation of
  Horn's method (an SVD of the 3x3 cross-covariance, with the reflection
  guard), then the per-pose position error is summarised
  (benchmark/evaluate_ate.py:47-77, printed statistics :150-166);
* relative pose error (RPE): for pose pairs (i, j) a fixed distance apart,
  with a (-) b = a^-1 b, E = (P_j (-) P_i) (-) (Q_j (-) Q_i) for estimated
  poses P and ground truth Q; translation error = |t(E)|, rotation error =
  arccos((trace(R(E)) - 1) / 2) (benchmark/evaluate_rpe.py:138-176,
  204-299);
* trajectory files in the benchmark's text format "stamp tx ty tz qx qy qz
  qw" and the greedy timestamp association of benchmark/associate.py:71-100.

Poses are 4x4 camera-to-world matrices (numpy float64)."""
import math

import numpy as np

_EPS = np.finfo(float).eps * 4.0


# ---------------------------------------------------------------- file formats
def read_file_list(path):
    """{stamp: [fields...]} of a benchmark text file; lines starting with '#'
    are comments, separators may be spaces, commas or tabs
    (benchmark/associate.py:49-69)."""
    out = {}
    with open(path) as f:
        for line in f:
            line = line.replace(",", " ").replace("\t", " ").strip()
            if not line or line.startswith("#"):
                continue
            v = line.split()
            out[float(v[0])] = v[1:]
    return out


def associate(first, second, offset=0.0, max_difference=0.02):
    """Pairs (a, b) of stamps of two {stamp: ...} dicts: candidate pairs closer
    than max_difference, taken greedily by increasing time difference, each
    stamp used once; returned sorted (benchmark/associate.py:71-100)."""
    cand = sorted((abs(a - (b + offset)), a, b) for a in first for b in second
                  if abs(a - (b + offset)) < max_difference)
    used_a, used_b, matches = set(), set(), []
    for _, a, b in cand:
        if a in used_a or b in used_b:
            continue
        used_a.add(a)
        used_b.add(b)
        matches.append((a, b))
    matches.sort()
    return matches


def quat_to_matrix(t, q):
    """4x4 pose from a position and a unit quaternion (qx, qy, qz, qw)
    (benchmark/evaluate_rpe.py:48-77)."""
    q = np.array(q, np.float64)
    nq = float(np.dot(q, q))
    T = np.eye(4)
    T[:3, 3] = t
    if nq < _EPS:
        return T
    q *= math.sqrt(2.0 / nq)
    q = np.outer(q, q)
    T[:3, :3] = [[1.0 - q[1, 1] - q[2, 2], q[0, 1] - q[2, 3], q[0, 2] + q[1, 3]],
                 [q[0, 1] + q[2, 3], 1.0 - q[0, 0] - q[2, 2], q[1, 2] - q[0, 3]],
                 [q[0, 2] - q[1, 3], q[1, 2] + q[0, 3], 1.0 - q[0, 0] - q[1, 1]]]
    return T


def matrix_to_quat(R):
    """Unit quaternion (qx, qy, qz, qw) of a rotation matrix, qw >= 0."""
    R = np.asarray(R, np.float64)
    tr = np.trace(R)
    if tr > 0:
        s = math.sqrt(tr + 1.0) * 2
        q = [(R[2, 1] - R[1, 2]) / s, (R[0, 2] - R[2, 0]) / s, (R[1, 0] - R[0, 1]) / s, 0.25 * s]
    else:
        i = int(np.argmax(np.diag(R)))
        j, k = (i + 1) % 3, (i + 2) % 3
        s = math.sqrt(1.0 + R[i, i] - R[j, j] - R[k, k]) * 2
        q = [0.0, 0.0, 0.0, (R[k, j] - R[j, k]) / s]
        q[i] = 0.25 * s
        q[j] = (R[j, i] + R[i, j]) / s
        q[k] = (R[k, i] + R[i, k]) / s
    q = np.array(q)
    q /= np.linalg.norm(q)
    return q if q[3] >= 0 else -q


def read_trajectory(path):
    """{stamp: 4x4 pose} of a trajectory file; lines with an all-zero
    quaternion or NaNs are skipped (benchmark/evaluate_rpe.py:79-112)."""
    out = {}
    for stamp, v in read_file_list(path).items():
        vals = [float(x) for x in v[:7]]
        if vals[3:7] == [0.0, 0.0, 0.0, 0.0] or any(math.isnan(x) for x in vals):
            continue
        out[stamp] = quat_to_matrix(vals[:3], vals[3:7])
    return out


def write_trajectory(path, stamps, poses):
    """Writes "stamp tx ty tz qx qy qz qw" lines (the benchmark's format)."""
    with open(path, "w") as f:
        for s, T in zip(stamps, poses):
            T = np.asarray(T, np.float64)
            q = matrix_to_quat(T[:3, :3])
            f.write("%.6f %.6f %.6f %.6f %.6f %.6f %.6f %.6f\n" % ((s,) + tuple(T[:3, 3]) + tuple(q)))


# ---------------------------------------------------------------- ATE
def align(model, data):
    """Rotation R and translation t minimising |R model + t - data| over
    3 x n point sets (Horn's closed form via SVD, benchmark/evaluate_ate.py:
    47-77); returns (R, t, per-point error after alignment)."""
    model = np.asarray(model, np.float64)
    data = np.asarray(data, np.float64)
    mz = model - model.mean(1, keepdims=True)
    dz = data - data.mean(1, keepdims=True)
    W = mz @ dz.T
    U, _, Vh = np.linalg.svd(W.T)
    S = np.eye(3)
    if np.linalg.det(U) * np.linalg.det(Vh) < 0:
        S[2, 2] = -1
    R = U @ S @ Vh
    t = data.mean(1, keepdims=True) - R @ model.mean(1, keepdims=True)
    err = np.sqrt(((R @ model + t - data) ** 2).sum(0))
    return R, t, err


def ate(gt_poses, est_poses):
    """Absolute trajectory error statistics (m) of two equally long pose
    sequences (already associated)."""
    gt = np.asarray([np.asarray(T)[:3, 3] for T in gt_poses]).T
    est = np.asarray([np.asarray(T)[:3, 3] for T in est_poses]).T
    _, _, e = align(est, gt)
    return {"pairs": int(e.size), "rmse": float(np.sqrt(np.dot(e, e) / e.size)), "mean": float(e.mean()),
            "median": float(np.median(e)), "std": float(e.std()), "min": float(e.min()), "max": float(e.max())}


def ate_rmse(gt_poses, est_poses):
    return ate(gt_poses, est_poses)["rmse"]


# ---------------------------------------------------------------- RPE
def ominus(a, b):
    """Relative transformation from a to b: a^-1 b (benchmark/evaluate_rpe.py:138-149)."""
    return np.linalg.inv(a) @ b


def _angle(T):
    return math.acos(min(1.0, max(-1.0, (np.trace(T[:3, :3]) - 1) / 2)))


def rpe(gt_poses, est_poses, delta=1, pairs=None):
    """Relative pose errors of two equally long pose sequences over pairs
    (i, i + delta) (the script's --fixed_delta with unit frames) or the given
    index pairs; returns RMSE / mean / median / max of the translational (m)
    and rotational (rad) errors and the per-pair arrays."""
    gt = [np.asarray(T, np.float64) for T in gt_poses]
    est = [np.asarray(T, np.float64) for T in est_poses]
    if pairs is None:
        pairs = [(i, i + delta) for i in range(len(est) - delta)]
    tr, rot = [], []
    for i, j in pairs:
        E = ominus(ominus(est[j], est[i]), ominus(gt[j], gt[i]))
        tr.append(float(np.linalg.norm(E[:3, 3])))
        rot.append(_angle(E))
    tr, rot = np.array(tr), np.array(rot)
    return {"pairs": len(pairs), "trans_rmse": float(np.sqrt(np.mean(tr ** 2))), "trans_mean": float(tr.mean()),
            "trans_median": float(np.median(tr)), "trans_max": float(tr.max()),
            "rot_rmse": float(np.sqrt(np.mean(rot ** 2))), "rot_mean": float(rot.mean()),
            "rot_median": float(np.median(rot)), "rot_max": float(rot.max()), "trans": tr, "rot": rot}


def evaluate_files(gt_path, est_path, offset=0.0, max_difference=0.02, delta=1):
    """ATE and RPE of two trajectory files after timestamp association."""
    gt = read_trajectory(gt_path)
    est = read_trajectory(est_path)
    m = associate(gt, est, offset, max_difference)
    if len(m) < 2:
        raise ValueError("fewer than two matching timestamps")
    G = [gt[a] for a, _ in m]
    E = [est[b] for _, b in m]
    return {"ate": ate(G, E), "rpe": {k: v for k, v in rpe(G, E, delta).items() if k not in ("trans", "rot")}}
