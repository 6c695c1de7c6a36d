"""Generates tests/golden/eval_golden.npz from the REFERENCE's own trajectory
metrics (benchmark/evaluate_ate.py align, benchmark/evaluate_rpe.py
transform44 / ominus / compute_distance / compute_angle, benchmark/associate.py
associate).  The scripts are Python 2 programs; their function bodies are
valid Python 3, so this script extracts each `def` block as text from the
checkout (read in place, nothing copied into the repository) and executes it
(two adaptations to Python 3 / numpy 2: numpy.linalg.linalg, through which
the ATE alignment calls svd, is pointed at numpy.linalg; the association is
given dicts whose keys() is a list, as in Python 2).
The fixture holds seeded trajectories, their quaternion rows, and the
reference's ATE errors, RPE errors (pairs (i, i + 1) and (i, i + 5)) and
timestamp matches; tests/test_evaluate.py checks slam_gb300/evaluate.py
against it.

usage: python tests/golden/make_eval_golden.py <reference checkout>"""
import os
import re
import sys

import numpy as np


def extract(path, names):
    src = open(path).read()
    out = []
    for name in names:
        m = re.search(r"^def %s\(.*?(?=^\S)" % name, src, re.S | re.M)
        if not m:
            raise SystemExit("no def %s in %s" % (name, path))
        out.append(m.group(0))
    return "\n".join(out)


def main(ref):
    bench = os.path.join(ref, "benchmark")
    # the scripts call numpy.linalg.linalg.svd, a module path numpy 2 no
    # longer has; it names the same function as numpy.linalg.svd
    if not hasattr(np.linalg, "linalg"):
        np.linalg.linalg = np.linalg
    ns = {"numpy": np, "_EPS": np.finfo(float).eps * 4.0}
    exec(extract(os.path.join(bench, "evaluate_ate.py"), ["align"]), ns)
    exec(extract(os.path.join(bench, "evaluate_rpe.py"),
                 ["transform44", "ominus", "compute_distance", "compute_angle"]), ns)
    exec(extract(os.path.join(bench, "associate.py"), ["associate"]), ns)
    rng = np.random.default_rng(2024)
    n = 60
    # ground truth: a smooth path; estimate: the truth moved rigidly plus noise
    t = np.cumsum(rng.normal(0, 0.02, (n, 3)), 0)
    q = rng.normal(0, 1, (n, 4)) * np.array([0.05, 0.05, 0.05, 1.0])
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    gt_rows = np.hstack([np.arange(n)[:, None] / 30.0, t, q])
    qe = q + rng.normal(0, 0.003, q.shape)
    qe /= np.linalg.norm(qe, axis=1, keepdims=True)
    te = t + rng.normal(0, 0.01, t.shape)
    est_rows = np.hstack([np.arange(n)[:, None] / 30.0 + 0.004, te, qe])
    G = [ns["transform44"](list(r)) for r in gt_rows]
    E = [ns["transform44"](list(r)) for r in est_rows]
    # a rigid offset of the whole estimate (ATE aligns it away)
    c, s = np.cos(0.3), np.sin(0.3)
    off = np.array([[c, -s, 0, 0.5], [s, c, 0, -0.2], [0, 0, 1, 0.1], [0, 0, 0, 1.0]])
    E = [off @ T for T in E]
    est_xyz = np.array([T[:3, 3] for T in E])
    _, _, ate_err = ns["align"](np.matrix(est_xyz.T), np.matrix(t.T))
    rpe = {}
    for d in (1, 5):
        tr, rot = [], []
        for i in range(n - d):
            e44 = ns["ominus"](ns["ominus"](E[i + d], E[i]), ns["ominus"](G[i + d], G[i]))
            tr.append(ns["compute_distance"](e44))
            rot.append(ns["compute_angle"](e44))
        rpe[d] = (np.array(tr), np.array(rot))
    class ListKeys(dict):  # Python 2 dicts: keys() is a list the function edits
        def keys(self):
            return list(super().keys())
    first = ListKeys({float(r[0]): list(r[1:]) for r in gt_rows})
    second = ListKeys({float(r[0]) + 0.001 * ((i % 7) - 3): list(r[1:]) for i, r in enumerate(est_rows[::2])})
    matches = np.array(ns["associate"](first, second, 0.0, 0.02), np.float64)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "eval_golden.npz")
    np.savez_compressed(out, gt_rows=gt_rows, est_rows=est_rows, offset=off, G=np.array(G), E=np.array(E),
                        ate_err=np.asarray(ate_err).ravel(), rpe1_trans=rpe[1][0], rpe1_rot=rpe[1][1],
                        rpe5_trans=rpe[5][0], rpe5_rot=rpe[5][1],
                        assoc_first=np.array(sorted(first)), assoc_second=np.array(sorted(second)), matches=matches)
    print(out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SLAM_REFERENCE", ""))
