"""slam_gb300/evaluate.py (ATE / RPE / trajectory files / timestamp
association) against the reference's own benchmark functions, recorded in
tests/golden/eval_golden.npz by tests/golden/make_eval_golden.py."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "eval_golden.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLDEN)


def test_quaternion_rows_to_poses(gold):
    from slam_gb300 import evaluate
    for rows, mats in ((gold["gt_rows"], gold["G"]),):
        for r, M in zip(rows, mats):
            assert np.allclose(evaluate.quat_to_matrix(r[1:4], r[4:8]), M, atol=1e-12)


def test_ate_matches_reference(gold):
    from slam_gb300 import evaluate
    G = gold["G"]
    E = gold["E"]
    _, _, err = evaluate.align(np.array([T[:3, 3] for T in E]).T, np.array([T[:3, 3] for T in G]).T)
    assert np.allclose(err, gold["ate_err"], rtol=1e-9, atol=1e-12)
    a = evaluate.ate(G, E)
    ref = gold["ate_err"]
    assert a["rmse"] == pytest.approx(np.sqrt(np.dot(ref, ref) / ref.size), rel=1e-9)
    assert a["median"] == pytest.approx(np.median(ref), rel=1e-9)


@pytest.mark.parametrize("delta", [1, 5])
def test_rpe_matches_reference(gold, delta):
    from slam_gb300 import evaluate
    r = evaluate.rpe(gold["G"], gold["E"], delta=delta)
    assert np.allclose(r["trans"], gold["rpe%d_trans" % delta], rtol=1e-9, atol=1e-12)
    assert np.allclose(r["rot"], gold["rpe%d_rot" % delta], rtol=1e-7, atol=1e-9)


def test_association_matches_reference(gold):
    from slam_gb300 import evaluate
    first = {float(s): [] for s in gold["assoc_first"]}
    second = {float(s): [] for s in gold["assoc_second"]}
    got = np.array(evaluate.associate(first, second, 0.0, 0.02))
    assert np.array_equal(got, gold["matches"])


def test_trajectory_file_round_trip(gold, tmp_path):
    from slam_gb300 import evaluate
    G, E = gold["G"], gold["E"]
    stamps = gold["gt_rows"][:, 0]
    evaluate.write_trajectory(str(tmp_path / "gt.txt"), stamps, G)
    evaluate.write_trajectory(str(tmp_path / "est.txt"), stamps, E)
    back = evaluate.read_trajectory(str(tmp_path / "gt.txt"))
    for s, T in zip(stamps, G):
        key = min(back, key=lambda k: abs(k - s))
        assert np.allclose(back[key], T, atol=2e-6)
    res = evaluate.evaluate_files(str(tmp_path / "gt.txt"), str(tmp_path / "est.txt"))
    assert res["ate"]["rmse"] == pytest.approx(evaluate.ate(G, E)["rmse"], rel=1e-4)
    assert res["rpe"]["trans_rmse"] == pytest.approx(evaluate.rpe(G, E)["trans_rmse"], rel=1e-3)


def test_identical_and_rigidly_moved_trajectories():
    from slam_gb300 import evaluate, synth
    T = synth.trajectory(3, 40)
    off = synth.pose(synth.rotvec_to_R([0.1, -0.2, 0.3]), np.array([1.0, 2.0, -0.5]))
    moved = [off @ P for P in T]
    assert evaluate.ate(T, moved)["rmse"] < 1e-9          # ATE aligns a rigid motion away
    r = evaluate.rpe(T, moved)
    assert r["trans_max"] < 1e-9 and r["rot_max"] < 1e-6  # relative motions are unchanged
