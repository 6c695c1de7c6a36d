"""The learned warm start: trained here on the GPU by the library's own
kernels, it must make the short-schedule tracker converge where the same
schedule without it does not (what the network gains over the method
without it), and the warm-started batch entry point must keep or improve the
plain tracker's accuracy."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def trained(gpu):
    from slam_gb300 import synth, warmstart as ws
    from slam_gb300.batch import BatchOdometry
    b = BatchOdometry(512)
    net = ws.WarmStartNet(max_batch=256)
    ts = ws.make_training_set(net, b, seed=7, n=16384)
    net.set_loss_metric(ts["metric"])
    x0, y0 = ts["inputs"][:256].contiguous(), ts["labels"][:256].contiguous()
    loss0 = net.gradients(x0, y0)[1]
    ws.train(net, ts["inputs"], ts["labels"], epochs=24, batch=256, lr=5e-4, lr_final=2e-5)
    loss1 = net.gradients(x0, y0)[1]
    ps = ws.make_room_pairs(4242, 256, synth.Camera(), 10.0, 0.10)
    return b, net, ps, float(np.median(ts["residuals"])), (loss0, loss1)


def _fail_rate(res, T2):
    from slam_gb300 import synth
    from slam_gb300.batch import result_pose
    e = np.array([synth.pose_error(result_pose(r), T2[i]) for i, r in enumerate(res)])
    return float(np.mean((e[:, 0] > np.radians(2.0)) | (e[:, 1] > 0.05))), e


def test_training_reduces_loss(trained):
    loss0, loss1 = trained[4]
    assert loss1 < 0.5 * loss0, (loss0, loss1)


def test_network_gain_over_no_network(trained):
    """Same short schedule (3 levels, 6/4/4 iterations, no SO3), started from
    the network's proposal vs from the identity: far fewer failures."""
    import torch
    b, net, ps, _, _ = trained
    fps = ps.frame_pairs(levels=3, iterations=(6, 4, 4))
    prop = net.propose(ps.frame_pairs())
    f_net, _ = _fail_rate(b.track_init(fps, prop), ps.T2)
    f_zero, _ = _fail_rate(b.track_init(fps, torch.zeros_like(prop)), ps.T2)
    assert f_net < 0.6 * f_zero, (f_net, f_zero)


def test_warm_batch_not_worse_than_plain(trained):
    b, net, ps, plain_res, _ = trained
    fps = ps.frame_pairs()
    f_plain, e_plain = _fail_rate(b.track(fps), ps.T2)
    res, fb = b.track_warm(net, fps, levels=3, iterations=(6, 4, 4), residual_limit=1.5 * plain_res,
                           max_disagree_deg=5.0)
    f_warm, e_warm = _fail_rate(res, ps.T2)
    assert f_warm <= f_plain + 0.02, (f_warm, f_plain)
    ok = (e_plain[:, 0] < np.radians(2.0)) & (e_warm[:, 0] < np.radians(2.0))
    assert np.median(e_warm[ok, 0]) <= 1.5 * np.median(e_plain[ok, 0])
    assert 0.0 <= fb.mean() < 1.0


def test_fallback_pairs_equal_plain_tracking(trained):
    """Pairs that fall back are re-tracked with the plain schedule on the
    warm call's preprocessed buffers: bit for bit what a plain batched call
    on those pairs returns."""
    from slam_gb300.batch import result_pose
    b, net, ps, plain_res, _ = trained
    fps = ps.frame_pairs()
    res, fb = b.track_warm(net, fps, levels=3, iterations=(2, 2, 2), residual_limit=1.0 * plain_res,
                           max_disagree_deg=5.0)
    idx = np.nonzero(fb)[0]
    assert 0 < len(idx) < len(fps)
    plain = b.track([fps[i] for i in idx])
    for k, i in enumerate(idx):
        assert np.array_equal(result_pose(res[i]), result_pose(plain[k])), i
        assert list(res[i].iterations) == list(plain[k].iterations)
