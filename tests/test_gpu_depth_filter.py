"""The depth pre-filter (the reference's depth_bilateral.frag and
depth_metric.frag, src/gl/shaders/) against the oracle's CPU restatement of
the shader arithmetic, and initICP on raw depth (filter + pyramid + maps)
against the filter followed by initICP.

Filtered depth is integer output: identical except where the oracle flags a
quotient within 2e-3 mm of a rounding boundary (expf differs between
libraries by an ulp or two).  Metric depth is an IEEE division: identical."""
import numpy as np
import pytest

from gpu_helpers import check_pose, dev, dev_u16, frame_runs, gpu_images, load_frame, new_gpu_odo, report, track

pytestmark = pytest.mark.gpu


def raw_depth(seed, cam):
    """Rendered depth (noise, 5 % holes) with some values beyond the far cut
    and below the 300 mm floor planted."""
    from slam_gb300 import synth
    p = synth.make_pair(seed, cam=cam)
    d = p["depth"].copy()
    rng = np.random.default_rng(seed)
    idx = rng.integers(0, d.size, size=d.size // 50)
    d.reshape(-1)[idx[: idx.size // 2]] = rng.integers(4001, 9000, size=idx.size // 2)
    d.reshape(-1)[idx[idx.size // 2:]] = rng.integers(1, 300, size=idx.size - idx.size // 2)
    return p, d


def host_u16(t):
    import torch
    return t.cpu().view(torch.int16).numpy().view(np.uint16)


@pytest.mark.parametrize("size", [(640, 480), (90, 66)], ids=["640x480", "90x66"])
@pytest.mark.parametrize("maxD", [4.0, 20.0])
def test_bilateral_filter_matches_oracle(gpu, size, maxD):
    from oracle import oracle
    from slam_gb300 import synth
    from slam_gb300.odometry import depth_metric, filter_depth
    p, d = raw_depth(7, synth.Camera().scaled(*size))
    got = host_u16(filter_depth(dev_u16(d), maxD))
    exp, tie = oracle.depth_bilateral(d, maxD, with_tie=True)
    mism = got != exp
    assert np.all(tie[mism] != 0), int((mism & (tie == 0)).sum())
    assert np.abs(got.astype(np.int32) - exp.astype(np.int32)).max() <= 1
    assert (got == 0).sum() > d.size // 100 and (got > 0).mean() > 0.5
    m = depth_metric(dev_u16(d), maxD).cpu().numpy()
    assert np.array_equal(m.view(np.uint32), oracle.depth_metric(d, maxD).view(np.uint32))
    report("depth filter %dx%d maxD %g: %d of %d pixels differ, all on flagged ties (%d flagged)"
           % (size + (maxD, int(mism.sum()), d.size, int(tie.sum()))))


def test_init_icp_raw_depth_equals_filter_then_init_icp(gpu):
    """initICP on raw depth = the filter followed by initICP(depth): the same
    level-0 depth, pyramid and maps, bit for bit; tracking from it matches the
    oracle's host loop on the oracle's filtered image."""
    from oracle import oracle
    from slam_gb300 import synth
    from slam_gb300.odometry import filter_depth
    p, d = raw_depth(11, synth.Camera().scaled(320, 240))
    p["depth"] = d
    a = new_gpu_odo(p["cam"])
    a.initFirstRGB(dev(p["prev_rgba"]))
    a.initICPModel(dev(p["model_vert"]), dev(p["model_norm"]), 20.0, p["T1"].astype(np.float32))
    a.initRGBModel(dev(p["model_rgba"]))
    a.initICPRawDepth(dev_u16(d), 4.0, 20.0)
    a.initRGB(dev(p["rgba"]))
    b = new_gpu_odo(p["cam"])
    pf = dict(p)
    pf["depth"] = host_u16(filter_depth(dev_u16(d), 4.0))
    load_frame(b, pf)
    for which in (0, 1, 2):
        for l in range(3):
            x, y = a.download(which, l), b.download(which, l)
            assert np.array_equal(np.asarray(x).view(np.uint8), np.asarray(y).view(np.uint8)), (which, l)
    images = gpu_images(a)
    tg, Rg = track(a, p)
    of = dict(p)
    of["depth"] = oracle.depth_bilateral(d, 4.0)
    ref = frame_runs(of, {}, images=images)
    to, Ro, o = ref.main
    check_pose("raw-depth tracking 320x240", tg, Rg, to, Ro, ref.tolerance)
