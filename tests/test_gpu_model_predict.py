"""Model prediction (IndexMap::combinedPredict as CUDA splatting,
src/model/shaders/splat.vert + combo_splat.frag) and fill-in
(src/gl/shaders/fill_*.frag) against the oracle's CPU restatement of the same
shader arithmetic: identical bits (both evaluate the same single-rounded FP32
operations in the same order with IEEE division and square root, and keep
the nearest fragment, the lower surfel index on equal depth)."""
import numpy as np
import pytest

from gpu_helpers import dev, dev_u16, report

pytestmark = pytest.mark.gpu


def surfel_map(cam, seed, views=3):
    """Surfels from `views` rendered views of one room (stride 2), with
    varied confidence and times so that the culling tests take both ways."""
    from slam_gb300 import model, synth
    rng = np.random.default_rng(seed)
    scene = synth.make_room(seed)
    T0 = synth.room_camera(rng)
    out = []
    for _ in range(views):
        T = T0 @ synth.random_motion(rng, 10.0, 0.2)
        m = synth.render(scene, T, cam, depth=False, rgba=True, model=True)
        S = model.surfels_from_view(m["vert"], m["norm"], m["rgba"], T, cam, stride=2)
        S[:, 3] = rng.uniform(5.0, 20.0, size=len(S)).astype(np.float32)      # confidence
        S[:, 6] = rng.integers(0, 50, size=len(S)).astype(np.float32)          # init time
        S[:, 7] = rng.integers(50, 100, size=len(S)).astype(np.float32)        # last update
        out.append(S)
    return T0, scene, np.concatenate(out)


def host(t):
    import torch
    t = t.cpu()
    return t.view(torch.int16).numpy().view(np.uint16) if t.dtype == torch.uint16 else t.numpy()


@pytest.mark.parametrize("size", [(640, 480), (90, 66)], ids=["640x480", "90x66"])
@pytest.mark.parametrize("cull", [dict(), dict(conf_threshold=12.0, time=100, time_delta=30, max_time=90)],
                         ids=["all", "culled"])
def test_prediction_matches_oracle(gpu, size, cull):
    from oracle import oracle
    from slam_gb300 import model, synth
    cam = synth.Camera().scaled(*size)
    T0, _, S = surfel_map(cam, 5)
    kw = dict(max_depth=20.0, conf_threshold=10.0, time=100, max_time=2 ** 30, time_delta=2 ** 30)
    kw.update(cull)
    params = model.predict_params(cam, **kw)
    img, v, n, t = (host(x) for x in model.predict(dev(S), T0, params))
    ei, ev, en, et = oracle.model_predict(S, model.t_inv_of(T0), cam, **kw)
    drawn = ev[..., 2] != 0
    assert drawn.mean() > 0.3
    assert np.array_equal(img, ei) and np.array_equal(t, et)
    assert np.array_equal(v.view(np.uint32), ev.view(np.uint32))
    assert np.array_equal(n.view(np.uint32), en.view(np.uint32))
    report("model prediction %dx%d %s: %d surfels, %.1f %% of pixels drawn, bit-identical"
           % (size + ("culled" if cull else "all", len(S), 100 * drawn.mean())))


def test_prediction_reproduces_the_view(gpu):
    """A surfel per pixel of one view, predicted at that view's pose, gives
    back its depth (to the half-pixel shift of the fragment centres and the
    disk intersection) on nearly every pixel."""
    from slam_gb300 import model, synth
    cam = synth.Camera().scaled(320, 240)
    T = synth.room_camera(np.random.default_rng(3))
    m = synth.render(synth.make_room(3), T, cam, depth=False, rgba=True, model=True)
    S = model.surfels_from_view(m["vert"], m["norm"], m["rgba"], T, cam)
    img, v, n, t = (host(x) for x in model.predict(dev(S), T, model.predict_params(cam, conf_threshold=0.0)))
    ok = (m["vert"][..., 2] > 0) & (v[..., 2] > 0)
    rel = np.abs(v[..., 2][ok] - m["vert"][..., 2][ok]) / m["vert"][..., 2][ok]
    assert ok.sum() > 0.95 * (m["vert"][..., 2] > 0).sum()
    assert np.median(rel) < 0.01


def test_fill_in_matches_oracle(gpu):
    from oracle import oracle
    from slam_gb300 import model, synth
    from slam_gb300.odometry import filter_depth
    cam = synth.Camera().scaled(160, 120)
    T0, scene, S = surfel_map(cam, 9, views=1)
    pi, pv, pn, _ = model.predict(dev(S), T0, model.predict_params(cam))
    live = synth.render(scene, T0, cam, noise_seed=4, depth=True, rgba=True)
    d = filter_depth(dev_u16(live["depth"]), 4.0)
    for passthrough in (False, True):
        ov, on, oi = (host(x) for x in model.fill_in(pv, pn, pi, d, dev(live["rgba"]), cam, passthrough))
        ev, en, ei = oracle.fill_in(host(pv), host(pn), host(pi), host(d), live["rgba"], cam, passthrough)
        assert np.array_equal(ov.view(np.uint32), ev.view(np.uint32)), passthrough
        nan_o, nan_e = np.isnan(on), np.isnan(en)
        assert np.array_equal(nan_o, nan_e), passthrough
        assert np.array_equal(on[~nan_o].view(np.uint32), en[~nan_e].view(np.uint32)), passthrough
        assert np.array_equal(oi, ei), passthrough
