"""Frame readers on the GPU: KLG logs with JPEG colour (decoded by nvJPEG
where the reference uses libjpeg, src/inputs/JPEGLoader.h) and a log read
back into the tracker (src/apps/elastic_fusion.cpp:336-340 uploads the
reader's depth and RGB; here they go through the depth pre-filter and
initRGB)."""
import numpy as np
import pytest

from gpu_helpers import dev, dev_u16, report

pytestmark = pytest.mark.gpu


def test_jpeg_round_trip_and_klg(gpu, tmp_path):
    from slam_gb300 import inputs, synth
    cam = synth.Camera().scaled(320, 240)
    scene = synth.make_room(3)
    T = synth.room_camera(np.random.default_rng(3))
    fr = synth.render(scene, T, cam, depth=True, rgba=True)
    rgb = fr["rgba"][..., :3].copy()
    codec = inputs.JpegCodec()
    jpg = codec.encode(rgb, quality=95)
    assert jpg[:2] == b"\xff\xd8" and jpg[-2:] == b"\xff\xd9"
    back = codec.decode(jpg).cpu().numpy()
    err = np.abs(back.astype(np.int32) - rgb.astype(np.int32))
    assert back.shape == rgb.shape and err.mean() < 2.0 and np.percentile(err, 99) < 16, (err.mean(), err.max())
    p = tmp_path / "jpeg.klg"
    inputs.write_klg(str(p), [(10, fr["depth"], jpg), (20, fr["depth"], rgb), (30, fr["depth"], None)],
                     cam.width, cam.height)
    r = inputs.RawLogReader(str(p), False, cam.width, cam.height)
    r.getNext()
    assert r.timestamp == 10 and np.array_equal(r.depth, fr["depth"]) and np.array_equal(r.rgb, back)
    r.getNext()
    assert np.array_equal(r.rgb, rgb)
    report("nvJPEG q95 round trip 320x240: mean abs error %.2f, p99 %d (libjpeg's IDCT may differ by a unit)"
           % (err.mean(), np.percentile(err, 99)))


def test_klg_frames_track_like_the_arrays(gpu, tmp_path):
    """A pair written to a KLG log and read back tracks to the same bits as
    the same pair given as arrays (the reader returns the stored frames
    exactly)."""
    from slam_gb300 import RGBDOdometry, inputs, synth
    pair = synth.make_pair(21, cam=synth.Camera().scaled(320, 240))
    cam = pair["cam"]
    p = tmp_path / "pair.klg"
    inputs.write_klg(str(p), [(1, pair["depth"], pair["rgba"][..., :3]), (2, pair["depth"], None)],
                     cam.width, cam.height)
    r = inputs.RawLogReader(str(p), False, cam.width, cam.height)
    r.getNext()
    T1 = pair["T1"].astype(np.float32)
    out = []
    for depth, rgba in ((r.depth, inputs.rgb_to_rgba(r.rgb)), (pair["depth"], inputs.rgb_to_rgba(pair["rgba"][..., :3]))):
        g = RGBDOdometry(cam.width, cam.height, cam.cx, cam.cy, cam.fx, cam.fy)
        g.initFirstRGB(dev(pair["prev_rgba"]))
        g.initICPModel(dev(pair["model_vert"]), dev(pair["model_norm"]), 20.0, T1)
        g.initRGBModel(dev(pair["model_rgba"]))
        g.initICPRawDepth(dev_u16(depth), 20.0)
        g.initRGB(dev(rgba))
        out.append(g.getIncrementalTransformation(T1[:3, 3], T1[:3, :3]))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
