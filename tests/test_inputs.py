"""Frame readers (slam_gb300.inputs) on the CPU: the KLG log layout of
src/inputs/RawLogReader.cpp:20-190 built byte by byte here, the TUM-style
file lists of src/inputs/FileReader.cpp:3-69, and the PNG scanline filters
against a direct restatement of the PNG format's reconstruction rules."""
import struct
import zlib

import numpy as np
import pytest

from slam_gb300 import inputs


def klg_bytes(frames, w, h):
    """A KLG log assembled field by field: int32 count; per frame int64
    timestamp, int32 depth size, int32 image size, depth, image."""
    out = struct.pack("<i", len(frames))
    for ts, depth_blob, image_blob in frames:
        out += struct.pack("<q", ts) + struct.pack("<i", len(depth_blob)) + struct.pack("<i", len(image_blob))
        out += depth_blob + image_blob
    return out


def test_klg_layout_compressed_raw_and_missing_images(tmp_path):
    w, h = 7, 5
    rng = np.random.default_rng(0)
    d = [rng.integers(0, 65535, size=(h, w)).astype(np.uint16) for _ in range(4)]
    c = [rng.integers(0, 256, size=(h, w, 3)).astype(np.uint8) for _ in range(4)]
    frames = [(1000, zlib.compress(d[0].astype("<u2").tobytes()), c[0].tobytes()),
              (2000, d[1].astype("<u2").tobytes(), c[1].tobytes()),         # raw depth (exactly 2 w h bytes)
              (3000, zlib.compress(d[2].astype("<u2").tobytes(), 9), b""),  # no image: black
              (4000, zlib.compress(d[3].astype("<u2").tobytes()), c[3].tobytes())]
    p = tmp_path / "log.klg"
    p.write_bytes(klg_bytes(frames, w, h))
    r = inputs.RawLogReader(str(p), False, w, h)
    assert r.getNumFrames() == 4 and r.rewound()
    seen = []
    while r.hasMore():                      # the reference never reads the last frame
        r.getNext()
        seen.append((r.timestamp, r.depth.copy(), r.rgb.copy()))
    assert [s[0] for s in seen] == [1000, 2000, 3000]
    for k in range(3):
        assert np.array_equal(seen[k][1], d[k])
    assert np.array_equal(seen[0][2], c[0]) and np.array_equal(seen[1][2], c[1])
    assert not seen[2][2].any()
    # getBack re-reads the frame last read and counts it, as the reference does
    n = r.currentFrame
    r.getBack()
    assert r.timestamp == 3000 and r.currentFrame == n + 1
    r.rewind()
    assert r.currentFrame == 0 and r.rewound()
    r.fastForward(2)
    assert r.currentFrame == 2
    r.getNext()
    assert r.timestamp == 3000 and np.array_equal(r.depth, d[2])
    r.close()


def test_klg_flip_colors_and_writer(tmp_path):
    w, h = 6, 4
    rng = np.random.default_rng(1)
    d = rng.integers(0, 5000, size=(h, w)).astype(np.uint16)
    c = rng.integers(0, 256, size=(h, w, 3)).astype(np.uint8)
    p = tmp_path / "w.klg"
    inputs.write_klg(str(p), [(5, d, c), (6, d, None), (7, d, c)], w, h)
    blob = p.read_bytes()
    assert struct.unpack("<i", blob[:4])[0] == 3
    ts, dsize, isize = struct.unpack("<qii", blob[4:20])
    assert ts == 5 and isize == w * h * 3 and zlib.decompress(blob[20:20 + dsize]) == d.astype("<u2").tobytes()
    r = inputs.RawLogReader(str(p), True, w, h)
    r.getNext()
    assert np.array_equal(r.rgb, c[..., ::-1])
    r2 = inputs.RawLogReader(str(p), False, w, h)
    r2.getNext()
    assert np.array_equal(r2.rgb, c)


def test_klg_truncated_and_corrupt(tmp_path):
    w, h = 4, 4
    d = (np.arange(16, dtype=np.uint16) % 3).reshape(4, 4)
    z = zlib.compress(d.tobytes())
    assert len(z) != 2 * w * h              # a blob of exactly 2 w h bytes is taken as raw depth
    p = tmp_path / "t.klg"
    p.write_bytes(klg_bytes([(1, z, b""), (2, b"xx", b"")], w, h)[:-1])
    r = inputs.RawLogReader(str(p), False, w, h)
    r.getNext()
    assert np.array_equal(r.depth, d)
    q = tmp_path / "c.klg"
    q.write_bytes(klg_bytes([(1, zlib.compress(b"\0" * 6), b""), (2, b"", b"")], w, h))
    r = inputs.RawLogReader(str(q), False, w, h)
    with pytest.raises(ValueError):
        r.getNext()


def unfilter_restated(raw, h, row_bytes, bpp):
    """The PNG format's reconstruction, byte by byte."""
    out = np.zeros((h, row_bytes), np.int64)
    for y in range(h):
        t = raw[y * (row_bytes + 1)]
        for i in range(row_bytes):
            x = int(raw[y * (row_bytes + 1) + 1 + i])
            a = int(out[y, i - bpp]) if i >= bpp else 0
            b = int(out[y - 1, i]) if y > 0 else 0
            c = int(out[y - 1, i - bpp]) if (y > 0 and i >= bpp) else 0
            if t == 1:
                x += a
            elif t == 2:
                x += b
            elif t == 3:
                x += (a + b) // 2
            elif t == 4:
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                x += a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            out[y, i] = x & 0xff
    return out.astype(np.uint8)


@pytest.mark.parametrize("bpp", [1, 2, 3, 4, 6, 8])
def test_png_unfilter_matches_the_format_rules(bpp):
    import ctypes
    from slam_gb300 import _native
    rng = np.random.default_rng(bpp)
    h, row_bytes = 11, bpp * 9
    raw = rng.integers(0, 256, size=h * (row_bytes + 1)).astype(np.uint8)
    raw[::row_bytes + 1] = np.arange(h) % 5
    out = np.empty(h * row_bytes, np.uint8)
    assert _native.load().odo_png_unfilter(raw.ctypes.data_as(ctypes.c_void_p), h, row_bytes, bpp,
                                           out.ctypes.data_as(ctypes.c_void_p)) == 0
    assert np.array_equal(out.reshape(h, row_bytes), unfilter_restated(raw, h, row_bytes, bpp))
    raw[0] = 5                                        # unknown filter type
    assert _native.load().odo_png_unfilter(raw.ctypes.data_as(ctypes.c_void_p), h, row_bytes, bpp,
                                           out.ctypes.data_as(ctypes.c_void_p)) != 0


@pytest.mark.parametrize("shape,dtype", [((9, 13), np.uint8), ((9, 13, 3), np.uint8), ((6, 5, 4), np.uint8),
                                         ((7, 11), np.uint16), ((5, 4, 3), np.uint16)])
def test_png_round_trip(shape, dtype):
    rng = np.random.default_rng(len(shape))
    img = rng.integers(0, np.iinfo(dtype).max + 1, size=shape).astype(dtype)
    for filters in (None, [4] * shape[0], [3] * shape[0]):
        back = inputs.decode_png(inputs.encode_png(img, filters=filters))
        assert back.dtype == dtype and np.array_equal(back, img)


def test_png_channel_order_is_imread_order():
    """A 3-channel PNG holds R, G, B; decoding returns B, G, R."""
    bgr = np.zeros((2, 2, 3), np.uint8)
    bgr[..., 0] = 10
    bgr[..., 2] = 200
    png = inputs.encode_png(bgr, filters=[0, 0])
    raw = zlib.decompress(png[png.index(b"IDAT") + 4:png.index(b"IEND") - 8])
    assert raw[1:4] == bytes([200, 0, 10])            # stored as R, G, B
    assert np.array_equal(inputs.decode_png(png), bgr)


def test_png_rejects_bad_input():
    img = np.zeros((3, 3), np.uint8)
    png = bytearray(inputs.encode_png(img))
    png[30] ^= 0xff                                   # inside IHDR: CRC fails
    with pytest.raises(ValueError):
        inputs.decode_png(bytes(png))
    with pytest.raises(ValueError):
        inputs.decode_png(b"notapng")


def test_tum_depth_scale():
    d = np.array([[0, 1, 2, 3, 5000], [7, 12, 13, 65535, 25000]], np.uint16)
    got = inputs.tum_depth_to_mm(d)
    # u16 * (float)0.2, round half to even: 1 -> 0.2 -> 0, 3 -> 0.6 -> 1, 12 -> 2.4 -> 2, 13 -> 2.6 -> 3
    assert got.tolist() == [[0, 0, 0, 1, 1000], [1, 2, 3, 13107, 5000]]


def test_file_reader(tmp_path):
    rng = np.random.default_rng(4)
    w, h = 8, 6
    (tmp_path / "rgb").mkdir()
    (tmp_path / "depth").mkdir()
    rgbs, depths = [], []
    rl, dl = [], []
    for k in range(3):
        c = rng.integers(0, 256, size=(h, w, 3)).astype(np.uint8)
        d = rng.integers(0, 60000, size=(h, w)).astype(np.uint16)
        inputs.write_png(str(tmp_path / "rgb" / ("%d.png" % k)), c)
        inputs.write_png(str(tmp_path / "depth" / ("%d.png" % k)), d)
        rgbs.append(c)
        depths.append(d)
        rl.append("%d.0 rgb/%d.png" % (k, k))
        dl.append("%d.0 depth/%d.png" % (k, k))
    (tmp_path / "rgb.txt").write_text("\n".join(rl) + "\n")
    (tmp_path / "depth.txt").write_text("\n".join(dl) + "\n")
    r = inputs.FileReader(str(tmp_path / "rgb.txt"), str(tmp_path / "depth.txt"), str(tmp_path) + "/", w, h)
    assert r.getNumFrames() == 3
    k = 0
    while r.hasMore():
        r.getNext()
        assert np.array_equal(r.rgb, rgbs[k])
        assert np.array_equal(r.depth, inputs.tum_depth_to_mm(depths[k]))
        k += 1
    assert k == 2


def test_rgb_to_rgba():
    c = np.arange(2 * 3 * 3, dtype=np.uint8).reshape(2, 3, 3)
    o = inputs.rgb_to_rgba(c)
    assert np.array_equal(o[..., :3], c) and (o[..., 3] == 255).all()
