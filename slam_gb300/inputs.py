"""Frame readers of the reference's input formats, producing the u16 depth
(mm) and RGB frames that the depth pre-filter and initRGB consume.

* KLG logs (RawLogReader, src/inputs/RawLogReader.cpp:20-190): an int32
  frame count, then per frame an int64 timestamp, int32 depth size, int32
  image size, the depth (raw u16 if it is exactly 2 w h bytes, else zlib)
  and the image (raw RGB if exactly 3 w h bytes, JPEG if non-empty, else
  black).  zlib is the same library the reference links; JPEG images are
  decoded on the GPU by nvJPEG instead of the reference's libjpeg
  (src/inputs/JPEGLoader.h), so JPEG frames agree to the decoders' IDCT
  rounding, not bit for bit.
* TUM-style association lists with PNG images (FileReader,
  src/inputs/FileReader.cpp:3-69): "timestamp filename" pairs read two
  tokens at a time from the rgb and depth lists, images read the way
  cv::imread(IMREAD_UNCHANGED) returns them (colour in BGR order), depth
  scaled by 1000 / 5000 with convertTo's saturating round-half-even.  The
  PNG decoding is restated here (zlib inflate, then the scanline filters in
  the library's host code, odo_png_unfilter).

Both keep the reference's frame-count quirk: hasMore() is
currentFrame + 1 < numFrames, so the last frame is never read."""
import ctypes
import ctypes.util
import os
import struct
import zlib

import numpy as np

from . import _native


# ---------------------------------------------------------------------------
# KLG
# ---------------------------------------------------------------------------
class RawLogReader:
    """src/inputs/RawLogReader.cpp.  After getNext(): .timestamp (int),
    .depth (u16 [h][w], mm), .rgb (u8 [h][w][3]); .currentFrame counts the
    frames read (getBack() also counts one, as the reference's does)."""

    def __init__(self, file, flipColors, width, height):
        if not os.path.isfile(file):
            raise FileNotFoundError(file)
        self.file = file
        self.flipColors = bool(flipColors)
        self.width, self.height = int(width), int(height)
        self.numPixels = self.width * self.height
        self.timestamp = 0
        self.depth = None
        self.rgb = None
        self._jpeg = None
        self._open()

    def _open(self):
        self._fp = open(self.file, "rb")
        self.numFrames = struct.unpack("<i", self._read(4))[0]
        self.currentFrame = 0
        self._positions = []

    def close(self):
        if self._fp:
            self._fp.close()
            self._fp = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _read(self, n):
        b = self._fp.read(n)
        if len(b) != n:
            raise EOFError("truncated KLG log %s" % self.file)
        return b

    def _header(self):
        ts, dsize, isize = struct.unpack("<qii", self._read(16))
        if dsize < 0 or isize < 0:
            raise ValueError("corrupt KLG frame header in %s" % self.file)
        return ts, dsize, isize

    def getNext(self):
        self._positions.append(self._fp.tell())
        self._core()

    def getBack(self):
        if not self._positions:
            raise IndexError("no frame to go back to")
        self._fp.seek(self._positions.pop())
        self._core()

    def _core(self):
        self.timestamp, dsize, isize = self._header()
        dbuf = self._read(dsize)
        ibuf = self._read(isize) if isize > 0 else b""
        n = self.numPixels
        if dsize == 2 * n:
            draw = dbuf
        else:
            draw = zlib.decompress(dbuf)
            if len(draw) != 2 * n:
                raise ValueError("KLG depth inflates to %d bytes, expected %d" % (len(draw), 2 * n))
        self.depth = np.frombuffer(draw, dtype="<u2").reshape(self.height, self.width).astype(np.uint16)
        if isize == 3 * n:
            rgb = np.frombuffer(ibuf, np.uint8).reshape(self.height, self.width, 3).copy()
        elif isize > 0:
            if self._jpeg is None:
                self._jpeg = JpegCodec()
            rgb = self._jpeg.decode(ibuf).cpu().numpy()
            if rgb.shape != (self.height, self.width, 3):
                raise ValueError("KLG JPEG image is %s, expected %dx%d" % (rgb.shape, self.width, self.height))
        else:
            rgb = np.zeros((self.height, self.width, 3), np.uint8)
        if self.flipColors:
            rgb = rgb[..., ::-1].copy()
        self.rgb = rgb
        self.currentFrame += 1

    def fastForward(self, frame):
        """Skips frames up to `frame` without decoding them."""
        while self.currentFrame < frame and self.hasMore():
            self._positions.append(self._fp.tell())
            _, dsize, isize = self._header()
            self._fp.seek(dsize + isize, os.SEEK_CUR)
            self.currentFrame += 1

    def getNumFrames(self):
        return self.numFrames

    def hasMore(self):
        return self.currentFrame + 1 < self.numFrames

    def rewind(self):
        self.close()
        self._open()

    def rewound(self):
        return len(self._positions) == 0

    def getFile(self):
        return self.file


def write_klg(path, frames, width, height, depth_level=1):
    """Writes a KLG log from (timestamp, depth u16 [h][w], image) tuples;
    image is u8 [h][w][3] (stored raw), JPEG bytes (stored as is) or None
    (no image).  Depth is zlib-compressed at `depth_level` (0 stores it
    raw), as the reference's loggers write it."""
    frames = list(frames)
    with open(path, "wb") as f:
        f.write(struct.pack("<i", len(frames)))
        for ts, depth, image in frames:
            d = np.ascontiguousarray(depth, dtype="<u2")
            if d.shape != (height, width):
                raise ValueError("depth must be %dx%d" % (width, height))
            db = d.tobytes() if depth_level == 0 else zlib.compress(d.tobytes(), depth_level)
            if image is None:
                ib = b""
            elif isinstance(image, (bytes, bytearray)):
                ib = bytes(image)
            else:
                im = np.ascontiguousarray(image, np.uint8)
                if im.shape != (height, width, 3):
                    raise ValueError("image must be %dx%dx3" % (width, height))
                ib = im.tobytes()
            f.write(struct.pack("<qii", int(ts), len(db), len(ib)))
            f.write(db)
            f.write(ib)


# ---------------------------------------------------------------------------
# JPEG through nvJPEG
# ---------------------------------------------------------------------------
class _NvjpegImage(ctypes.Structure):
    _fields_ = [("channel", ctypes.c_void_p * 4), ("pitch", ctypes.c_size_t * 4)]


_NVJPEG_OUTPUT_RGBI = 5
_NVJPEG_INPUT_RGBI = 5
_NVJPEG_CSS_444 = 0


def _load_nvjpeg():
    names = ["libnvjpeg.so.13", "libnvjpeg.so"]
    found = ctypes.util.find_library("nvjpeg")
    if found:
        names.append(found)
    for d in ("/usr/local/cuda/lib64", "/usr/local/cuda/targets/sbsa-linux/lib",
              "/usr/local/cuda/targets/x86_64-linux/lib"):
        names += [os.path.join(d, "libnvjpeg.so.13"), os.path.join(d, "libnvjpeg.so")]
    for n in names:
        try:
            return ctypes.CDLL(n)
        except OSError:
            continue
    raise _native.NativeError("nvJPEG (libnvjpeg) not found: KLG logs with JPEG images cannot be read")


class JpegCodec:
    """Baseline JPEG decode (and encode, for writing test logs) on the GPU
    with nvJPEG, on the current torch stream."""

    def __init__(self):
        self._L = _load_nvjpeg()
        self._h = ctypes.c_void_p()
        self._check(self._L.nvjpegCreateSimple(ctypes.byref(self._h)), "nvjpegCreateSimple")
        self._state = ctypes.c_void_p()
        self._check(self._L.nvjpegJpegStateCreate(self._h, ctypes.byref(self._state)), "nvjpegJpegStateCreate")

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise _native.NativeError("%s failed with nvJPEG status %d" % (what, rc))

    @staticmethod
    def _stream():
        import torch
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def decode(self, data):
        """JPEG bytes -> CUDA u8 [h][w][3] (RGB)."""
        import torch
        data = bytes(data)
        buf = (ctypes.c_ubyte * len(data)).from_buffer_copy(data)
        nc, ss = ctypes.c_int(), ctypes.c_int()
        ws, hs = (ctypes.c_int * 4)(), (ctypes.c_int * 4)()
        self._check(self._L.nvjpegGetImageInfo(self._h, buf, ctypes.c_size_t(len(data)), ctypes.byref(nc),
                                               ctypes.byref(ss), ws, hs), "nvjpegGetImageInfo")
        w, h = ws[0], hs[0]
        out = torch.empty((h, w, 3), dtype=torch.uint8, device="cuda")
        img = _NvjpegImage()
        img.channel[0] = out.data_ptr()
        img.pitch[0] = 3 * w
        self._check(self._L.nvjpegDecode(self._h, self._state, buf, ctypes.c_size_t(len(data)), _NVJPEG_OUTPUT_RGBI,
                                         ctypes.byref(img), self._stream()), "nvjpegDecode")
        torch.cuda.current_stream().synchronize()
        return out

    def encode(self, rgb, quality=95):
        """CUDA (or host) u8 [h][w][3] RGB -> JPEG bytes (4:4:4)."""
        import torch
        rgb = torch.as_tensor(rgb).cuda().contiguous()
        h, w = rgb.shape[:2]
        s = self._stream()
        st, par = ctypes.c_void_p(), ctypes.c_void_p()
        self._check(self._L.nvjpegEncoderStateCreate(self._h, ctypes.byref(st), s), "nvjpegEncoderStateCreate")
        try:
            self._check(self._L.nvjpegEncoderParamsCreate(self._h, ctypes.byref(par), s), "nvjpegEncoderParamsCreate")
            self._check(self._L.nvjpegEncoderParamsSetQuality(par, int(quality), s), "nvjpegEncoderParamsSetQuality")
            self._check(self._L.nvjpegEncoderParamsSetSamplingFactors(par, _NVJPEG_CSS_444, s),
                        "nvjpegEncoderParamsSetSamplingFactors")
            img = _NvjpegImage()
            img.channel[0] = rgb.data_ptr()
            img.pitch[0] = 3 * w
            self._check(self._L.nvjpegEncodeImage(self._h, st, par, ctypes.byref(img), _NVJPEG_INPUT_RGBI, w, h, s),
                        "nvjpegEncodeImage")
            n = ctypes.c_size_t()
            self._check(self._L.nvjpegEncodeRetrieveBitstream(self._h, st, None, ctypes.byref(n), s),
                        "nvjpegEncodeRetrieveBitstream")
            buf = (ctypes.c_ubyte * n.value)()
            self._check(self._L.nvjpegEncodeRetrieveBitstream(self._h, st, buf, ctypes.byref(n), s),
                        "nvjpegEncodeRetrieveBitstream")
            torch.cuda.current_stream().synchronize()
            return bytes(buf[:n.value])
        finally:
            if par:
                self._L.nvjpegEncoderParamsDestroy(par)
            self._L.nvjpegEncoderStateDestroy(st)

    def close(self):
        if self._state:
            self._L.nvjpegJpegStateDestroy(self._state)
            self._state = None
        if self._h:
            self._L.nvjpegDestroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# PNG (the subset a TUM-style dataset uses: 8/16-bit grey, RGB, RGBA, no
# interlacing)
# ---------------------------------------------------------------------------
_PNG_SIG = b"\x89PNG\r\n\x1a\n"
_CHANNELS = {0: 1, 2: 3, 6: 4}


def _chunks(data):
    if data[:8] != _PNG_SIG:
        raise ValueError("not a PNG file")
    pos = 8
    while pos + 8 <= len(data):
        n, kind = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if len(body) != n:
            raise ValueError("truncated PNG chunk")
        crc = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        if zlib.crc32(kind + body) & 0xffffffff != crc:
            raise ValueError("PNG chunk %r fails its CRC" % kind)
        yield kind, body
        pos += 12 + n
        if kind == b"IEND":
            return
    raise ValueError("PNG without IEND")


def decode_png(data):
    """PNG bytes -> array as cv::imread(IMREAD_UNCHANGED) returns it: grey
    [h][w], colour [h][w][3] BGR, with alpha [h][w][4] BGRA; u8 or u16."""
    ihdr, idat = None, []
    for kind, body in _chunks(data):
        if kind == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat.append(body)
    if ihdr is None:
        raise ValueError("PNG without IHDR")
    w, h, depth, ctype, comp, filt, interlace = ihdr
    if ctype not in _CHANNELS or depth not in (8, 16) or comp != 0 or filt != 0:
        raise ValueError("unsupported PNG (colour type %d, bit depth %d)" % (ctype, depth))
    if interlace != 0:
        raise ValueError("interlaced PNG is not supported")
    ch = _CHANNELS[ctype]
    bpp = ch * depth // 8
    row_bytes = w * bpp
    raw = zlib.decompress(b"".join(idat))
    if len(raw) != h * (row_bytes + 1):
        raise ValueError("PNG image data has %d bytes, expected %d" % (len(raw), h * (row_bytes + 1)))
    src = np.frombuffer(raw, np.uint8)
    out = np.empty(h * row_bytes, np.uint8)
    rc = _native.load().odo_png_unfilter(src.ctypes.data_as(ctypes.c_void_p), h, row_bytes, bpp,
                                         out.ctypes.data_as(ctypes.c_void_p))
    if rc != 0:
        raise ValueError("PNG scanline with an unknown filter type")
    img = out.view(">u2").astype(np.uint16) if depth == 16 else out
    img = img.reshape(h, w, ch) if ch > 1 else img.reshape(h, w)
    if ch == 3:
        img = img[..., ::-1]
    elif ch == 4:
        img = img[..., [2, 1, 0, 3]]
    return np.ascontiguousarray(img)


def read_png(path):
    with open(path, "rb") as f:
        return decode_png(f.read())


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
    return np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))


def encode_png(img, filters=None, level=6):
    """Array in cv::imwrite order (grey, BGR or BGRA; u8 or u16) -> PNG
    bytes.  filters: per-row filter types 0-4 (default: the rows cycle
    through all five, which is what the decoder's tests need)."""
    img = np.asarray(img)
    if img.dtype not in (np.uint8, np.uint16):
        raise ValueError("PNG needs u8 or u16 pixels")
    h, w = img.shape[:2]
    ch = 1 if img.ndim == 2 else img.shape[2]
    ctype = {1: 0, 3: 2, 4: 6}[ch]
    if ch == 3:
        img = img[..., ::-1]
    elif ch == 4:
        img = img[..., [2, 1, 0, 3]]
    depth = 16 if img.dtype == np.uint16 else 8
    rows = np.ascontiguousarray(img.astype(">u2") if depth == 16 else img).view(np.uint8).reshape(h, -1)
    bpp = ch * depth // 8
    filters = [y % 5 for y in range(h)] if filters is None else list(filters)
    out = bytearray()
    prev = np.zeros(rows.shape[1], np.int32)
    for y in range(h):
        r = rows[y].astype(np.int32)
        a = np.concatenate([np.zeros(bpp, np.int32), r[:-bpp]])
        c = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]])
        t = filters[y]
        pred = [np.zeros_like(r), a, prev, (a + prev) >> 1, _paeth(a, prev, c)][t]
        out.append(t)
        out += ((r - pred) & 0xff).astype(np.uint8).tobytes()
        prev = r
    chunk = lambda kind, body: (struct.pack(">I", len(body)) + kind + body +
                                struct.pack(">I", zlib.crc32(kind + body) & 0xffffffff))
    return (_PNG_SIG + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0)) +
            chunk(b"IDAT", zlib.compress(bytes(out), level)) + chunk(b"IEND", b""))


def write_png(path, img, **kw):
    with open(path, "wb") as f:
        f.write(encode_png(img, **kw))


# ---------------------------------------------------------------------------
# TUM-style file lists
# ---------------------------------------------------------------------------
def tum_depth_to_mm(depth):
    """depth.convertTo(depth, CV_16UC1, 1000 * 1.0 / 5000)
    (src/inputs/FileReader.cpp:52): u16 * (float)0.2, rounded half to even,
    saturated to u16."""
    v = np.asarray(depth, np.uint16).astype(np.float32) * np.float32(1000 * 1.0 / 5000)
    return np.clip(np.rint(v), 0, 65535).astype(np.uint16)


class FileReader:
    """src/inputs/FileReader.cpp.  After getNext(): .rgb (as cv::imread
    returns it: BGR), .depth (u16 mm) and the frame's .timestamp token."""

    def __init__(self, rgb_info, depth_info, dataset_dir, width, height):
        for p in (rgb_info, depth_info):
            if not os.path.isfile(p):
                raise FileNotFoundError(p)
        self.dataset_dir = dataset_dir
        self.width, self.height = int(width), int(height)
        with open(rgb_info, "rb") as f:
            self.numFrames = f.read().count(b"\n")
        self.currentFrame = 0
        with open(rgb_info) as f:
            self._rgb_tokens = f.read().split()
        with open(depth_info) as f:
            self._depth_tokens = f.read().split()
        self.rgb = self.depth = None
        self.timestamp = None

    def getNext(self):
        if not self.hasMore():
            return
        k = 2 * self.currentFrame
        if k + 1 >= len(self._rgb_tokens) or k + 1 >= len(self._depth_tokens):
            raise EOFError("file list shorter than its line count")
        self.timestamp = self._rgb_tokens[k]
        self.rgb = read_png(self.dataset_dir + self._rgb_tokens[k + 1])
        self.depth = tum_depth_to_mm(read_png(self.dataset_dir + self._depth_tokens[k + 1]))
        self.currentFrame += 1

    def getNumFrames(self):
        return self.numFrames

    def hasMore(self):
        return self.currentFrame + 1 < self.numFrames


def rgb_to_rgba(rgb):
    """The RGB upload into the RGBA texture initRGB reads (GL fills alpha
    with 255)."""
    rgb = np.asarray(rgb, np.uint8)
    out = np.empty(rgb.shape[:2] + (4,), np.uint8)
    out[..., :3] = rgb
    out[..., 3] = 255
    return out
