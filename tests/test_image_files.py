"""Image files written on the host (vcr_write_exr, vcr_write_png; no GPU):
each file is parsed here by a reader written from the formats'
specifications (OpenEXR 2.0 single-part scan-line layout; PNG with a zlib
stream, checked by Python's zlib) and its pixels compared with the input.
HALF channels are compared bit for bit with numpy's float16 rounding
(round to nearest, ties to even) over every halfway case of the half range."""
import struct
import zlib

import numpy as np
import pytest

import vcr
from vcr import _abi


def read_exr(path):
    """Minimal OpenEXR reader for single-part, uncompressed scan-line files:
    (header attributes, [H, W, 3] float64 RGB, raw channel arrays)."""
    b = open(path, "rb").read()
    assert b[:4] == b"\x76\x2f\x31\x01"
    version = struct.unpack("<I", b[4:8])[0]
    pos, attrs = 8, {}
    while b[pos] != 0:
        end = b.index(b"\0", pos)
        name = b[pos:end].decode()
        pos = end + 1
        end = b.index(b"\0", pos)
        typ = b[pos:end].decode()
        pos = end + 1
        size = struct.unpack("<i", b[pos:pos + 4])[0]
        pos += 4
        attrs[name] = (typ, b[pos:pos + size])
        pos += size
    pos += 1
    chl, q, channels = attrs["channels"][1], 0, []
    while chl[q] != 0:
        end = chl.index(b"\0", q)
        name = chl[q:end].decode()
        ptype, plinear, xs, ys = struct.unpack("<iB3xii", chl[end + 1:end + 17])
        channels.append((name, ptype, plinear, xs, ys))
        q = end + 17
    assert q == len(chl) - 1
    x0, y0, x1, y1 = struct.unpack("<4i", attrs["dataWindow"][1])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    offsets = struct.unpack(f"<{h}Q", b[pos:pos + 8 * h])
    raw = {c[0]: np.zeros((h, w), np.float16 if c[1] == 1 else np.float32) for c in channels}
    for i, off in enumerate(offsets):
        y, size = struct.unpack("<iI", b[off:off + 8])
        assert y == y0 + i
        p = off + 8
        for name, ptype, *_ in channels:
            dt = np.dtype("<f2") if ptype == 1 else np.dtype("<f4")
            raw[name][i] = np.frombuffer(b[p:p + w * dt.itemsize], dt)
            p += w * dt.itemsize
        assert p == off + 8 + size
    assert offsets[-1] + 8 + size == len(b)
    img = np.stack([raw["R"], raw["G"], raw["B"]], axis=-1).astype(np.float64)
    return version, attrs, channels, img, raw


def test_exr_float_round_trip_and_header(tmp_path):
    rng = np.random.default_rng(4)
    img = (rng.standard_normal((37, 53, 3)) * 10.0 ** rng.integers(-8, 8, (37, 53, 3))).astype(np.float32)
    img[0, 0] = [0.0, -0.0, np.inf]
    path = str(tmp_path / "a.exr")
    vcr.write_exr(path, img)
    version, attrs, channels, back, raw = read_exr(path)
    assert version == 2  # single part, scan lines, short names
    assert [c[0] for c in channels] == ["B", "G", "R"]
    assert all(c[1:] == (2, 0, 1, 1) for c in channels)
    assert attrs["compression"] == ("compression", b"\x00")
    assert attrs["lineOrder"] == ("lineOrder", b"\x00")
    assert attrs["dataWindow"] == attrs["displayWindow"] == ("box2i", struct.pack("<4i", 0, 0, 52, 36))
    assert struct.unpack("<f", attrs["pixelAspectRatio"][1]) == (1.0,)
    assert struct.unpack("<2f", attrs["screenWindowCenter"][1]) == (0.0, 0.0)
    assert struct.unpack("<f", attrs["screenWindowWidth"][1]) == (1.0,)
    assert set(attrs) == {"channels", "compression", "dataWindow", "displayWindow", "lineOrder", "pixelAspectRatio",
                          "screenWindowCenter", "screenWindowWidth"}
    for c, name in enumerate("RGB"):
        np.testing.assert_array_equal(raw[name].view(np.uint32), img[..., c].view(np.uint32))
    assert np.signbit(raw["G"][0, 0])


def _halfway_cases():
    """Every finite half, the midpoints between neighbours, one float step
    either side of each midpoint, overflow, underflow and the specials."""
    h = np.arange(0, 0x7C00, dtype=np.uint32).astype(np.uint16).view(np.float16).astype(np.float64)
    nxt = np.append(h[1:], 65536.0)  # the step past 65504 is where rounding overflows
    mid = ((h + nxt) / 2).astype(np.float32)
    up = np.nextafter(mid, np.float32(np.inf))
    down = np.nextafter(mid, np.float32(0))
    vals = np.concatenate([h.astype(np.float32), mid, up, down,
                           np.array([65504, 65519.99, 65520, 1e9, 3e38, np.inf, 2.0 ** -25, 2.0 ** -26, 1e-30,
                                     1e-45, 2.0 ** -14, 2.0 ** -24, 5.960464477539063e-08], np.float32)])
    return np.concatenate([vals, -vals])


def test_exr_half_channels_round_like_numpy(tmp_path):
    vals = _halfway_cases()
    w = 1024
    n = (len(vals) + 3 * w - 1) // (3 * w) * 3 * w
    flat = np.zeros(n, np.float32)
    flat[:len(vals)] = vals
    img = flat.reshape(-1, w, 3)
    path = str(tmp_path / "h.exr")
    vcr.write_exr(path, img, half=True)
    _, _, channels, _, raw = read_exr(path)
    assert all(c[1] == 1 for c in channels)
    got = np.stack([raw["R"], raw["G"], raw["B"]], axis=-1).reshape(-1)[:len(vals)]
    with np.errstate(over="ignore"):  # overflow to infinity is among the cases
        want = vals.astype(np.float16)
    np.testing.assert_array_equal(got.view(np.uint16), want.view(np.uint16))


def test_exr_half_nan_stays_nan(tmp_path):
    img = np.array([[[np.nan, -np.nan, 1.0]]], np.float32)
    img[0, 0, 2] = np.frombuffer(struct.pack("<I", 0x7F800001), np.float32)[0]  # signalling, low payload bit
    path = str(tmp_path / "n.exr")
    vcr.write_exr(path, img, half=True)
    _, _, _, back, raw = read_exr(path)
    assert np.isnan(back).all()
    assert np.signbit(raw["G"][0, 0]) == np.signbit(img[0, 0, 1])


def test_exr_and_png_refuse_bad_arguments(tmp_path):
    L = vcr.lib()
    img = np.zeros((2, 2, 3), np.float32)
    p = str(tmp_path / "x.exr").encode()
    assert L.vcr_write_exr(p, 2, 2, img.ctypes.data, 3) == _abi.ERR_INVALID
    assert L.vcr_write_exr(p, 0, 2, img.ctypes.data, _abi.EXR_FLOAT) == _abi.ERR_INVALID
    assert L.vcr_write_exr(p, 2, 2, None, _abi.EXR_FLOAT) == _abi.ERR_INVALID
    bad = str(tmp_path / "no" / "such" / "dir.exr").encode()
    assert L.vcr_write_exr(bad, 2, 2, img.ctypes.data, _abi.EXR_FLOAT) == _abi.ERR_IO
    assert b"cannot create" in L.vcr_last_error(None)
    px = np.zeros((2, 2, 4), np.uint8)
    assert L.vcr_write_png(bad, 2, 2, px.ctypes.data) == _abi.ERR_IO
    assert L.vcr_write_png(p, 2, 0, px.ctypes.data) == _abi.ERR_INVALID


def _png_chunks(raw):
    assert raw[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, []
    while pos < len(raw):
        n = struct.unpack(">I", raw[pos:pos + 4])[0]
        kind, data = raw[pos + 4:pos + 8], raw[pos + 8:pos + 8 + n]
        assert struct.unpack(">I", raw[pos + 8 + n:pos + 12 + n])[0] == zlib.crc32(kind + data) & 0xFFFFFFFF
        chunks.append((kind, data))
        pos += 12 + n
    return chunks


@pytest.mark.parametrize("shape", [(1, 1), (7, 5), (255, 64), (64, 256), (200, 130)])
def test_png_writer_stored_blocks(tmp_path, shape):
    """Filtered rows below one 65,535-byte block, exactly one (255 rows of
    257 bytes), just over one and well over one."""
    h, w = shape
    rng = np.random.default_rng(h * 1000 + w)
    img = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    path = tmp_path / "c.png"
    vcr.check(vcr.lib().vcr_write_png(str(path).encode(), w, h, img.ctypes.data))
    chunks = _png_chunks(path.read_bytes())
    assert [k for k, _ in chunks] == [b"IHDR", b"IDAT", b"IEND"]
    assert struct.unpack(">IIBBBBB", chunks[0][1]) == (w, h, 8, 6, 0, 0, 0)
    rows = zlib.decompress(chunks[1][1])  # checks the zlib header and the Adler-32
    back = np.frombuffer(rows, np.uint8).reshape(h, 1 + 4 * w)
    assert (back[:, 0] == 0).all()
    np.testing.assert_array_equal(back[:, 1:].reshape(h, w, 4), img)
    blocks = (h * (1 + 4 * w) + 65534) // 65535
    assert len(chunks[1][1]) == 2 + h * (1 + 4 * w) + 5 * blocks + 4
