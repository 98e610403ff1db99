"""Display image on the CPU: the oracle's sRGB encode against the transfer
function of IEC 61966-2-1 (the B8G8R8A8_SRGB swapchain the reference blits
into, VulkanSwapchain.cpp:72), its packing, and the PNG writer."""
import struct
import zlib

import numpy as np

import vcr
from oracle import oracle as orc


def _srgb64(v):
    v = np.asarray(v, np.float64)
    return np.where(v <= 0.0031308, 12.92 * v, 1.055 * np.power(v, 1.0 / 2.4) - 0.055)


def test_srgb_encode_follows_the_transfer_function():
    vs = np.concatenate([np.linspace(0.0, 1.0, 20001), np.geomspace(1e-7, 1.0, 2000)]).astype(np.float32)
    ours = np.array([orc.srgb_encode(float(v)) for v in vs], np.float64)
    assert np.abs(ours - _srgb64(vs)).max() < 1e-6
    # 8-bit known answers: black, white, mid grey, 18 % grey, the linear segment's end
    q = lambda v: int(orc.srgb_encode(v) * 255.0 + 0.5)
    assert (q(0.0), q(1.0), q(0.5), q(0.18), q(0.0031308)) == (0, 255, 188, 118, 10)


def test_display_packing_order_clamp_and_exposure():
    s = np.array([[[0.5, 0.18, 0.0], [2.0, -1.0, 1.0]]], np.float64) * 4  # sums over 4 samples
    rgba = orc.display(s, 4)
    np.testing.assert_array_equal(rgba[0, 0], [188, 118, 0, 255])
    np.testing.assert_array_equal(rgba[0, 1], [255, 0, 255, 255])  # clamped to [0, 1]
    bgra = orc.display(s, 4, order=vcr.ORDER_BGRA)
    np.testing.assert_array_equal(bgra[..., [2, 1, 0, 3]], rgba)
    half = orc.display(s, 4, exposure=0.5)
    assert half[0, 0, 0] == int(orc.srgb_encode(0.25) * 255 + 0.5)
    np.testing.assert_array_equal(orc.display(s, 0)[..., :3], 0)  # no samples yet: black


def test_png_writer_round_trip(tmp_path):
    rng = np.random.default_rng(2)
    img = rng.integers(0, 256, (7, 5, 4), dtype=np.uint8)
    path = tmp_path / "a.png"
    vcr.write_png(str(path), img)
    raw = path.read_bytes()
    assert raw[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, {}
    while pos < len(raw):
        n = struct.unpack(">I", raw[pos:pos + 4])[0]
        kind, data = raw[pos + 4:pos + 8], raw[pos + 8:pos + 8 + n]
        assert struct.unpack(">I", raw[pos + 8 + n:pos + 12 + n])[0] == zlib.crc32(kind + data) & 0xFFFFFFFF
        chunks[kind] = data
        pos += 12 + n
    w, h, depth, color = struct.unpack(">IIBB", chunks[b"IHDR"][:10])
    assert (w, h, depth, color) == (5, 7, 8, 6)
    rows = zlib.decompress(chunks[b"IDAT"])
    assert len(rows) == 7 * (1 + 5 * 4)
    back = np.frombuffer(rows, np.uint8).reshape(7, 21)
    assert (back[:, 0] == 0).all()
    np.testing.assert_array_equal(back[:, 1:].reshape(7, 5, 4), img)
