"""The present step without a canvas: rgba8 frames written as PPM (C ABI) and PNG (Python), read back
byte for byte. Host only."""
import struct
import zlib

import numpy as np
import pytest

import webgs


def _frame(h=37, w=53):
    rng = np.random.default_rng(3)
    img = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    img[..., 3] = 255
    return img


def test_ppm_round_trip(tmp_path):
    img = _frame()
    p = tmp_path / "frame.ppm"
    webgs.save_ppm(p, img)
    data = p.read_bytes()
    header = b"P6\n53 37\n255\n"
    assert data.startswith(header)
    body = np.frombuffer(data[len(header):], np.uint8).reshape(37, 53, 3)
    np.testing.assert_array_equal(body, img[..., :3])


def test_ppm_rejects_bad_arguments(tmp_path):
    with pytest.raises(ValueError):
        webgs.save_ppm(tmp_path / "x.ppm", np.zeros((4, 4, 3), np.uint8))
    with pytest.raises(webgs.GsError):
        webgs.save_ppm(tmp_path / "missing_dir" / "x.ppm", _frame())


def test_png_round_trip(tmp_path):
    img = _frame()
    p = tmp_path / "frame.png"
    webgs.save_png(p, img)
    data = p.read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, {}
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        tag, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        (crc,) = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(tag + body) & 0xFFFFFFFF
        chunks[tag] = body
        pos += 12 + n
    w, h, depth, ctype = struct.unpack(">IIBB", chunks[b"IHDR"][:10])
    assert (w, h, depth, ctype) == (53, 37, 8, 6)
    raw = np.frombuffer(zlib.decompress(chunks[b"IDAT"]), np.uint8).reshape(37, 1 + 53 * 4)
    assert not raw[:, 0].any()
    np.testing.assert_array_equal(raw[:, 1:].reshape(37, 53, 4), img)
