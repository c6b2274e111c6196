"""Image output (sr_write_image): PNG, PPM and PAM files read back to the
same pixels.  Host code only."""
import struct
import zlib

import numpy as np
import pytest


def _read_png(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, []
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        crc = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        assert crc == zlib.crc32(typ + body) & 0xFFFFFFFF
        chunks.append((typ, body))
        pos += 12 + n
    assert [c[0] for c in chunks] == [b"IHDR", b"IDAT", b"IEND"]
    w, h, depth, ctype = struct.unpack(">IIBB", chunks[0][1][:10])
    assert (depth, ctype) == (8, 6)
    raw = zlib.decompress(chunks[1][1])
    rows = np.frombuffer(raw, np.uint8).reshape(h, 1 + 4 * w)
    assert np.all(rows[:, 0] == 0)
    return rows[:, 1:].reshape(h, w, 4)


@pytest.mark.parametrize("shape", [(1, 1), (23, 37), (300, 250)])
def test_png_round_trip(srlib, tmp_path, shape):
    rng = np.random.default_rng(shape[0])
    img = rng.integers(0, 256, size=shape + (4,), dtype=np.uint8)
    p = tmp_path / "f.png"
    srlib.write_image(p, img)
    assert np.array_equal(_read_png(p), img)


def test_ppm_and_pam_round_trip(srlib, tmp_path):
    img = np.random.default_rng(3).integers(0, 256, size=(17, 29, 4), dtype=np.uint8)
    srlib.write_image(tmp_path / "f.ppm", img)
    data = open(tmp_path / "f.ppm", "rb").read()
    head = b"P6\n29 17\n255\n"
    assert data.startswith(head)
    assert np.array_equal(np.frombuffer(data[len(head):], np.uint8).reshape(17, 29, 3), img[:, :, :3])
    srlib.write_image(tmp_path / "f.pam", img)
    data = open(tmp_path / "f.pam", "rb").read()
    end = data.index(b"ENDHDR\n") + 7
    assert b"TUPLTYPE RGB_ALPHA" in data[:end]
    assert np.array_equal(np.frombuffer(data[end:], np.uint8).reshape(17, 29, 4), img)


def test_bad_arguments_are_rejected(srlib, tmp_path):
    L = srlib.lib()
    img = np.zeros((2, 2, 4), np.uint8)
    assert L.sr_write_image(str(tmp_path / "x.png").encode(), img.ctypes.data, 0, 2, 0) == 1
    assert L.sr_write_image(str(tmp_path / "x.png").encode(), img.ctypes.data, 2, 2, 9) == 1
    assert L.sr_write_image(str(tmp_path / "nodir" / "x.png").encode(), img.ctypes.data, 2, 2, 0) == 1
    assert b"cannot open" in L.sr_last_error()
