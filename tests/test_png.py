"""SavePNG (util.go:56-63) on the host: the encoder's bytes decode back to the
frame's NRGBA pixels. The decoder here is written for the test from the PNG
specification (chunk layout, CRC-32, zlib stream, per-row filter type 0)."""
import struct
import zlib

import numpy as np

from fauxgl_gb300.png import SavePNG, encode_png


def decode_png(data):
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, []
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        tag, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert zlib.crc32(tag + body) & 0xFFFFFFFF == crc, tag
        chunks.append((tag, body))
        pos += 12 + n
    assert chunks[0][0] == b"IHDR" and chunks[-1][0] == b"IEND"
    w, h, depth, ctype, comp, filt, inter = struct.unpack(">IIBBBBB", chunks[0][1])
    assert (depth, ctype, comp, filt, inter) == (8, 6, 0, 0, 0)  # 8-bit RGBA, not interlaced
    raw = zlib.decompress(b"".join(b for t, b in chunks if t == b"IDAT"))
    rows = np.frombuffer(raw, dtype=np.uint8).reshape(h, 1 + 4 * w)
    assert (rows[:, 0] == 0).all()  # filter type 0 on every row
    return rows[:, 1:].reshape(h, w, 4)


def test_png_round_trip(tmp_path):
    rng = np.random.default_rng(7)
    for h, w in ((1, 1), (3, 5), (61, 97), (270, 480)):
        img = rng.integers(0, 256, size=(h, w, 4), dtype=np.uint8)
        img[: h // 2, : w // 3, 3] = 0  # transparent pixels keep their colour bytes (NRGBA)
        assert np.array_equal(decode_png(encode_png(img)), img)
        p = tmp_path / ("f%dx%d.png" % (w, h))
        SavePNG(str(p), img)
        assert np.array_equal(decode_png(p.read_bytes()), img)
