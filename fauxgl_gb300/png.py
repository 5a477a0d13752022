"""Minimal PNG encoder for NRGBA frames (SavePNG, util.go:56-63).

Writes 8-bit RGBA, non-interlaced, filter type 0 per row, zlib level 6;
the bytes differ from Go's image/png encoder (which picks filters
adaptively) but decode to the same pixels.
"""
import struct
import zlib

import numpy as np


def encode_png(nrgba):
    img = np.ascontiguousarray(np.asarray(nrgba, dtype=np.uint8))
    h, w = img.shape[:2]
    raw = np.zeros((h, 1 + w * 4), dtype=np.uint8)
    raw[:, 1:] = img.reshape(h, w * 4)

    def chunk(tag, data):
        body = tag + data
        return struct.pack(">I", len(data)) + body + struct.pack(">I", zlib.crc32(body) & 0xFFFFFFFF)

    ihdr = struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)
    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", ihdr) + chunk(b"IDAT", zlib.compress(raw.tobytes(), 6))
            + chunk(b"IEND", b""))


def SavePNG(path, nrgba):
    with open(path, "wb") as f:
        f.write(encode_png(nrgba))
