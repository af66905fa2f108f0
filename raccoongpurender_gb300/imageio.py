"""Headless image output: PNG (8-bit RGBA) and PFM (float RGB), for
contest-style runs that write the final image to a file (the reference's
Render app writes a PNG after its time budget, Render/src/ofApp.cpp:123-147)."""
from __future__ import annotations

import struct
import zlib

import numpy as np


def write_png(path: str, rgba8: np.ndarray) -> None:
    """Write an (H, W, 4) uint8 image as a PNG (filter 0, zlib level 6)."""
    img = np.ascontiguousarray(rgba8, dtype=np.uint8)
    if img.ndim != 3 or img.shape[2] != 4:
        raise ValueError("expected an (H, W, 4) uint8 array")
    h, w = img.shape[:2]
    raw = b"".join(b"\x00" + img[y].tobytes() for y in range(h))

    def chunk(tag: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    out = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)) + \
        chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b"")
    with open(path, "wb") as f:
        f.write(out)


def read_png(path: str) -> np.ndarray:
    """Read back a PNG written by write_png (8-bit RGBA, filter 0 only)."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        tag = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        if tag == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
        elif tag == b"IDAT":
            idat += body
        pos += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), dtype=np.uint8).reshape(h, 1 + 4 * w)
    assert (raw[:, 0] == 0).all()
    return raw[:, 1:].reshape(h, w, 4).copy()


def write_pfm(path: str, rgb: np.ndarray) -> None:
    """Write an (H, W, 3) float image as little-endian PFM (bottom row first)."""
    img = np.ascontiguousarray(rgb, dtype="<f4")
    h, w = img.shape[:2]
    with open(path, "wb") as f:
        f.write(f"PF\n{w} {h}\n-1.0\n".encode())
        f.write(img[::-1].tobytes())
