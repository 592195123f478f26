"""Frame output: the PNG encoder (stored deflate blocks) read back with
Python's zlib and chunk CRCs checked; rows are written top row first."""
import struct
import zlib

import numpy as np


def read_png(data):
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, []
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        kind = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(kind + body) & 0xFFFFFFFF
        chunks.append((kind, body))
        pos += 12 + n
    assert [k for k, _ in chunks] == [b"IHDR", b"IDAT", b"IEND"]
    W, H, depth, ctype, comp, filt, inter = struct.unpack(">IIBBBBB", chunks[0][1])
    assert (depth, ctype, comp, filt, inter) == (8, 6, 0, 0, 0)
    raw = zlib.decompress(chunks[1][1])
    rows = np.frombuffer(raw, np.uint8).reshape(H, 1 + 4 * W)
    assert (rows[:, 0] == 0).all()
    return rows[:, 1:].reshape(H, W, 4)


def test_png_round_trip(native):
    import livre_gb300 as lv
    rng = np.random.default_rng(3)
    for H, W in [(1, 1), (7, 13), (300, 301)]:  # the last spans several stored blocks
        img = rng.integers(0, 256, (H, W, 4), dtype=np.uint8)
        back = read_png(lv.encode_png(img))
        assert np.array_equal(back, img[::-1])
