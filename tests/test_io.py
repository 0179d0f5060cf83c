"""PNG and raw-stream I/O (CPU): round trips through every row filter, the
colour types the reader decodes, and the y-up adaptor."""
import struct
import zlib

import numpy as np
import pytest

from depix import io, synth


def _png(w, h, depth, ctype, rows, extra=b""):
    """A PNG from already filtered rows (filter byte + data per row)."""
    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)
    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0)) + extra +
            chunk(b"IDAT", zlib.compress(rows)) + chunk(b"IEND", b""))


@pytest.mark.parametrize("filt", [0, 1, 2, 3, 4])
def test_round_trip_through_every_filter(filt):
    img = synth.sprites(1, seed=filt)[0]
    data = io.write_png(None, img, filter_type=filt)
    assert np.array_equal(io.read_png(data), img)


def test_rgb_grey_and_grey_alpha():
    rng = np.random.default_rng(0)
    rgb = rng.integers(0, 256, (5, 7, 3), dtype=np.uint8)
    got = io.read_png(_png(7, 5, 8, 2, b"".join(b"\x00" + r.tobytes() for r in rgb)))
    assert np.array_equal(got[..., :3], rgb) and (got[..., 3] == 255).all()
    grey = rng.integers(0, 256, (4, 6), dtype=np.uint8)
    got = io.read_png(_png(6, 4, 8, 0, b"".join(b"\x00" + r.tobytes() for r in grey)))
    assert np.array_equal(got[..., 0], grey) and np.array_equal(got[..., 2], grey)
    ga = rng.integers(0, 256, (3, 5, 2), dtype=np.uint8)
    got = io.read_png(_png(5, 3, 8, 4, b"".join(b"\x00" + r.tobytes() for r in ga)))
    assert np.array_equal(got[..., 1], ga[..., 0]) and np.array_equal(got[..., 3], ga[..., 1])


def test_palette_at_two_bits_with_transparency():
    pal = np.array([[10, 20, 30], [200, 0, 0], [0, 200, 0], [1, 2, 3]], np.uint8)
    idx = np.array([[0, 1, 2, 3, 3], [3, 2, 1, 0, 1]], np.uint8)
    packed = []
    for r in idx:
        bits = 0
        for k, v in enumerate(r):
            bits |= int(v) << (2 * (3 - k % 4)) << (8 * (1 - k // 4))
        packed.append(b"\x00" + bits.to_bytes(2, "big"))
    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)
    extra = chunk(b"PLTE", pal.tobytes()) + chunk(b"tRNS", bytes([255, 0]))
    got = io.read_png(_png(5, 2, 2, 3, b"".join(packed), extra))
    assert np.array_equal(got[..., :3], pal[idx])
    assert np.array_equal(got[..., 3], np.where(idx == 1, 0, 255))


def test_corrupt_and_unsupported_files_raise():
    img = synth.frame(0, w=8, h=8)
    data = bytearray(io.write_png(None, img))
    data[40] ^= 0xFF  # inside IHDR or IDAT: CRC mismatch
    with pytest.raises(ValueError):
        io.read_png(bytes(data))
    with pytest.raises(ValueError):
        io.read_png(b"GIF89a")


def test_frame_adaptor_flips_rows(tmp_path):
    img = synth.frame(2, w=16, h=12)  # y-up, as the frame path wants it
    io.save_raster(tmp_path / "r.png", img)
    top_down = io.read_png(tmp_path / "r.png")
    assert np.array_equal(top_down, img[::-1])
    assert np.array_equal(io.load_frame(tmp_path / "r.png"), img)


def test_raw_stream_frames(tmp_path):
    frames = synth.stream(3, seed=1, n_sprites=2, w=20, h=10)
    top_down = frames[:, ::-1]
    (tmp_path / "s.rgba").write_bytes(np.ascontiguousarray(top_down).tobytes())
    got = list(io.read_raw_frames(tmp_path / "s.rgba", 20, 10))
    assert len(got) == 3 and all(np.array_equal(g, f) for g, f in zip(got, frames))
    bgr = np.ascontiguousarray(top_down[..., [2, 1, 0]])
    (tmp_path / "s.bgr").write_bytes(bgr.tobytes())
    got = list(io.read_raw_frames(tmp_path / "s.bgr", 20, 10, layout="bgr"))
    assert all(np.array_equal(g[..., :3], f[..., :3]) for g, f in zip(got, frames))
