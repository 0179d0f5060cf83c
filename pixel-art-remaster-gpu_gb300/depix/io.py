"""Image I/O for real inputs: PNG files and raw frame streams, with the
y-up row order the frame path works in.

The reference loads images with OpenCV as BGR rows with a 4-byte-aligned
stride (Image.cpp:42-48) and turns them upside down before the frame path
(Image::reverses, Image.cpp:21-38). OpenCV is not available here; this module
reads and writes PNG itself (zlib from the standard library) and gives
images as RGBA8 ``(H, W, 4)`` arrays. ``load_frame`` returns them with row 0
at the bottom (the order ``depix_frame`` and the raster use), and
``save_raster`` writes a raster back top-down. ``synth.rgba_to_bgr`` makes the
reference's own BGR layout from such an array.

PNG support: bit depth 8 for every colour type (grey, RGB, palette, grey +
alpha, RGBA), bit depths 1/2/4 for grey and palette, no interlacing; all
five row filters.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

__all__ = ["read_png", "write_png", "load_frame", "save_raster", "read_raw_frames"]

_SIG = b"\x89PNG\r\n\x1a\n"
_CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


def _chunks(data):
    off = len(_SIG)
    while off + 8 <= len(data):
        n, kind = struct.unpack(">I4s", data[off:off + 8])
        body = data[off + 8:off + 8 + n]
        crc, = struct.unpack(">I", data[off + 8 + n:off + 12 + n])
        if zlib.crc32(kind + body) & 0xFFFFFFFF != crc:
            raise ValueError(f"PNG chunk {kind!r}: CRC mismatch")
        yield kind, body
        off += 12 + n


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _unfilter(raw, height, stride, bpp):
    """Undo the per-row filters (PNG spec 9.2) of `height` rows of `stride`
    bytes, `bpp` bytes per complete pixel (at least 1)."""
    out = np.zeros((height, stride), np.uint8)
    prev = np.zeros(stride, np.int64)
    pos = 0
    for y in range(height):
        ftype = raw[pos]
        row = np.frombuffer(raw, np.uint8, stride, pos + 1).astype(np.int64)
        pos += 1 + stride
        if ftype == 0:
            cur = row
        elif ftype == 1:  # Sub: a running sum per byte lane
            cur = row.copy()
            for lane in range(bpp):
                cur[lane::bpp] = np.cumsum(row[lane::bpp]) & 0xFF
        elif ftype == 2:  # Up
            cur = (row + prev) & 0xFF
        elif ftype == 3:  # Average
            cur = row.copy()
            for x in range(stride):
                left = cur[x - bpp] if x >= bpp else 0
                cur[x] = (row[x] + ((left + prev[x]) >> 1)) & 0xFF
        elif ftype == 4:  # Paeth
            cur = row.copy()
            for x in range(stride):
                a = cur[x - bpp] if x >= bpp else 0
                c = prev[x - bpp] if x >= bpp else 0
                cur[x] = (row[x] + _paeth(int(a), int(prev[x]), int(c))) & 0xFF
        else:
            raise ValueError(f"PNG: unknown filter type {ftype}")
        out[y] = cur
        prev = cur
    return out


def read_png(path_or_bytes) -> np.ndarray:
    """A PNG file (path or bytes) as an RGBA8 (H, W, 4) array, top row first."""
    data = path_or_bytes if isinstance(path_or_bytes, (bytes, bytearray)) else open(path_or_bytes, "rb").read()
    if data[:8] != _SIG:
        raise ValueError("not a PNG file")
    idat, palette, trns = [], None, None
    w = h = depth = ctype = None
    for kind, body in _chunks(data):
        if kind == b"IHDR":
            w, h, depth, ctype, comp, filt, interlace = struct.unpack(">IIBBBBB", body)
            if comp != 0 or filt != 0:
                raise ValueError("PNG: unknown compression or filter method")
            if interlace != 0:
                raise ValueError("PNG: interlaced images are not supported")
            if ctype not in _CHANNELS:
                raise ValueError(f"PNG: colour type {ctype}")
            if depth != 8 and not (ctype in (0, 3) and depth in (1, 2, 4)):
                raise ValueError(f"PNG: bit depth {depth} with colour type {ctype} is not supported")
        elif kind == b"PLTE":
            palette = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"tRNS":
            trns = body
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
    if w is None:
        raise ValueError("PNG: no IHDR")
    ch = _CHANNELS[ctype]
    bits_per_px = ch * depth
    stride = (w * bits_per_px + 7) // 8
    raw = zlib.decompress(b"".join(idat))
    if len(raw) < h * (stride + 1):
        raise ValueError("PNG: image data too short")
    rows = _unfilter(raw, h, stride, max(1, bits_per_px // 8))
    if depth < 8:  # unpack 1/2/4-bit samples, most significant first
        per = 8 // depth
        shifts = np.arange(per - 1, -1, -1) * depth
        samples = ((rows[:, :, None] >> shifts) & ((1 << depth) - 1)).reshape(h, -1)[:, :w]
    else:
        samples = rows.reshape(h, w, ch)
    out = np.empty((h, w, 4), np.uint8)
    if ctype == 3:
        if palette is None:
            raise ValueError("PNG: palette image without PLTE")
        idx = samples.reshape(h, w)
        out[..., :3] = palette[idx]
        alpha = np.full(len(palette), 255, np.uint8)
        if trns is not None:
            alpha[:len(trns)] = np.frombuffer(trns, np.uint8)[:len(palette)]
        out[..., 3] = alpha[idx]
    elif ctype == 0:
        g = samples.reshape(h, w)
        if depth < 8:
            g = (g.astype(np.int64) * 255 // ((1 << depth) - 1)).astype(np.uint8)
        out[..., :3] = g[..., None]
        out[..., 3] = 255
        if trns is not None:
            out[..., 3][samples.reshape(h, w) == struct.unpack(">H", trns[:2])[0]] = 0
    elif ctype == 2:
        out[..., :3] = samples
        out[..., 3] = 255
        if trns is not None:
            key = np.array(struct.unpack(">HHH", trns[:6]))
            out[..., 3][np.all(samples == key, axis=-1)] = 0
    elif ctype == 4:
        out[..., :3] = samples[..., :1]
        out[..., 3] = samples[..., 1]
    else:
        out[...] = samples
    return out


def write_png(path, img: np.ndarray, filter_type: int = 0) -> bytes:
    """Write an RGBA8 (H, W, 4) array, top row first, as a PNG (colour type 6)
    with one row filter for every row; returns the file's bytes (path None:
    only returns them)."""
    img = np.ascontiguousarray(img, np.uint8)
    if img.ndim != 3 or img.shape[2] != 4:
        raise ValueError("write_png wants an (H, W, 4) uint8 array")
    h, w = img.shape[:2]
    rows = img.reshape(h, w * 4).astype(np.int64)
    out = bytearray()
    prev = np.zeros(w * 4, np.int64)
    for y in range(h):
        cur = rows[y]
        left = np.concatenate([np.zeros(4, np.int64), cur[:-4]])
        upleft = np.concatenate([np.zeros(4, np.int64), prev[:-4]])
        if filter_type == 0:
            f = cur
        elif filter_type == 1:
            f = cur - left
        elif filter_type == 2:
            f = cur - prev
        elif filter_type == 3:
            f = cur - ((left + prev) >> 1)
        elif filter_type == 4:
            pred = np.array([_paeth(int(a), int(b), int(c)) for a, b, c in zip(left, prev, upleft)], np.int64)
            f = cur - pred
        else:
            raise ValueError("filter_type must be 0..4")
        out.append(filter_type)
        out += (f & 0xFF).astype(np.uint8).tobytes()
        prev = cur

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)

    data = (_SIG + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)) +
            chunk(b"IDAT", zlib.compress(bytes(out), 9)) + chunk(b"IEND", b""))
    if path is not None:
        with open(path, "wb") as fh:
            fh.write(data)
    return data


def load_frame(path) -> np.ndarray:
    """A PNG as the frame path's input: RGBA8 with row 0 at the bottom."""
    return np.ascontiguousarray(read_png(path)[::-1])


def save_raster(path, raster: np.ndarray) -> bytes:
    """Write a raster (row 0 at the bottom, as the raster produces it) as a
    PNG with its top row first."""
    return write_png(path, np.ascontiguousarray(np.asarray(raster)[::-1]))


def read_raw_frames(path, w: int, h: int, layout: str = "rgba", top_down: bool = True, widthstep: int = 0,
                    skip: int = 0):
    """Frames of a headerless stream of w x h images (``rgba``: 4 bytes per
    pixel; ``bgr``: 3), yielded as RGBA8 with row 0 at the bottom (flipped
    when the stream stores the top row first). Rows are ``widthstep`` bytes
    apart (0: packed); the reference's raw video held its image loader's BGR
    rows with their 4-byte-aligned stride and was read from frame 40 on
    (main.cpp:67-75): ``layout="bgr", widthstep=(3 * w + 3) & ~3, skip=40``.
    ``skip`` frames are passed over first."""
    bpp = {"rgba": 4, "bgr": 3}[layout]
    stride = widthstep or w * bpp
    if stride < w * bpp:
        raise ValueError("widthstep smaller than a row")
    size = stride * h
    with open(path, "rb") as fh:
        fh.seek(size * skip)
        while True:
            buf = fh.read(size)
            if len(buf) < size:
                return
            px = np.frombuffer(buf, np.uint8).reshape(h, stride)[:, :w * bpp].reshape(h, w, bpp)
            if layout == "bgr":
                img = np.empty((h, w, 4), np.uint8)
                img[..., 0], img[..., 1], img[..., 2], img[..., 3] = px[..., 2], px[..., 1], px[..., 0], 255
            else:
                img = px.copy()
            yield np.ascontiguousarray(img[::-1]) if top_down else img
