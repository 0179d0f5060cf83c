"""Frame streams through the batched path.

The reference's application kept a commented-out raw-video reader
(main.cpp:67-75). It read a file of back-to-back frames in its image
loader's layout, meant to be drawn one by one. ``upscale_stream`` takes such
a stream (``io.read_raw_frames`` reads the files) or any iterable of RGBA8
frames, row 0 at the bottom and of any sizes. It runs the frames through
``depix_batch_host`` ``batch`` at a time: one call per batch, host buffers
in and out. Rasters come back in frame order.
"""
from __future__ import annotations

import itertools

import numpy as np

__all__ = ["upscale_stream", "pack_batch"]


def _align16(n: int) -> int:
    return (n + 15) // 16 * 16


def pack_batch(frames, scale: int):
    """Host layout of one batch: the frames' widths and heights, 16-byte
    aligned input and output offsets, the packed input bytes, the output
    size and the label count."""
    ws = np.array([f.shape[1] for f in frames], np.int32)
    hs = np.array([f.shape[0] for f in frames], np.int32)
    in_off = np.zeros(len(frames), np.uint64)
    out_off = np.zeros(len(frames), np.uint64)
    oi = oo = 0
    for k, (w, h) in enumerate(zip(ws.tolist(), hs.tolist())):
        in_off[k], out_off[k] = oi, oo
        oi += _align16(w * h * 4)
        oo += _align16(w * h * 4 * scale * scale)
    buf = np.zeros(oi, np.uint8)
    for k, f in enumerate(frames):
        a = np.ascontiguousarray(f, np.uint8).reshape(-1)
        if a.size != int(ws[k]) * int(hs[k]) * 4:
            raise ValueError("frames must be RGBA8 (H, W, 4) arrays")
        buf[int(in_off[k]):int(in_off[k]) + a.size] = a
    return ws, hs, in_off, out_off, buf, oo, int((ws.astype(np.int64) * hs).sum())


def upscale_stream(frames, params, batch: int = 8, labels: bool = False, ctx=None):
    """Yield every frame's raster ((H*s, W*s, 4) uint8, row 0 at the bottom),
    or (raster, labels) with labels=True, in order. The frames go through
    the batched path `batch` at a time; the last batch may be shorter. With
    ctx None a context is made (and grown for larger frames) and closed at
    the end; a given context must hold the batch's largest frame."""
    from . import Context
    if batch < 1:
        raise ValueError("batch must be >= 1")
    s = int(params.scale)
    it = iter(frames)
    owned = ctx is None
    cap = 0
    try:
        while True:
            chunk = list(itertools.islice(it, batch))
            if not chunk:
                return
            ws, hs, in_off, out_off, buf, out_bytes, npx = pack_batch(chunk, s)
            need = int((ws.astype(np.int64) * hs).max())
            if owned and need > cap:
                if ctx is not None:
                    ctx.close()
                cap = max(need, 2 * cap)
                ctx = Context(cap, batch)
            h_out = np.empty(max(out_bytes, 16), np.uint8)
            h_lab = np.empty(max(npx, 1), np.int32) if labels else None
            ctx.batch_host(ws, hs, in_off, out_off, buf, buf.size, params, h_out, h_out.size, h_lab)
            px = 0
            for k in range(len(chunk)):
                w, h = int(ws[k]), int(hs[k])
                o = int(out_off[k])
                raster = h_out[o:o + w * h * 4 * s * s].reshape(h * s, w * s, 4).copy()
                if labels:
                    yield raster, h_lab[px:px + w * h].copy()
                else:
                    yield raster
                px += w * h
    finally:
        if owned and ctx is not None:
            ctx.close()
