"""The stream front end's batching on CPU: a stand-in context runs each
batch call through the oracle, so frame order, offsets, labels and the
short last batch are checked without a GPU; and a raw stream file in the
reference's BGR layout read back through the front end."""
import numpy as np
import pytest

import oracle as O
from depix import io, stream, synth


class OracleContext:
    """batch_host through the oracle (the CUDA library's contract)."""

    def __init__(self):
        self.calls = []

    def batch_host(self, ws, hs, in_off, out_off, h_img, in_bytes, p, h_out, out_bytes, h_labels=None):
        s = p.scale
        assert all(int(o) % 16 == 0 for o in in_off) and all(int(o) % 16 == 0 for o in out_off)
        self.calls.append(len(ws))
        px = 0
        for k, (w, h) in enumerate(zip(ws.tolist(), hs.tolist())):
            img = h_img[int(in_off[k]):int(in_off[k]) + w * h * 4].reshape(h, w, 4)
            bgr, wstep = synth.rgba_to_bgr(img)
            f = O.frame(bgr, w, h, wstep, p.subdivide, (p.tr_y, p.tr_u, p.tr_v), yuv=p.yuv)
            r = O.raster(f.pos, f.col, w, h, s).reshape(-1)
            assert int(out_off[k]) + r.size <= out_bytes
            h_out[int(out_off[k]):int(out_off[k]) + r.size] = r
            if h_labels is not None:
                h_labels[px:px + w * h] = O.label_cc(f.graph, w, h)
            px += w * h


class Params:
    tr_y, tr_u, tr_v, subdivide, scale, yuv = 48, 7, 6, 1, 2, 0


def _expected(img, s):
    h, w = img.shape[:2]
    bgr, ws = synth.rgba_to_bgr(img)
    f = O.frame(bgr, w, h, ws, 1, (48, 7, 6))
    return O.raster(f.pos, f.col, w, h, s), O.label_cc(f.graph, w, h)


def test_frames_come_back_in_order_with_labels():
    imgs = synth.sprites(7, seed=5)  # uneven sizes
    ctx = OracleContext()
    out = list(stream.upscale_stream(imgs, Params(), batch=3, labels=True, ctx=ctx))
    assert ctx.calls == [3, 3, 1]
    assert len(out) == len(imgs)
    for img, (raster, lab) in zip(imgs, out):
        r, l = _expected(img, 2)
        assert np.array_equal(raster, r) and np.array_equal(lab, l)


def test_pack_batch_layout():
    imgs = [np.zeros((3, 5, 4), np.uint8), np.ones((2, 7, 4), np.uint8)]
    ws, hs, in_off, out_off, buf, out_bytes, npx = stream.pack_batch(imgs, 3)
    assert ws.tolist() == [5, 7] and hs.tolist() == [3, 2]
    assert in_off.tolist() == [0, 64] and out_off.tolist() == [0, 544]
    assert out_bytes == 544 + 512 and npx == 29
    assert (buf[64:64 + 56] == 1).all()
    with pytest.raises(ValueError):
        stream.pack_batch([np.zeros((3, 5, 3), np.uint8)], 2)


def test_raw_reference_stream_through_the_front_end(tmp_path):
    """BGR rows with the 4-byte-aligned stride, top row first, read from a
    given frame on, as the reference's raw video was."""
    frames = synth.stream(5, seed=2, n_sprites=3, w=21, h=13)
    wstep = (3 * 21 + 3) & ~3
    raw = bytearray()
    for f in frames:
        top = f[::-1]
        rows = np.zeros((13, wstep), np.uint8)
        rows[:, :63] = top[..., [2, 1, 0]].reshape(13, 63)
        raw += rows.tobytes()
    (tmp_path / "v.bin").write_bytes(bytes(raw))
    got = list(io.read_raw_frames(tmp_path / "v.bin", 21, 13, layout="bgr", widthstep=wstep, skip=2))
    assert len(got) == 3
    assert all(np.array_equal(g[..., :3], f[..., :3]) for g, f in zip(got, frames[2:]))
    out = list(stream.upscale_stream(got, Params(), batch=2, ctx=OracleContext()))
    assert all(np.array_equal(o, _expected(f, 2)[0]) for o, f in zip(out, got))
