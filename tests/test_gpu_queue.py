"""Uneven batches through the persistent tile-queue path (depix_batch with
frames of different sizes, or at uneven strides), called through the C ABI
and compared with the oracle frame by frame: rasters within the raster budget
(they come out bit-exact), component labels bit-exact. Every forced launch
shape (tiles per queue step, raster tile) must give the same bytes as the
tuned one."""
import numpy as np
import pytest

import oracle as O
from depix import synth

from test_gpu_parity import assert_raster_close

pytestmark = pytest.mark.gpu

# sizes that cut tiles at every stage's edges: 1-pixel frames, frames
# narrower than one tile, wider than two graph tiles, taller than a label tile
EDGE = [(1, 1), (1, 37), (53, 1), (130, 9), (3, 70), (65, 33), (33, 65), (16, 16), (17, 31)]


def _images(count=24, seed=11):
    imgs = synth.sprites(count, seed=seed)
    imgs += [synth.frame(300 + w * 5 + h, w=w, h=h) for w, h in EDGE]
    return imgs


_ORACLE = {}


def _oracle(img, scale):
    key = (img.tobytes(), img.shape, scale)
    if key not in _ORACLE:
        h, w = img.shape[:2]
        bgr, ws = synth.rgba_to_bgr(img)
        f = O.frame(bgr, w, h, ws, 1, (48, 7, 6))
        _ORACLE[key] = (O.raster(f.pos, f.col, w, h, scale), O.label_cc(f.graph, w, h))
    return _ORACLE[key]


def _pack(imgs, scale, gap=0):
    """Input and output offsets (16-byte aligned, `gap` extra bytes between
    frames) and the packed input buffer."""
    in_off, out_off, oi, oo = [], [], 0, 0
    for img in imgs:
        h, w = img.shape[:2]
        in_off.append(oi)
        out_off.append(oo)
        oi += (w * h * 4 + 15) // 16 * 16 + gap
        oo += (w * h * 4 * scale * scale + 15) // 16 * 16 + gap
    buf = np.zeros(oi, np.uint8)
    for k, img in enumerate(imgs):
        a = np.ascontiguousarray(img).reshape(-1)
        buf[in_off[k]:in_off[k] + a.size] = a
    return buf, in_off, out_off, oo


def _run(torch, ctx, imgs, scale, labels=True, gap=0, stream=None):
    import depix
    buf, in_off, out_off, out_bytes = _pack(imgs, scale, gap)
    d_in = torch.from_numpy(buf).cuda()
    d_out = torch.full((out_bytes,), 7, dtype=torch.uint8, device="cuda")
    npx = sum(i.shape[0] * i.shape[1] for i in imgs)
    d_lab = torch.full((npx,), -5, dtype=torch.int32, device="cuda") if labels else None
    ctx.batch([i.shape[1] for i in imgs], [i.shape[0] for i in imgs], in_off, out_off, d_in,
              depix.params(scale=scale), d_out, d_lab, stream=stream)
    torch.cuda.synchronize()
    out = d_out.cpu().numpy()
    rasters = []
    for k, img in enumerate(imgs):
        h, w = img.shape[:2]
        rasters.append(out[out_off[k]:out_off[k] + w * h * 4 * scale * scale].reshape(h * scale, w * scale, 4))
    labs = []
    if labels:
        lab = d_lab.cpu().numpy()
        o = 0
        for img in imgs:
            n = img.shape[0] * img.shape[1]
            labs.append(lab[o:o + n])
            o += n
    return rasters, labs


def _check(imgs, scale, rasters, labs):
    for k, img in enumerate(imgs):
        r, lab = _oracle(img, scale)
        assert_raster_close(rasters[k], r)
        if labs:
            assert np.array_equal(labs[k], lab), f"labels of frame {k} {img.shape}"


@pytest.mark.parametrize("scale", [4, 8, 3])
def test_uneven_batch_tuned_matches_oracle(cuda, scale):
    import depix
    torch = cuda
    imgs = _images()
    ctx = depix.Context(max(i.shape[0] * i.shape[1] for i in imgs), len(imgs))
    rasters, labs = _run(torch, ctx, imgs, scale)
    gran, tw, th = ctx.launch_shape()
    assert all(g in (1, 2, 4, 8) for g in gran) and (tw, th) in ((32, 32), (32, 16), (16, 16), (0, 0))
    _check(imgs, scale, rasters, labs)
    ctx.close()


@pytest.mark.parametrize("tile", [(32, 32), (32, 16), (16, 16), (0, 0)])
@pytest.mark.parametrize("gran", [1, 8])
def test_every_forced_shape_gives_the_same_bytes(cuda, tile, gran):
    import depix
    torch = cuda
    imgs = _images(12, seed=12)
    ctx = depix.Context(max(i.shape[0] * i.shape[1] for i in imgs), len(imgs))
    ctx.set_launch_shape(gran, *tile)
    rasters, labs = _run(torch, ctx, imgs, 4)
    assert ctx.launch_shape() == ((gran,) * 4, tile[0], tile[1])
    _check(imgs, 4, rasters, labs)
    ctx.close()


def test_graph_replays_follow_new_descriptors(cuda):
    """One context, three batches of different compositions in a row (the
    second replays the first's graph with new descriptors), then the first
    again; a batch without labels in between."""
    import depix
    torch = cuda
    a = _images(10, seed=21)
    b = _images(6, seed=22)[::-1]
    ctx = depix.Context(max(i.shape[0] * i.shape[1] for i in a + b), len(a) + len(b))
    ra, la = _run(torch, ctx, a, 4)
    rb, lb = _run(torch, ctx, b, 4)
    rn, _ = _run(torch, ctx, a + b, 4, labels=False)
    ra2, la2 = _run(torch, ctx, a, 4)
    _check(a, 4, ra, la)
    _check(b, 4, rb, lb)
    _check(a + b, 4, rn, [])
    for x, y in zip(ra, ra2):
        assert np.array_equal(x, y)
    for x, y in zip(la, la2):
        assert np.array_equal(x, y)
    ctx.close()


def test_equal_sizes_at_uneven_strides_match_the_grid_path(cuda):
    """Frames of one size at a constant stride take the grid path; with a gap
    that varies between frames they take the queue path. Same bytes."""
    import depix
    torch = cuda
    imgs = [synth.frame(60 + k, w=72, h=56) for k in range(9)]
    ctx = depix.Context(72 * 56, len(imgs))
    grid_r, grid_l = _run(torch, ctx, imgs, 4)
    # uneven strides: the packing below adds 16 bytes after every other frame
    buf, in_off, out_off, out_bytes = _pack(imgs, 4)
    in_off = [o + 16 * (k // 2) for k, o in enumerate(in_off)]
    out_off = [o + 16 * (k // 2) for k, o in enumerate(out_off)]
    buf2 = np.zeros(in_off[-1] + 72 * 56 * 4, np.uint8)
    for k, img in enumerate(imgs):
        buf2[in_off[k]:in_off[k] + 72 * 56 * 4] = np.ascontiguousarray(img).reshape(-1)
    d_out = torch.zeros(out_off[-1] + 72 * 56 * 64, dtype=torch.uint8, device="cuda")
    d_lab = torch.zeros(72 * 56 * len(imgs), dtype=torch.int32, device="cuda")
    ctx.batch([72] * 9, [56] * 9, in_off, out_off, torch.from_numpy(buf2).cuda(), depix.params(), d_out, d_lab)
    torch.cuda.synchronize()
    out = d_out.cpu().numpy()
    lab = d_lab.cpu().numpy()
    for k in range(9):
        q = out[out_off[k]:out_off[k] + 72 * 56 * 64].reshape(56 * 4, 72 * 4, 4)
        assert np.array_equal(q, grid_r[k])
        assert np.array_equal(lab[k * 72 * 56:(k + 1) * 72 * 56], grid_l[k])
    ctx.close()


def test_uneven_batch_from_host_buffers(cuda):
    import depix
    torch = cuda
    imgs = _images(8, seed=31)
    buf, in_off, out_off, out_bytes = _pack(imgs, 4)
    h_out = np.zeros(out_bytes, np.uint8)
    npx = sum(i.shape[0] * i.shape[1] for i in imgs)
    h_lab = np.zeros(npx, np.int32)
    ctx = depix.Context(max(i.shape[0] * i.shape[1] for i in imgs), len(imgs))
    ctx.batch_host([i.shape[1] for i in imgs], [i.shape[0] for i in imgs], in_off, out_off, buf, buf.size,
                   depix.params(), h_out, out_bytes, h_lab)
    o = 0
    for k, img in enumerate(imgs):
        h, w = img.shape[:2]
        r, lab = _oracle(img, 4)
        assert_raster_close(h_out[out_off[k]:out_off[k] + w * h * 64].reshape(h * 4, w * 4, 4), r)
        assert np.array_equal(h_lab[o:o + w * h], lab)
        o += w * h
    ctx.close()


def test_uneven_batch_inside_a_stream_capture(cuda):
    """While the caller's stream captures, the batch takes one launch per
    stage and frame (nothing on the host may change under a captured copy);
    the replayed graph gives the oracle's bytes."""
    import depix
    torch = cuda
    imgs = _images(5, seed=41)
    buf, in_off, out_off, out_bytes = _pack(imgs, 4)
    d_in = torch.from_numpy(buf).cuda()
    d_out = torch.zeros(out_bytes, dtype=torch.uint8, device="cuda")
    ctx = depix.Context(max(i.shape[0] * i.shape[1] for i in imgs), len(imgs))
    ws, hs = [i.shape[1] for i in imgs], [i.shape[0] for i in imgs]
    ctx.batch(ws, hs, in_off, out_off, d_in, depix.params(), d_out)  # tables built before the capture
    torch.cuda.synchronize()
    d_out.zero_()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            ctx.batch(ws, hs, in_off, out_off, d_in, depix.params(), d_out, stream=s)
    torch.cuda.synchronize()
    assert int(d_out.sum().item()) == 0  # capture records, it does not run
    g.replay()
    torch.cuda.synchronize()
    out = d_out.cpu().numpy()
    for k, img in enumerate(imgs):
        h, w = img.shape[:2]
        assert_raster_close(out[out_off[k]:out_off[k] + w * h * 64].reshape(h * 4, w * 4, 4), _oracle(img, 4)[0])
    ctx.close()


def test_scale_beyond_the_mask_raster_uses_per_frame_launches(cuda):
    import depix
    torch = cuda
    imgs = _images(3, seed=51)[:2] + [synth.frame(9, w=20, h=13)]
    ctx = depix.Context(max(i.shape[0] * i.shape[1] for i in imgs), len(imgs))
    rasters, labs = _run(torch, ctx, imgs, 13)
    _check(imgs, 13, rasters, labs)
    ctx.close()


@pytest.mark.parametrize("kind", ["uniform", "uneven"])
def test_host_batch_in_chunks_equals_the_device_batch(cuda, kind):
    """Batches of 32 or more frames in order go through depix_batch_host in
    chunks whose copy-back overlaps the next chunk's kernels: same bytes as
    the device-buffer call, labels included."""
    import depix
    torch = cuda
    if kind == "uniform":
        imgs = [synth.frame(90 + k, w=40, h=24) for k in range(48)]
    else:
        imgs = synth.sprites(40, seed=77)
    buf, in_off, out_off, out_bytes = _pack(imgs, 4)
    ws, hs = [i.shape[1] for i in imgs], [i.shape[0] for i in imgs]
    npx = sum(w * h for w, h in zip(ws, hs))
    ctx = depix.Context(max(w * h for w, h in zip(ws, hs)), len(imgs))
    d_out = torch.zeros(out_bytes, dtype=torch.uint8, device="cuda")
    d_lab = torch.zeros(npx, dtype=torch.int32, device="cuda")
    ctx.batch(ws, hs, in_off, out_off, torch.from_numpy(buf).cuda(), depix.params(), d_out, d_lab)
    h_out = torch.zeros(out_bytes, dtype=torch.uint8).pin_memory()
    h_lab = torch.zeros(npx, dtype=torch.int32).pin_memory()
    h_in = torch.from_numpy(buf).pin_memory()
    ctx.batch_host(ws, hs, in_off, out_off, h_in, buf.size, depix.params(), h_out, out_bytes, h_lab)
    torch.cuda.synchronize()
    assert torch.equal(h_out, d_out.cpu())
    assert torch.equal(h_lab, d_lab.cpu())
    ctx.close()


def test_stream_front_end(cuda):
    """depix.stream.upscale_stream with its own context: uneven frames in
    batches of 4 through depix_batch_host, rasters and labels in order."""
    import depix
    from depix import stream
    imgs = synth.sprites(9, seed=41)
    out = list(stream.upscale_stream(imgs, depix.params(), batch=4, labels=True))
    assert len(out) == len(imgs)
    for img, (raster, lab) in zip(imgs, out):
        r, l = _oracle(img, 4)
        assert_raster_close(raster, r)
        assert np.array_equal(lab, l)
