"""The benchmarked configurations themselves against the oracle, frame by
frame, through the same calls the benchmark times:
  - the uniform batch of 256x224 RGBA8 frames (seeded benchmark generator),
    x4, subdivision, component labels and the default crossing decision
    (the reference's ordered tests), 16 distinct frames through depix_batch:
    the grid kernels of the headline leg (TMA graph, heuristics with fused
    local labels, label merge and flatten, TMA raster);
  - the full 4096-sprite uneven batch (sides ~ U[8, 64], 30 % transparent
    backgrounds), x4 with labels, through the tuned persistent tile-queue
    path, every sprite;
  - the labels of both, bit-exact in every one of repeated runs (the tile
    unions run concurrently: a race shows in some runs only).
Rasters bit-exact (budget: 1 LSB on 0.1 % of pixels), labels bit-exact."""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import oracle as O
from depix import synth

from test_gpu_parity import assert_raster_close
from test_gpu_queue import _pack

pytestmark = pytest.mark.gpu


def _oracle(img, scale=4):
    h, w = img.shape[:2]
    bgr, ws = synth.rgba_to_bgr(img)
    f = O.frame(bgr, w, h, ws, 1, (48, 7, 6))
    return O.raster(f.pos, f.col, w, h, scale), O.label_cc(f.graph, w, h)


def _check_all(imgs, rasters, labels):
    with ThreadPoolExecutor(max_workers=16) as ex:  # the oracle's C calls release the GIL
        want = list(ex.map(_oracle, imgs))
    for k, (wr, wl) in enumerate(want):
        assert_raster_close(rasters[k], wr)
        assert np.array_equal(labels[k], wl), f"frame {k}: labels differ"


def _run_batch(torch, imgs, scale=4):
    import depix
    buf, in_off, out_off, out_bytes = _pack(imgs, scale)
    d_in = torch.from_numpy(buf).cuda()
    d_out = torch.full((out_bytes,), 7, dtype=torch.uint8, device="cuda")
    npx = sum(i.shape[0] * i.shape[1] for i in imgs)
    d_lab = torch.full((npx,), -5, dtype=torch.int32, device="cuda")
    ctx = depix.Context(max(i.shape[0] * i.shape[1] for i in imgs), len(imgs))
    ws = np.array([i.shape[1] for i in imgs], np.int32)
    hs = np.array([i.shape[0] for i in imgs], np.int32)
    ctx.batch(ws, hs, np.array(in_off, np.uint64), np.array(out_off, np.uint64), d_in, depix.params(scale=scale),
              d_out, d_lab)
    torch.cuda.synchronize()
    assert depix.take_device_faults() == 0
    shape = ctx.launch_shape()
    ctx.close()
    out, lab = d_out.cpu().numpy(), d_lab.cpu().numpy()
    rasters, labels, o = [], [], 0
    for k, img in enumerate(imgs):
        h, w = img.shape[:2]
        rasters.append(out[out_off[k]:out_off[k] + w * h * 4 * scale * scale].reshape(h * scale, w * scale, 4))
        labels.append(lab[o:o + w * h])
        o += w * h
    return rasters, labels, shape


def test_uniform_256x224_batch_with_labels_default_decision(cuda):
    imgs = [np.ascontiguousarray(synth.frame(seed)) for seed in range(16)]
    rasters, labels, _ = _run_batch(cuda, imgs)
    _check_all(imgs, rasters, labels)


def test_4096_sprite_batch_every_sprite(cuda):
    imgs = [np.ascontiguousarray(i) for i in synth.sprites(4096, seed=0)]
    assert len(imgs) == 4096
    rasters, labels, shape = _run_batch(cuda, imgs)
    _check_all(imgs, rasters, labels)


def _labels_only(img):
    h, w = img.shape[:2]
    bgr, ws = synth.rgba_to_bgr(img)
    return O.label_cc(O.frame(bgr, w, h, ws, 1, (48, 7, 6)).graph, w, h)


def test_sprite_batch_labels_every_run(cuda):
    """The component labels of the 4096-sprite batch, bit-exact in every one
    of repeated runs at each queue granularity: the tile unions run
    concurrently, and a union lost to a race shows up only in some runs
    (with path compression inside the concurrent unions, about one run in
    ten of this batch had a wrong label). The rasters of all runs are
    byte-identical (the raster's tile tables are built with atomics too)."""
    import depix
    from test_gpu_queue import _pack
    imgs = [np.ascontiguousarray(i) for i in synth.sprites(4096, seed=0)]
    with ThreadPoolExecutor(max_workers=16) as ex:
        want = np.concatenate(list(ex.map(_labels_only, imgs)))
    buf, in_off, out_off, out_bytes = _pack(imgs, 4)
    d_in = cuda.from_numpy(buf).cuda()
    d_out = cuda.empty((out_bytes,), dtype=cuda.uint8, device="cuda")
    d_lab = cuda.empty((want.size,), dtype=cuda.int32, device="cuda")
    ws = np.array([i.shape[1] for i in imgs], np.int32)
    hs = np.array([i.shape[0] for i in imgs], np.int32)
    io, oo = np.array(in_off, np.uint64), np.array(out_off, np.uint64)
    ctx = depix.Context(max(i.shape[0] * i.shape[1] for i in imgs), len(imgs))
    first = None
    try:
        for gran in (1, 2, 4, 8):
            ctx.set_launch_shape(gran, 32, 32)
            for rep in range(8):
                d_lab.fill_(-5)
                d_out.fill_(rep)
                ctx.batch(ws, hs, io, oo, d_in, depix.params(scale=4), d_out, d_lab)
                cuda.cuda.synchronize()
                got = d_lab.cpu().numpy()
                assert np.array_equal(got, want), f"granularity {gran}, run {rep}: {np.count_nonzero(got != want)} labels differ"
                # the rasters of every run identical too
                if first is None:
                    first = d_out.clone()
                else:
                    assert cuda.equal(d_out, first), f"granularity {gran}, run {rep}: raster differs from the first run"
    finally:
        ctx.close()
    assert depix.take_device_faults() == 0


def test_uniform_batch_labels_every_run(cuda):
    """The same for the uniform 256x224 batch (grid kernels), 16 frames, 10 runs;
    the rasters of all runs byte-identical."""
    import depix
    W, H, N = 256, 224, 16
    frames = [np.ascontiguousarray(synth.frame(seed)) for seed in range(N)]
    with ThreadPoolExecutor(max_workers=16) as ex:
        want = np.concatenate(list(ex.map(_labels_only, frames)))
    d_in = cuda.from_numpy(np.stack(frames).reshape(-1)).cuda()
    d_out = cuda.empty((N * W * H * 64,), dtype=cuda.uint8, device="cuda")
    d_lab = cuda.empty((N * W * H,), dtype=cuda.int32, device="cuda")
    ctx = depix.Context(W * H, N)
    first = None
    try:
        for rep in range(10):
            d_lab.fill_(-5)
            d_out.fill_(rep)
            ctx.batch(np.full(N, W, np.int32), np.full(N, H, np.int32), np.arange(N, dtype=np.uint64) * np.uint64(W * H * 4),
                      np.arange(N, dtype=np.uint64) * np.uint64(W * H * 64), d_in, depix.params(), d_out, d_lab)
            cuda.cuda.synchronize()
            assert np.array_equal(d_lab.cpu().numpy(), want), f"run {rep}: labels differ"
            if first is None:
                first = d_out.clone()
            else:
                assert cuda.equal(d_out, first), f"run {rep}: raster differs from the first run"
    finally:
        ctx.close()
    assert depix.take_device_faults() == 0


@pytest.mark.parametrize("w,h", [(256, 224), (250, 98)])
def test_large_uniform_batch_labels(cuda, w, h):
    """A uniform batch of 144 frames (16 distinct, frame widths a multiple
    of 64 and not): every frame's labels bit-exact against the oracle, the
    same frame in every copy, over two runs."""
    import depix
    N, distinct = 144, 16
    frames = [np.ascontiguousarray(synth.frame(seed, w=w, h=h)) for seed in range(distinct)]
    with ThreadPoolExecutor(max_workers=16) as ex:
        want = list(ex.map(_labels_only, frames))
    batch = np.stack([frames[k % distinct] for k in range(N)])
    d_in = cuda.from_numpy(batch.reshape(-1)).cuda()
    d_out = cuda.empty((N * w * h * 64,), dtype=cuda.uint8, device="cuda")
    d_lab = cuda.empty((N * w * h,), dtype=cuda.int32, device="cuda")
    ctx = depix.Context(w * h, N)
    try:
        for rep in range(2):
            d_lab.fill_(-5)
            ctx.batch(np.full(N, w, np.int32), np.full(N, h, np.int32),
                      np.arange(N, dtype=np.uint64) * np.uint64(w * h * 4),
                      np.arange(N, dtype=np.uint64) * np.uint64(w * h * 64), d_in, depix.params(), d_out, d_lab)
            cuda.cuda.synchronize()
            got = d_lab.cpu().numpy().reshape(N, -1)
            for k in range(N):
                assert np.array_equal(got[k], want[k % distinct]), f"run {rep}, frame {k}: labels differ"
    finally:
        ctx.close()
    assert depix.take_device_faults() == 0
