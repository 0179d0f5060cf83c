"""The weighted-vote heuristics (depix_params.vote = 1) on the GPU against
the oracle's vote. The vote is not in the reference, so the oracle is the
target: resolved graphs bit-exact through the stage entry point (widths that
take the TMA window and widths that do not), component labels bit-exact and
rasters within the raster budget through the frame path, the uniform batch
and the uneven batch (tile queue), and vote and reference calls interleaved
on one context (each keeps its own captured graph)."""
import numpy as np
import pytest

import oracle as O
from depix import synth

from test_gpu_parity import _upload, assert_raster_close
from test_gpu_queue import _pack

pytestmark = pytest.mark.gpu

# 256 and 64 are multiples of 16 bytes (TMA graph window), the rest are not
SIZES = [(256, 224), (64, 16), (97, 61), (300, 17), (1, 40), (33, 2)]

_CACHE = {}


def _oracle(img, vote, scale=4):
    key = (img.tobytes(), img.shape, vote, scale)
    if key not in _CACHE:
        h, w = img.shape[:2]
        bgr, ws = synth.rgba_to_bgr(img)
        _, triv, res = O.graph(bgr, w, h, ws, vote=vote)
        f = O.frame(bgr, w, h, ws, 1, (48, 7, 6), graph_in=res)
        _CACHE[key] = dict(triv=triv, graph=res, raster=O.raster(f.pos, f.col, w, h, scale),
                           labels=O.label_cc(res, w, h))
    return _CACHE[key]


@pytest.mark.parametrize("w,h", SIZES)
def test_stage_entry_point(cuda, w, h):
    import depix
    torch = cuda
    img = synth.frame(900 + w + h, w=w, h=h)
    o = _oracle(img, True)
    snap = torch.from_numpy(o["triv"].copy()).cuda()
    out = torch.empty_like(snap)
    depix.resolve_heuristics(snap, w, h, out, vote=True)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), o["graph"])
    depix.resolve_heuristics(snap, w, h, out)  # the default stays the reference's decision
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), O.heuristics(o["triv"], w, h))


@pytest.mark.parametrize("w,h", [(256, 224), (97, 61)])
def test_frame_path(cuda, w, h):
    import depix
    torch = cuda
    img = synth.frame(910 + w, w=w, h=h)
    o = _oracle(img, True)
    d_img, ws = _upload(torch, img, depix.LAYOUT_RGBA)
    ctx = depix.Context(w * h, 1)
    out = torch.empty(w * h * 64, dtype=torch.uint8, device="cuda")
    graph = torch.empty(w * h, dtype=torch.uint8, device="cuda")
    labels = torch.empty(w * h, dtype=torch.int32, device="cuda")
    ctx.frame(d_img, w, h, ws, depix.LAYOUT_RGBA, depix.params(vote=True), out, graph, labels)
    torch.cuda.synchronize()
    assert np.array_equal(graph.cpu().numpy(), o["graph"])
    assert np.array_equal(labels.cpu().numpy(), o["labels"])
    assert_raster_close(out.cpu().numpy().reshape(h * 4, w * 4, 4), o["raster"])
    ctx.close()


def _batch(torch, ctx, imgs, vote):
    import depix
    buf, in_off, out_off, out_bytes = _pack(imgs, 4)
    d_in = torch.from_numpy(buf).cuda()
    d_out = torch.zeros(out_bytes, dtype=torch.uint8, device="cuda")
    npx = sum(i.shape[0] * i.shape[1] for i in imgs)
    d_lab = torch.full((npx,), -5, dtype=torch.int32, device="cuda")
    ctx.batch([i.shape[1] for i in imgs], [i.shape[0] for i in imgs], in_off, out_off, d_in,
              depix.params(vote=vote), d_out, d_lab)
    torch.cuda.synchronize()
    out, lab = d_out.cpu().numpy(), d_lab.cpu().numpy()
    px = 0
    for k, img in enumerate(imgs):
        h, w = img.shape[:2]
        o = _oracle(img, vote)
        assert np.array_equal(lab[px:px + w * h], o["labels"]), (vote, k)
        assert_raster_close(out[out_off[k]:out_off[k] + w * h * 64].reshape(h * 4, w * 4, 4), o["raster"])
        px += w * h


def test_uniform_batch(cuda):
    import depix
    imgs = [synth.frame(920 + k) for k in range(4)]
    ctx = depix.Context(256 * 224, len(imgs))
    _batch(cuda, ctx, imgs, True)
    ctx.close()


def test_uneven_batch_interleaved_with_reference_decision(cuda):
    import depix
    imgs = synth.sprites(12, seed=21) + [synth.frame(930 + w, w=w, h=h) for w, h in ((65, 33), (1, 37), (130, 9))]
    ctx = depix.Context(max(i.shape[0] * i.shape[1] for i in imgs), len(imgs))
    for vote in (False, True, False, True):
        _batch(cuda, ctx, imgs, vote)
    ctx.close()


def test_vote_is_rejected_outside_0_1(cuda):
    import depix
    torch = cuda
    img = synth.frame(940, w=16, h=16)
    d_img, ws = _upload(torch, img, depix.LAYOUT_RGBA)
    ctx = depix.Context(256, 1)
    p = depix.params()
    p.vote = 7
    out = torch.empty(16 * 16 * 64, dtype=torch.uint8, device="cuda")
    with pytest.raises(depix.DepixError):
        ctx.frame(d_img, 16, 16, ws, depix.LAYOUT_RGBA, p, out)
    ctx.close()
