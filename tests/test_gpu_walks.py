"""Border walks on the GPU (depix_border_walks through the C ABI) against
the walks the reference recorded for its 24x24 image and against the oracle
on seeded frames, one frame per call and in batches; node lists and chain
codes bit-exact, capacities reported."""
import json
import os

import numpy as np
import pytest

import oracle as O
from depix import synth

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _graph(img):
    h, w = img.shape[:2]
    bgr, ws = synth.rgba_to_bgr(img)
    return O.graph(bgr, w, h, ws)[2]


def test_recorded_walks(cuda):
    import depix
    z = np.load(os.path.join(GOLDEN, "dumps.npz"))
    b = json.load(open(os.path.join(GOLDEN, "borders.json")))
    g = cuda.from_numpy(z["alex/graph"].copy()).cuda()
    (walks, trunc), = depix.border_walk_lists(g, 24, 24)
    assert not trunc and len(walks) == 21
    assert all(nodes == b["walks"][str(k)] for k, (nodes, _) in enumerate(walks))
    n = len(b["chain_from_5"]["edges"])
    assert walks[1][1][:n] == b["chain_from_5"]["edges"]


SIZES = [(256, 224), (97, 61), (1, 1), (1, 9), (13, 1), (64, 16)]


@pytest.mark.parametrize("w,h", SIZES)
def test_single_frames_equal_oracle(cuda, w, h):
    import depix
    img = synth.frame(700 + w + h, w=w, h=h)
    g = _graph(img)
    (walks, trunc), = depix.border_walk_lists(cuda.from_numpy(g.copy()).cuda(), w, h)
    assert not trunc
    assert walks == [(list(a), list(b)) for a, b in O.border_walks(g, w, h)]


def test_batch_equals_oracle(cuda):
    import depix
    frames = [synth.frame(710 + k, w=80, h=48) for k in range(9)]
    gs = [_graph(f) for f in frames]
    d = cuda.from_numpy(np.concatenate(gs)).cuda()
    res = depix.border_walk_lists(d, 80, 48, nframes=len(gs))
    for g, (walks, trunc) in zip(gs, res):
        assert not trunc
        assert walks == [(list(a), list(b)) for a, b in O.border_walks(g, 80, 48)]


def test_walks_of_the_frame_path_graph(cuda):
    """The graph the frame path writes, walked on the device."""
    import depix
    torch = cuda
    img = synth.frame(720)
    h, w = img.shape[:2]
    d_img = torch.from_numpy(np.ascontiguousarray(img).reshape(-1)).cuda()
    ctx = depix.Context(w * h, 1)
    out = torch.empty(w * h * 64, dtype=torch.uint8, device="cuda")
    graph = torch.empty(w * h, dtype=torch.uint8, device="cuda")
    ctx.frame(d_img, w, h, 4 * w, depix.LAYOUT_RGBA, depix.params(), out, graph)
    (walks, trunc), = depix.border_walk_lists(graph, w, h)
    ctx.close()
    assert not trunc
    assert walks == [(list(a), list(b)) for a, b in O.border_walks(graph.cpu().numpy(), w, h)]


def test_capacities(cuda):
    import depix
    g = _graph(synth.frame(730, w=64, h=40))
    d = cuda.from_numpy(g.copy()).cuda()
    full = O.border_walks(g, 64, 40)
    for max_nodes, max_walks in ((50, 10 ** 6), (10 ** 5, 7)):
        (walks, trunc), = depix.border_walk_lists(d, 64, 40, max_nodes=max_nodes, max_walks=max_walks)
        assert trunc and len(walks) < len(full)
        assert walks == [(list(a), list(b)) for a, b in full[:len(walks)]]
        assert sum(len(n) for n, _ in walks) <= max_nodes and len(walks) <= max_walks


@pytest.mark.parametrize("kind", ["symmetric", "bytes"])
def test_random_graphs_equal_oracle(cuda, kind):
    """Random graphs in one batch: symmetric ones like the pipeline's, and
    arbitrary bytes (links outside the image, asymmetric links, walks that
    never close)."""
    import depix
    from test_walks_random import _symmetric
    rng = np.random.default_rng(7 if kind == "symmetric" else 8)
    w, h, n = 23, 17, 6
    gs = [(_symmetric(rng, w, h, 0.6) if kind == "symmetric" else rng.integers(0, 256, w * h).astype(np.uint8))
          for _ in range(n)]
    d = cuda.from_numpy(np.concatenate(gs)).cuda()
    res = depix.border_walk_lists(d, w, h, nframes=n, max_nodes=8 * w * h + 8, max_walks=w * h)
    for g, (walks, trunc) in zip(gs, res):
        assert not trunc
        assert walks == [(list(a), list(b)) for a, b in O.border_walks(g, w, h)]
