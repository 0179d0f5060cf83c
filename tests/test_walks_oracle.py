"""Border walks of the oracle (CPU) against what the reference recorded for
its 24x24 image (alex_png.txt: 21 walks and the chain code of the walk from
node 5), and the properties every walk keeps on seeded frames."""
import json
import os

import numpy as np

import oracle as O
from depix import synth

from conftest import GOLDEN

DI = [-1, 0, 1, -1, 1, -1, 0, 1]
DJ = [1, 1, 1, 0, 0, -1, -1, -1]


def _alex():
    z = np.load(os.path.join(GOLDEN, "dumps.npz"))
    return z["alex/graph"], json.load(open(os.path.join(GOLDEN, "borders.json")))


def test_walks_equal_the_recorded_walks():
    g, b = _alex()
    walks = O.border_walks(g, 24, 24)
    assert len(walks) == len(b["walks"]) == 21
    for k, (nodes, _) in enumerate(walks):
        assert nodes == b["walks"][str(k)], k
    chain = b["chain_from_5"]
    nodes, edges = walks[1]
    n = len(chain["nodes"])
    assert nodes[:n] == chain["nodes"] and edges[:n] == chain["edges"]


def test_format_matches_the_recorded_lines():
    import depix
    g, b = _alex()
    text = depix.format_walks(O.border_walks(g, 24, 24))
    lines = text.splitlines(keepends=True)
    assert len(lines) == 21
    assert lines[3] == "Spline: 3 -  30,  55,  56,  57,  33,  32,  31, \n"
    assert lines[19] == "Spline: 19 -  370,  394, \n"


def _check_walks(g, w, h, walks):
    g = g.reshape(-1)
    lab = O.label_cc(g, w, h)
    starts = [nodes[0] for nodes, _ in walks]
    assert starts == sorted(starts)
    seen = set()
    for nodes, edges in walks:
        assert len(nodes) == len(edges)
        if edges == [-1]:  # a node without links
            assert g[nodes[0]] == 0
            continue
        assert len({int(lab[v]) for v in nodes}) == 1
        for i, (v, e) in enumerate(zip(nodes, edges)):
            assert g[v] != 90 and (g[v] >> e) & 1
            x, y = v % w + DI[e], v // w + DJ[e]
            assert 0 <= x < w and 0 <= y < h
            nxt = nodes[(i + 1) % len(nodes)]
            assert y * w + x == nxt  # the last link closes on the start
        assert not seen & set(nodes)  # no node in two recorded walks
        seen |= set(nodes)


def test_walk_properties_on_frames():
    imgs = [synth.frame(s, w=w, h=h) for s, (w, h) in enumerate([(96, 80), (37, 21), (1, 9), (13, 1), (1, 1)])]
    imgs += synth.sprites(6, seed=4)
    for img in imgs:
        h, w = img.shape[:2]
        bgr, ws = synth.rgba_to_bgr(img)
        _, _, g = O.graph(bgr, w, h, ws)
        walks = O.border_walks(g, w, h)
        assert walks is not None
        _check_walks(g, w, h, walks)


def test_capacity_is_reported():
    g, _ = _alex()
    assert O.border_walks(g, 24, 24, max_nodes=100) is None
    assert O.border_walks(g, 24, 24, max_walks=5) is None
    assert len(O.border_walks(g, 24, 24, max_walks=21)) == 21
