"""The oracle's border walks against a second, independent restatement of
the same rules (written here in Python) on random graphs: symmetric graphs
like the pipeline's resolved graphs, and arbitrary byte graphs. The latter
exercise the cases the reference leaves undefined: nodes without links,
links that point outside the image, asymmetric links and walks that never
close."""
import numpy as np
import pytest

import oracle as O

# clock position c (0..7, clockwise from up-left) -> node bit, and back
REAL = [0, 1, 2, 4, 7, 6, 5, 3]
CLOCK = {r: c for c, r in enumerate(REAL)}
DI = [-1, 0, 1, -1, 1, -1, 0, 1]
DJ = [1, 1, 1, 0, 0, -1, -1, -1]


def _inside(x, y, w, h):
    m = 0xFF
    if x == 0:
        m &= ~0x29
    if x == w - 1:
        m &= ~0x94
    if y == 0:
        m &= ~0xE0
    if y == h - 1:
        m &= ~0x07
    return m


def _walks(g, w, h):
    node = lambda x, y: int(g[y * w + x]) & _inside(x, y, w, h)
    ones = lambda v: bin(v).count("1")

    def turn_cw(v, e):  # the link left by after arriving along e
        back = 7 - e
        if ones(v) == 1:
            return back
        c = CLOCK[back]
        for k in range(c + 1, c + 8):
            if v >> REAL[k % 8] & 1:
                return REAL[k % 8]
        return back

    def turn_ccw(v, e):
        if ones(v) == 1:
            return e
        c = CLOCK[e]
        for k in range(c + 7, c, -1):
            if v >> REAL[k % 8] & 1:
                return REAL[k % 8]
        return e

    listed, discarded, out = set(), set(), []
    limit = 8 * w * h + 8
    for y in range(h):
        for x in range(w):
            p, v0 = y * w + x, node(x, y)
            if v0 == 90 or p in listed:
                continue
            if v0 == 0:
                out.append(([p], [-1]))
                listed.add(p)
                continue
            listed.add(p)
            e = next(REAL[c] for c in range(8) if v0 >> REAL[c] & 1)
            arr = turn_ccw(v0, e)
            nodes, edges, cx, cy, steps, ok = [p], [e], x, y, 0, True
            while not (cx + DI[e] == x and cy + DJ[e] == y and 7 - e == arr):
                cx, cy = cx + DI[e], cy + DJ[e]
                v = node(cx, cy)
                e = turn_cw(v, e)
                steps += 1
                q = cy * w + cx
                if v == 90 or q in listed or q in discarded or steps > limit:
                    discarded.add(nodes[-1])
                    listed.discard(p)
                    ok = False
                    break
                nodes.append(q)
                edges.append(e)
            if ok:
                out.append((nodes, edges))
                listed.update(nodes)
    return out


def _symmetric(rng, w, h, p_edge):
    """A random symmetric graph without crossing diagonals."""
    g = np.zeros((h, w), np.int64)
    for y in range(h):
        for x in range(w):
            for e, (dx, dy) in ((4, (1, 0)), (1, (0, 1))):
                if x + dx < w and y + dy < h and rng.random() < p_edge:
                    g[y, x] |= 1 << e
                    g[y + dy, x + dx] |= 1 << (7 - e)
            if x + 1 < w and y + 1 < h:  # at most one diagonal per 2x2 block
                r = rng.random()
                if r < p_edge / 2:
                    g[y, x] |= 1 << 2
                    g[y + 1, x + 1] |= 1 << 5
                elif r < p_edge:
                    g[y, x + 1] |= 1 << 0
                    g[y + 1, x] |= 1 << 7
    return g.astype(np.uint8).reshape(-1)


@pytest.mark.parametrize("seed", range(40))
def test_random_symmetric_graphs(seed):
    rng = np.random.default_rng(seed)
    w, h = int(rng.integers(1, 24)), int(rng.integers(1, 24))
    g = _symmetric(rng, w, h, float(rng.uniform(0.2, 0.9)))
    assert O.border_walks(g, w, h) == _walks(g, w, h)


@pytest.mark.parametrize("seed", range(40))
def test_random_byte_graphs(seed):
    rng = np.random.default_rng(1000 + seed)
    w, h = int(rng.integers(1, 16)), int(rng.integers(1, 16))
    g = rng.integers(0, 256, w * h).astype(np.uint8)
    g[rng.random(w * h) < 0.2] = 90
    assert O.border_walks(g, w, h) == _walks(g, w, h)
