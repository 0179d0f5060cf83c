"""The oracle's weighted-vote heuristics against a second, independent
restatement (written here in Python) on random few-colour images, which
leave many crossings for the vote to decide."""
import numpy as np
import pytest

import oracle as O
from depix import synth

DI = [-1, 0, 1, -1, 1, -1, 0, 1]
DJ = [1, 1, 1, 0, 0, -1, -1, -1]


def _others(v, e):
    """links of v other than e, and the last of them in the order e+1 .. e+7"""
    n, last = 0, 0
    for k in range(e + 1, e + 8):
        if v >> (k % 8) & 1:
            n, last = n + 1, k % 8
    return n, last


def _vote(g, w, h):
    at = lambda i, j: int(g[j, i]) if 0 <= i < w and 0 <= j < h else 0

    def walk(i, j, e, acc):
        while True:
            n, last = _others(at(i, j), e)
            if acc > 30 or n != 1:
                return acc
            acc += 1
            i, j, e = i + DI[last], j + DJ[last], 7 - last

    def component(wi, wj, si, sj):
        seen, todo = {(si, sj)}, [(si, sj)]
        while todo:
            x, y = todo.pop()
            for e in range(8):
                if at(x, y) >> e & 1:
                    q = (x + DI[e], y + DJ[e])
                    if wi <= q[0] < wi + 8 and wj <= q[1] < wj + 8 and q not in seen:
                        seen.add(q)
                        todo.append(q)
        return len(seen)

    def decide(i, j):  # set of diagonals to remove: "/" and/or "\\"
        n1, n2, n3, n4 = at(i, j), at(i, j + 1), at(i + 1, j), at(i + 1, j + 1)
        keep_slash = keep_back = 0
        seg = walk(i + 1, j + 1, 5, walk(i, j, 2, 0))
        seg2 = walk(i, j + 1, 7, walk(i + 1, j, 0, 0))
        if seg > seg2:
            keep_slash += seg - seg2
        else:
            keep_back += seg2 - seg
        if _others(n1, 2)[0] == 0 or _others(n4, 5)[0] == 0:
            keep_slash += 5
        if _others(n3, 0)[0] == 0 or _others(n2, 7)[0] == 0:
            keep_back += 5
        a, b = component(i - 3, j - 3, i, j), component(i - 3, j - 3, i, j + 1)
        if a < b:
            keep_slash += b - a
        else:
            keep_back += a - b
        if keep_slash > keep_back:
            return {"\\"}
        if keep_back > keep_slash:
            return {"/"}
        return {"/", "\\"}

    out = g.copy()
    for j in range(h - 1):
        for i in range(w - 1):
            if at(i, j) >> 2 & 1 and at(i, j + 1) >> 7 & 1 and at(i + 1, j) & 1 and at(i + 1, j + 1) >> 5 & 1:
                d = decide(i, j)
                if "/" in d:
                    out[j, i] &= 0xFB
                    out[j + 1, i + 1] &= 0xDF
                if "\\" in d:
                    out[j, i + 1] &= 0xFE
                    out[j + 1, i] &= 0x7F
    return out


@pytest.mark.parametrize("seed", range(12))
def test_vote_equals_independent_restatement(seed):
    rng = np.random.default_rng(seed)
    w, h = int(rng.integers(4, 40)), int(rng.integers(4, 40))
    palette = rng.integers(0, 256, (int(rng.integers(2, 4)), 3))
    img = np.full((h, w, 4), 255, np.uint8)
    img[..., :3] = palette[rng.integers(0, len(palette), (h, w))]
    bgr, ws = synth.rgba_to_bgr(img)
    _, triv, res = O.graph(bgr, w, h, ws, vote=True)
    expect = _vote(triv.reshape(h, w), w, h).reshape(-1)
    assert np.array_equal(res, expect)
