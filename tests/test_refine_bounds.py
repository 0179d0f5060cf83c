"""The worst-case sizes the refinement setup reserves so that it reads only
the edge and node counts back (CPU, no GPU): a cell's split curve edges are
at most the quarter-unit lattice steps around its hull's bounding box, 2
(width + height), so a frame has at most w h max_split of them, max_split
taken over every cell pattern's hull; samples are at most the output
pixels."""
from math import gcd

import numpy as np
import pytest

import oracle as O
import refine_oracle as R
from depix import synth


def _max_split():
    counts, pts = O.hull_table()
    best = 0
    for pat in range(4096):
        k = int(counts[pat])
        if k == 0:
            continue
        x, y = pts[pat, :k, 0].astype(int), pts[pat, :k, 1].astype(int)
        best = max(best, 2 * ((x.max() - x.min()) + (y.max() - y.min())))
    return max(best, 1)


def test_lattice_steps_of_each_hull_bound_its_split_edges():
    """Around a convex hull, each edge has at most max(|dx|, |dy|) lattice
    steps, and their sum is at most 2 (width + height) of its box."""
    counts, pts = O.hull_table()
    for pat in range(4096):
        k = int(counts[pat])
        if k < 2:
            continue
        P = [(int(pts[pat, t, 0]), int(pts[pat, t, 1])) for t in range(k)]
        steps = sum(gcd(abs(P[(t + 1) % k][0] - P[t][0]), abs(P[(t + 1) % k][1] - P[t][1])) for t in range(k))
        xs, ys = [p[0] for p in P], [p[1] for p in P]
        assert steps <= 2 * ((max(xs) - min(xs)) + (max(ys) - min(ys))), pat


@pytest.mark.parametrize("seed,w,h", [(0, 48, 40), (3, 64, 32), (5, 40, 56)])
def test_frame_counts_within_reserved_sizes(seed, w, h):
    img = synth.frame(seed, w=w, h=h)
    bgr, ws = synth.rgba_to_bgr(img)
    raw, _, res = O.graph(bgr, w, h, ws, (48, 7, 6))
    top = R.topology(img, res, raw, 4)
    n = w * h
    E, N = len(top.eu), len(top.qx)
    assert E <= n * _max_split()
    # nodes are vertices of the (4w + 3) x (4h + 3) quarter-unit grid
    assert N <= (4 * w + 3) * (4 * h + 3)
    # samples: at most one per output pixel
    assert len(top.samp_idx) <= n * 16
    assert len(np.unique(top.samp_idx)) == len(top.samp_idx)
