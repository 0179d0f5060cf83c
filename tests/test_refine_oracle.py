"""The refinement stage's CPU specification on its own (no GPU): its
analytic gradient against float64 central differences, and the topology's
invariants (every split cell edge pairs with a reversed twin or lies on the
frame; free nodes have two neighbours; segment colours follow the edges)."""
from math import gcd

import numpy as np
import pytest

import oracle as O
import refine_oracle as R
from depix import synth


def _frame(seed=0, w=48, h=40):
    img = synth.frame(seed, w=w, h=h)
    bgr, ws = synth.rgba_to_bgr(img)
    raw, _, res = O.graph(bgr, w, h, ws, (48, 7, 6))
    return img, raw, res


@pytest.fixture(scope="module")
def small():
    img, raw, res = _frame()
    return img, R.topology(img, res, raw, 4)


def test_gradient_matches_central_differences(small):
    img, top = small
    P0 = R.initial_positions(top)
    rng = np.random.default_rng(1)
    free = np.nonzero(top.free)[0]
    P = P0.copy()
    P[free] += rng.normal(0, 0.05, (len(free), 2))
    _, _, G = R.energy_grad(top, P, P0, img)
    sel = rng.choice(free, 64, replace=False)
    fd = R.central_differences(top, P, P0, img, sel, h=1e-4)
    assert np.linalg.norm(G[sel] - fd) <= 1e-6 * np.linalg.norm(fd)
    assert np.all(G[~top.free] == 0)


def test_local_central_differences_equal_full_ones(small):
    """The per-node differences from only the terms touching the node equal
    the differences of the whole energy (the other terms cancel)."""
    img, top = small
    P0 = R.initial_positions(top)
    rng = np.random.default_rng(2)
    free = np.nonzero(top.free)[0]
    P = P0.copy()
    P[free] += rng.normal(0, 0.05, (len(free), 2))
    sel = np.concatenate([rng.choice(free, 24, replace=False), np.nonzero(~top.free)[0][:4]])
    full = R.central_differences(top, P, P0, img, sel, h=1e-4)
    local = R.central_differences_local(top, P, P0, img, sel, h=1e-4)
    assert np.abs(full - local).max() <= 1e-9 * max(np.abs(full).max(), 1e-12) + 1e-11


def test_topology_invariants(small):
    img, top = small
    assert len(top.qx) > 100 and top.free.sum() > 50
    deg = top.flags >> 4
    free = top.free
    assert np.all(deg[free] == 2)
    assert np.all(top.nbr[free] >= 0) and np.all(top.nbr[free, 0] < top.nbr[free, 1])
    # every edge joins two distinct nodes at most one quarter-pixel lattice step apart
    du = np.abs(top.qx[top.eu] - top.qx[top.ev])
    dv = np.abs(top.qy[top.eu] - top.qy[top.ev])
    assert np.all(du + dv > 0) and np.all(np.maximum(du, dv) <= 4)
    # free-node corner slots take the colours of their first edge
    S = len(top.seg_type)
    E = len(top.eu)
    assert S == 3 * E + len(top.qx)
    assert np.all(top.seg_type[3 * E:][free] == R.SEG_CORNER)
    assert np.all(top.seg_type[3 * np.arange(E) + 1] == R.SEG_MID)
    # samples: unique, in range, assigned to live slots
    assert len(np.unique(top.samp_idx)) == len(top.samp_idx)
    assert np.all(top.seg_type[top.samp_seg] > 0)


def test_cells_tile_the_frame_once_edges_are_split():
    """The property the twin search relies on: after splitting hull edges at
    the hull vertices inside them, every edge off the frame has a reversed
    twin, and the cells' areas add up to the frame."""
    img, raw, res = _frame(3, 40, 36)
    h, w = img.shape[:2]
    cnt, pts = R.cell_hulls(res, w, h)
    edges, verts, area = [], set(), 0
    for idx in range(w * h):
        i, j = idx % w, idx // w
        P = [(4 * i + int(pts[idx, t, 0]), 4 * j + int(pts[idx, t, 1])) for t in range(cnt[idx])]
        verts.update(P)
        edges += [(P[t], P[(t + 1) % len(P)]) for t in range(len(P))]
        area += sum(P[t][0] * P[(t + 1) % len(P)][1] - P[(t + 1) % len(P)][0] * P[t][1] for t in range(len(P)))
    assert area == 2 * 16 * w * h
    split = set()
    for a, b in edges:
        dx, dy = b[0] - a[0], b[1] - a[1]
        g = gcd(abs(dx), abs(dy))
        pts_on = [a] + [(a[0] + dx * t // g, a[1] + dy * t // g) for t in range(1, g)
                        if (a[0] + dx * t // g, a[1] + dy * t // g) in verts] + [b]
        split.update(zip(pts_on[:-1], pts_on[1:]))
    on_frame = lambda a, b: (a[0] == b[0] and a[0] in (0, 4 * w)) or (a[1] == b[1] and a[1] in (0, 4 * h))
    assert all((b, a) in split or on_frame(a, b) for a, b in split)


def test_adam_lowers_the_energy(small):
    img, top = small
    _, e0, e1 = R.adam(top, img, steps=40)
    assert e1[1] < e0[1]
