"""The weighted-vote heuristics of the oracle (CPU): hand-made crossings
whose answer is known, and the properties every resolution must keep (only
diagonals of crossing blocks removed, symmetric edges, no crossing left) on
seeded synthetic frames. The vote is not in the reference, so these pin the
oracle's vote to its published definition, not to reference outputs."""
import numpy as np
import pytest

import oracle as O
from depix import synth

DI = [-1, 0, 1, -1, 1, -1, 0, 1]
DJ = [1, 1, 1, 0, 0, -1, -1, -1]


def _resolve(img, vote):
    h, w = img.shape[:2]
    bgr, ws = synth.rgba_to_bgr(img)
    raw, triv, res = O.graph(bgr, w, h, ws, vote=vote)
    return triv.reshape(h, w), res.reshape(h, w)


def _two_colour(mask):
    img = np.full(mask.shape + (4,), 255, np.uint8)
    img[mask] = (0, 0, 0, 255)
    return img


def test_checkerboard_tie_removes_both_diagonals():
    i, j = np.meshgrid(np.arange(16), np.arange(16))
    img = _two_colour((i + j) % 2 == 0)
    _, ref = _resolve(img, False)
    _, vote = _resolve(img, True)
    # interior nodes: every block within 4 pixels around is a crossing with
    # equal curves (none), equal window components (32 and 32), no islands
    inner = vote[5:11, 5:11]
    assert not (inner & 0b10100101).any()
    # the reference's tie rule removes "/" only: "\" edges stay
    assert (ref[5:11, 5:11] & 0b10000001).all() and not (ref[5:11, 5:11] & 0b00100100).any()


def test_thin_line_is_kept():
    k = np.arange(16)
    mask = np.zeros((16, 16), bool)
    mask[k, k] = True  # a dark "/" line, row index = j
    img = _two_colour(mask)
    for vote in (False, True):
        _, res = _resolve(img, vote)
        for t in range(2, 13):
            assert res[t, t] & 4, (vote, t)           # (t, t) keeps its up-right edge
            assert not res[t + 1, t] & 128, (vote, t)  # the light "\" through the line is cut


def _check_resolution(triv, res):
    h, w = res.shape
    assert not (res & ~triv).any()                       # removals only
    assert np.array_equal(res & 0b01011010, triv & 0b01011010)  # orthogonal bits unchanged
    for e in range(8):
        jj, ii = np.nonzero(res >> e & 1)
        ni, nj = ii + DI[e], jj + DJ[e]
        assert ((ni >= 0) & (nj >= 0) & (ni < w) & (nj < h)).all()
        assert (res[nj, ni] >> (7 - e) & 1).all()        # symmetric
    # no block keeps both diagonals
    both = (res[:-1, :-1] >> 2 & 1) & (res[:-1, 1:] & 1)
    assert not both.any()


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_vote_keeps_the_resolution_properties(seed):
    img = synth.frame(seed, w=96, h=80)
    triv, ref = _resolve(img, False)
    _, vote = _resolve(img, True)
    _check_resolution(triv, ref)
    _check_resolution(triv, vote)


def test_vote_changes_some_decisions():
    changed = 0
    for seed in range(3):
        img = synth.frame(seed, w=128, h=96)
        _, ref = _resolve(img, False)
        _, vote = _resolve(img, True)
        changed += int((ref != vote).sum())
    assert changed > 0
