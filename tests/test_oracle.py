"""The CPU oracle against the reference: committed golden fixtures made by the
reference's own stage bodies in both of its builds (host: frames.npz,
yuv.json, luma arithmetic YUV_HOST; CUDA: frames_cuda.npz, yuv_cuda.json,
YUV_CUDA), its known-answer graph dumps and border walks, and (when built in
this checkout) the reference's host build directly."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle as O
from depix import synth

from conftest import GOLDEN

CELL = 45


def _defined_pos(pos, ec):
    n = ec.shape[0]
    lim = np.maximum((ec - 2) * 3, 0)
    mask = np.arange(CELL)[None, :] < lim[:, None]
    return pos.reshape(n, CELL, 2)[mask].reshape(-1)


def _defined_hull(diag, ec):
    n = ec.shape[0]
    mask = np.arange(CELL)[None, :] < ec[:, None]
    return diag.reshape(n, CELL, 2)[mask].reshape(-1)


def _golden_runs():
    z = np.load(os.path.join(GOLDEN, "frames.npz"))
    names = sorted({k.split("/")[0] for k in z.files})
    for name in names:
        for tr in (5, 48):
            for sub in (0, 1):
                yield name, tr, sub


@pytest.fixture(scope="module")
def frames():
    return np.load(os.path.join(GOLDEN, "frames.npz"))


@pytest.mark.parametrize("name,tr,sub", list(_golden_runs()))
def test_oracle_matches_reference_golden(frames, name, tr, sub):
    img = frames[f"{name}/rgba"]
    h, w = img.shape[:2]
    bgr, ws = synth.rgba_to_bgr(img)
    f = O.frame(bgr, w, h, ws, sub, (tr, 7, 6), yuv=O.YUV_HOST)
    key = f"{name}/tr{tr}/sub{sub}"
    assert np.array_equal(f.graph_trivial, frames[key + "/graph_trivial"])
    assert np.array_equal(f.graph, frames[key + "/graph"])
    assert np.array_equal(f.ec_cells, frames[key + "/ec_cells"])
    assert np.array_equal(_defined_hull(f.diag_cells, f.ec_cells), frames[key + "/hull"])
    assert np.array_equal(f.ec, frames[key + "/ec"])
    assert np.array_equal(_defined_pos(f.pos, f.ec), frames[key + "/pos"])
    assert f.fails == 0


def test_hull_table_matches_reference():
    z = np.load(os.path.join(GOLDEN, "patterns.npz"))
    counts, pts = O.hull_table()
    assert np.array_equal(counts, z["counts"])
    for k in range(4096):
        c = counts[k]
        assert np.array_equal(pts[k, :c].astype(np.float32) * 0.25, z["points"][k, :c]), k


@pytest.mark.parametrize("name", ["c_pattern", "alex"])
def test_known_answer_graph_dumps(name):
    z = np.load(os.path.join(GOLDEN, "dumps.npz"))
    g = z[f"{name}/graph"]
    w, h = (int(v) for v in z[f"{name}/size"])
    f = O.frame(np.zeros(3 * w * h + 64, np.uint8), w, h, 3 * w, 0, (5, 7, 6), graph_in=g)
    assert np.array_equal(f.ec, z[f"{name}/ec"])
    assert np.array_equal(_defined_pos(f.pos, f.ec), z[f"{name}/pos"])


def test_component_labels_contain_reference_border_walks():
    """Every per-component border walk the reference recorded for its 24x24
    image (alex_png.txt) lies inside one labelled component of that image's
    resolved graph (kernel.cu:296)."""
    z = np.load(os.path.join(GOLDEN, "dumps.npz"))
    b = json.load(open(os.path.join(GOLDEN, "borders.json")))
    lab = O.label_cc(z["alex/graph"], 24, 24)
    for walk in b["walks"].values():
        assert len({int(lab[i]) for i in walk}) == 1
    # and labels are the component minima
    assert all(lab[k] <= k and lab[lab[k]] == lab[k] for k in range(576))


def _all_colours():
    allc = np.stack(np.meshgrid(np.arange(256), np.arange(256), np.arange(256), indexing="ij"), -1)
    return allc.reshape(-1, 3).astype(np.uint8)


def test_yuv_words_exhaustive_against_reference():
    y = json.load(open(os.path.join(GOLDEN, "yuv.json")))
    words = O.yuv_words(_all_colours(), yuv=O.YUV_HOST)
    assert hashlib.sha256(words.astype("<u4").tobytes()).hexdigest() == y["sha256_u32le"]
    assert words[np.array(y["sample_index"])].tolist() == y["sample_word"]


def test_yuv_words_exhaustive_against_reference_cuda_build():
    """The luma of the CUDA build: the oracle's fused multiply-add order gives
    the CUDA build's word for all 2^24 colours, and differs from the host
    build exactly on the colours the fixture lists."""
    y = json.load(open(os.path.join(GOLDEN, "yuv_cuda.json")))
    allc = _all_colours()
    words = O.yuv_words(allc, yuv=O.YUV_CUDA)
    assert hashlib.sha256(words.astype("<u4").tobytes()).hexdigest() == y["sha256_u32le"]
    host = O.yuv_words(allc, yuv=O.YUV_HOST)
    assert np.nonzero(words != host)[0].tolist() == y["differs_from_host_build"]
    assert len(y["differs_from_host_build"]) == 2490
    # every such colour has an exact integer sum 0.299 r + 0.587 g + 0.114 b
    d = np.array(y["differs_from_host_build"])
    r, g, b = allc[d, 0].astype(np.int64), allc[d, 1].astype(np.int64), allc[d, 2].astype(np.int64)
    assert ((299 * r + 587 * g + 114 * b) % 1000 == 0).all()


def _cuda_golden_runs():
    z = np.load(os.path.join(GOLDEN, "frames_cuda.npz"))
    for name in sorted({k.split("/")[0] for k in z.files}):
        for tr in (5, 48):
            for sub in (0, 1):
                yield name, tr, sub


@pytest.fixture(scope="module")
def frames_cuda():
    return np.load(os.path.join(GOLDEN, "frames_cuda.npz"))


@pytest.mark.parametrize("name,tr,sub", list(_cuda_golden_runs()))
def test_oracle_matches_reference_cuda_build_golden(frames_cuda, name, tr, sub):
    z = frames_cuda
    img = z[f"{name}/rgba"]
    h, w = img.shape[:2]
    bgr, ws = synth.rgba_to_bgr(img)
    f = O.frame(bgr, w, h, ws, sub, (tr, 7, 6), yuv=O.YUV_CUDA)
    key = f"{name}/tr{tr}/sub{sub}"
    assert np.array_equal(f.graph_trivial, z[key + "/graph_trivial"])
    assert np.array_equal(f.graph, z[key + "/graph"])
    assert np.array_equal(f.ec_cells, z[key + "/ec_cells"])
    assert np.array_equal(_defined_hull(f.diag_cells, f.ec_cells), z[key + "/hull"])
    assert np.array_equal(f.ec, z[key + "/ec"])
    assert np.array_equal(_defined_pos(f.pos, f.ec), z[key + "/pos"])


def test_the_two_builds_differ_on_grey_frames(frames_cuda):
    """The fixtures of the two builds are not the same data: on the grey
    frames the CUDA build's graphs differ from the host build's."""
    z = frames_cuda
    img = z["grey_k/rgba"]
    h, w = img.shape[:2]
    bgr, ws = synth.rgba_to_bgr(img)
    host = O.frame(bgr, w, h, ws, 0, (5, 7, 6), yuv=O.YUV_HOST)
    assert not np.array_equal(host.graph_trivial, z["grey_k/tr5/sub0/graph_trivial"])


def _bfs_labels(g, w, h):
    di = [-1, 0, 1, -1, 1, -1, 0, 1]
    dj = [1, 1, 1, 0, 0, -1, -1, -1]
    adj = [[] for _ in range(w * h)]
    for k in range(w * h):
        i, j = k % w, k // w
        for e in range(8):
            if (g[k] >> e) & 1:
                ni, nj = i + di[e], j + dj[e]
                if 0 <= ni < w and 0 <= nj < h:
                    adj[k].append(nj * w + ni)
                    adj[nj * w + ni].append(k)
    lab = [-1] * (w * h)
    for k in range(w * h):
        if lab[k] >= 0:
            continue
        comp, stack = [k], [k]
        lab[k] = k
        while stack:
            x = stack.pop()
            for y in adj[x]:
                if lab[y] < 0:
                    lab[y] = k
                    comp.append(y)
                    stack.append(y)
    return np.array(lab, np.int32)


def test_component_labels_equal_bfs():
    img = synth.frame(3, w=48, h=40)
    bgr, ws = synth.rgba_to_bgr(img)
    _, _, res = O.graph(bgr, 48, 40, ws)
    assert np.array_equal(O.label_cc(res, 48, 40), _bfs_labels(res, 48, 40))


def test_raster_uniform_image_is_flat():
    img = np.zeros((6, 7, 4), np.uint8)
    img[...] = (10, 200, 30, 255)
    bgr, ws = synth.rgba_to_bgr(img)
    f = O.frame(bgr, 7, 6, ws, 1)
    out = O.raster(f.pos, f.col, 7, 6, 4)
    assert (out.reshape(-1, 4) == np.array([10, 200, 30, 255], np.uint8)).all()


def test_raster_painter_order_and_edges():
    """Two overlapping triangles: the later one wins on the overlap; top-left
    rule on a shared vertical edge; uncovered samples keep the clear colour."""
    w, h, s = 2, 1, 4
    pos = np.full((w * h * CELL, 2), -100.0, np.float32)
    col = np.zeros((w * h * CELL, 4), np.uint8)
    # cell 0: triangle covering x in [0, 1.5], cell 1: triangle x in [1, 2]
    pos[0:3] = [(0, 0), (1.5, 0), (0, 1)]
    col[0:CELL] = (255, 0, 0, 255)
    pos[CELL:CELL + 3] = [(1, 0), (2, 0), (1, 1)]
    col[CELL:2 * CELL] = (0, 0, 255, 255)
    out = O.raster(pos.reshape(-1), col.reshape(-1), w, h, s)
    # sample (0.5,0.5)/4: inside the first triangle only
    assert out[0, 0].tolist() == [255, 0, 0, 255]
    # sample x=4.5/4=1.125, y=0.125: inside both -> the later (blue) wins
    assert out[0, 4].tolist() == [0, 0, 255, 255]
    # sample (7.5/4, 3.5/4): outside both
    assert out[3, 7].tolist() == [0, 0, 0, 255]


@pytest.mark.skipif(not (O.ref_available(5) and O.ref_available(48)), reason="reference host build not present")
@pytest.mark.parametrize("seed", [0, 1])
@pytest.mark.parametrize("tr", [5, 48])
def test_oracle_equals_reference_build_full_frames(seed, tr):
    for img in (synth.frame(seed), synth.frame_large(seed, w=160, h=120)):
        h, w = img.shape[:2]
        bgr, ws = synth.rgba_to_bgr(img)
        for sub in (0, 1):
            a = O.frame(bgr, w, h, ws, sub, (tr, 7, 6), yuv=O.YUV_HOST)
            b = O.ref_frame(bgr, w, h, ws, sub, tr)
            assert np.array_equal(a.graph_trivial, b.graph_trivial)
            assert np.array_equal(a.graph, b.graph)
            assert np.array_equal(a.ec, b.ec)
            assert np.array_equal(a.pos, b.pos)
            assert np.array_equal(a.col, b.col)
