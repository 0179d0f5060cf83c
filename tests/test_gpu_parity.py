"""CUDA library (through its C ABI) against the oracle and the reference's
golden fixtures of its host build (frames.npz, yuv.json: luma arithmetic
DEPIX_YUV_HOST); the CUDA build's fixtures and the CUDA build itself are
compared in test_gpu_refcuda.py. Tolerances: the similarity graph, resolved graph, component
labels, cell counts and cell topology are compared bit-exact; vertex
positions are compared bit-exact too (the pipeline is exact on 1/64-cell
multiples, far inside the 1e-5 px budget); rasters are compared bit-exact
(budget: at most 1 LSB on at most 0.1 % of pixels)."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle as O
from depix import synth

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
CELL = 45
RASTER_MAX_LSB = 1
RASTER_MAX_FRAC = 0.001


def _defined_pos(pos, ec):
    n = ec.shape[0]
    lim = np.maximum((ec - 2) * 3, 0)
    mask = np.arange(CELL)[None, :] < lim[:, None]
    return pos.reshape(n, CELL, 2)[mask].reshape(-1)


def _defined_hull(diag, ec):
    n = ec.shape[0]
    mask = np.arange(CELL)[None, :] < ec[:, None]
    return diag.reshape(n, CELL, 2)[mask].reshape(-1)


def _upload(torch, img, layout):
    import depix
    h, w = img.shape[:2]
    if layout == depix.LAYOUT_BGR:
        buf, ws = synth.rgba_to_bgr(img)
    else:
        buf, ws = np.ascontiguousarray(img).reshape(-1), 4 * w
    return torch.from_numpy(buf.copy()).cuda(), ws


def gpu_stages(torch, img, tr, sub, layout, scale=4, yuv=0):
    """Runs every stage entry point the way the reference driver chains its kernels."""
    import depix
    h, w = img.shape[:2]
    n = w * h
    d_img, ws = _upload(torch, img, layout)
    p = depix.params(tr, 7, 6, sub, scale, yuv=yuv)
    u8 = dict(dtype=torch.uint8, device="cuda")
    raw = torch.empty(n, **u8)
    depix.graph(d_img, w, h, ws, layout, p, raw, fuse_trivial=False)
    triv = raw.clone()
    depix.resolve_trivial(triv, w, h)
    fused = torch.empty(n, **u8)
    depix.graph(d_img, w, h, ws, layout, p, fused, fuse_trivial=True)
    res = torch.empty(n, **u8)
    depix.resolve_heuristics(fused, w, h, res)
    diag = torch.zeros(n * CELL * 2, dtype=torch.float32, device="cuda")
    ec = torch.zeros(n, dtype=torch.int32, device="cuda")
    depix.cells(res, w, h, diag, ec)
    hull, ec_cells = diag.clone(), ec.clone()
    if sub:
        depix.subdivide(d_img, w, h, ws, layout, res, hull, ec_cells, diag, ec)
    ec_final = ec.clone()
    depix.triangulate(diag, ec, w, h)
    pos = torch.empty(n * CELL * 2, dtype=torch.float32, device="cuda")
    col = torch.empty(n * CELL * 4, **u8)
    depix.emit_vbo(d_img, w, h, ws, layout, diag, ec, pos, col)
    labels = torch.empty(n, dtype=torch.int32, device="cuda")
    depix.label_components(res, w, h, labels)
    out = torch.empty(n * scale * scale * 4, **u8)
    depix.raster(d_img, w, h, ws, layout, res, p, out)
    torch.cuda.synchronize()
    c = lambda t: t.cpu().numpy()
    return dict(raw=c(raw), triv=c(triv), fused=c(fused), graph=c(res), ec_cells=c(ec_cells), hull=c(hull),
                ec=c(ec_final), pos=c(pos), col=c(col), labels=c(labels),
                raster=c(out).reshape(h * scale, w * scale, 4))


def oracle_all(img, tr, sub, scale=4, yuv=0):
    h, w = img.shape[:2]
    bgr, ws = synth.rgba_to_bgr(img)
    raw, triv, res = O.graph(bgr, w, h, ws, (tr, 7, 6), yuv=yuv)
    f = O.frame(bgr, w, h, ws, sub, (tr, 7, 6), yuv=yuv)
    assert np.array_equal(f.graph, res)
    return dict(raw=raw, triv=triv, f=f, labels=O.label_cc(res, w, h), raster=O.raster(f.pos, f.col, w, h, scale))


def assert_raster_close(a, b):
    d = np.abs(a.astype(np.int16) - b.astype(np.int16)).max(axis=-1)
    bad = np.count_nonzero(d > 0)
    assert d.max() <= RASTER_MAX_LSB or bad == 0, f"max diff {d.max()}"
    assert bad <= RASTER_MAX_FRAC * d.size, f"{bad} of {d.size} pixels differ"


def compare(g, o):
    f = o["f"]
    assert np.array_equal(g["raw"], o["raw"])
    assert np.array_equal(g["triv"], o["triv"])
    assert np.array_equal(g["fused"], o["triv"])
    assert np.array_equal(g["graph"], f.graph)
    assert np.array_equal(g["ec_cells"], f.ec_cells)
    assert np.array_equal(_defined_hull(g["hull"], g["ec_cells"]), _defined_hull(f.diag_cells, f.ec_cells))
    assert np.array_equal(g["ec"], f.ec)
    assert np.array_equal(g["pos"], f.pos)
    assert np.array_equal(g["col"], f.col)
    assert np.array_equal(g["labels"], o["labels"])
    assert_raster_close(g["raster"], o["raster"])


# ----------------------------------------------------------------- tables


def test_pattern_tables_match_reference(cuda):
    import depix
    hull = np.zeros(4096, np.uint64)
    tri = np.zeros(4096, np.uint64)
    depix.pattern_tables(hull, tri)
    z = np.load(os.path.join(GOLDEN, "patterns.npz"))
    counts = (hull & np.uint64(0xF)).astype(np.int64)
    assert np.array_equal(counts, z["counts"])
    for k in range(4096):
        e = int(hull[k])
        for t in range(counts[k]):
            v = (e >> (4 + 6 * t)) & 63
            x, y = ((v & 7) - 1) * 0.25, ((v >> 3) - 1) * 0.25
            assert (x, y) == tuple(z["points"][k, t]), (k, t)


@pytest.mark.parametrize("yuv,fixture", [(1, "yuv.json"), (0, "yuv_cuda.json")])
def test_yuv_words_exhaustive(cuda, yuv, fixture):
    """All 2^24 words against the reference's host build (yuv.json) and its
    CUDA build (yuv_cuda.json)."""
    import depix
    torch = cuda
    y = json.load(open(os.path.join(GOLDEN, fixture)))
    a = torch.arange(1 << 24, dtype=torch.int32, device="cuda")
    px = torch.stack([(a >> 16) & 255, (a >> 8) & 255, a & 255], dim=1).to(torch.uint8).contiguous()
    out = torch.empty(1 << 24, dtype=torch.int32, device="cuda")
    depix.yuv_words(px, 1 << 24, out, yuv=yuv)
    words = out.cpu().numpy().view(np.uint32)
    assert hashlib.sha256(words.astype("<u4").tobytes()).hexdigest() == y["sha256_u32le"]


# ---------------------------------------------------------- golden frames


def _golden_cases():
    z = np.load(os.path.join(GOLDEN, "frames.npz"))
    return sorted({k.split("/")[0] for k in z.files})


@pytest.mark.parametrize("name", _golden_cases())
@pytest.mark.parametrize("layout", [0, 1])
def test_golden_frames_all_stages(cuda, name, layout):
    z = np.load(os.path.join(GOLDEN, "frames.npz"))
    img = z[f"{name}/rgba"]
    for tr in (5, 48):
        for sub in (0, 1):
            g = gpu_stages(cuda, img, tr, sub, layout, yuv=1)
            key = f"{name}/tr{tr}/sub{sub}"
            assert np.array_equal(g["fused"], z[key + "/graph_trivial"])
            assert np.array_equal(g["triv"], z[key + "/graph_trivial"])
            assert np.array_equal(g["graph"], z[key + "/graph"])
            assert np.array_equal(g["ec_cells"], z[key + "/ec_cells"])
            assert np.array_equal(_defined_hull(g["hull"], g["ec_cells"]), z[key + "/hull"])
            assert np.array_equal(g["ec"], z[key + "/ec"])
            assert np.array_equal(_defined_pos(g["pos"], g["ec"]), z[key + "/pos"])
            compare(g, oracle_all(img, tr, sub, yuv=1))


@pytest.mark.parametrize("name", ["c_pattern", "alex"])
def test_known_answer_graph_dumps(cuda, name):
    import depix
    torch = cuda
    z = np.load(os.path.join(GOLDEN, "dumps.npz"))
    g = torch.from_numpy(z[f"{name}/graph"].copy()).cuda()
    w, h = (int(v) for v in z[f"{name}/size"])
    diag = torch.zeros(w * h * CELL * 2, dtype=torch.float32, device="cuda")
    ec = torch.zeros(w * h, dtype=torch.int32, device="cuda")
    depix.cells(g, w, h, diag, ec)
    depix.triangulate(diag, ec, w, h)
    img = torch.zeros(3 * w * h, dtype=torch.uint8, device="cuda")
    pos = torch.empty(w * h * CELL * 2, dtype=torch.float32, device="cuda")
    depix.emit_vbo(img, w, h, 3 * w, depix.LAYOUT_BGR, diag, ec, pos, None)
    ecn = ec.cpu().numpy()
    assert np.array_equal(ecn, z[f"{name}/ec"])
    assert np.array_equal(_defined_pos(pos.cpu().numpy(), ecn), z[f"{name}/pos"])


# ------------------------------------------------------- synthetic frames

EDGE_SIZES = [(1, 1), (1, 9), (9, 1), (2, 2), (3, 5), (31, 7), (33, 9), (64, 8), (65, 17), (97, 41), (129, 33)]


@pytest.mark.parametrize("wh", EDGE_SIZES)
def test_edge_sizes(cuda, wh):
    w, h = wh
    img = synth.frame(100 + w * 7 + h, w=w, h=h)
    for layout in (0, 1):
        compare(gpu_stages(cuda, img, 48, 1, layout), oracle_all(img, 48, 1))


@pytest.mark.parametrize("seed", [0, 1])
def test_benchmark_frame_256x224(cuda, seed):
    img = synth.frame(seed)
    for tr in (5, 48):
        compare(gpu_stages(cuda, img, tr, 1, 1), oracle_all(img, tr, 1))


def test_sprites_with_transparent_backgrounds(cuda):
    for img in synth.sprites(12, seed=9):
        compare(gpu_stages(cuda, img, 48, 1, 1), oracle_all(img, 48, 1))


@pytest.mark.parametrize("scale", [1, 2, 3, 5, 8, 12, 13, 16])
def test_raster_scales(cuda, scale):
    img = synth.frame(21, w=70, h=50)
    g = gpu_stages(cuda, img, 48, 1, 1, scale=scale)
    o = oracle_all(img, 48, 1, scale=scale)
    assert_raster_close(g["raster"], o["raster"])


def test_context_frame_path_matches_stages(cuda):
    import depix
    torch = cuda
    img = synth.frame(5)
    h, w = img.shape[:2]
    d_img, ws = _upload(torch, img, 1)
    ctx = depix.Context(w * h, 1)
    out = torch.empty(w * h * 16 * 4, dtype=torch.uint8, device="cuda")
    graph = torch.empty(w * h, dtype=torch.uint8, device="cuda")
    labels = torch.empty(w * h, dtype=torch.int32, device="cuda")
    ctx.frame(d_img, w, h, ws, 1, depix.params(), out, graph, labels)
    torch.cuda.synchronize()
    o = oracle_all(img, 48, 1)
    assert np.array_equal(graph.cpu().numpy(), o["f"].graph)
    assert np.array_equal(labels.cpu().numpy(), o["labels"])
    assert_raster_close(out.cpu().numpy().reshape(h * 4, w * 4, 4), o["raster"])
    ctx.close()


def test_batch_uniform_and_uneven(cuda):
    import depix
    torch = cuda
    p = depix.params()
    frames = [synth.frame(40 + k, w=48, h=40) for k in range(5)]
    sprites = synth.sprites(7, seed=3)
    for imgs in (frames, sprites):
        in_off, out_off, ins, oi, oo = [], [], [], 0, 0
        for img in imgs:
            h, w = img.shape[:2]
            in_off.append(oi)
            out_off.append(oo)
            ins.append(np.ascontiguousarray(img).reshape(-1))
            oi += (w * h * 4 + 15) // 16 * 16
            oo += (w * h * 64 + 15) // 16 * 16
        buf = np.zeros(oi, np.uint8)
        for k, a in enumerate(ins):
            buf[in_off[k]:in_off[k] + a.size] = a
        d_in = torch.from_numpy(buf).cuda()
        d_out = torch.zeros(oo, dtype=torch.uint8, device="cuda")
        ctx = depix.Context(max(i.shape[0] * i.shape[1] for i in imgs), len(imgs))
        ctx.batch([i.shape[1] for i in imgs], [i.shape[0] for i in imgs], in_off, out_off, d_in, p, d_out)
        res = d_out.cpu().numpy()
        for k, img in enumerate(imgs):
            h, w = img.shape[:2]
            o = oracle_all(img, 48, 1)
            got = res[out_off[k]:out_off[k] + w * h * 64].reshape(h * 4, w * 4, 4)
            assert_raster_close(got, o["raster"])
        ctx.close()


def test_drop_in_launch_kernel(cuda):
    """launch_kernel's own argument list: device VBOs, host image and host
    outputs, malloc'd diagram returned."""
    import ctypes
    import depix
    torch = cuda
    for img, sub in ((synth.frame(7, w=61, h=45), 1), (synth.frame(8, w=50, h=30), 0)):
        h, w = img.shape[:2]
        bgr, ws = synth.rgba_to_bgr(img)
        bgr = np.ascontiguousarray(bgr)
        pos = torch.empty(w * h * CELL * 2, dtype=torch.float32, device="cuda")
        col = torch.empty(w * h * CELL * 4, dtype=torch.uint8, device="cuda")
        ec = np.zeros(w * h, np.int32)
        graph = np.zeros(w * h, np.uint8)
        r = depix.lib().launch_kernel(depix.ptr(pos), depix.ptr(col), 0.0, depix.ptr(bgr), w, h, ws,
                                      depix.ptr(ec), depix.ptr(graph), bool(sub))
        assert r
        diag = np.ctypeslib.as_array(ctypes.cast(r, ctypes.POINTER(ctypes.c_float)), shape=(w * h * CELL * 2,)).copy()
        ctypes.CDLL(None).free(ctypes.c_void_p(r))
        f = O.frame(bgr, w, h, ws, sub, (5, 7, 6))
        assert np.array_equal(graph, f.graph)
        assert np.array_equal(ec, f.ec)
        assert np.array_equal(pos.cpu().numpy(), f.pos)
        assert np.array_equal(col.cpu().numpy(), f.col)
        assert np.array_equal(_defined_pos(diag, ec), _defined_pos(f.pos, f.ec))


# ---------------------------------------------------- full-size properties


def test_large_frame_640x480_x8_matches_oracle(cuda):
    """The 640x480 workload end to end at its own size and scale."""
    img = synth.frame_large(0)
    g = gpu_stages(cuda, img, 48, 1, 1, scale=8)
    o = oracle_all(img, 48, 1, scale=8)
    compare(g, o)


def test_resolved_graph_is_symmetric_and_labels_are_minima(cuda):
    img = synth.frame_large(1)
    g = gpu_stages(cuda, img, 48, 1, 1, scale=1)
    h, w = img.shape[:2]
    gr = g["graph"].reshape(h, w).astype(np.int64)
    di = [-1, 0, 1, -1, 1, -1, 0, 1]
    dj = [1, 1, 1, 0, 0, -1, -1, -1]
    for e in range(8):
        bit = (gr >> e) & 1
        jj, ii = np.nonzero(bit)
        nj, ni = jj + dj[e], ii + di[e]
        assert ((ni >= 0) & (ni < w) & (nj >= 0) & (nj < h)).all()
        assert (((gr[nj, ni] >> (7 - e)) & 1) == 1).all()
    lab = g["labels"]
    assert (lab <= np.arange(w * h)).all() and (lab[lab] == lab).all()
