"""Generates the committed golden fixtures from the reference itself.

Run in a checkout where the reference is mounted (default /root/reference)
after ``oracle/build_ref.sh`` has built the host build of the reference's own
stage bodies (oracle/_ref). Writes, next to this script:

* ``frames.npz``   -- small seeded inputs (RGBA8) and, for Y thresholds 5 and
                      48 with subdivision off and on, the reference's graph
                      after trivial removal, resolved graph, cell and final
                      vertex counts, and the defined VBO position slots;
* ``patterns.npz`` -- the reference's reshaped-cell hull for every one of the
                      4096 cell patterns (node byte + two bits of each row
                      neighbour), read off one reference run over a graph that
                      holds every pattern;
* ``dumps.npz``    -- the resolved graphs the reference keeps as known answers
                      (kernel.cu:291-293, an 8x8 image; kernel.cu:296, a 24x24
                      image) and the reference's cells/triangles for them;
* ``borders.json`` -- the per-component border walks of the 24x24 image
                      (alex_png.txt:1-21) and the chain code recorded for
                      its walk from node 5 (alex_png.txt:25-44);
* ``yuv.json``     -- SHA-256 of the reference's packed YUV word for all 2^24
                      colours (graph_functions.cu:80-131) plus a sample.

usage: python tests/golden/make_golden.py [REFERENCE_DIR]
       python tests/golden/make_golden.py --borders [REFERENCE_DIR]   (borders.json only)
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "pixel-art-remaster-gpu_gb300"))

import oracle as O  # noqa: E402
from depix import synth  # noqa: E402

CELL = 45


def golden_inputs():
    """name -> RGBA8 image (row 0 at the bottom)."""
    rng = np.random.default_rng(1234)
    cases = {
        "frame_a": synth.frame(11, w=40, h=32),
        "frame_b": synth.frame(12, w=37, h=23),
        "large_c": synth.frame_large(3, w=48, h=40),
        "sprite_d": synth.sprites(6, seed=5)[5],
    }
    # low contrast: small steps around one colour, to sit on the thresholds
    base = rng.integers(40, 200, size=3)
    sub = np.clip(base[None, None, :] + rng.integers(-24, 25, size=(24, 32, 3)), 0, 255).astype(np.uint8)
    cases["subtle_e"] = np.concatenate([sub, np.full((24, 32, 1), 255, np.uint8)], axis=2)
    # grays and near-grays: the Y sums that land on exact integers
    g = np.zeros((16, 32, 4), np.uint8)
    v = rng.integers(0, 256, size=(16, 32))
    g[..., 0] = v
    g[..., 1] = np.clip(v + rng.integers(-1, 2, size=v.shape), 0, 255)
    g[..., 2] = v
    g[..., 3] = 255
    cases["gray_f"] = g
    cases["thin_g"] = synth.frame(13, w=1, h=17)
    cases["thin_h"] = synth.frame(14, w=19, h=1)
    cases["dot_i"] = synth.frame(15, w=1, h=1)
    cases["tiny_j"] = synth.frame(16, w=2, h=2)
    for k, img in cases.items():
        cases[k] = np.ascontiguousarray(img)
    return cases


def defined_pos(pos, ec):
    """Concatenation of every cell's defined VBO position slots."""
    n = ec.shape[0]
    p = pos.reshape(n, CELL, 2)
    lim = np.maximum((ec - 2) * 3, 0)
    mask = np.arange(CELL)[None, :] < lim[:, None]
    return p[mask].reshape(-1)


def defined_hull(diag, ec):
    n = ec.shape[0]
    d = diag.reshape(n, CELL, 2)
    mask = np.arange(CELL)[None, :] < ec[:, None]
    return d[mask].reshape(-1)


def pattern_graph():
    """A 96x128 graph whose cell 3k+1 has pattern k (left at 3k, right at 3k+2)."""
    g = np.zeros(96 * 128, np.uint8)
    for k in range(4096):
        node = k & 0xFF
        left = (((k >> 8) & 1) << 2) | (((k >> 9) & 1) << 7)
        right = ((k >> 10) & 1) | (((k >> 11) & 1) << 5)
        g[3 * k] = left
        g[3 * k + 1] = node
        g[3 * k + 2] = right
    return g


def parse_dump(src, label, size):
    m = re.search(r"/\* " + re.escape(label) + r" \*/(.*?)\};", src, re.S)
    body = m.group(1).replace("//", " ").replace("(char)", " ")
    body = body.split("{", 1)[1]
    vals = [int(t) for t in re.findall(r"-?\d+", body)]
    assert len(vals) == size, (label, len(vals))
    return np.array(vals, np.int64).astype(np.uint8)


def write_borders(ref_dir):
    """borders.json from alex_png.txt: the walks ("Spline: k - ..." lines)
    and the chain code the file records for the walk from node 5 ("index: i,
    edge: e" lines)."""
    walks, chain = {}, {"nodes": [], "edges": []}
    for line in open(os.path.join(ref_dir, "alex_png.txt")):
        m = re.match(r"Spline: (\d+) -(.*)", line)
        if m:
            walks[int(m.group(1))] = [int(t) for t in re.findall(r"\d+", m.group(2))]
        m = re.match(r"index: (\d+), edge: (\d+)", line)
        if m:
            chain["nodes"].append(int(m.group(1)))
            chain["edges"].append(int(m.group(2)))
    with open(os.path.join(HERE, "borders.json"), "w") as fh:
        json.dump({"image": "alex", "size": [24, 24], "walks": walks, "chain_from_5": chain}, fh, indent=0)


def main(ref_dir="/root/reference"):
    for tr in (5, 48):
        if not O.ref_available(tr):
            sys.exit("reference host build missing: run oracle/build_ref.sh first")
    out = {}
    for name, img in golden_inputs().items():
        h, w = img.shape[:2]
        bgr, ws = synth.rgba_to_bgr(img)
        out[f"{name}/rgba"] = img
        for tr in (5, 48):
            for sub in (0, 1):
                f = O.ref_frame(bgr, w, h, ws, sub, tr)
                key = f"{name}/tr{tr}/sub{sub}"
                out[key + "/graph_trivial"] = f.graph_trivial
                out[key + "/graph"] = f.graph
                out[key + "/ec_cells"] = f.ec_cells
                out[key + "/ec"] = f.ec
                out[key + "/hull"] = defined_hull(f.diag_cells, f.ec_cells)
                out[key + "/pos"] = defined_pos(f.pos, f.ec)
    np.savez_compressed(os.path.join(HERE, "frames.npz"), **out)

    g = pattern_graph()
    f = O.ref_frame(np.zeros(3 * 96 * 128 + 128, np.uint8), 96, 128, 3 * 96, 0, 5, graph_in=g)
    idx = 3 * np.arange(4096) + 1
    counts = f.ec_cells[idx]
    diag = f.diag_cells.reshape(-1, CELL, 2)[idx]
    pts = np.zeros((4096, 8, 2), np.float32)
    for k in range(4096):
        pts[k, :counts[k]] = diag[k, :counts[k]]
    np.savez_compressed(os.path.join(HERE, "patterns.npz"), counts=counts, points=pts)

    src = open(os.path.join(ref_dir, "kernel.cu")).read()
    dumps = {"c_pattern": (parse_dump(src, "c_pattern.png", 64), 8, 8),
             "alex": (parse_dump(src, "alex.png", 576), 24, 24)}
    dz = {}
    for name, (graph, w, h) in dumps.items():
        f = O.ref_frame(np.zeros(3 * w * h + 64, np.uint8), w, h, 3 * w, 0, 5, graph_in=graph)
        dz[f"{name}/graph"] = graph
        dz[f"{name}/size"] = np.array([w, h])
        dz[f"{name}/ec"] = f.ec
        dz[f"{name}/pos"] = defined_pos(f.pos, f.ec)
    np.savez_compressed(os.path.join(HERE, "dumps.npz"), **dz)

    write_borders(ref_dir)

    allc = np.stack(np.meshgrid(np.arange(256), np.arange(256), np.arange(256), indexing="ij"), -1)
    allc = allc.reshape(-1, 3).astype(np.uint8)
    words = O.yuv_words(allc, ref_tr_y=5)
    sample = np.arange(0, 1 << 24, 65537)
    with open(os.path.join(HERE, "yuv.json"), "w") as fh:
        json.dump({"order": "b0 + 256*b1 + 65536*b2 runs over the last byte fastest: index = b0*65536 + b1*256 + b2",
                   "sha256_u32le": hashlib.sha256(words.astype("<u4").tobytes()).hexdigest(),
                   "sample_index": sample.tolist(), "sample_word": words[sample].tolist()}, fh)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    if sys.argv[1:2] == ["--borders"]:
        write_borders(*(sys.argv[2:] or ["/root/reference"]))
    else:
        main(*sys.argv[1:])
