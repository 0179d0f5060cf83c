"""Generates the golden fixtures of the reference's CUDA build.

The reference ships as a CUDA program (depixel_gpu.pro: nvcc with
-use_fast_math and nvcc's default FMA contraction). Its stage bodies, built
that way for the GPU by ``oracle/build_ref.sh`` (``oracle/ref_gpu.cu`` ->
``oracle/_ref/libdepix_refgpu{5,48}.so``), differ from the host build of the
same sources (``make_golden.py``) in the luma of 2490 colours: nvcc fuses
y = 0.299 r + 0.587 g + 0.114 b into fused multiply-adds. Run on a machine
with a CUDA GPU after ``oracle/build_ref.sh`` (``__graft_entry__.build()``
runs it). Writes, next to this script:

* ``frames_cuda.npz`` -- the inputs of ``frames.npz`` plus grey-level frames,
  for Y thresholds 5 and 48 with subdivision off and on: the CUDA build's
  graph after trivial removal, resolved graph, cell and final vertex counts,
  hull points and defined VBO position slots;
* ``yuv_cuda.json``   -- SHA-256 of the CUDA build's packed YUV word for all
  2^24 colours (index order of ``yuv.json``), and the colours where it
  differs from the host build's word.

usage: python tests/golden/make_golden_cuda.py [OUT_DIR]
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "pixel-art-remaster-gpu_gb300"))
sys.path.insert(0, HERE)

import oracle as O  # noqa: E402
from depix import synth  # noqa: E402
from make_golden import defined_hull, defined_pos, golden_inputs  # noqa: E402


def grey_inputs():
    """Frames of grey levels in 2x2 blocks: every grey level the two builds
    evaluate differently appears next to its neighbours."""
    rng = np.random.default_rng(4321)
    out = {}
    levels = rng.permutation(256)
    v = np.repeat(np.repeat(levels.reshape(16, 16), 2, 0), 2, 1)
    out["grey_k"] = np.dstack([v, v, v, np.full_like(v, 255)]).astype(np.uint8)
    v = rng.integers(0, 256, (24, 20))
    v = np.repeat(np.repeat(v, 2, 0), 2, 1)[:45, :37]
    near = np.clip(v[..., None] + rng.integers(-1, 2, (45, 37, 3)) * (rng.random((45, 37, 1)) < 0.3), 0, 255)
    out["grey_l"] = np.dstack([near, np.full((45, 37, 1), 255)]).astype(np.uint8)
    return {k: np.ascontiguousarray(x) for k, x in out.items()}


def main(out_dir=HERE):
    import torch  # noqa: F401  (creates the CUDA context the harness shares)
    for tr in (5, 48):
        if not O.refgpu_available(tr):
            sys.exit("reference CUDA build missing: run oracle/build_ref.sh on a machine with nvcc")
    out = {}
    cases = dict(golden_inputs())
    cases.update(grey_inputs())
    for name, img in cases.items():
        h, w = img.shape[:2]
        bgr, ws = synth.rgba_to_bgr(img)
        out[f"{name}/rgba"] = img
        for tr in (5, 48):
            for sub in (0, 1):
                f = O.refgpu_frame(bgr, w, h, ws, sub, tr)
                key = f"{name}/tr{tr}/sub{sub}"
                out[key + "/graph_trivial"] = f.graph_trivial
                out[key + "/graph"] = f.graph
                out[key + "/ec_cells"] = f.ec_cells
                out[key + "/ec"] = f.ec
                out[key + "/hull"] = defined_hull(f.diag_cells, f.ec_cells)
                out[key + "/pos"] = defined_pos(f.pos, f.ec)
    np.savez_compressed(os.path.join(out_dir, "frames_cuda.npz"), **out)

    # word of (b0, b1, b2) at index b0*65536 + b1*256 + b2, as in yuv.json
    gpu = O.refgpu_yuv_words(5)  # harness order: b0 | b1 << 8 | b2 << 16
    i = np.arange(1 << 24, dtype=np.int64)
    b0, b1, b2 = i >> 16, (i >> 8) & 255, i & 255
    words = gpu[b0 | (b1 << 8) | (b2 << 16)]
    px = np.stack([b0, b1, b2], 1).astype(np.uint8)
    host = O.yuv_words(px, yuv=O.YUV_HOST)
    diff = np.nonzero(words != host)[0]
    grey = sorted({int(k >> 16) for k in diff if (k >> 16) == ((k >> 8) & 255) == (k & 255)})
    with open(os.path.join(out_dir, "yuv_cuda.json"), "w") as fh:
        json.dump({"order": "index = b0*65536 + b1*256 + b2 (as yuv.json)",
                   "sha256_u32le": hashlib.sha256(words.astype("<u4").tobytes()).hexdigest(),
                   "differs_from_host_build": diff.tolist(), "grey_levels_differing": grey}, fh)
    print(f"CUDA-build fixtures written to {out_dir}: {len(cases)} frames, {diff.size} words differ from the host build")


if __name__ == "__main__":
    main(*sys.argv[1:])
