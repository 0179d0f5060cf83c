"""The CUDA library against the reference's own CUDA build.

The reference is a CUDA program; its stage bodies built for the GPU with its
own flags (oracle/build_ref.sh -> oracle/_ref/libdepix_refgpu{5,48}.so, from
the reference sources staged beside it) run here on the same inputs as the
library, through the library's C ABI with the default luma arithmetic
(DEPIX_YUV_CUDA). Compared:
  - packed YUV words: all 2^24 colours, bit-exact;
  - graph after trivial removal, resolved graph, cell counts and hull
    vertices, subdivided counts: bit-exact;
  - VBO positions: within POS_TOL = 1e-5 px (observed: identical), colours
    bit-exact;
  - component labels against the minimum-index labelling of the reference's
    resolved graph: bit-exact;
  - the raster against the raster contract applied to the reference's VBO:
    at most RASTER_MAX_LSB on at most RASTER_MAX_FRAC of the pixels (observed:
    identical).
Inputs: the committed golden inputs, grey-level frames (where the builds'
luma differs), the 256x224 benchmark frames, the 640x480 frame and the
sprites. The same comparisons against the committed fixtures of the CUDA
build (frames_cuda.npz) run without the harness.
"""
import json
import os

import numpy as np
import pytest

import oracle as O
from depix import synth

from conftest import GOLDEN
from test_gpu_parity import _defined_hull, _defined_pos, assert_raster_close, gpu_stages

pytestmark = pytest.mark.gpu
CELL = 45
POS_TOL = 1e-5

needs_harness = pytest.mark.skipif(not (O.refgpu_available(5) and O.refgpu_available(48)),
                                   reason="reference CUDA build not present (oracle/build_ref.sh stages and builds it)")


def _grey_frame(seed, w=64, h=48):
    rng = np.random.default_rng(seed)
    v = np.repeat(np.repeat(rng.integers(0, 256, (h // 2 + 1, w // 2 + 1)), 2, 0), 2, 1)[:h, :w]
    return np.ascontiguousarray(np.dstack([v, v, v, np.full_like(v, 255)]).astype(np.uint8))


def _inputs():
    z = np.load(os.path.join(GOLDEN, "frames_cuda.npz"))
    cases = {name: z[f"{name}/rgba"] for name in sorted({k.split("/")[0] for k in z.files})}
    cases["grey_64x48"] = _grey_frame(3)
    cases["frame_256x224_s0"] = synth.frame(0)
    cases["frame_256x224_s1"] = synth.frame(1)
    for k, s in enumerate(synth.sprites(4, seed=11)):
        cases[f"sprite_{k}"] = np.ascontiguousarray(s)
    return cases


def _compare_with_reference(g, r, w, h, scale=4):
    """g: library stage outputs (gpu_stages); r: the reference CUDA build's Frame."""
    assert np.array_equal(g["triv"], r.graph_trivial)
    assert np.array_equal(g["fused"], r.graph_trivial)
    assert np.array_equal(g["graph"], r.graph)
    assert np.array_equal(g["ec_cells"], r.ec_cells)
    assert np.array_equal(_defined_hull(g["hull"], g["ec_cells"]), _defined_hull(r.diag_cells, r.ec_cells))
    assert np.array_equal(g["ec"], r.ec)
    a, b = _defined_pos(g["pos"], g["ec"]), _defined_pos(r.pos, r.ec)
    assert a.shape == b.shape and (a.size == 0 or np.abs(a - b).max() <= POS_TOL)
    # unused slots: (-100, -100) in both
    assert np.array_equal(g["pos"] == -100.0, r.pos == -100.0)
    assert np.array_equal(g["col"], r.col)
    assert np.array_equal(g["labels"], O.label_cc(r.graph, w, h))
    assert_raster_close(g["raster"], O.raster(r.pos, r.col, w, h, scale))


@needs_harness
def test_yuv_words_all_colours_equal_reference_cuda_build(cuda):
    import depix
    torch = cuda
    ref = O.refgpu_yuv_words(5)  # index b0 | b1 << 8 | b2 << 16
    a = torch.arange(1 << 24, dtype=torch.int32, device="cuda")
    px = torch.stack([a & 255, (a >> 8) & 255, (a >> 16) & 255], dim=1).to(torch.uint8).contiguous()
    out = torch.empty(1 << 24, dtype=torch.int32, device="cuda")
    depix.yuv_words(px, 1 << 24, out, yuv=depix.YUV_CUDA)
    ours = out.cpu().numpy().view(np.uint32)
    assert np.array_equal(ours, ref)
    # and the host-build arithmetic differs from it exactly where the fixture says
    depix.yuv_words(px, 1 << 24, out, yuv=depix.YUV_HOST)
    host = out.cpu().numpy().view(np.uint32)
    d = np.nonzero(host != ref)[0]
    y = json.load(open(os.path.join(GOLDEN, "yuv_cuda.json")))
    listed = np.array(y["differs_from_host_build"])  # index b0*65536 + b1*256 + b2
    as_harness = (listed >> 16) | (((listed >> 8) & 255) << 8) | ((listed & 255) << 16)
    assert np.array_equal(np.sort(as_harness), d)


@needs_harness
@pytest.mark.parametrize("name", list(_inputs()))
def test_stages_equal_reference_cuda_build(cuda, name):
    img = _inputs()[name]
    h, w = img.shape[:2]
    bgr, ws = synth.rgba_to_bgr(img)
    for tr in (5, 48):
        for sub in (0, 1):
            for layout in (0, 1):
                g = gpu_stages(cuda, img, tr, sub, layout)
                _compare_with_reference(g, O.refgpu_frame(bgr, w, h, ws, sub, tr), w, h)


@needs_harness
def test_large_frame_640x480_x8_equals_reference_cuda_build(cuda):
    img = synth.frame_large(0)
    h, w = img.shape[:2]
    bgr, ws = synth.rgba_to_bgr(img)
    g = gpu_stages(cuda, img, 48, 1, 1, scale=8)
    _compare_with_reference(g, O.refgpu_frame(bgr, w, h, ws, 1, 48), w, h, scale=8)


@needs_harness
def test_frame_and_batch_paths_equal_reference_cuda_build(cuda):
    """The fused frame path and the uniform batch path (default params: Y 48,
    subdivision, x4) against the reference's CUDA build."""
    import depix
    torch = cuda
    imgs = [synth.frame(s) for s in (2, 3, 4)] + [np.ascontiguousarray(np.resize(_grey_frame(9), (224, 256, 4)))]
    W, H = 256, 224
    p = depix.params()
    ctx = depix.Context(W * H, len(imgs))
    d_in = torch.from_numpy(np.stack(imgs).reshape(-1).copy()).cuda()
    d_out = torch.empty(len(imgs) * W * H * 64, dtype=torch.uint8, device="cuda")
    d_lab = torch.empty(len(imgs) * W * H, dtype=torch.int32, device="cuda")
    ctx.batch([W] * len(imgs), [H] * len(imgs), [k * W * H * 4 for k in range(len(imgs))],
              [k * W * H * 64 for k in range(len(imgs))], d_in, p, d_out, d_lab)
    f_out = torch.empty(W * H * 64, dtype=torch.uint8, device="cuda")
    f_graph = torch.empty(W * H, dtype=torch.uint8, device="cuda")
    f_lab = torch.empty(W * H, dtype=torch.int32, device="cuda")
    for k, img in enumerate(imgs):
        bgr, ws = synth.rgba_to_bgr(img)
        r = O.refgpu_frame(bgr, W, H, ws, 1, 48)
        want_raster = O.raster(r.pos, r.col, W, H, 4)
        want_lab = O.label_cc(r.graph, W, H)
        ctx1 = depix.Context(W * H, 1)
        ctx1.frame(d_in[k * W * H * 4:], W, H, 4 * W, depix.LAYOUT_RGBA, p, f_out, f_graph, f_lab)
        torch.cuda.synchronize()
        ctx1.close()
        assert np.array_equal(f_graph.cpu().numpy(), r.graph)
        assert np.array_equal(f_lab.cpu().numpy(), want_lab)
        assert_raster_close(f_out.cpu().numpy().reshape(H * 4, W * 4, 4), want_raster)
        got = d_out[k * W * H * 64:(k + 1) * W * H * 64].cpu().numpy().reshape(H * 4, W * 4, 4)
        assert_raster_close(got, want_raster)
        assert np.array_equal(d_lab[k * W * H:(k + 1) * W * H].cpu().numpy(), want_lab)
    ctx.close()


@needs_harness
@pytest.mark.parametrize("sub", [0, 1])
def test_drop_in_launch_kernel_equals_reference_cuda_build(cuda, sub):
    """The reference's own symbol and argument list (Y 5, luma of the CUDA
    build) on a benchmark frame and a grey frame."""
    import ctypes
    import depix
    torch = cuda
    for img in (synth.frame(6), _grey_frame(4, 72, 40)):
        h, w = img.shape[:2]
        bgr, ws = synth.rgba_to_bgr(img)
        bgr = np.ascontiguousarray(bgr)
        pos = torch.empty(w * h * CELL * 2, dtype=torch.float32, device="cuda")
        col = torch.empty(w * h * CELL * 4, dtype=torch.uint8, device="cuda")
        ec = np.zeros(w * h, np.int32)
        graph = np.zeros(w * h, np.uint8)
        res = depix.lib().launch_kernel(depix.ptr(pos), depix.ptr(col), 0.0, depix.ptr(bgr), w, h, ws,
                                        depix.ptr(ec), depix.ptr(graph), bool(sub))
        assert res
        diag = np.ctypeslib.as_array(ctypes.cast(res, ctypes.POINTER(ctypes.c_float)),
                                     shape=(w * h * CELL * 2,)).copy()
        ctypes.CDLL(None).free(ctypes.c_void_p(res))
        r = O.refgpu_frame(bgr, w, h, ws, sub, 5)
        assert np.array_equal(graph, r.graph)
        assert np.array_equal(ec, r.ec)
        assert np.array_equal(col.cpu().numpy(), r.col)
        got = pos.cpu().numpy()
        assert np.array_equal(got == -100.0, r.pos == -100.0)
        assert np.abs(got - r.pos).max() <= POS_TOL
        a, b = _defined_pos(diag, ec), _defined_pos(r.pos, r.ec)
        assert np.abs(a - b).max() <= POS_TOL


@pytest.mark.parametrize("layout", [0, 1])
def test_stages_equal_reference_cuda_build_fixtures(cuda, layout):
    """Without the harness: the committed outputs of the reference's CUDA build."""
    z = np.load(os.path.join(GOLDEN, "frames_cuda.npz"))
    for name in sorted({k.split("/")[0] for k in z.files}):
        img = z[f"{name}/rgba"]
        for tr in (5, 48):
            for sub in (0, 1):
                g = gpu_stages(cuda, img, tr, sub, layout)
                key = f"{name}/tr{tr}/sub{sub}"
                assert np.array_equal(g["fused"], z[key + "/graph_trivial"]), key
                assert np.array_equal(g["graph"], z[key + "/graph"]), key
                assert np.array_equal(g["ec_cells"], z[key + "/ec_cells"]), key
                assert np.array_equal(_defined_hull(g["hull"], g["ec_cells"]), z[key + "/hull"]), key
                assert np.array_equal(g["ec"], z[key + "/ec"]), key
                assert np.array_equal(_defined_pos(g["pos"], g["ec"]), z[key + "/pos"]), key
