"""depix_resolve_heuristics_static: in-place heuristic resolution whose graph
snapshot lives in a fixed device array inside the library, for callers that
cannot allocate device memory. Called through the C ABI and compared, bit for
bit, with depix_resolve_heuristics (which takes the snapshot from the caller)
on consecutive calls. This file is collected last on purpose, after
test_zz_device_faults.py."""
import ctypes

import numpy as np
import pytest

import oracle as O
from depix import synth

pytestmark = pytest.mark.gpu


def _entry(depix):
    fn = depix.lib().depix_resolve_heuristics_static
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


def test_static_snapshot_equals_caller_snapshot_on_consecutive_calls(cuda):
    import depix
    torch = cuda
    fn = _entry(depix)
    p = depix.params()
    # calls in a row, each on a smaller frame: whatever the previous call
    # left in the shared array must not leak into the next; the last frame's
    # width is not a multiple of 16, so the heuristics read the array with
    # plain loads instead of a TMA tile load
    for img in (synth.frame_large(5, w=320, h=240), synth.frame(31), synth.frame(7, w=250, h=97)):
        h, w = img.shape[:2]
        d_img = torch.from_numpy(np.ascontiguousarray(img).reshape(-1).copy()).cuda()
        after_trivial = torch.empty(w * h, dtype=torch.uint8, device="cuda")
        depix.graph(d_img, w, h, 4 * w, depix.LAYOUT_RGBA, p, after_trivial, fuse_trivial=True)
        expected = torch.empty_like(after_trivial)
        depix.resolve_heuristics(after_trivial, w, h, expected)
        in_place = after_trivial.clone()
        status = fn(depix.ptr(in_place), w, h, depix.stream_ptr())
        assert status == 0, depix.lib().depix_last_error()
        torch.cuda.synchronize()
        assert torch.equal(in_place, expected)
        bgr, ws = synth.rgba_to_bgr(img)
        assert np.array_equal(in_place.cpu().numpy(), O.graph(bgr, w, h, ws)[2])
    # no bounded wait of the TMA tile loads (which read the array) gave up
    assert depix.take_device_faults() == 0


def test_static_snapshot_rejects_frames_beyond_its_size(cuda):
    import depix
    torch = cuda
    fn = _entry(depix)
    g = torch.zeros(16, dtype=torch.uint8, device="cuda")
    status = fn(depix.ptr(g), 4097, 1024, depix.stream_ptr())  # 4,195,328 > 4,194,304 pixels
    assert status == 4  # DEPIX_ERR_TOO_LARGE, before any device work
    assert b"larger than the fixed snapshot" in depix.lib().depix_last_error()
