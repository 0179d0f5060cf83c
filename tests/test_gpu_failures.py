"""Error paths of the C ABI, with failures made on the host or by a wait that
nothing completes, never by a GPU fault:
  - depix_batch_host rejects frames outside its host buffers (including a
    corrupt offset near 2^64) before any allocation or copy;
  - an allocation failure injected through the library's allocator hook
    (depix_debug_fail_allocations) in context creation and in staging growth
    returns DEPIX_ERR_ALLOC, leaks nothing, and leaves the context usable;
  - the graph stage's bounded TMA wait, made to run out with no load issued
    (depix_debug_tma_timeout), sets fault bit 1 and makes
    depix_take_device_faults return DEPIX_ERR_TIMEOUT; the next frame is
    correct again."""
import ctypes

import numpy as np
import pytest

import oracle as O
from depix import synth

pytestmark = pytest.mark.gpu
W, H = 64, 48


def _frames(n, seed=0):
    return [np.ascontiguousarray(synth.frame(seed + k, w=W, h=H)) for k in range(n)]


def _host_batch(imgs, scale=4):
    ws = np.full(len(imgs), W, np.int32)
    hs = np.full(len(imgs), H, np.int32)
    in_off = np.arange(len(imgs), dtype=np.uint64) * np.uint64(W * H * 4)
    out_off = np.arange(len(imgs), dtype=np.uint64) * np.uint64(W * H * 4 * scale * scale)
    h_in = np.ascontiguousarray(np.stack(imgs).reshape(-1))
    h_out = np.zeros(len(imgs) * W * H * 4 * scale * scale, np.uint8)
    return ws, hs, in_off, out_off, h_in, h_out


def _expected(img, scale=4):
    bgr, ws = synth.rgba_to_bgr(img)
    f = O.frame(bgr, W, H, ws, 1, (48, 7, 6))
    return O.raster(f.pos, f.col, W, H, scale).reshape(-1)


def test_batch_host_rejects_frames_outside_its_buffers(cuda):
    import depix
    ctx = depix.Context(W * H, 4)
    p = depix.params()
    imgs = _frames(2)
    ws, hs, in_off, out_off, h_in, h_out = _host_batch(imgs)
    live = depix.debug_live_allocations()
    h_out[:] = 77
    bad_cases = [
        (np.array([0, (1 << 64) - 16], np.uint64), out_off),             # wraps around 2^64
        (np.array([0, h_in.size], np.uint64), out_off),                  # starts at the end
        (in_off, np.array([0, h_out.size - 16], np.uint64)),             # output runs past the end
        (in_off, np.array([0, (1 << 64) - 4096], np.uint64)),            # output offset wraps
    ]
    for i_off, o_off in bad_cases:
        with pytest.raises(depix.DepixError) as e:
            ctx.batch_host(ws, hs, i_off, o_off, h_in, h_in.size, p, h_out, h_out.size)
        assert e.value.status == depix.ERR_INVALID_ARG
        assert b"outside the host buffers" in depix.lib().depix_last_error()
    # rejected before any staging allocation or copy
    assert depix.debug_live_allocations() == live
    assert (h_out == 77).all()
    ctx.batch_host(ws, hs, in_off, out_off, h_in, h_in.size, p, h_out, h_out.size)
    assert np.array_equal(h_out[:W * H * 64], _expected(imgs[0]))
    ctx.close()


def test_injected_allocation_failure_in_context_create(cuda):
    import depix
    base = depix.debug_live_allocations()
    try:
        for after in (0, 1):  # the first or the second scratch allocation fails
            depix.debug_fail_allocations(after)
            with pytest.raises(depix.DepixError) as e:
                depix.Context(W * H, 2)
            assert e.value.status == depix.ERR_ALLOC
            assert depix.debug_live_allocations() == base  # nothing leaked
    finally:
        depix.debug_fail_allocations(-1)
    ctx = depix.Context(W * H, 2)
    assert depix.debug_live_allocations() > base
    ctx.close()
    assert depix.debug_live_allocations() == base


def test_injected_allocation_failure_in_staging_growth(cuda):
    import depix
    ctx = depix.Context(W * H, 8)
    p = depix.params()
    small = _host_batch(_frames(1))
    ctx.batch_host(*small[:5], small[4].size, p, small[5], small[5].size)
    live = depix.debug_live_allocations()
    imgs = _frames(8, seed=3)
    big = _host_batch(imgs)
    try:
        depix.debug_fail_allocations(0)
        with pytest.raises(depix.DepixError) as e:
            ctx.batch_host(*big[:5], big[4].size, p, big[5], big[5].size)
        assert e.value.status == depix.ERR_ALLOC
        assert b"staging" in depix.lib().depix_last_error()
        # the failed growth released the old staging buffer it replaced
        assert depix.debug_live_allocations() <= live
    finally:
        depix.debug_fail_allocations(-1)
    # the context is still usable: the same batch now succeeds and is correct
    ctx.batch_host(*big[:5], big[4].size, p, big[5], big[5].size)
    for k, img in enumerate(imgs):
        assert np.array_equal(big[5][k * W * H * 64:(k + 1) * W * H * 64], _expected(img))
    ctx.close()


def test_graph_stage_wait_that_runs_out_reports_timeout(cuda):
    import depix
    torch = cuda
    img = np.ascontiguousarray(synth.frame(4))  # 256x224 RGBA: the TMA graph kernel
    h, w = img.shape[:2]
    d_img = torch.from_numpy(img.reshape(-1).copy()).cuda()
    out = torch.empty(w * h * 64, dtype=torch.uint8, device="cuda")
    graph = torch.empty(w * h, dtype=torch.uint8, device="cuda")
    ctx = depix.Context(w * h, 1)
    p = depix.params()
    torch.cuda.synchronize()
    assert depix.take_device_faults() == 0
    try:
        depix.debug_tma_timeout(True)
        ctx.frame(d_img, w, h, 4 * w, depix.LAYOUT_RGBA, p, out, graph, None)
        torch.cuda.synchronize()  # the launch ends: every wait is bounded
    finally:
        depix.debug_tma_timeout(False)
    flags = ctypes.c_int(0)
    status = depix.lib().depix_take_device_faults(ctypes.byref(flags))
    assert status == depix.ERR_TIMEOUT
    assert flags.value & 2  # the graph stage
    assert b"gave up" in depix.lib().depix_last_error()
    assert depix.take_device_faults() == 0  # cleared
    # the context and the device are still usable: the next frame is correct
    ctx.frame(d_img, w, h, 4 * w, depix.LAYOUT_RGBA, p, out, graph, None)
    torch.cuda.synchronize()
    bgr, ws = synth.rgba_to_bgr(img)
    f = O.frame(bgr, w, h, ws, 1, (48, 7, 6))
    assert np.array_equal(graph.cpu().numpy(), f.graph)
    assert np.array_equal(out.cpu().numpy().reshape(h * 4, w * 4, 4), O.raster(f.pos, f.col, w, h, 4))
    assert depix.take_device_faults() == 0
    ctx.close()
