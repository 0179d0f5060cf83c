"""Spline refinement on the GPU (depix_refine_*, through the C ABI) against
its CPU specification (oracle/refine_oracle.py, float64):
  * the frozen topology bit-exact: nodes, flags, neighbours, curve edges,
    segment slots and colours, sample assignment;
  * energies within 1e-5 relative, the adjoint gradient within 1e-4
    relative (2-norm) of the float64 analytic gradient and of float64
    central differences (h = 1e-4) on 256 random free nodes;
  * Adam on the GPU against Adam in float64;
  * a torch.autograd.Function over the adjoint (test harness only) driving
    torch's Adam, against the library's own loop;
  * the energy cut of 200 steps on the 256x224 frame."""
import numpy as np
import pytest

import oracle as O
import refine_oracle as R
from depix import synth

pytestmark = pytest.mark.gpu

GRAD_RTOL = 1e-4
ENERGY_RTOL = 1e-5


def _setup(torch, img, scale=4, rp=None):
    import depix
    h, w = img.shape[:2]
    bgr, ws = synth.rgba_to_bgr(img)
    raw, _, res = O.graph(bgr, w, h, ws, (48, 7, 6))
    d_img = torch.from_numpy(np.ascontiguousarray(img).reshape(-1).copy()).cuda()
    d_graph = torch.from_numpy(res.copy()).cuda()
    rf = depix.Refiner(w * h)
    rp = rp or depix.refine_params()
    rf.setup(d_img, w, h, 4 * w, depix.LAYOUT_RGBA, d_graph, depix.params(scale=scale), rp)
    return rf, rp, raw, res


def _compare_topology(g, top):
    assert np.array_equal(g["q"], np.stack([top.qx, top.qy], 1))
    assert np.array_equal(g["flags"], top.flags)
    assert np.array_equal(g["nbr"], top.nbr)
    assert np.array_equal(g["edges"], np.concatenate([top.eu[:, None], top.ev[:, None], top.ecell], 1))
    assert np.array_equal(g["segs"][:, :3], top.seg_nodes)
    assert np.array_equal(g["segs"][:, 3], top.seg_type)
    live = top.seg_type > 0
    packed = top.seg_col[..., 0] | top.seg_col[..., 1] << 8 | top.seg_col[..., 2] << 16
    assert np.array_equal(g["cols"][live].astype(np.int64), packed[live])
    order = np.argsort(g["samples"][:, 0], kind="stable")
    assert np.array_equal(g["samples"][order, 0], top.samp_idx)
    assert np.array_equal(g["samples"][order, 1], top.samp_seg)


@pytest.mark.parametrize("case", ["frame64x48", "sprite", "odd17x9", "scale3", "flat"])
def test_topology_matches_oracle(cuda, case):
    torch = cuda
    scale = 4
    if case == "frame64x48":
        img = synth.frame(0, w=64, h=48)
    elif case == "sprite":
        img = synth.sprites(6, seed=4)[5]
    elif case == "odd17x9":
        img = synth.frame(17, w=17, h=9)
    elif case == "scale3":
        img = synth.frame(2, w=40, h=30)
        scale = 3
    else:
        img = np.zeros((12, 20, 4), np.uint8)
        img[..., 3] = 255
    rf, rp, raw, res = _setup(torch, img, scale)
    top = R.topology(img, res, raw, scale)
    c = rf.counts()
    assert (c["nodes"], c["edges"], c["samples"]) == (len(top.qx), len(top.eu), len(top.samp_idx))
    assert c["free"] == int(top.free.sum())
    _compare_topology(rf.export(), top)
    rf.close()


def test_topology_of_the_256x224_frame(cuda):
    img = synth.frame(0)
    rf, rp, raw, res = _setup(cuda, img)
    top = R.topology(img, res, raw, 4)
    _compare_topology(rf.export(), top)
    rf.close()


@pytest.fixture(scope="module")
def small(cuda):
    img = synth.frame(0, w=64, h=48)
    rf, rp, raw, res = _setup(cuda, img)
    top = R.topology(img, res, raw, 4)
    yield cuda, img, rf, rp, top
    rf.close()


def _perturbed(torch, top, rf, seed=1, amp=0.05):
    N = len(top.qx)
    d_pos = torch.empty(N * 2, dtype=torch.float32, device="cuda")
    rf.initial(d_pos)
    P0 = d_pos.cpu().numpy().reshape(N, 2).astype(np.float64)
    assert np.array_equal(P0, R.initial_positions(top))
    rng = np.random.default_rng(seed)
    P = P0.copy()
    free = np.nonzero(top.free)[0]
    P[free] += rng.normal(0, amp, (len(free), 2))
    P = P.astype(np.float32).astype(np.float64)
    d_pos.copy_(torch.from_numpy(P.astype(np.float32).reshape(-1)))
    return d_pos, P, P0


@pytest.mark.parametrize("amp", [0.0, 0.05])
def test_energy_and_adjoint_match_float64(small, amp):
    torch, img, rf, rp, top = small
    d_pos, P, P0 = _perturbed(torch, top, rf, amp=amp)
    d_grad = torch.zeros_like(d_pos)
    e = rf.energy_grad(rp, d_pos, d_grad)
    parts, total, G = R.energy_grad(top, P, P0, img)
    for k in range(3):
        assert abs(e[k] - parts[k]) <= ENERGY_RTOL * max(abs(parts[k]), 1e-12) + 1e-12, (k, e[k], parts[k])
    assert abs(e[3] - total) <= ENERGY_RTOL * total
    g = d_grad.cpu().numpy().reshape(-1, 2).astype(np.float64)
    assert np.linalg.norm(g - G) <= GRAD_RTOL * np.linalg.norm(G)
    assert np.all(g[~top.free] == 0)


def test_adjoint_matches_central_differences(small):
    torch, img, rf, rp, top = small
    d_pos, P, P0 = _perturbed(torch, top, rf, seed=7)
    d_grad = torch.zeros_like(d_pos)
    rf.energy_grad(rp, d_pos, d_grad)
    g = d_grad.cpu().numpy().reshape(-1, 2).astype(np.float64)
    free = np.nonzero(top.free)[0]
    sel = np.random.default_rng(3).choice(free, 256, replace=False)
    fd = R.central_differences(top, P, P0, img, sel, h=1e-4)
    assert np.linalg.norm(g[sel] - fd) <= GRAD_RTOL * np.linalg.norm(fd)


def test_adjoint_on_the_256x224_frame(cuda):
    """The check of the workload's own frame (256x224, seed 0, x4): the
    adjoint at perturbed positions against the float64 analytic gradient on
    every node, and against float64 central differences (h = 1e-4) on 256
    random free nodes, each difference formed from the energy terms that
    touch its node (the rest cancel exactly)."""
    torch = cuda
    img = synth.frame(0)
    rf, rp, raw, res = _setup(torch, img)
    top = R.topology(img, res, raw, 4)
    d_pos, P, P0 = _perturbed(torch, top, rf, seed=11)
    d_grad = torch.zeros_like(d_pos)
    e = rf.energy_grad(rp, d_pos, d_grad)
    parts, total, G = R.energy_grad(top, P, P0, img)
    assert abs(e[3] - total) <= ENERGY_RTOL * total
    g = d_grad.cpu().numpy().reshape(-1, 2).astype(np.float64)
    assert np.linalg.norm(g - G) <= GRAD_RTOL * np.linalg.norm(G)
    free = np.nonzero(top.free)[0]
    sel = np.random.default_rng(5).choice(free, 256, replace=False)
    fd = R.central_differences_local(top, P, P0, img, sel, h=1e-4)
    assert np.linalg.norm(g[sel] - fd) <= GRAD_RTOL * np.linalg.norm(fd)
    assert np.linalg.norm(G[sel] - fd) <= 1e-6 * np.linalg.norm(fd)
    rf.close()


def test_adam_on_the_gpu_follows_float64_adam(small):
    """One step moves every node whose gradient is clear of float32 noise by
    the same amount as float64 Adam (the first Adam step is lr * g / (|g| +
    eps) per coordinate, so a gradient near zero may take either sign);
    after 40 steps the energies agree."""
    torch, img, rf, rp, top = small
    import depix
    N = len(top.qx)
    P0 = R.initial_positions(top)
    _, _, G = R.energy_grad(top, P0, P0, img)
    d_pos = torch.empty(N * 2, dtype=torch.float32, device="cuda")
    rf.initial(d_pos)
    rf.run(depix.refine_params(steps=1), d_pos)
    P1, _, _ = R.adam(top, img, steps=1)
    clear = np.abs(G) > 1e-3 * np.abs(G).max()
    got = d_pos.cpu().numpy().reshape(N, 2)
    assert clear.sum() > N // 4
    assert np.abs(got - P1)[clear].max() <= 1e-5
    rf.initial(d_pos)
    before, after = rf.run(depix.refine_params(steps=40), d_pos)
    _, e0, e1 = R.adam(top, img, steps=40)
    assert abs(before[3] - e0[1]) <= ENERGY_RTOL * e0[1]
    assert abs(after[3] - e1[1]) <= 1e-3 * e1[1]
    assert after[3] < before[3]


def test_autograd_function_with_torch_adam_matches_the_library_loop(small):
    torch, img, rf, rp, top = small
    import depix

    class RefineEnergy(torch.autograd.Function):
        @staticmethod
        def forward(ctx, pos):
            grad = torch.empty_like(pos)
            e = rf.energy_grad(rp, pos.detach(), grad)
            ctx.save_for_backward(grad)
            return pos.new_tensor(e[3])

        @staticmethod
        def backward(ctx, go):
            (grad,) = ctx.saved_tensors
            return go * grad

    N = len(top.qx)
    start = torch.empty(N * 2, dtype=torch.float32, device="cuda")
    rf.initial(start)
    g0 = torch.empty_like(start)
    rf.energy_grad(rp, start, g0)
    # coordinates whose gradient is clear of float32 noise (near zero, an
    # Adam step may take either sign, and the adjoint sums in any order)
    clear = g0.abs() > 1e-3 * g0.abs().max()
    for steps in (3, 10):
        pos = start.clone().requires_grad_(True)
        opt = torch.optim.Adam([pos], lr=0.05, betas=(0.9, 0.999), eps=1e-8)
        for _ in range(steps):
            opt.zero_grad()
            RefineEnergy.apply(pos).backward()
            opt.step()
        lib_pos = start.clone()
        _, after = rf.run(depix.refine_params(steps=steps), lib_pos)
        torch.cuda.synchronize()
        if steps == 3:
            assert torch.allclose(pos.detach()[clear], lib_pos[clear], atol=1e-4, rtol=0)
        e_torch = rf.energy_grad(rp, pos.detach())[3]
        assert abs(e_torch - after[3]) <= 1e-3 * after[3]


def test_200_steps_cut_the_energy_of_the_256x224_frame(cuda):
    img = synth.frame(0)
    rf, rp, raw, res = _setup(cuda, img)
    c = rf.counts()
    assert c["nodes"] > 5000
    before, after = rf.run(rp)
    assert after[3] <= 0.7 * before[3], (before, after)
    rf.close()


def test_setup_rejects_bad_arguments(cuda):
    import depix
    torch = cuda
    img = synth.frame(1, w=16, h=16)
    rf = depix.Refiner(16 * 16)
    d_img = torch.from_numpy(img.reshape(-1).copy()).cuda()
    d_graph = torch.zeros(256, dtype=torch.uint8, device="cuda")
    with pytest.raises(depix.DepixError):
        rf.setup(d_img, 16, 16, 64, depix.LAYOUT_RGBA, d_graph, depix.params(scale=13), depix.refine_params())
    with pytest.raises(depix.DepixError):
        rf.setup(d_img, 32, 16, 128, depix.LAYOUT_RGBA, d_graph, depix.params(), depix.refine_params())
    rf.setup(d_img, 16, 16, 64, depix.LAYOUT_RGBA, d_graph, depix.params(), depix.refine_params())
    pos = torch.zeros(2 * max(rf.counts()["nodes"], 1), dtype=torch.float32, device="cuda")
    with pytest.raises(depix.DepixError):
        rf.energy_grad(depix.refine_params(sigma=1.0), pos)
    rf.close()


def test_warm_start_from_the_previous_frame(cuda):
    """Two frames of a stream: the second warm-starts from the first's
    refined nodes in tiles whose signature is unchanged (checked against the
    float64 specification's rule and its own tile signatures)."""
    import depix
    torch = cuda
    frames = synth.stream(3, seed=2, n_sprites=2, w=128, h=96)  # 19 of 48 tiles unchanged
    a, b = frames[0], frames[2]
    rfa, rp, raw_a, res_a = _setup(torch, a)
    rfb, _, raw_b, res_b = _setup(torch, b)
    top_a = R.topology(a, res_a, raw_a, 4)
    top_b = R.topology(b, res_b, raw_b, 4)
    pos_a = torch.empty(2 * len(top_a.qx), dtype=torch.float32, device="cuda")
    rfa.initial(pos_a)
    rfa.run(depix.refine_params(steps=50), pos_a)
    pos_b = torch.empty(2 * len(top_b.qx), dtype=torch.float32, device="cuda")
    reused = rfb.warm_start(rfa, pos_a, pos_b)
    sig_a, tx = R.tile_signatures(a, res_a)
    sig_b, _ = R.tile_signatures(b, res_b)
    same = sum(x == y for x, y in zip(sig_a, sig_b))
    assert reused == same and 0 < same < len(sig_a)
    want = R.warm_positions(top_b, sig_b, top_a, sig_a, pos_a.cpu().numpy().reshape(-1, 2).astype(np.float64), tx)
    got = pos_b.cpu().numpy().reshape(-1, 2).astype(np.float64)
    assert np.array_equal(got, want)
    moved = np.any(want != R.initial_positions(top_b), axis=1)
    assert moved.sum() > 10  # some nodes really carried over
    # refinement from the warm start
    before, after = rfb.run(depix.refine_params(steps=20), pos_b)
    assert after[3] < before[3]
    rfa.close()
    rfb.close()


def test_setup_resolves_the_graph_itself(cuda):
    import depix
    torch = cuda
    img = synth.frame(3, w=64, h=40)
    rf, rp, raw, res = _setup(torch, img)
    g1 = rf.export()
    d_img = torch.from_numpy(np.ascontiguousarray(img).reshape(-1).copy()).cuda()
    rf2 = depix.Refiner(64 * 40)
    rf2.setup(d_img, 64, 40, 256, depix.LAYOUT_RGBA, None, depix.params(), rp)
    g2 = rf2.export()
    for k in g1:
        assert np.array_equal(g1[k], g2[k]), k
    rf.close()
    rf2.close()


def test_setups_on_side_streams_then_a_warm_started_chain(cuda):
    """Setups that return before their work is done: four frames of a stream
    set up at once, each on its own stream (the graph resolved by the
    refiner), then initial / warm start and 20 steps frame after frame on a
    third stream that waits on each setup's event. Topologies bit-exact
    against the specification; every frame's energy lowered by its steps and
    within 1 % of the same calls made one after another on one stream (the
    coverage gradient is summed with float atomics, whose order, and through
    Adam's normalised step the positions, depend on what else runs);
    positions finite and within Adam's reach of their start."""
    import depix
    torch = cuda
    w, h = 128, 96
    frames = synth.stream(4, seed=1, n_sprites=2, w=w, h=h)
    d_imgs = [torch.from_numpy(np.ascontiguousarray(f).reshape(-1).copy()).cuda() for f in frames]
    rp = depix.refine_params(steps=20)
    p = depix.params()
    cap = 2 * (4 * w + 3) * (4 * h + 3)

    def chain(rfs, setup_streams, main):
        done = []
        for k, rf in enumerate(rfs):
            rf.setup(d_imgs[k], w, h, 4 * w, depix.LAYOUT_RGBA, None, p, rp, stream=setup_streams[k])
            ev = torch.cuda.Event()
            ev.record(setup_streams[k])
            done.append(ev)
        pos = [torch.zeros(cap, dtype=torch.float32, device="cuda") for _ in rfs]
        start = [torch.zeros(cap, dtype=torch.float32, device="cuda") for _ in rfs]
        for k, rf in enumerate(rfs):
            main.wait_event(done[k])
            if k == 0:
                rf.initial(pos[k], stream=main)
            else:
                rf.warm_start(rfs[k - 1], pos[k - 1], pos[k], stream=main, count=False)
            with torch.cuda.stream(main):
                start[k].copy_(pos[k])
            rf.run(rp, pos[k], stream=main, energies=False)
        torch.cuda.synchronize()
        return pos, start

    side = [torch.cuda.Stream() for _ in frames]
    main = torch.cuda.Stream()
    rfs = [depix.Refiner(w * h) for _ in frames]
    got, got_start = chain(rfs, side, main)
    one = torch.cuda.current_stream()
    rfs_seq = [depix.Refiner(w * h) for _ in frames]
    want, _ = chain(rfs_seq, [one] * len(frames), one)
    for k, f in enumerate(frames):
        bgr, ws = synth.rgba_to_bgr(f)
        raw, _, res = O.graph(bgr, w, h, ws, (48, 7, 6))
        top = R.topology(f, res, raw, 4)
        _compare_topology(rfs[k].export(), top)
        n = 2 * len(top.qx)
        assert bool(torch.isfinite(got[k][:n]).all()), f"frame {k}"
        # an Adam step moves a coordinate by at most lr (1 - beta1) / sqrt(1 - beta2) = 3.16 lr
        assert float((got[k][:n] - got_start[k][:n]).abs().max()) <= 20 * rp.lr * 3.2, f"frame {k}"
        assert bool(torch.all(got[k][n:] == 0)), f"frame {k}: written past its nodes"
        e_start = rfs[k].energy_grad(rp, got_start[k])[3]
        e_got = rfs[k].energy_grad(rp, got[k])[3]
        e_want = rfs_seq[k].energy_grad(rp, want[k])[3]
        assert e_got < e_start, f"frame {k}"
        assert abs(e_got - e_want) <= 1e-2 * e_want, f"frame {k}: {e_got} against {e_want}"
    for rf in rfs + rfs_seq:
        rf.close()
