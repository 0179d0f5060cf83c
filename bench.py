#!/usr/bin/env python
"""Benchmark of the depixelization frame path on GB300.

Workload: 256x224 RGBA8 frames from the seeded benchmark-frame generator
(16 colours, 40 rectangles + 30 ellipses, dark outlines, 5 % dither),
similarity graph (Y 48, U 7, V 6) -> crossing resolution -> component labels
-> reshaped cells -> one subdivision round -> triangles -> x4 raster
(1024x896 RGBA8). A step is one batch of frames through depix_batch.

Prints one JSON line. ``value`` is frames/s of the batched path with inputs
resident in HBM; ``e2e`` is the same through depix_batch_host with the copies
from and to pinned host memory inside the timed region; ``plain`` is the
per-frame path (one launch per stage and frame) with its p50/p99 latency;
``roofline`` covers the dominant kernel (the fused cells/subdivision/
triangle/raster kernel); ``cpu_baseline`` is the CPU oracle (a C restatement
of the reference's per-pixel stage bodies) on this host's cores.

--impl reference times that CPU implementation itself on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "pixel-art-remaster-gpu_gb300")
ORACLE = os.path.join(REPO, "oracle")
sys.path.insert(0, PKG)

W, H, SCALE = 256, 224, 4
METRIC = "frames/s, 256x224 RGBA8 -> x4 (1024x896), batched"
UNIT = "frames/s"
DISTINCT = 64


def workload_config(batch):
    return {
        "workload": "256x224 RGBA8 synthetic frames (16 colours, 40 rects + 30 ellipses, 50% outlined, 5% dither), "
                    "graph Y48/U7/V6 + trivial + heuristics, component labels, cells + 1 subdivision round + "
                    "triangles, x4 raster to 1024x896 RGBA8",
        "frames_per_step": batch,
        "distinct_frames": DISTINCT,
        "l2_policy": "inputs larger than L2: %.0f MB read and %.0f MB written per step vs 129 MB L2"
                     % (batch * W * H * 5 / 1e6, batch * W * H * (SCALE * SCALE * 4 + 4) / 1e6),
        "parallelism": "replicas",
    }


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=1024, help="frames per step")
    ap.add_argument("--plain-frames", type=int, default=300)
    ap.add_argument("--e2e-steps", type=int, default=0, help="default: max(200, steps // 5)")
    ap.add_argument("--cpu-sample", type=int, default=0, help="frames in the CPU-baseline sample (default 4 x cores)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--sprites", type=int, default=4096, help="sprites in the uneven-batch leg")
    ap.add_argument("--no-sprites", action="store_true")
    ap.add_argument("--no-refine", action="store_true")
    ap.add_argument("--no-stream", action="store_true")
    ap.add_argument("--no-vote", action="store_true")
    ap.add_argument("--no-walks", action="store_true")
    ap.add_argument("--no-large", action="store_true")
    ap.add_argument("--large-frames", type=int, default=16, help="640x480 frames per step in the x8 leg")
    ap.add_argument("--large-only", action="store_true", help="run only the 640x480 x8 leg (for profiling)")
    ap.add_argument("--stream-frames", type=int, default=512)
    ap.add_argument("--latency-frames", type=int, default=400, help="plain calls in the latency sweep")
    return ap.parse_args()


def make_frames(n_distinct):
    import numpy as np
    from depix import synth
    return np.stack([synth.frame(seed) for seed in range(n_distinct)])


# ------------------------------------------------------------- CPU baseline


def cpu_path_frame(img, kind):
    """The whole path on one frame on the CPU. kind "reference": the
    reference's own per-pixel stage bodies (its host build, oracle/_ref) from
    the graph to the VBO, then the component labels and the x4 raster of that
    VBO through the CPU oracle (the reference draws with OpenGL, unavailable
    here, and has no labelling stage). kind "port": all of it through the CPU
    oracle (oracle/depix_oracle.c, a C restatement of the same stages)."""
    import oracle as O
    from depix import synth
    bgr, ws = synth.rgba_to_bgr(img)
    if kind == "reference":
        graph, pos, col = O.ref_frame_vbo(bgr, W, H, ws, 1, 48)
    else:
        f = O.frame(bgr, W, H, ws, 1, (48, 7, 6))
        graph, pos, col = f.graph, f.pos, f.col
    O.label_cc(graph, W, H)
    O.raster(pos, col, W, H, SCALE)


def cpu_run(frames, n_frames, threads, kind):
    """frames/s of the CPU path over n_frames frames on `threads` threads
    (the C calls release the GIL)."""
    from concurrent.futures import ThreadPoolExecutor
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(lambda k: cpu_path_frame(frames[k % len(frames)], kind), range(n_frames)))
    return n_frames / (time.perf_counter() - t0)


def cpu_setup():
    """Builds the CPU oracle and the reference's host build (from the staged
    reference sources, for this machine's CPU); returns the core count and
    the kind of CPU path available ("reference" when the host build is)."""
    if ORACLE not in sys.path:
        sys.path.insert(0, ORACLE)
    import oracle as O
    O.build()
    kind = "reference" if O.build_ref(gpu=False) else "port"
    return os.cpu_count() or 1, kind


CPU_SAMPLE = {
    "reference": "the reference's own per-pixel stage bodies (graph_functions.cu, diagram_functions.cu, "
                 "subdivision_functions.cu, triangulate_functions.cu, point.cu; host build with g++ -O2, Y 48, "
                 "oracle/ref_driver.cpp replaying launch_kernel's stage order) from the graph to the VBO, then "
                 "labels and the x4 raster of that VBO through the CPU oracle (the reference's raster is an OpenGL "
                 "draw, unavailable here; it has no labelling stage)",
    "port": "the CPU oracle (oracle/depix_oracle.c, a C restatement of the reference's stage bodies: graph, "
            "resolution, cells, subdivision, ear clip, VBO fill, labels, x4 raster)",
}


# ------------------------------------------------------------------- clocks


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- our arm


def measured_peak():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes per frame of the raster kernel from the committed ncu summary."""
    path = os.path.join(REPO, "profiles", "k_mask_raster_tma_256x224_x4.md")
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_frame:"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def run_ours(args, rank, world, local_rank):
    import numpy as np
    import torch
    import depix
    from depix import replicas

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    depix.init_device()
    B = args.batch
    frames = make_frames(DISTINCT)
    tiled = np.ascontiguousarray(np.resize(frames, (B, H, W, 4)))
    in_bytes, out_px = W * H * 4, W * H * SCALE * SCALE
    d_in = torch.from_numpy(tiled.reshape(-1)).to(dev)
    d_out = torch.empty(B * out_px * 4, dtype=torch.uint8, device=dev)
    d_lab = torch.empty(B * W * H, dtype=torch.int32, device=dev)
    ctx = depix.Context(W * H, B)
    p = depix.params(48, 7, 6, True, SCALE)
    ws, hs = np.full(B, W, np.int32), np.full(B, H, np.int32)
    in_off = np.arange(B, dtype=np.uint64) * np.uint64(in_bytes)
    out_off = np.arange(B, dtype=np.uint64) * np.uint64(out_px * 4)
    stream = torch.cuda.current_stream(dev)

    def step():
        ctx.batch(ws, hs, in_off, out_off, d_in, p, d_out, d_lab, stream=stream)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    ctx.stage_times()  # reset

    clocks = ClockSampler(local_rank)
    clocks.start()
    ctx.set_timing(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ctx.set_timing(False)
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    stages = ctx.stage_times()
    # replicas: every rank ran its own B frames per step; the job's time is the slowest rank's
    ms = replicas.max_over_ranks(ms, dev)
    value = replicas.job_throughput(B * args.steps, ms / 1e3, dev)

    # roofline of the kernel that writes the output (the raster stage: one
    # kernel per call); algorithmic bytes: image and graph in, raster out
    r_ms, r_launches, r_calls = stages["raster"]
    raster_ms = r_ms / max(r_calls, 1)
    alg_bytes = B * (W * H * 4 + W * H * 1 + out_px * 4)
    achieved = alg_bytes / (raster_ms / 1e3) / 1e9
    peak, peak_kind = measured_peak()
    tpf = profiled_traffic()
    roofline = {"kernel": "k_mask_raster_tma (TMA pixel windows, cell masks, block resolution, 16-byte output stores)", "bound": "hbm",
                "achieved": round(achieved, 1), "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": (tpf * B if tpf else None),
                "alg_bytes_per_launch": alg_bytes, "avg_launch_ms": round(raster_ms, 4),
                "stage_ms_per_step": {k: round(v[0] / max(v[2], 1), 4) for k, v in stages.items()}}
    launches = sum(v[1] for v in stages.values())

    # end to end through the host-buffer call, copies inside the timed region
    e2e = None
    e2e_steps = args.e2e_steps or max(200, args.steps // 5)  # ~4 s: one stall of the shared link weighs little
    h_in = torch.from_numpy(tiled.reshape(-1)).pin_memory()
    h_out = torch.empty(B * out_px * 4, dtype=torch.uint8).pin_memory()
    h_lab = torch.empty(B * W * H, dtype=torch.int32).pin_memory()
    for _ in range(2):
        ctx.batch_host(ws, hs, in_off, out_off, h_in, h_in.numel(), p, h_out, h_out.numel(), h_lab, stream=stream)
    barrier()
    step_ms = []
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ts = time.perf_counter()
        # returns when the step's last copy to host memory is done
        ctx.batch_host(ws, hs, in_off, out_off, h_in, h_in.numel(), p, h_out, h_out.numel(), h_lab, stream=stream)
        step_ms.append((time.perf_counter() - ts) * 1e3)
    e2e_s = time.perf_counter() - t0
    e2e_v = replicas.job_throughput(B * e2e_steps, e2e_s, dev)
    step_ms.sort()
    # value: all timed steps; the per-step spread shows when the shared host
    # link was busy with other traffic during some steps
    e2e = {"value": round(e2e_v, 1), "unit": UNIT, "h2d_bytes_per_step": B * in_bytes,
           "d2h_bytes_per_step": B * (out_px * 4 + W * H * 4), "steps": e2e_steps,
           "timed_s": round(e2e_s, 3), "step_ms": {"min": round(step_ms[0], 2),
                                                  "median": round(step_ms[len(step_ms) // 2], 2),
                                                  "max": round(step_ms[-1], 2)}}

    # frames of both paths against the CPU oracle (a C restatement of the
    # reference's stage bodies): rasters and labels of a few frames of the
    # last device-resident batch and of the last host-buffer batch
    check = check_against_oracle(frames, d_out, d_lab, h_out, h_lab, B)

    # per-frame latency, plain and batched: from the start of a frame's (or
    # batch's) upload from pinned host memory to its last kernel, on the
    # stream, over back-to-back calls; frames/s over the same calls
    latency = run_latency(args, dev, stream, ctx, frames, B)

    # plain per-frame path, device-resident input: one launch per stage and frame
    pf = max(args.plain_frames, 10)
    ctx1 = depix.Context(W * H, 1)
    lat = []
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(pf)]
    for k in range(5):
        ctx1.frame(d_in[k * in_bytes:], W, H, 4 * W, depix.LAYOUT_RGBA, p, d_out, None, d_lab, stream=stream)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(pf):
        a, b = evs[k]
        a.record(stream)
        f = k % B
        ctx1.frame(d_in[f * in_bytes:], W, H, 4 * W, depix.LAYOUT_RGBA, p, d_out[f * out_px * 4:], None,
                   d_lab[f * W * H:], stream=stream)
        b.record(stream)
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - t0
    lat = sorted(a.elapsed_time(b) for a, b in evs)
    plain = {"frames_per_s": round(pf / plain_s, 1), "p50_ms_per_frame": round(lat[len(lat) // 2], 4),
             "p99_ms_per_frame": round(lat[min(len(lat) - 1, int(0.99 * len(lat)))], 4), "frames": pf}
    ctx1.close()

    # the same batch with the weighted-vote heuristics (depix_params.vote)
    vote = None
    if not args.no_vote:
        pv = depix.params(48, 7, 6, True, SCALE, vote=True)
        for _ in range(3):
            ctx.batch(ws, hs, in_off, out_off, d_in, pv, d_out, d_lab, stream=stream)
        torch.cuda.synchronize()
        ctx.stage_times()
        ctx.set_timing(True)
        vsteps = max(10, args.steps // 10)
        e0.record(stream)
        for _ in range(vsteps):
            ctx.batch(ws, hs, in_off, out_off, d_in, pv, d_out, d_lab, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ctx.set_timing(False)
        vst = ctx.stage_times()
        vms = e0.elapsed_time(e1)
        vote = {"frames_per_s": round(B * vsteps / (vms / 1e3), 1), "ms_per_step": round(vms / vsteps, 4),
                "steps": vsteps, "stage_ms_per_step": {k: round(v[0] / max(v[2], 1), 4) for k, v in vst.items()}}

    walks = None if args.no_walks else run_walks(args, dev, stream, d_in, cpu=(rank == 0 and world == 1 and not args.no_cpu))
    large = None if args.no_large else run_large(args, dev, stream)

    sprites = None if args.no_sprites else run_sprites(args, dev, stream)
    refine = None if args.no_refine else run_refine(args, dev, stream, cpu=(rank == 0 and world == 1 and not args.no_cpu))
    stream_leg = None if args.no_stream else run_stream(args, dev, stream)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cores, kind = cpu_setup()
        n = args.cpu_sample or 4 * cores
        cpu_run(frames, min(cores, n), cores, kind)  # warm
        v = cpu_run(frames, n, cores, kind)
        v1 = cpu_run(frames, 4, 1, kind)
        cpu = {"value": round(v, 2), "unit": UNIT, "cores": cores, "kind": kind,
               "sample": f"{n} frames of the same workload, {cores} threads, one frame each: " + CPU_SAMPLE[kind],
               "single_thread_value": round(v1, 2)}
        if kind == "reference":
            cpu["port_value"] = round(cpu_run(frames, n, cores, "port"), 2)
    ctx.close()
    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic (seeded generator)",
                "config": workload_config(B), "e2e": e2e, "plain": plain, "latency": latency,
                "oracle_check": check, "roofline": roofline,
                "cpu_baseline": cpu, "clocks": clk, "gpu_launches": launches, "sprites": sprites,
                "refine": refine, "stream": stream_leg, "vote": vote, "border_walks": walks,
                "large_x8": large}
        print(json.dumps(line))


def check_against_oracle(frames, d_out, d_lab, h_out, h_lab, B):
    """Frames 0, 1 and B-1 of the device-resident batch (d_out, d_lab) and of
    the host-buffer batch (h_out, h_lab) against the CPU oracle: raster and
    labels bit-exact. Raises on a mismatch."""
    import numpy as np
    if ORACLE not in sys.path:
        sys.path.insert(0, ORACLE)
    import oracle as O
    from depix import synth
    O.build()
    out_px = W * H * SCALE * SCALE
    checked = []
    for k in sorted({0, 1, B - 1}):
        img = frames[k % len(frames)]
        bgr, ws = synth.rgba_to_bgr(img)
        f = O.frame(bgr, W, H, ws, 1, (48, 7, 6))
        want_r = O.raster(f.pos, f.col, W, H, SCALE).reshape(-1)
        want_l = O.label_cc(f.graph, W, H)
        for name, r, l in (("device", d_out, d_lab), ("host", h_out, h_lab)):
            got_r = r[k * out_px * 4:(k + 1) * out_px * 4].cpu().numpy()
            got_l = l[k * W * H:(k + 1) * W * H].cpu().numpy()
            assert np.array_equal(got_r, want_r), f"{name} batch frame {k}: raster differs from the oracle"
            assert np.array_equal(got_l, want_l), f"{name} batch frame {k}: labels differ from the oracle"
        checked.append(k)
    return {"frames": checked, "paths": ["device batch", "host-buffer batch"],
            "compared": "x4 raster and component labels, bit-exact, against the CPU oracle"}


def run_latency(args, dev, stream, ctx, frames, B_max):
    """Per-frame latency of the plain path (one depix_frame call per frame)
    and of batches of 8, 32, 128 and 1024 frames through depix_batch, each
    call preceded by the upload of its frames from pinned host memory. A
    frame's latency is its call's: from the start of the upload to the end
    of the call's last kernel (CUDA events on the stream). frames/s: frames
    over the wall time of the back-to-back calls."""
    import numpy as np
    import torch
    import depix
    in_bytes, out_px = W * H * 4, W * H * SCALE * SCALE
    p = depix.params(48, 7, 6, True, SCALE)
    n_frames = max(args.latency_frames, 64)
    h_all = torch.from_numpy(np.ascontiguousarray(np.resize(frames, (max(B_max, 1024), H, W, 4))).reshape(-1))
    h_all = h_all.pin_memory()
    d_in = torch.empty(max(B_max, 1024) * in_bytes, dtype=torch.uint8, device=dev)
    d_out = torch.empty(max(B_max, 1024) * out_px * 4, dtype=torch.uint8, device=dev)
    d_lab = torch.empty(max(B_max, 1024) * W * H, dtype=torch.int32, device=dev)
    ev = lambda: torch.cuda.Event(enable_timing=True)
    pct = lambda v, q: round(float(v[min(len(v) - 1, int(q * len(v)))]), 4)

    def measure(b, calls, run):
        marks = [(ev(), ev()) for _ in range(calls)]
        for k in range(3):
            run(k % max(1, (1024 // b)))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(calls):
            a, e = marks[k]
            a.record(stream)
            run(k % max(1, (1024 // b)))
            e.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        lat = sorted(a.elapsed_time(e) for a, e in marks)
        return {"frames_per_s": round(b * calls / wall, 1), "p50_ms": pct(lat, 0.5), "p99_ms": pct(lat, 0.99),
                "calls": calls}

    ctx1 = depix.Context(W * H, 1)

    def plain(slot):
        d = d_in[slot * in_bytes:(slot + 1) * in_bytes]
        d.copy_(h_all[slot * in_bytes:(slot + 1) * in_bytes], non_blocking=True)
        ctx1.frame(d, W, H, 4 * W, depix.LAYOUT_RGBA, p, d_out[slot * out_px * 4:], None, d_lab[slot * W * H:],
                   stream=stream)

    out = {"definition": "frame latency = its call's time from the start of the upload of the call's frames "
                         "(pinned host -> device) to the end of its last kernel; frames/s over back-to-back calls",
           "plain": dict(measure(1, n_frames, plain), batch=1)}
    out["plain"]["frames"] = n_frames
    rows = []
    for b in (8, 32, 128, 1024):
        if b > B_max:
            continue
        ws_b, hs_b = np.full(b, W, np.int32), np.full(b, H, np.int32)
        io = np.arange(b, dtype=np.uint64) * np.uint64(in_bytes)
        oo = np.arange(b, dtype=np.uint64) * np.uint64(out_px * 4)

        def batched(slot, b=b, ws_b=ws_b, hs_b=hs_b, io=io, oo=oo):
            base = slot * b
            d_in[base * in_bytes:(base + b) * in_bytes].copy_(h_all[base * in_bytes:(base + b) * in_bytes],
                                                              non_blocking=True)
            ctx.batch(ws_b, hs_b, io, oo, d_in[base * in_bytes:], p, d_out[base * out_px * 4:], d_lab[base * W * H:],
                      stream=stream)

        calls = max(8, min(200, (n_frames * 4) // b))
        r = measure(b, calls, batched)
        r["batch"] = b
        r["beats_plain_frames_per_s"] = r["frames_per_s"] > out["plain"]["frames_per_s"]
        r["p99_under_1ms"] = r["p99_ms"] < 1.0
        rows.append(r)
    ctx1.close()
    out["batched"] = rows
    ok = [r["batch"] for r in rows if r["beats_plain_frames_per_s"] and r["p99_under_1ms"]]
    out["batches_beating_plain_with_p99_under_1ms"] = ok
    return out


def run_large(args, dev, stream):
    """The 640x480 workload upscaled x8 (5120x3840 per frame), batched with
    labels: frames/s, per-stage times and the raster's roofline."""
    import numpy as np
    import torch
    import depix
    from depix import synth
    B, LW, LH, LS = args.large_frames, 640, 480, 8
    imgs = np.stack([synth.frame_large(s) for s in range(B)])
    in_bytes, out_px = LW * LH * 4, LW * LH * LS * LS
    d_img = torch.from_numpy(imgs.reshape(-1)).to(dev)
    d_out = torch.empty(B * out_px * 4, dtype=torch.uint8, device=dev)
    d_lab = torch.empty(B * LW * LH, dtype=torch.int32, device=dev)
    ctx = depix.Context(LW * LH, B)
    p = depix.params(48, 7, 6, True, LS)
    ws, hs = np.full(B, LW, np.int32), np.full(B, LH, np.int32)
    in_off = np.arange(B, dtype=np.uint64) * np.uint64(in_bytes)
    out_off = np.arange(B, dtype=np.uint64) * np.uint64(out_px * 4)

    def step():
        ctx.batch(ws, hs, in_off, out_off, d_img, p, d_out, d_lab, stream=stream)

    for _ in range(3):
        step()
    torch.cuda.synchronize()
    steps = max(3, min(args.steps, 20))
    ctx.stage_times()
    ctx.set_timing(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ctx.set_timing(False)
    ms = e0.elapsed_time(e1) / steps
    st = {k: round(v[0] / max(v[2], 1), 4) for k, v in ctx.stage_times().items()}
    ctx.close()
    alg = B * (LW * LH * (4 + 1) + out_px * 4)
    peak, peak_kind = measured_peak()
    achieved = alg / (st["raster"] / 1e3) / 1e9
    return {"workload": f"{B} frames 640x480 RGBA8 (64 colours, 200 shapes, 10% dither, 2% noise) -> x8 5120x3840, "
                        "labels, subdivision", "frames_per_s": round(B / (ms / 1e3), 1), "ms_per_step": round(ms, 3),
            "out_mpix_per_s": round(B * out_px / (ms / 1e3) / 1e6, 1), "steps": steps, "stage_ms_per_step": st,
            "raster_roofline": {"achieved": round(achieved, 1), "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                                "frac": round(achieved / peak, 4), "alg_bytes_per_step": alg}}


def run_walks(args, dev, stream, d_in, cpu):
    """Border walks (the spline export's input) of a batch of resolved
    graphs: the graphs of the distinct frames tiled to the batch size, one
    warp per frame; CUDA-event time per batch."""
    import numpy as np
    import torch
    import depix
    B, N = args.batch, W * H
    p = depix.params(48, 7, 6, True, SCALE)
    fused = torch.empty(N, dtype=torch.uint8, device=dev)
    graphs = torch.empty(B * N, dtype=torch.uint8, device=dev)
    for k in range(DISTINCT):
        depix.graph(d_in[k * N * 4:], W, H, 4 * W, depix.LAYOUT_RGBA, p, fused, stream=stream)
        depix.resolve_heuristics(fused, W, H, graphs[k * N:], stream=stream)
    for k in range(DISTINCT, B):
        graphs[k * N:(k + 1) * N].copy_(graphs[(k % DISTINCT) * N:(k % DISTINCT + 1) * N])
    max_nodes, max_walks = N, N // 4
    scratch = torch.empty(B * N, dtype=torch.uint8, device=dev)
    nodes = torch.empty(B * max_nodes, dtype=torch.int32, device=dev)
    edges = torch.empty(B * max_nodes, dtype=torch.int8, device=dev)
    offs = torch.empty(B * (max_walks + 1), dtype=torch.int32, device=dev)
    counts = torch.empty(3 * B, dtype=torch.int32, device=dev)

    def step():
        depix.border_walks(graphs, W, H, B, scratch, nodes, edges, offs, max_nodes, max_walks, counts, stream)

    for _ in range(3):
        step()
    torch.cuda.synchronize()
    steps = 5
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    c = counts.cpu().numpy().reshape(B, 3)
    assert not c[:, 2].any(), "border-walk capacity ran out"
    out = {"workload": f"{B} resolved graphs {W}x{H} ({DISTINCT} distinct frames), one warp per frame",
           "frames_per_s": round(B / (ms / 1e3), 1), "ms_per_batch": round(ms, 3), "steps": steps,
           "walks_per_frame": round(float(c[:, 0].mean()), 1), "nodes_per_frame": round(float(c[:, 1].mean()), 1)}
    if cpu:
        if ORACLE not in sys.path:
            sys.path.insert(0, ORACLE)
        import oracle as O
        g0 = graphs[:N].cpu().numpy()
        t0 = time.perf_counter()
        n = 0
        while n < 8 or time.perf_counter() - t0 < 1.0:
            O.border_walks(g0, W, H)
            n += 1
        out["cpu_baseline"] = {"frames_per_s": round(n / (time.perf_counter() - t0), 1), "cores": 1, "kind": "port",
                               "sample": f"{n} walks of one frame through the CPU oracle (oracle/depix_oracle.c)"}
    return out


def run_sprites(args, dev, stream):
    """Uneven batch: 4096 sprites with sides ~ U[8, 64] (30 % transparent
    backgrounds), x4, with labels, in one depix_batch call per step (the
    persistent tile-queue path, replayed as a graph, launch shape tuned on
    the first call), against one plain per-frame call per sprite."""
    import numpy as np
    import torch
    import depix
    from depix import synth

    imgs = synth.sprites(args.sprites, seed=0)
    ws, hs = [i.shape[1] for i in imgs], [i.shape[0] for i in imgs]
    in_off, out_off, oi, oo = [], [], 0, 0
    for w, h in zip(ws, hs):
        in_off.append(oi)
        out_off.append(oo)
        oi += (w * h * 4 + 15) // 16 * 16
        oo += (w * h * 64 + 15) // 16 * 16
    # per-frame arrays as numpy: the binding passes them by pointer
    ws_a, hs_a = np.array(ws, np.int32), np.array(hs, np.int32)
    in_a, out_a = np.array(in_off, np.uint64), np.array(out_off, np.uint64)
    buf = np.zeros(oi, np.uint8)
    for k, img in enumerate(imgs):
        buf[in_off[k]:in_off[k] + img.size] = img.reshape(-1)
    npx = sum(w * h for w, h in zip(ws, hs))
    d_in = torch.from_numpy(buf).to(dev)
    d_out = torch.empty(oo, dtype=torch.uint8, device=dev)
    d_lab = torch.empty(npx, dtype=torch.int32, device=dev)
    p = depix.params(48, 7, 6, True, SCALE)
    ctx = depix.Context(64 * 64, len(imgs))

    def step():
        ctx.batch(ws_a, hs_a, in_a, out_a, d_in, p, d_out, d_lab, stream=stream)

    t0 = time.perf_counter()
    step()  # tunes the launch shape for this size bucket
    torch.cuda.synchronize()
    tune_s = time.perf_counter() - t0
    for _ in range(3):
        step()
    steps = max(10, args.steps // 3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    ctx.set_timing(True)
    for _ in range(5):
        step()
    torch.cuda.synchronize()
    ctx.set_timing(False)
    st = ctx.stage_times()
    gran, tw, th = ctx.launch_shape()

    # plain: one depix_frame call (one launch per stage) per sprite
    ctx1 = depix.Context(64 * 64, 1)

    def plain():
        for k in range(len(imgs)):
            ctx1.frame(d_in[in_off[k]:], ws[k], hs[k], 4 * ws[k], depix.LAYOUT_RGBA, p, d_out[out_off[k]:], None,
                       d_lab, stream=stream)

    plain()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    t0 = time.perf_counter()
    plain()
    b.record(stream)
    torch.cuda.synchronize()
    plain_wall = time.perf_counter() - t0
    plain_ms = a.elapsed_time(b)
    ctx1.close()
    ctx.close()
    n = len(imgs)
    return {"workload": f"{n} sprites, sides ~ U[8,64] (seeded generator), {npx} px in, x4 RGBA8 out, labels",
            "frames_per_s": round(n / (ms / 1e3), 1), "ms_per_batch": round(ms, 4),
            "out_mpix_per_s": round(npx * SCALE * SCALE / (ms / 1e3) / 1e6, 1), "steps": steps,
            "stage_ms_per_batch": {k: round(v[0] / max(v[2], 1), 4) for k, v in st.items()},
            "launch_shape": {"gran": list(gran), "raster_tile": [tw, th]}, "first_call_s": round(tune_s, 3),
            "plain_frames_per_s": round(n / (plain_ms / 1e3), 1), "plain_host_wall_s": round(plain_wall, 3)}


def run_refine(args, dev, stream, cpu):
    """Spline refinement of the 256x224 frame: topology setup, then 200 Adam
    steps of the curvature + deviation + soft-coverage energy (x4, sigma 0.5
    output px) through the adjoint kernel; steps/s, ms per frame, energy cut;
    the float64 CPU specification timed on a few steps beside it."""
    import numpy as np
    import torch
    import depix

    img = make_frames(1)[0]
    d_img = torch.from_numpy(np.ascontiguousarray(img).reshape(-1)).to(dev)
    ctx = depix.Context(W * H, 1)
    p = depix.params(48, 7, 6, True, SCALE)
    d_graph = torch.empty(W * H, dtype=torch.uint8, device=dev)
    ctx.frame(d_img, W, H, 4 * W, depix.LAYOUT_RGBA, p, None, d_graph, None, stream=stream)
    rp = depix.refine_params()
    rf = depix.Refiner(W * H)
    rf.setup(d_img, W, H, 4 * W, depix.LAYOUT_RGBA, d_graph, p, rp, stream=stream)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    reps = 5
    for _ in range(reps):
        rf.setup(d_img, W, H, 4 * W, depix.LAYOUT_RGBA, d_graph, p, rp, stream=stream)
    torch.cuda.synchronize()
    setup_ms = (time.perf_counter() - t0) / reps * 1e3
    c = rf.counts()
    pos = torch.empty(2 * max(c["nodes"], 1), dtype=torch.float32, device=dev)
    rf.initial(pos, stream=stream)
    before, after = rf.run(rp, pos, stream=stream)
    for _ in range(2):
        rf.run(rp, None, stream=stream, energies=False)
    torch.cuda.synchronize()
    runs = 10
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(runs):
        rf.run(rp, None, stream=stream, energies=False)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / runs
    out = {"workload": f"256x224 frame (seeded generator), x4 coverage, {c['nodes']} nodes ({c['free']} free), "
                       f"{c['edges']} curve edges, {c['samples']} samples, {rp.steps} Adam steps",
           "node_definition": "nodes are the cell-hull vertices on curve edges (edges between dissimilar cells); "
                              "the workload's 'about 20k nodes' is an estimate: the distinct vertices of every "
                              "subdivided cell polygon of this frame number 45,846, the curve-edge vertices "
                              f"{c['nodes']}",
           "steps_per_s": round(rp.steps / (ms / 1e3), 1), "ms_per_frame": round(ms, 3),
           "setup_ms": round(setup_ms, 3), "energy_before": round(before[3], 6), "energy_after": round(after[3], 6),
           "energy_cut": round(1 - after[3] / before[3], 4),
           "terms_after": {"curvature": round(after[0], 6), "deviation": round(after[1], 6),
                           "coverage": round(after[2], 6)}}
    rf.close()
    ctx.close()
    if cpu:
        sys.path.insert(0, ORACLE)
        import oracle as O
        import refine_oracle as R
        from depix import synth
        bgr, ws = synth.rgba_to_bgr(img)
        raw, _, res = O.graph(bgr, W, H, ws, (48, 7, 6))
        top = R.topology(img, res, raw, SCALE)
        k = 5
        P0 = R.initial_positions(top)
        t0 = time.perf_counter()
        for _ in range(k):  # an Adam step is one energy + gradient evaluation and an update
            R.energy_grad(top, P0, P0, img)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"steps_per_s": round(k / dt, 2), "cores": 1, "kind": "port",
                               "sample": f"{k} Adam steps of the float64 numpy specification "
                                         f"(oracle/refine_oracle.py) on the same frame and topology"}
    return out


def run_stream(args, dev, stream):
    """A stream of 256x224 frames (background + 24 moving sprites), x4: the
    plain path (one depix_frame call per frame) against batches of 8 through
    depix_batch followed, per frame, by topology setup, a warm start from the
    previous frame's refined nodes (tiles with unchanged signatures) and 20
    Adam steps. Frame latency: from the batch's (or frame's) upload to its
    last kernel; uploads from pinned host memory are inside the timed region."""
    import numpy as np
    import torch
    import depix
    from depix import synth

    n = args.stream_frames
    B = 8
    frames = synth.stream(n, seed=0)
    h_frames = torch.from_numpy(frames.reshape(n, -1)).pin_memory()
    fb = W * H * 4
    out_px = W * H * SCALE * SCALE
    p = depix.params(48, 7, 6, True, SCALE)
    rp = depix.refine_params(steps=20)
    ev = lambda: torch.cuda.Event(enable_timing=True)

    # plain: one frame at a time
    ctx1 = depix.Context(W * H, 1)
    d_in1 = torch.empty(fb, dtype=torch.uint8, device=dev)
    d_out1 = torch.empty(out_px * 4, dtype=torch.uint8, device=dev)
    for f in range(3):
        d_in1.copy_(h_frames[f], non_blocking=True)
        ctx1.frame(d_in1, W, H, 4 * W, depix.LAYOUT_RGBA, p, d_out1, None, None, stream=stream)
    torch.cuda.synchronize()
    marks = [(ev(), ev()) for _ in range(n)]
    t0 = time.perf_counter()
    for f in range(n):
        a, b = marks[f]
        a.record(stream)
        d_in1.copy_(h_frames[f], non_blocking=True)
        ctx1.frame(d_in1, W, H, 4 * W, depix.LAYOUT_RGBA, p, d_out1, None, None, stream=stream)
        b.record(stream)
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - t0
    plain_lat = sorted(a.elapsed_time(b) for a, b in marks)
    ctx1.close()

    # batched + refined with warm start: a batch's eight topology setups run
    # at once (each refiner on its own stream, driven from its own host
    # thread: a setup reads two counts back), then warm start and Adam steps
    # frame after frame (each frame starts from the previous frame's nodes),
    # on a stream above the setups' in priority
    from concurrent.futures import ThreadPoolExecutor
    ctx = depix.Context(W * H, B)
    d_in = torch.empty(B * fb, dtype=torch.uint8, device=dev)
    d_out = torch.empty(B * out_px * 4, dtype=torch.uint8, device=dev)
    rfs = [[depix.Refiner(W * H) for _ in range(B)] for _ in range(2)]  # one set per batch parity
    cap = (4 * W + 3) * (4 * H + 3)  # nodes are vertices of the quarter-unit grid
    pos = [[torch.empty(2 * cap, dtype=torch.float32, device=dev) for _ in range(B)] for _ in range(2)]
    # priorities: the refinement chain first (each frame waits for the one
    # before it), then the setups in the order the chain needs them
    try:
        lo, hi = torch.cuda.Stream.priority_range()
    except Exception:
        lo, hi = 0, 0
    side = [torch.cuda.Stream(dev, priority=min(lo, hi + 1 + k)) for k in range(B)]
    stream = torch.cuda.Stream(dev, priority=hi)
    caller_stream = torch.cuda.current_stream()
    torch.cuda.set_stream(stream)
    pool = ThreadPoolExecutor(max_workers=B)
    in_off = [k * fb for k in range(B)]
    out_off = [k * out_px * 4 for k in range(B)]

    def setup(rf, k, uploaded):
        side[k].wait_event(uploaded)
        rf.setup(d_in[k * fb:], W, H, 4 * W, depix.LAYOUT_RGBA, None, p, rp, stream=side[k])
        done = torch.cuda.Event(enable_timing=True)
        done.record(side[k])
        return done

    def run_all(count_reuse):
        reused, tiles = 0, 0
        prev = None
        for bi, b0 in enumerate(range(0, n, B)):
            start = ev()
            start.record(stream)
            d_in.copy_(h_frames[b0:b0 + B].reshape(-1), non_blocking=True)
            uploaded = torch.cuda.Event()
            uploaded.record(stream)
            ctx.batch([W] * B, [H] * B, in_off, out_off, d_in, p, d_out, None, stream=stream)
            rastered = ev()
            rastered.record(stream)
            cur = rfs[bi % 2]
            futs = [pool.submit(setup, cur[k], k, uploaded) for k in range(B)]
            marks = (start, rastered, [], [])
            batch_marks.append(marks)
            for k in range(B):
                rf, ps = cur[k], pos[bi % 2][k]
                set_up = futs[k].result()
                marks[2].append(set_up)
                stream.wait_event(set_up)
                if prev is None:
                    rf.initial(ps, stream=stream)
                else:
                    r = rf.warm_start(prev[0], prev[1], ps, stream=stream, count=count_reuse)
                    if count_reuse:
                        reused += r
                        tiles += ((W + 15) // 16) * ((H + 15) // 16)
                rf.run(rp, ps, stream=stream, energies=False)
                done = ev()
                done.record(stream)
                lat_marks.append((start, done))
                marks[3].append(done)
                prev = (rf, ps)
            # the next batch's upload is ordered after these steps on the main
            # stream, and its setups (the other refiner set) wait for that upload
        return reused, tiles

    lat_marks, batch_marks = [], []
    run_all(False)  # warm-up pass
    torch.cuda.synchronize()
    lat_marks, batch_marks = [], []
    t0 = time.perf_counter()
    run_all(False)
    torch.cuda.synchronize()
    batched_s = time.perf_counter() - t0
    lat = sorted(a.elapsed_time(b) for a, b in lat_marks)
    # where a batch's time goes: upload + batch raster, the eight topology
    # setups (concurrent, each with host readbacks of its counts), then warm
    # start + Adam steps frame after frame
    med = lambda v: round(float(np.median(v)), 4)
    breakdown = {
        "upload_raster_ms": med([m[0].elapsed_time(m[1]) for m in batch_marks]),
        "setups_done_ms": med([max(m[0].elapsed_time(e) for e in m[2]) for m in batch_marks]),
        "first_frame_done_ms": med([m[0].elapsed_time(m[3][0]) for m in batch_marks]),
        "refine_per_frame_ms": med([(m[3][0].elapsed_time(m[3][-1])) / (B - 1) for m in batch_marks]),
    }
    lat_marks = []
    reused, tiles = run_all(True)
    torch.cuda.synchronize()
    pool.shutdown()
    rfs_flat = [r for st in rfs for r in st]
    rfs = [rfs_flat[0], rfs_flat[1]]
    pos = [pos[0][0], pos[0][1]]

    # warm against cold start: energy after 20 steps on a few frames, and the
    # cold-start steps that reach the warm start's 20-step energy
    warm_e, cold_e, cold_steps = [], [], []
    ladder = [20, 25, 30, 40, 50, 60, 80, 100, 150, 200]
    for f in range(1, 17):
        rf, ps = rfs[f % 2], pos[f % 2]
        prv = rfs[(f - 1) % 2]
        prv.setup(torch.from_numpy(frames[f - 1].reshape(-1)).to(dev), W, H, 4 * W, depix.LAYOUT_RGBA, None, p, rp,
                  stream=stream)
        pp = pos[(f - 1) % 2]
        prv.initial(pp, stream=stream)
        prv.run(depix.refine_params(steps=200), pp, stream=stream, energies=False)
        rf.setup(torch.from_numpy(frames[f].reshape(-1)).to(dev), W, H, 4 * W, depix.LAYOUT_RGBA, None, p, rp,
                 stream=stream)
        rf.warm_start(prv, pp, ps, stream=stream, count=False)
        warm_e.append(rf.run(rp, ps, stream=stream)[1][3])
        cold_e.append(rf.run(rp, None, stream=stream)[1][3])
        need = None
        for k in ladder:
            if rf.run(depix.refine_params(steps=k), None, stream=stream)[1][3] <= warm_e[-1]:
                need = k
                break
        cold_steps.append(need if need is not None else 10 ** 9)
    for r in rfs_flat:
        r.close()
    ctx.close()
    torch.cuda.synchronize()
    torch.cuda.set_stream(caller_stream)
    pct = lambda v, q: round(v[min(len(v) - 1, int(q * len(v)))], 4)
    return {"workload": f"{n} frames 256x224 (background + 24 sprites at 0-3 px/frame, wrap-around), x4; "
                        f"refinement: 20 Adam steps per frame, warm start by 16x16 tile signature",
            "plain": {"frames_per_s": round(n / plain_s, 1), "p50_ms": pct(plain_lat, 0.5),
                      "p99_ms": pct(plain_lat, 0.99)},
            "batched_refined": {"frames_per_s": round(n / batched_s, 1), "p50_ms": pct(lat, 0.5),
                                "p99_ms": pct(lat, 0.99), "batch": B, "reused_tile_frac": round(reused / max(tiles, 1), 4)},
            "energy_after_20_steps": {"warm_start": round(float(np.mean(warm_e)), 6),
                                      "cold_start": round(float(np.mean(cold_e)), 6), "frames": len(warm_e),
                                      "cold_steps_to_warm_energy_median": int(np.median(cold_steps)),
                                      "cold_steps_to_warm_energy": [int(c) if c < 10 ** 9 else None
                                                                    for c in cold_steps],
                                      "ladder": ladder},
            "batch_breakdown": breakdown}


# ---------------------------------------------------------- reference arm


def run_reference(args, rank, world):
    if rank != 0:
        return
    cores, kind = cpu_setup()
    frames = make_frames(min(DISTINCT, max(cores, 8)))
    per_step = cores
    for _ in range(max(args.warmup, 1)):
        cpu_run(frames, per_step, cores, kind)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cpu_run(frames, per_step, cores, kind)
    dt = time.perf_counter() - t0
    value = per_step * args.steps / dt
    sample = f"{per_step} frames per step ({cores} threads, one frame each): " + CPU_SAMPLE[kind]
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * dt / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
            "data": "synthetic (seeded generator)", "config": workload_config(per_step),
            "cpu_baseline": {"value": round(value, 2), "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": round(value, 2), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if kind == "reference":
        line["cpu_baseline"]["single_thread_value"] = round(cpu_run(frames, 2, 1, kind), 2)
    print(json.dumps(line))


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import torch
    if world > 1:
        torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group("nccl")
    if rank == 0 or world == 1:
        import build as depix_build
        depix_build.build()
    if world > 1:
        torch.distributed.barrier()
    if args.large_only:
        import torch
        torch.cuda.set_device(local_rank)
        import depix
        depix.init_device()
        print(json.dumps({"large_x8": run_large(args, torch.device("cuda", local_rank),
                                                torch.cuda.current_stream())}))
        return
    run_ours(args, rank, world, local_rank)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
