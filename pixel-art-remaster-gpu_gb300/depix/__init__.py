"""Python binding of libdepix.so (the C ABI declared in include/depix.h).

Device buffers are passed as torch CUDA tensors (or raw integer addresses);
streams as torch.cuda.Stream (default: torch's current stream). There is no
CPU fallback: when the library is missing every call raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG, "libdepix.so")

LAYOUT_BGR = 0
LAYOUT_RGBA = 1
# depix_status codes
OK, ERR_INVALID_ARG, ERR_CUDA, ERR_ALLOC, ERR_TOO_LARGE, ERR_TIMEOUT, ERR_CAPTURING, ERR_STATE = range(8)
# luma arithmetic (depix_yuv): the reference's CUDA build, or its host build
YUV_CUDA = 0
YUV_HOST = 1
CELL = 45


class DepixError(RuntimeError):
    def __init__(self, status, where, detail=""):
        self.status = status
        super().__init__(f"{where}: status {status} ({_status_name(status)}) {detail}".strip())


class Params(ctypes.Structure):
    _fields_ = [("tr_y", ctypes.c_int), ("tr_u", ctypes.c_int), ("tr_v", ctypes.c_int),
                ("subdivide", ctypes.c_int), ("scale", ctypes.c_int), ("vote", ctypes.c_int),
                ("yuv", ctypes.c_int)]


class RefineParams(ctypes.Structure):
    _fields_ = [("w_curvature", ctypes.c_float), ("w_deviation", ctypes.c_float), ("w_coverage", ctypes.c_float),
                ("sigma", ctypes.c_float), ("lr", ctypes.c_float), ("steps", ctypes.c_int)]


def refine_params(w_curvature=1.0, w_deviation=0.25, w_coverage=1.0, sigma=0.5, lr=0.05, steps=200):
    return RefineParams(w_curvature, w_deviation, w_coverage, sigma, lr, steps)


def params(tr_y=48, tr_u=7, tr_v=6, subdivide=True, scale=4, vote=False, yuv=YUV_CUDA) -> Params:
    """Frame-path parameters; vote=True resolves ambiguous crossings by the
    weighted vote (curves, sparse pixels, islands) instead of the
    reference's ordered tests; yuv selects the luma arithmetic of the
    reference's CUDA build (YUV_CUDA, the default) or of its host build
    (YUV_HOST)."""
    return Params(tr_y, tr_u, tr_v, int(bool(subdivide)), scale, int(bool(vote)), int(yuv))


_lib = None
_vp = ctypes.c_void_p
_i = ctypes.c_int


def _sig(L, name, args, res=ctypes.c_int):
    fn = getattr(L, name)
    fn.argtypes = args
    fn.restype = res


def lib():
    """Load libdepix.so (raises when it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FileNotFoundError(f"{LIB_PATH} not built: run pixel-art-remaster-gpu_gb300/build.py")
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER(Params)
        _sig(L, "depix_default_params", [P], None)
        _sig(L, "depix_status_string", [_i], ctypes.c_char_p)
        _sig(L, "depix_last_error", [], ctypes.c_char_p)
        _sig(L, "depix_init_device", [])
        _sig(L, "depix_take_device_faults", [_vp])
        _sig(L, "depix_debug_fail_allocations", [_i])
        _sig(L, "depix_debug_live_allocations", [_vp])
        _sig(L, "depix_debug_tma_timeout", [_i])
        _sig(L, "depix_graph", [_vp, _i, _i, _i, _i, P, _i, _vp, _vp])
        _sig(L, "depix_resolve_trivial", [_vp, _i, _i, _vp])
        _sig(L, "depix_resolve_heuristics", [_vp, _i, _i, _vp, _vp])
        _sig(L, "depix_resolve_heuristics_vote", [_vp, _i, _i, _vp, _vp])
        _sig(L, "depix_cells", [_vp, _i, _i, _vp, _vp, _vp])
        _sig(L, "depix_subdivide", [_vp, _i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp])
        _sig(L, "depix_triangulate", [_vp, _vp, _i, _i, _vp])
        _sig(L, "depix_emit_vbo", [_vp, _i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp])
        _sig(L, "depix_label_components", [_vp, _i, _i, _vp, _vp])
        _sig(L, "depix_border_walks", [_vp, _i, _i, _i, _vp, _vp, _vp, _vp, _i, _i, _vp, _vp])
        _sig(L, "depix_raster", [_vp, _i, _i, _i, _i, _vp, P, _vp, _vp])
        _sig(L, "depix_context_create", [ctypes.POINTER(_vp), ctypes.c_size_t, _i])
        _sig(L, "depix_context_destroy", [_vp])
        _sig(L, "depix_frame", [_vp, _vp, _i, _i, _i, _i, P, _vp, _vp, _vp, _vp])
        _sig(L, "depix_batch", [_vp, _i, _vp, _vp, _vp, _vp, _vp, P, _vp, _vp, _vp])
        _sig(L, "depix_batch_host", [_vp, _i, _vp, _vp, _vp, _vp, _vp, ctypes.c_size_t, P, _vp, ctypes.c_size_t,
                                     _vp, _vp])
        _sig(L, "depix_context_set_timing", [_vp, _i])
        _sig(L, "depix_context_set_launch_shape", [_vp, _i, _i, _i])
        _sig(L, "depix_context_launch_shape", [_vp, _vp, _vp, _vp])
        _sig(L, "depix_context_stage_times", [_vp, _vp, _vp, _vp])
        _sig(L, "depix_launch_kernel_compat", [_vp, _vp, ctypes.c_float, _vp, _i, _i, _i, _vp, _vp, _i, P], _vp)
        _sig(L, "launch_kernel", [_vp, _vp, ctypes.c_float, _vp, _i, _i, _i, _vp, _vp, ctypes.c_bool], _vp)
        RP = ctypes.POINTER(RefineParams)
        _sig(L, "depix_refine_default_params", [RP], None)
        _sig(L, "depix_refiner_create", [ctypes.POINTER(_vp), ctypes.c_size_t])
        _sig(L, "depix_refiner_destroy", [_vp])
        _sig(L, "depix_refine_setup", [_vp, _vp, _i, _i, _i, _i, _vp, P, RP, _vp])
        _sig(L, "depix_refine_counts", [_vp, _vp])
        _sig(L, "depix_refine_export", [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp])
        _sig(L, "depix_refine_initial", [_vp, _vp, _vp])
        _sig(L, "depix_refine_energy_grad", [_vp, RP, _vp, _vp, _vp, _vp])
        _sig(L, "depix_refine_warm_start", [_vp, _vp, _vp, _vp, _vp, _vp])
        _sig(L, "depix_refine_run", [_vp, RP, _vp, _vp, _vp, _vp])
        _sig(L, "depix_yuv_words", [_vp, ctypes.c_size_t, _i, _vp, _vp])
        _sig(L, "depix_pattern_tables", [_vp, _vp])
        _lib = L
    return _lib


def _status_name(s):
    try:
        return lib().depix_status_string(s).decode()
    except Exception:
        return "?"


def _check(status, where):
    if status != 0:
        raise DepixError(status, where, lib().depix_last_error().decode())


def ptr(t):
    """Device/host address of a torch tensor, numpy array or int."""
    if t is None:
        return None
    if isinstance(t, int):
        return _vp(t)
    if hasattr(t, "data_ptr"):
        return _vp(t.data_ptr())
    if hasattr(t, "ctypes"):
        return _vp(t.ctypes.data)
    raise TypeError(type(t))


def stream_ptr(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return _vp(s.cuda_stream)


def init_device():
    _check(lib().depix_init_device(), "depix_init_device")


def graph(img, w, h, ws, layout, p, out, fuse_trivial=True, stream=None):
    _check(lib().depix_graph(ptr(img), w, h, ws, layout, ctypes.byref(p), int(fuse_trivial), ptr(out),
                             stream_ptr(stream)), "depix_graph")


def resolve_trivial(g, w, h, stream=None):
    _check(lib().depix_resolve_trivial(ptr(g), w, h, stream_ptr(stream)), "depix_resolve_trivial")


def resolve_heuristics(snap, w, h, out, stream=None, vote=False):
    if vote:
        _check(lib().depix_resolve_heuristics_vote(ptr(snap), w, h, ptr(out), stream_ptr(stream)),
               "depix_resolve_heuristics_vote")
    else:
        _check(lib().depix_resolve_heuristics(ptr(snap), w, h, ptr(out), stream_ptr(stream)),
               "depix_resolve_heuristics")


def cells(g, w, h, diagram, ec, stream=None):
    _check(lib().depix_cells(ptr(g), w, h, ptr(diagram), ptr(ec), stream_ptr(stream)), "depix_cells")


def subdivide(img, w, h, ws, layout, g, snap, ec_snap, diagram, ec, stream=None):
    _check(lib().depix_subdivide(ptr(img), w, h, ws, layout, ptr(g), ptr(snap), ptr(ec_snap), ptr(diagram),
                                 ptr(ec), stream_ptr(stream)), "depix_subdivide")


def triangulate(diagram, ec, w, h, stream=None):
    _check(lib().depix_triangulate(ptr(diagram), ptr(ec), w, h, stream_ptr(stream)), "depix_triangulate")


def emit_vbo(img, w, h, ws, layout, diagram, ec, pos, col, stream=None):
    _check(lib().depix_emit_vbo(ptr(img), w, h, ws, layout, ptr(diagram), ptr(ec), ptr(pos), ptr(col),
                                stream_ptr(stream)), "depix_emit_vbo")


def label_components(g, w, h, labels, stream=None):
    _check(lib().depix_label_components(ptr(g), w, h, ptr(labels), stream_ptr(stream)), "depix_label_components")


def border_walks(g, w, h, nframes, scratch, nodes, edges, offsets, max_nodes, max_walks, counts, stream=None):
    _check(lib().depix_border_walks(ptr(g), w, h, nframes, ptr(scratch), ptr(nodes), ptr(edges), ptr(offsets),
                                    max_nodes, max_walks, ptr(counts), stream_ptr(stream)), "depix_border_walks")


def border_walk_lists(g, w, h, nframes=1, max_nodes=None, max_walks=None, stream=None):
    """Border walks of nframes resolved graphs on the device (a torch uint8
    tensor, frames w*h bytes apart): per frame, a list of (nodes, edges)
    walks and whether a capacity ran out."""
    import torch
    n = w * h
    max_nodes = 4 * n + 16 if max_nodes is None else max_nodes
    max_walks = n if max_walks is None else max_walks
    dev = g.device
    scratch = torch.empty(n * nframes, dtype=torch.uint8, device=dev)
    nodes = torch.empty(max_nodes * nframes, dtype=torch.int32, device=dev)
    edges = torch.empty(max_nodes * nframes, dtype=torch.int8, device=dev)
    offsets = torch.empty((max_walks + 1) * nframes, dtype=torch.int32, device=dev)
    counts = torch.empty(3 * nframes, dtype=torch.int32, device=dev)
    border_walks(g, w, h, nframes, scratch, nodes, edges, offsets, max_nodes, max_walks, counts, stream)
    c = counts.cpu().numpy().reshape(nframes, 3)
    nd, ed, of = nodes.cpu().numpy(), edges.cpu().numpy(), offsets.cpu().numpy()
    out = []
    for f in range(nframes):
        o = of[f * (max_walks + 1):f * (max_walks + 1) + c[f, 0] + 1]
        base = f * max_nodes
        out.append(([(nd[base + o[k]:base + o[k + 1]].tolist(), ed[base + o[k]:base + o[k + 1]].tolist())
                     for k in range(c[f, 0])], bool(c[f, 2])))
    return out


def format_walks(walks) -> str:
    """Walks as the reference's spline export wrote them (alex_png.txt):
    one line 'Spline: k - ' with ' node, ' per node."""
    return "".join(f"Spline: {k} - " + "".join(f" {v}, " for v in nodes) + "\n" for k, (nodes, _) in enumerate(walks))


def raster(img, w, h, ws, layout, g, p, out, stream=None):
    _check(lib().depix_raster(ptr(img), w, h, ws, layout, ptr(g), ctypes.byref(p), ptr(out), stream_ptr(stream)),
           "depix_raster")


def yuv_words(px, n, out, stream=None, yuv=YUV_CUDA):
    _check(lib().depix_yuv_words(ptr(px), n, int(yuv), ptr(out), stream_ptr(stream)), "depix_yuv_words")


def pattern_tables(hull_out, tri_out):
    _check(lib().depix_pattern_tables(ptr(hull_out), ptr(tri_out)), "depix_pattern_tables")


class Context:
    """Owns the scratch of the frame and batch paths."""

    def __init__(self, max_pixels, max_frames=1):
        h = _vp()
        _check(lib().depix_context_create(ctypes.byref(h), max_pixels, max_frames), "depix_context_create")
        self.handle = h

    def close(self):
        if self.handle:
            lib().depix_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def frame(self, img, w, h, ws, layout, p, out, graph_out=None, labels=None, stream=None):
        _check(lib().depix_frame(self.handle, ptr(img), w, h, ws, layout, ctypes.byref(p), ptr(out), ptr(graph_out),
                                 ptr(labels), stream_ptr(stream)), "depix_frame")

    @staticmethod
    def _arrays(ws, hs, in_off, out_off):
        """ctypes views of the per-frame arrays: numpy int32 / uint64 arrays
        pass by pointer (no per-call conversion), other sequences are copied."""
        import numpy as np
        n = len(ws)

        def view(a, dtype, ctype):
            if isinstance(a, np.ndarray) and a.dtype == dtype and a.flags.c_contiguous:
                return a.ctypes.data_as(ctypes.POINTER(ctype))
            return (ctype * n)(*a)

        return (n, view(ws, np.int32, ctypes.c_int), view(hs, np.int32, ctypes.c_int),
                view(in_off, np.uint64, ctypes.c_uint64), view(out_off, np.uint64, ctypes.c_uint64))

    def batch(self, ws, hs, in_off, out_off, img, p, out, labels=None, stream=None):
        """ws/hs/in_off/out_off: host int sequences (frame sizes, byte offsets)."""
        n, W, H, I, O = self._arrays(ws, hs, in_off, out_off)
        _check(lib().depix_batch(self.handle, n, W, H, I, O, ptr(img), ctypes.byref(p), ptr(out), ptr(labels),
                                 stream_ptr(stream)), "depix_batch")

    def batch_host(self, ws, hs, in_off, out_off, h_img, in_bytes, p, h_out, out_bytes, h_labels=None,
                   stream=None):
        n, W, H, I, O = self._arrays(ws, hs, in_off, out_off)
        _check(lib().depix_batch_host(self.handle, n, W, H, I, O, ptr(h_img), in_bytes, ctypes.byref(p),
                                      ptr(h_out), out_bytes, ptr(h_labels), stream_ptr(stream)),
               "depix_batch_host")

    def set_launch_shape(self, gran=0, tile_w=32, tile_h=32):
        """Queue-path shape for uneven batches; gran 0 returns to tuning."""
        _check(lib().depix_context_set_launch_shape(self.handle, gran, tile_w, tile_h),
               "depix_context_set_launch_shape")

    def launch_shape(self):
        """(gran per stage, raster tile w, h) of the last queue-path batch."""
        g = (ctypes.c_int * 4)()
        tw, th = ctypes.c_int(), ctypes.c_int()
        _check(lib().depix_context_launch_shape(self.handle, g, ctypes.byref(tw), ctypes.byref(th)),
               "depix_context_launch_shape")
        return tuple(g), tw.value, th.value

    def set_timing(self, on=True):
        _check(lib().depix_context_set_timing(self.handle, int(bool(on))), "depix_context_set_timing")

    STAGES = ("graph", "heuristics", "labels", "raster")

    def stage_times(self):
        """{stage: (ms, launches, calls)} accumulated since the last call."""
        ms = (ctypes.c_double * 4)()
        la = (ctypes.c_longlong * 4)()
        ca = (ctypes.c_longlong * 4)()
        _check(lib().depix_context_stage_times(self.handle, ms, la, ca), "depix_context_stage_times")
        return {name: (ms[k], la[k], ca[k]) for k, name in enumerate(self.STAGES)}


def take_device_faults() -> int:
    """Sticky device-side fault bits since the last call (0: none); the C
    call returns DEPIX_ERR_TIMEOUT (5) whenever a bit is set, which is
    reported here through the bits, not raised."""
    f = ctypes.c_int(0)
    st = lib().depix_take_device_faults(ctypes.byref(f))
    if st != ERR_TIMEOUT:
        _check(st, "depix_take_device_faults")
    return f.value


def debug_fail_allocations(after: int) -> None:
    """Testing hook: after `after` more device allocations by the library
    succeed, every later one fails until called with a negative value."""
    _check(lib().depix_debug_fail_allocations(int(after)), "depix_debug_fail_allocations")


def debug_live_allocations() -> int:
    """Testing hook: device allocations the library holds now."""
    n = ctypes.c_longlong(0)
    _check(lib().depix_debug_live_allocations(ctypes.byref(n)), "depix_debug_live_allocations")
    return n.value


def debug_tma_timeout(enable: bool) -> None:
    """Testing hook: the TMA graph kernel issues no tile load and gives up
    its bounded wait after a few polls (nothing in flight)."""
    _check(lib().depix_debug_tma_timeout(int(bool(enable))), "depix_debug_tma_timeout")


class Refiner:
    """Spline refinement of one frame at a time (topology frozen at setup)."""

    def __init__(self, max_pixels):
        h = _vp()
        _check(lib().depix_refiner_create(ctypes.byref(h), max_pixels), "depix_refiner_create")
        self.handle = h

    def close(self):
        if self.handle:
            lib().depix_refiner_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def setup(self, img, w, h, ws, layout, graph, p, rp, stream=None):
        _check(lib().depix_refine_setup(self.handle, ptr(img), w, h, ws, layout, ptr(graph), ctypes.byref(p),
                                        ctypes.byref(rp), stream_ptr(stream)), "depix_refine_setup")

    def counts(self):
        """dict of nodes, free, edges, segments (slots), samples (the first
        call after a setup synchronises the device)."""
        c = (ctypes.c_longlong * 5)()
        _check(lib().depix_refine_counts(self.handle, c), "depix_refine_counts")
        return dict(zip(("nodes", "free", "edges", "segments", "samples"), list(c)))

    def export(self):
        import numpy as np
        c = self.counts()
        N, E, S, M = c["nodes"], c["edges"], c["segments"], c["samples"]
        out = dict(q=np.zeros((N, 2), np.int32), flags=np.zeros(N, np.int32), nbr=np.zeros((N, 2), np.int32),
                   edges=np.zeros((E, 4), np.int32), segs=np.zeros((S, 4), np.int32),
                   cols=np.zeros((S, 2), np.uint32), samples=np.zeros((M, 2), np.int32))
        _check(lib().depix_refine_export(self.handle, *(ptr(out[k]) for k in
                                                        ("q", "flags", "nbr", "edges", "segs", "cols", "samples"))),
               "depix_refine_export")
        return out

    def initial(self, pos, stream=None):
        _check(lib().depix_refine_initial(self.handle, ptr(pos), stream_ptr(stream)), "depix_refine_initial")

    def warm_start(self, prev, prev_pos, pos, stream=None, count=True):
        """Start positions from the previous frame's refiner; returns the
        number of unchanged tiles (None with count=False)."""
        n = ctypes.c_int(0)
        _check(lib().depix_refine_warm_start(self.handle, prev.handle, ptr(prev_pos), ptr(pos),
                                             ctypes.byref(n) if count else None, stream_ptr(stream)),
               "depix_refine_warm_start")
        return n.value if count else None

    def energy_grad(self, rp, pos, grad=None, stream=None):
        e = (ctypes.c_double * 4)()
        _check(lib().depix_refine_energy_grad(self.handle, ctypes.byref(rp), ptr(pos), ptr(grad), e,
                                              stream_ptr(stream)), "depix_refine_energy_grad")
        return tuple(e)

    def run(self, rp, pos=None, stream=None, energies=True):
        """Adam; returns (energy before, energy after) as 4-tuples, or None
        without the (synchronising) energy evaluations."""
        b = (ctypes.c_double * 4)()
        a = (ctypes.c_double * 4)()
        _check(lib().depix_refine_run(self.handle, ctypes.byref(rp), ptr(pos), b if energies else None,
                                      a if energies else None, stream_ptr(stream)), "depix_refine_run")
        return (tuple(b), tuple(a)) if energies else None


def launch_kernel_compat(pos, col, img_host, w, h, ws, edge_count_host, graph_host, subdivide, p=None):
    """Drop-in frame driver; returns the host address of the malloc'd points
    (free it with libc free) or raises."""
    r = lib().depix_launch_kernel_compat(ptr(pos), ptr(col), 0.0, ptr(img_host), w, h, ws, ptr(edge_count_host),
                                         ptr(graph_host), int(bool(subdivide)),
                                         ctypes.byref(p) if p is not None else None)
    if not r:
        raise DepixError(-1, "depix_launch_kernel_compat", lib().depix_last_error().decode())
    return r
