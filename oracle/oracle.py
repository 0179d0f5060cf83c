"""ctypes bindings of the CPU oracle (depix_oracle.c) and, when it has been
built in this checkout, of the host build of the reference's own stage bodies
(oracle/_ref). TEST INFRASTRUCTURE ONLY: imported by tests/, by
__graft_entry__.smoke() and by bench.py's CPU-baseline leg, never by the
product library.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libdepix_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")
CELL = 45
# luma arithmetic of the packed Y/U/V word (the library's depix_yuv): the
# reference's CUDA build (fused multiply-adds) or its host build
YUV_CUDA = 0
YUV_HOST = 1

_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_i8p = np.ctypeslib.ndpointer(np.int8, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    """Compile the oracle with IEEE semantics (no FMA contraction)."""
    src = os.path.join(HERE, "depix_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
                               "-o", LIB_PATH, src, "-lm"])
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_yuv_word.restype = ctypes.c_uint32
        L.orc_yuv_word.argtypes = [ctypes.c_uint8] * 3 + [ctypes.c_int]
        L.orc_graph.argtypes = [_u8p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                ctypes.c_int, ctypes.c_int, _u8p]
        L.orc_trivial.argtypes = [_u8p, ctypes.c_int, ctypes.c_int]
        L.orc_heuristics.argtypes = [_u8p, ctypes.c_int, ctypes.c_int, _u8p]
        L.orc_heuristics_vote.argtypes = [_u8p, ctypes.c_int, ctypes.c_int, _u8p]
        L.orc_hull_table.argtypes = [_i32p, _i8p]
        L.orc_raster.argtypes = [_f32p, _u8p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _u8p]
        L.orc_label_cc.argtypes = [_u8p, ctypes.c_int, ctypes.c_int, _i32p]
        L.orc_border_walks.restype = ctypes.c_int
        L.orc_border_walks.argtypes = [_u8p, ctypes.c_int, ctypes.c_int, _i32p, _i8p, _i32p, ctypes.c_int,
                                       ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        vp = ctypes.c_void_p
        L.orc_frame.restype = ctypes.c_int
        L.orc_frame.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                ctypes.c_int, ctypes.c_int, ctypes.c_int] + [vp] * 9
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Frame:
    """All outputs of one run of the path on one frame."""

    def __init__(self, w, h):
        n = w * h
        self.w, self.h = w, h
        self.graph_trivial = np.zeros(n, np.uint8)
        self.graph = np.zeros(n, np.uint8)
        self.ec_cells = np.zeros(n, np.int32)
        self.diag_cells = np.zeros(n * CELL * 2, np.float32)
        self.ec = np.zeros(n, np.int32)
        self.diag = np.zeros(n * CELL * 2, np.float32)
        self.pos = np.zeros(n * CELL * 2, np.float32)
        self.col = np.zeros(n * CELL * 4, np.uint8)
        self.fails = 0

    def _args(self):
        return [_ptr(self.graph_trivial), _ptr(self.graph), _ptr(self.ec_cells), _ptr(self.diag_cells),
                _ptr(self.ec), _ptr(self.diag), _ptr(self.pos), _ptr(self.col)]


def frame(bgr, w, h, ws, subdivide=True, tr=(48, 7, 6), graph_in=None, yuv=YUV_CUDA) -> Frame:
    """Run the oracle's whole path on a reference-layout BGR buffer (luma
    arithmetic of the reference's CUDA build unless yuv=YUV_HOST)."""
    bgr = np.ascontiguousarray(bgr, np.uint8)
    f = Frame(w, h)
    gi = None if graph_in is None else np.ascontiguousarray(graph_in, np.uint8)
    f.fails = lib().orc_frame(_ptr(bgr), w, h, ws, int(bool(subdivide)), tr[0], tr[1], tr[2], int(yuv), _ptr(gi),
                              *f._args())
    return f


def yuv_word(b0, b1, b2, yuv=YUV_CUDA) -> int:
    return int(lib().orc_yuv_word(b0, b1, b2, int(yuv)))


def graph(bgr, w, h, ws, tr=(48, 7, 6), vote=False, yuv=YUV_CUDA):
    """Similarity graph, then trivial and heuristic resolution (the
    reference's ordered tests, or the weighted vote): returns
    (raw, after_trivial, resolved)."""
    bgr = np.ascontiguousarray(bgr, np.uint8)
    raw = np.zeros(w * h, np.uint8)
    lib().orc_graph(bgr, w, h, ws, tr[0], tr[1], tr[2], int(yuv), raw)
    triv = raw.copy()
    lib().orc_trivial(triv, w, h)
    return raw, triv, heuristics(triv, w, h, vote)


def heuristics(snap, w, h, vote=False):
    """Heuristic resolution of a graph after trivial removal."""
    res = np.zeros(w * h, np.uint8)
    fn = lib().orc_heuristics_vote if vote else lib().orc_heuristics
    fn(np.ascontiguousarray(snap, np.uint8).reshape(-1), w, h, res)
    return res


def hull_table():
    counts = np.zeros(4096, np.int32)
    pts = np.zeros(4096 * 16 * 2, np.int8)
    lib().orc_hull_table(counts, pts)
    return counts, pts.reshape(4096, 16, 2)


def raster(pos, col, w, h, scale):
    out = np.zeros(w * scale * h * scale * 4, np.uint8)
    lib().orc_raster(np.ascontiguousarray(pos, np.float32), np.ascontiguousarray(col, np.uint8), w, h, scale, out)
    return out.reshape(h * scale, w * scale, 4)


def label_cc(graph_resolved, w, h):
    out = np.zeros(w * h, np.int32)
    lib().orc_label_cc(np.ascontiguousarray(graph_resolved, np.uint8), w, h, out)
    return out


def border_walks(graph, w, h, max_nodes=None, max_walks=None):
    """Border walks of a resolved graph: a list of (nodes, edges) per walk, or
    None when the capacities run out."""
    n = w * h
    max_nodes = 8 * n + 8 if max_nodes is None else max_nodes
    max_walks = n if max_walks is None else max_walks
    nodes = np.zeros(max(max_nodes, 1), np.int32)
    edges = np.zeros(max(max_nodes, 1), np.int8)
    offs = np.zeros(max_walks + 1, np.int32)
    used = ctypes.c_int(0)
    k = lib().orc_border_walks(np.ascontiguousarray(graph, np.uint8).reshape(-1), w, h, nodes, edges, offs,
                               max_nodes, max_walks, ctypes.byref(used))
    if k < 0:
        return None
    return [(nodes[offs[i]:offs[i + 1]].tolist(), edges[offs[i]:offs[i + 1]].tolist()) for i in range(k)]


# ----------------------------------------------------------- reference build

_ref = {}


def ref_available(tr_y: int) -> bool:
    return os.path.exists(os.path.join(REF_DIR, f"libdepix_ref{tr_y}.so"))


def ref_lib(tr_y: int):
    """Host build of the reference's own stage bodies (Y threshold 5 or 48)."""
    if tr_y not in _ref:
        L = ctypes.CDLL(os.path.join(REF_DIR, f"libdepix_ref{tr_y}.so"))
        vp = ctypes.c_void_p
        L.ref_frame.restype = ctypes.c_int
        L.ref_frame.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int] + [vp] * 9
        L.ref_yuv_word.restype = ctypes.c_uint32
        L.ref_yuv_word.argtypes = [ctypes.c_uint8] * 3
        _ref[tr_y] = L
    return _ref[tr_y]


def ref_frame(bgr, w, h, ws, subdivide=True, tr_y=48, graph_in=None) -> Frame:
    bgr = np.ascontiguousarray(bgr, np.uint8)
    f = Frame(w, h)
    gi = None if graph_in is None else np.ascontiguousarray(graph_in, np.uint8)
    ref_lib(tr_y).ref_frame(_ptr(bgr), w, h, ws, int(bool(subdivide)), _ptr(gi), *f._args())
    return f


def ref_frame_vbo(bgr, w, h, ws, subdivide=True, tr_y=48):
    """The reference's host build on one frame, returning only what the frame
    path hands on (resolved graph, VBO positions and colours)."""
    bgr = np.ascontiguousarray(bgr, np.uint8)
    n = w * h
    graph = np.zeros(n, np.uint8)
    pos = np.zeros(n * CELL * 2, np.float32)
    col = np.zeros(n * CELL * 4, np.uint8)
    ref_lib(tr_y).ref_frame(_ptr(bgr), w, h, ws, int(bool(subdivide)), None, None, _ptr(graph), None, None, None,
                            None, _ptr(pos), _ptr(col))
    return graph, pos, col


def build_ref(gpu: bool = False) -> bool:
    """Runs oracle/build_ref.sh (host build only unless gpu) and reports
    whether the host build of the reference's stage bodies is present."""
    env = dict(os.environ)
    if not gpu:
        env["DEPIX_REF_NO_GPU"] = "1"
    subprocess.run([os.path.join(HERE, "build_ref.sh")], env=env, check=False, stdout=subprocess.DEVNULL)
    return ref_available(5) and ref_available(48)


def yuv_words(px3: np.ndarray, ref_tr_y: int = 0, yuv=YUV_CUDA) -> np.ndarray:
    """Packed YUV words of an (n, 3) byte array by the oracle (luma
    arithmetic yuv); with ref_tr_y set, computed by the reference's own
    functions in its host build instead."""
    px3 = np.ascontiguousarray(px3, np.uint8)
    n = px3.shape[0]
    out = np.zeros(n, np.uint32)
    if ref_tr_y:
        fn = ref_lib(ref_tr_y).ref_yuv_words
        fn.restype = None
        fn.argtypes = [ctypes.c_void_p, ctypes.c_long, ctypes.c_void_p]
        fn(_ptr(px3), n, _ptr(out))
    else:
        fn = lib().orc_yuv_words
        fn.restype = None
        fn.argtypes = [ctypes.c_void_p, ctypes.c_long, ctypes.c_int, ctypes.c_void_p]
        fn(_ptr(px3), n, int(yuv), _ptr(out))
    return out


# ------------------------------------------------------ reference CUDA build

_refgpu = {}


def refgpu_available(tr_y: int) -> bool:
    return os.path.exists(os.path.join(REF_DIR, f"libdepix_refgpu{tr_y}.so"))


def refgpu_lib(tr_y: int):
    """The reference's own stage bodies built for the GPU with its own device
    flags (oracle/ref_gpu.cu; Y threshold 5 or 48). Needs a CUDA device."""
    if tr_y not in _refgpu:
        L = ctypes.CDLL(os.path.join(REF_DIR, f"libdepix_refgpu{tr_y}.so"))
        vp = ctypes.c_void_p
        L.refgpu_frame.restype = ctypes.c_int
        L.refgpu_frame.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int] + [vp] * 9
        L.refgpu_yuv_words.restype = ctypes.c_int
        L.refgpu_yuv_words.argtypes = [vp]
        L.refgpu_last_error.restype = ctypes.c_char_p
        _refgpu[tr_y] = L
    return _refgpu[tr_y]


def _refgpu_check(L, rc):
    if rc != 0:
        raise RuntimeError("reference CUDA build: " + L.refgpu_last_error().decode())


def refgpu_frame(bgr, w, h, ws, subdivide=True, tr_y=48, graph_in=None) -> Frame:
    """All stage outputs of one frame from the reference's CUDA build."""
    bgr = np.ascontiguousarray(bgr, np.uint8)
    f = Frame(w, h)
    gi = None if graph_in is None else np.ascontiguousarray(graph_in, np.uint8)
    L = refgpu_lib(tr_y)
    _refgpu_check(L, L.refgpu_frame(_ptr(bgr), w, h, ws, int(bool(subdivide)), _ptr(gi), *f._args()))
    return f


def refgpu_yuv_words(tr_y: int = 5) -> np.ndarray:
    """The packed YUV word of every byte triple b0 | b1 << 8 | b2 << 16 (2^24
    entries) as the reference's CUDA build computes it."""
    out = np.zeros(1 << 24, np.uint32)
    L = refgpu_lib(tr_y)
    _refgpu_check(L, L.refgpu_yuv_words(_ptr(out)))
    return out
