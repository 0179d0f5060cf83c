"""The C ABI without a GPU: the library loads, exports every function that
include/depix.h declares, and rejects bad arguments before touching CUDA."""
import ctypes
import os
import re

import pytest

from conftest import REPO

HEADER = os.path.join(REPO, "include", "depix.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w \*]*?\b([A-Za-z_]\w*)\s*\(", src, flags=re.M)
    return sorted({n for n in names if n not in ("defined",)})


@pytest.fixture(scope="module")
def L():
    import build
    build.build()
    import depix
    return depix.lib()


def test_header_declares_the_drop_in_symbol():
    names = declared_functions()
    assert "launch_kernel" in names and "depix_raster" in names and len(names) >= 20


def test_library_exports_every_declared_function(L):
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_status_strings(L):
    assert L.depix_status_string(0) == b"ok"
    assert L.depix_status_string(1) == b"invalid argument"


def test_bad_arguments_are_rejected_before_cuda(L):
    import depix
    p = depix.params()
    # NULL image
    assert L.depix_graph(None, 4, 4, 16, 1, ctypes.byref(p), 1, ctypes.c_void_p(16), None) == 1
    # zero size
    assert L.depix_graph(ctypes.c_void_p(16), 0, 4, 16, 1, ctypes.byref(p), 1, ctypes.c_void_p(16), None) == 1
    # RGBA stride too small
    assert L.depix_graph(ctypes.c_void_p(16), 4, 4, 8, 1, ctypes.byref(p), 1, ctypes.c_void_p(16), None) == 1
    # bad scale
    bad = depix.params(scale=0)
    assert L.depix_raster(ctypes.c_void_p(16), 4, 4, 16, 1, ctypes.c_void_p(16), ctypes.byref(bad),
                          ctypes.c_void_p(16), None) == 1
    # aliasing snapshot and output
    assert L.depix_resolve_heuristics(ctypes.c_void_p(16), 4, 4, ctypes.c_void_p(16), None) == 1
    assert L.depix_resolve_heuristics_vote(ctypes.c_void_p(16), 4, 4, ctypes.c_void_p(16), None) == 1
    # heuristics decision other than 0 / 1
    bad = depix.params()
    bad.vote = 2
    assert L.depix_graph(ctypes.c_void_p(16), 4, 4, 16, 1, ctypes.byref(bad), 1, ctypes.c_void_p(16), None) == 1
    assert b"vote" in L.depix_last_error()
    # empty context
    h = ctypes.c_void_p()
    assert L.depix_context_create(ctypes.byref(h), 0, 1) == 1
    assert b"capacity" in L.depix_last_error()
    # launch shape of a missing context
    assert L.depix_context_set_launch_shape(None, 1, 32, 32) == 1
    # border walks: no frames, no capacity, a NULL buffer
    v = ctypes.c_void_p(16)
    assert L.depix_border_walks(v, 8, 8, 0, v, v, v, v, 16, 16, v, None) == 1
    assert L.depix_border_walks(v, 8, 8, 1, v, v, v, v, 0, 16, v, None) == 1
    assert L.depix_border_walks(v, 8, 8, 1, v, v, v, None, 16, 16, v, None) == 1
    assert L.depix_border_walks(v, 0, 8, 1, v, v, v, v, 16, 16, v, None) == 1


def test_default_params(L):
    import depix
    p = depix.Params()
    L.depix_default_params(ctypes.byref(p))
    assert (p.tr_y, p.tr_u, p.tr_v, p.subdivide, p.scale, p.vote) == (48, 7, 6, 1, 4, 0)
