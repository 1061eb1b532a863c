"""The allocation-free direct-rule filter, dcf_filter_direct_noalloc.

It serves callers that cannot allocate device memory while they filter (a host
framework whose caching allocator already holds the free device memory, or a
real-time loop that must not wait on an allocation): its scratch is a fixed device
array inside the library instead of context buffers.  These tests call it through
the C ABI and check that it returns exactly what the ordinary dcf_filter returns
(filtered images are compared bit-exactly everywhere in this suite), on two calls
in a row that share the array, and that it refuses trees larger than its array.

This file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

import disccofan_gb300 as dcf

pytestmark = pytest.mark.gpu

MAX_PIXELS = 1 << 23


def _noalloc(lib):
    fn = lib.dcf_filter_direct_noalloc
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_int, C.c_void_p]
    fn.restype = C.c_int
    return fn


def _image(shape, seed):
    rng = np.random.default_rng(seed)
    base = rng.integers(0, 4000, shape).astype(np.float64)
    k = np.ones(5) / 5.0
    for ax in range(2):
        base = np.apply_along_axis(lambda v: np.convolve(v, k, mode="same"), ax, base)
    return np.rint(base).astype(np.uint16)


def test_noalloc_matches_dcf_filter_on_consecutive_calls():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = dcf.Context(0)
    lib = ctx.lib
    noalloc = _noalloc(lib)
    img = _image((700, 900), 11)
    tree = ctx.build(img, connectivity=8, tree_type="max", attribute=0)
    n = img.size
    ref = torch.empty(n, dtype=torch.float32, device="cuda")
    got = torch.empty(n, dtype=torch.float32, device="cuda")
    for lam, extract in ((40.0, 0), (400.0, 1)):
        ctx.check(lib.dcf_filter(ctx.h, tree.h, 0, 0, lam, extract, C.c_void_p(ref.data_ptr()), 1), "dcf_filter")
        got.fill_(-1.0)
        ctx.check(noalloc(ctx.h, tree.h, 0, lam, extract, C.c_void_p(got.data_ptr())), "noalloc")
        ctx.synchronize()
        assert torch.equal(got, ref), (lam, extract)
    # a third call repeats the first: results must not depend on the previous contents
    ctx.check(lib.dcf_filter(ctx.h, tree.h, 0, 0, 40.0, 0, C.c_void_p(ref.data_ptr()), 1), "dcf_filter")
    ctx.check(noalloc(ctx.h, tree.h, 0, 40.0, 0, C.c_void_p(got.data_ptr())), "noalloc")
    ctx.synchronize()
    assert torch.equal(got, ref)
    tree.close()
    ctx.close()


def test_noalloc_rejects_trees_beyond_its_array():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = dcf.Context(0)
    noalloc = _noalloc(ctx.lib)
    side = 2900  # 8,410,000 pixels > 8,388,608
    assert side * side > MAX_PIXELS
    img = np.zeros((side, side), np.uint8)
    img[::7, ::5] = 3
    tree = ctx.build(img, connectivity=4, tree_type="max", attribute=0)
    out = torch.empty(side * side, dtype=torch.float32, device="cuda")
    st = noalloc(ctx.h, tree.h, 0, 10.0, 0, C.c_void_p(out.data_ptr()))
    assert st == 1
    assert b"exceed" in ctx.lib.dcf_ctx_last_error(ctx.h)
    tree.close()
    ctx.close()
