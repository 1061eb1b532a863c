"""disccofan_gb300 -- GB300 component-forest hot path behind a C ABI.

Python view of ``libdcf_gb300.so`` (declared in ``include/dcf.h``).  It mirrors the
reference's operator surface for this path -- tree type, connectivity, attribute
index, lambda, filter rule, lambda-vector bins -- with the reference's names:

    ctx  = Context()
    tree = ctx.build(image, connectivity=4, tree_type="max", attribute=0)
    out  = tree.filter(attribute=0, lam=200.0, rule="direct")      # tree_filtering
    chk  = tree.check(attribute=0)                                 # tree_attribute_check
    spec = tree.pattern_spectrum(0, lvec)                          # tree_pattern_spectrum
    spec = tree.pattern_spectrum2d(14, lvec1, 0, lvec2)            # tree_pattern_spectrum2d

Images are numpy arrays (host memory) or CUDA torch tensors (device memory, used in
place).  Every computation runs in the CUDA library; there is no CPU fallback, and
importing this module fails loudly when the library has not been built.
"""
from __future__ import annotations

import contextlib
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdcf_gb300.so")

DTYPES = {np.dtype(np.uint8): 0, np.dtype(np.uint16): 1, np.dtype(np.uint32): 2, np.dtype(np.float32): 3}
RULES = {"direct": 0, "min": 1, "max": 2, "subtractive": 3}
TREE_TYPES = {"max": 0, "min": 1}
STATUS = {0: "ok", 1: "invalid argument", 2: "out of memory", 3: "CUDA error", 4: "device loop bound exceeded",
          5: "image contains NaN", 6: "invalid state", 7: "I/O error", 8: "unsupported"}

# attribute names, in the reference's AttribsArray order (attributes.c:1224-1248) + 18
ATTRIBUTES = ["area", "rectarea", "rectdiag", "xext", "yext", "zext", "xmean", "ymean", "zmean", "xwmean",
              "ywmean", "zwmean", "flux", "inertiatrace", "elong", "flat", "spars", "ncomp", "bboxelong"]
ATTR_GROUP = [0, 1, 1, 1, 1, 1, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 4, 1]


class DcfError(RuntimeError):
    def __init__(self, status: int, detail: str = ""):
        self.status = status
        super().__init__(f"dcf: {STATUS.get(status, status)}" + (f" ({detail})" if detail else ""))


class _Image(C.Structure):
    _fields_ = [("data", C.c_void_p), ("dtype", C.c_int), ("on_device", C.c_int), ("dims", C.c_uint64 * 3),
                ("connectivity", C.c_int), ("tree_type", C.c_int), ("pixdim", C.c_float * 3)]


class OpSet(C.Structure):
    """dcf_op_set: the operations of a batch run / an adjoint."""
    _fields_ = [("filter_attr", C.c_int), ("lam", C.c_double), ("spec_attr1", C.c_int), ("lvec1", C.c_void_p),
                ("n1", C.c_int), ("spec_attr2", C.c_int), ("lvec2", C.c_void_p), ("n2", C.c_int),
                ("use_graph", C.c_int)]


def make_ops(filter_attr=-1, lam=0.0, spectrum=None, use_graph=False):
    """OpSet plus the lambda arrays it points to (keep both alive).  spectrum =
    (attr1, lvec1, attr2, lvec2) with lvecs including the leading 0."""
    keep = []
    ops = OpSet(filter_attr, float(lam), -1, None, 0, 0, None, 0, int(use_graph))
    if spectrum is not None:
        a1, l1, a2, l2 = spectrum
        l1 = np.ascontiguousarray(l1, np.float32)
        l2 = np.ascontiguousarray(l2, np.float32)
        keep += [l1, l2]
        ops.spec_attr1, ops.lvec1, ops.n1 = a1, l1.ctypes.data, l1.size
        ops.spec_attr2, ops.lvec2, ops.n2 = a2, l2.ctypes.data, l2.size
    return ops, keep


_lib = None
_exiting = False


def _at_exit():
    # objects finalised during interpreter shutdown must not call into CUDA
    global _exiting
    _exiting = True


import atexit  # noqa: E402

atexit.register(_at_exit)


def library() -> C.CDLL:
    """Load libdcf_gb300.so (raises if it was not built: no fallback path exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing; run `python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(LIB_PATH)
    vp, i, d, u64 = C.c_void_p, C.c_int, C.c_double, C.c_uint64
    sig = {
        "dcf_ctx_create": [i, vp, C.POINTER(vp)],
        "dcf_ctx_destroy": [vp],
        "dcf_ctx_synchronize": [vp],
        "dcf_tree_build": [vp, C.POINTER(_Image), i, C.POINTER(vp)],
        "dcf_tree_set_attribute": [vp, vp, i],
        "dcf_tree_destroy": [vp],
        "dcf_tree_info": [vp, C.POINTER(u64), C.POINTER(u64), C.POINTER(i), C.POINTER(C.c_float)],
        "dcf_tree_parent": [vp, vp, vp, i],
        "dcf_tree_gval": [vp, vp, vp, i],
        "dcf_node_attribute": [vp, vp, i, i, vp, i],
        "dcf_filter": [vp, vp, i, i, d, i, vp, i],
        "dcf_filter_as": [vp, vp, i, i, d, i, i, vp, i],
        "dcf_image_stage": [vp, C.POINTER(_Image), C.POINTER(_Image)],
        "dcf_attribute_check": [vp, vp, i, vp, i],
        "dcf_dmp": [vp, vp, i, i, vp, i, vp, i],
        "dcf_pattern_spectrum": [vp, vp, i, vp, i, vp, i],
        "dcf_pattern_spectrum2d": [vp, vp, i, vp, i, i, vp, i, vp, i],
        "dcf_lvec_read": [C.c_char_p, d, vp, i, C.POINTER(i)],
        "dcf_tree_export": [vp, vp, i, C.c_char_p],
        "dcf_csl": [vp, vp, i, vp, i, vp, vp, vp, i],
        "dcf_fits_read": [C.c_char_p, vp, u64, C.POINTER(u64 * 3), C.POINTER(i)],
        "dcf_fits_read_raw": [C.c_char_p, vp, u64, C.POINTER(u64 * 3), C.POINTER(i)],
        "dcf_batch_create": [vp, i, vp, vp, i, i, i, vp, C.POINTER(vp)],
        "dcf_batch_destroy": [vp],
        "dcf_batch_info": [vp, C.POINTER(u64), C.POINTER(u64), vp, C.POINTER(u64)],
        "dcf_batch_set_schedule": [vp, vp, i, i, i, i],
        "dcf_batch_set_merge": [vp, vp, i, i],
        "dcf_batch_autotune": [vp, vp, vp, i, i, C.POINTER(d)],
        "dcf_batch_run": [vp, vp, vp, i, C.POINTER(OpSet), vp, vp, i],
        "dcf_batch_parent": [vp, vp, vp, i],
        "dcf_batch_node_attribute": [vp, vp, i, vp, i],
        "dcf_batch_adjoint": [vp, vp, vp, vp, vp, i],
        "dcf_tree_adjoint": [vp, vp, C.POINTER(OpSet), vp, vp, vp, i],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = C.c_int
    L.dcf_ctx_last_error.argtypes = [vp]
    L.dcf_ctx_last_error.restype = C.c_char_p
    L.dcf_status_string.argtypes = [C.c_int]
    L.dcf_status_string.restype = C.c_char_p
    L.dcf_ctx_launch_count.argtypes = [vp]
    L.dcf_ctx_launch_count.restype = C.c_uint64
    L.dcf_ctx_stream.argtypes = [vp]
    L.dcf_ctx_stream.restype = C.c_void_p
    L.dcf_ctx_set_profiling.argtypes = [vp, i]
    L.dcf_ctx_set_profiling.restype = C.c_int
    L.dcf_ctx_profile.argtypes = [vp, i, C.POINTER(d), C.POINTER(u64)]
    L.dcf_ctx_profile.restype = C.c_int
    L.dcf_profile_num_kernels.restype = C.c_int
    L.dcf_profile_kernel_name.argtypes = [i]
    L.dcf_profile_kernel_name.restype = C.c_char_p
    _lib = L
    return L


def _is_torch_cuda(x) -> bool:
    return type(x).__module__.startswith("torch") and getattr(x, "is_cuda", False)


def lvec_from_values(values, imscale: float = 1.0) -> np.ndarray:
    """The bins lambda_vector_read builds from file values: [0, v1/imscale, ...] (float32)."""
    out = [np.float32(0.0)]
    for v in values:
        out.append(np.float32(np.float64(np.float32(v)) / imscale))
    return np.array(out, dtype=np.float32)


def read_lvec(path: str, imscale: float = 1.0) -> np.ndarray:
    """Read a "#LambdaVector file..." file exactly as the reference does (lambdavec.c:35)."""
    L = library()
    n = C.c_int(0)
    st = L.dcf_lvec_read(path.encode(), imscale, None, 0, C.byref(n))
    if st:
        raise DcfError(st, path)
    out = np.empty(n.value, np.float32)
    st = L.dcf_lvec_read(path.encode(), imscale, out.ctypes.data, out.size, C.byref(n))
    if st:
        raise DcfError(st, path)
    return out


def read_fits(path: str) -> np.ndarray:
    """Primary FITS image as the reference reads it (float32, BZERO + BSCALE * raw),
    shaped (H, W) or (D, H, W)."""
    L = library()
    dims = (C.c_uint64 * 3)()
    bp = C.c_int()
    st = L.dcf_fits_read(path.encode(), None, 0, C.byref(dims), C.byref(bp))
    if st:
        raise DcfError(st, path)
    w, h, d = dims[0], dims[1], dims[2]
    out = np.empty(w * h * d, np.float32)
    st = L.dcf_fits_read(path.encode(), out.ctypes.data, out.size, C.byref(dims), C.byref(bp))
    if st:
        raise DcfError(st, path)
    return out.reshape((h, w) if d == 1 else (d, h, w))


def read_fits_raw(path: str) -> np.ndarray:
    """Primary FITS image in its own pixel type (uint8, uint16 with BZERO 32768,
    uint32 with BZERO 2^31, float32), for a build without a float copy; raises
    DcfError (status unsupported) for other scalings, which read_fits handles."""
    L = library()
    dims = (C.c_uint64 * 3)()
    dt = C.c_int()
    st = L.dcf_fits_read_raw(path.encode(), None, 0, C.byref(dims), C.byref(dt))
    if st:
        raise DcfError(st, path)
    w, h, d = dims[0], dims[1], dims[2]
    out = np.empty(w * h * d, (np.uint8, np.uint16, np.uint32, np.float32)[dt.value])
    st = L.dcf_fits_read_raw(path.encode(), out.ctypes.data, out.nbytes, C.byref(dims), C.byref(dt))
    if st:
        raise DcfError(st, path)
    return out.reshape((h, w) if d == 1 else (d, h, w))


class Context:
    """One GPU, one CUDA stream, reusable device workspace (dcf_ctx)."""

    def __init__(self, device: int = 0, stream=None):
        self.lib = library()
        h = C.c_void_p()
        st = self.lib.dcf_ctx_create(device, C.c_void_p(stream) if stream else None, C.byref(h))
        if st:
            raise DcfError(st, "dcf_ctx_create")
        self.h = h
        self.device = device
        self._torch_stream = None

    @contextlib.contextmanager
    def ordered(self, *arrays):
        """Around a call that reads or writes CUDA tensors: this context's stream first
        waits for the work queued on torch's current stream (the tensors' producers),
        and torch's current stream then waits for the call (its consumers, and the
        caching allocator's reuse of the tensors).  Nothing to do for host arrays, or
        when torch's current stream is this context's stream."""
        if not any(_is_torch_cuda(a) for a in arrays):
            yield
            return
        import torch
        cur = torch.cuda.current_stream(self.device)
        if self._torch_stream is None:
            self._torch_stream = torch.cuda.ExternalStream(self.lib.dcf_ctx_stream(self.h), device=self.device)
        own = self._torch_stream
        same = cur.cuda_stream == own.cuda_stream
        if not same:
            own.wait_stream(cur)
        try:
            yield
        finally:
            if not same:
                cur.wait_stream(own)

    def close(self):
        if getattr(self, "h", None) and not _exiting:
            self.lib.dcf_ctx_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, st: int, what: str = ""):
        if st:
            detail = self.lib.dcf_ctx_last_error(self.h).decode(errors="replace")
            raise DcfError(st, f"{what}: {detail}" if what else detail)

    def synchronize(self):
        self.check(self.lib.dcf_ctx_synchronize(self.h), "synchronize")

    @property
    def launches(self) -> int:
        return int(self.lib.dcf_ctx_launch_count(self.h))

    def set_profiling(self, enable: bool = True):
        """Per-kernel CUDA-event timing on this context's stream (resets totals)."""
        self.check(self.lib.dcf_ctx_set_profiling(self.h, int(enable)), "set_profiling")

    def profile(self) -> dict:
        """{kernel name: (total device ms, launch groups)} since profiling was enabled."""
        out = {}
        for k in range(self.lib.dcf_profile_num_kernels()):
            ms, n = C.c_double(), C.c_uint64()
            self.check(self.lib.dcf_ctx_profile(self.h, k, C.byref(ms), C.byref(n)), "profile")
            if n.value:
                out[self.lib.dcf_profile_kernel_name(k).decode()] = (ms.value, n.value)
        return out

    def build(self, image, connectivity: int = 4, tree_type: str = "max", attribute: int = 0,
              pixdim=(1.0, 1.0, 1.0)) -> "Tree":
        """build_tree_with_attributes: tree of a 2-D (H, W) or 3-D (D, H, W) image
        (numpy array, CUDA tensor, or a StagedImage from stage())."""
        return Tree(self, image, connectivity, tree_type, attribute, pixdim)

    def stage(self, image) -> "StagedImage":
        """dcf_image_stage: copy a host image to this context's device buffer once,
        for several builds (valid until the next stage() on this context)."""
        arr = np.ascontiguousarray(image)
        if arr.dtype not in DTYPES:
            raise TypeError(f"unsupported image dtype {arr.dtype} (u8, u16, u32, f32)")
        if arr.ndim not in (2, 3):
            raise ValueError("image must be 2-D or 3-D")
        d, h, w = (1,) + arr.shape if arr.ndim == 2 else arr.shape
        im = _Image(arr.ctypes.data, DTYPES[arr.dtype], 0, (C.c_uint64 * 3)(w, h, d), 4, 0,
                    (C.c_float * 3)(1.0, 1.0, 1.0))
        out = _Image()
        self.check(self.lib.dcf_image_stage(self.h, C.byref(im), C.byref(out)), "dcf_image_stage")
        return StagedImage(out, arr.shape, arr.dtype, arr)


    def batch(self, shapes, dtype=np.float32, connectivity: int = 8, attribute: int = 0,
              pixdim=(1.0, 1.0, 1.0)) -> "Batch":
        """A batch of 2-D cutouts; shapes = [(height, width), ...]."""
        return Batch(self, shapes, dtype, connectivity, attribute, pixdim)


class StagedImage:
    """An image copied to a context's device buffer by Context.stage()."""

    def __init__(self, im, shape, dtype, host):
        self.im = im
        self.shape = tuple(shape)
        self.dtype = np.dtype(dtype)
        self._host = host  # the copy is stream-ordered: keep the source alive


class Tree:
    def __init__(self, ctx: Context, image, connectivity, tree_type, attribute, pixdim):
        self.ctx = ctx
        L = ctx.lib
        on_dev = _is_torch_cuda(image)
        if isinstance(image, StagedImage):
            on_dev = True
            dt = image.dtype
            ptr = image.im.data
            shape = image.shape
            self._keep = image
        elif on_dev:
            import torch
            tdt = {torch.uint8: np.uint8, torch.uint16: np.uint16, torch.int32: None,
                   torch.float32: np.float32}.get(image.dtype)
            if image.dtype == getattr(torch, "uint32", None):
                tdt = np.uint32
            if tdt is None:
                raise TypeError(f"unsupported tensor dtype {image.dtype}")
            if not image.is_contiguous():
                raise ValueError("device image must be contiguous")
            dt = np.dtype(tdt)
            ptr = image.data_ptr()
            shape = tuple(image.shape)
            self._keep = image
        else:
            arr = np.ascontiguousarray(image)
            if arr.dtype not in DTYPES:
                raise TypeError(f"unsupported image dtype {arr.dtype} (u8, u16, u32, f32)")
            dt = arr.dtype
            ptr = arr.ctypes.data
            shape = arr.shape
            self._keep = arr
        if len(shape) == 2:
            d, h, w = 1, shape[0], shape[1]
        elif len(shape) == 3:
            d, h, w = shape
        else:
            raise ValueError("image must be 2-D or 3-D")
        self.shape = tuple(shape)
        im = _Image(ptr, DTYPES[dt], int(on_dev), (C.c_uint64 * 3)(w, h, d), connectivity,
                    TREE_TYPES[tree_type], (C.c_float * 3)(*pixdim))
        hnd = C.c_void_p()
        with ctx.ordered(image):
            ctx.check(L.dcf_tree_build(ctx.h, C.byref(im), attribute, C.byref(hnd)), "dcf_tree_build")
        self.h = hnd
        self.n = w * h * d
        self.attribute = attribute
        self.tree_type = tree_type

    def close(self):
        if getattr(self, "h", None) and not _exiting:
            self.ctx.lib.dcf_tree_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- helpers -----------------------------------------------------------
    def _out(self, dtype, out=None, count=None):
        count = self.n if count is None else count
        if out is not None:
            if _is_torch_cuda(out):
                return out, out.data_ptr(), 1
            return out, out.ctypes.data, 0
        a = np.empty(count, dtype)
        return a, a.ctypes.data, 0

    def _shape(self, a, lead=()):
        return a.reshape(lead + self.shape) if isinstance(a, np.ndarray) else a

    def set_attribute(self, attribute: int):
        """flood_attributes: accumulate a new attribute group on this tree."""
        self.ctx.check(self.ctx.lib.dcf_tree_set_attribute(self.ctx.h, self.h, attribute), "set_attribute")
        self.attribute = attribute

    def _ensure_group(self, attribute: int):
        # area (0) is readable from every group's records
        if attribute != 0 and ATTR_GROUP[attribute] != ATTR_GROUP[self.attribute]:
            self.set_attribute(attribute)

    def csl(self, attribute: int, lvec):
        """CSL segmentation (perform_csl): (contrast, scale, luminance) images;
        lvec includes the leading 0 (read_lvec / lvec_from_values)."""
        self._ensure_group(attribute)
        lv = np.ascontiguousarray(lvec, np.float32)
        outs = [np.empty(self.n, np.float32) for _ in range(3)]
        self.ctx.check(self.ctx.lib.dcf_csl(self.ctx.h, self.h, attribute, lv.ctypes.data, lv.size,
                                            *[o.ctypes.data for o in outs], 0), "csl")
        return tuple(self._shape(o) for o in outs)

    def export(self, path: str, attribute: int | None = None):
        """Write the tree file (write_tree's format) for an attribute of the current group."""
        a = self.attribute if attribute is None else attribute
        self._ensure_group(a)
        self.ctx.check(self.ctx.lib.dcf_tree_export(self.ctx.h, self.h, a, path.encode()), "tree_export")

    def info(self):
        n, m, c, g = C.c_uint64(), C.c_uint64(), C.c_int(), C.c_float()
        self.ctx.check(self.ctx.lib.dcf_tree_info(self.h, C.byref(n), C.byref(m), C.byref(c), C.byref(g)), "info")
        return {"pixels": n.value, "nodes": m.value, "connectivity": c.value, "max_gval": g.value}

    # -- tree data ---------------------------------------------------------
    def parent(self, out=None):
        a, p, dev = self._out(np.int64, out)
        with self.ctx.ordered(a):
            self.ctx.check(self.ctx.lib.dcf_tree_parent(self.ctx.h, self.h, p, dev), "parent")
        return a

    def gval(self, out=None):
        a, p, dev = self._out(np.float32, out)
        with self.ctx.ordered(a):
            self.ctx.check(self.ctx.lib.dcf_tree_gval(self.ctx.h, self.h, p, dev), "gval")
        return a

    def node_attribute(self, attribute: int, area: bool = False, out=None):
        self._ensure_group(attribute)
        a, p, dev = self._out(np.float64, out)
        with self.ctx.ordered(a):
            self.ctx.check(self.ctx.lib.dcf_node_attribute(self.ctx.h, self.h, attribute, int(area), p, dev),
                           "node_attribute")
        return a

    # -- operations (operation.c) ------------------------------------------
    def filter(self, attribute: int, lam: float, rule="direct", extract: bool = False, out=None, out_dtype=None):
        """tree_filtering (+ extract, min-tree re-inversion).  The output is float32,
        or, with out_dtype (or an `out` array) of the input's own uint8/uint16 type,
        that type (dcf_filter_as)."""
        self._ensure_group(attribute)
        r = RULES[rule] if isinstance(rule, str) else int(rule)
        if out is not None and out_dtype is None:
            odt = getattr(out, "dtype", None)
            if odt is not None and "uint16" in str(odt):
                out_dtype = np.uint16
            elif odt is not None and "uint8" in str(odt):
                out_dtype = np.uint8
        if out_dtype is None or np.dtype(out_dtype) == np.float32:
            a, p, dev = self._out(np.float32, out)
            with self.ctx.ordered(a):
                self.ctx.check(self.ctx.lib.dcf_filter(self.ctx.h, self.h, attribute, r, float(lam), int(extract), p,
                                                       dev), "filter")
            return self._shape(a)
        odt = np.dtype(out_dtype)
        if odt not in DTYPES:
            raise TypeError(f"unsupported output dtype {odt}")
        a, p, dev = self._out(odt, out)
        with self.ctx.ordered(a):
            self.ctx.check(self.ctx.lib.dcf_filter_as(self.ctx.h, self.h, attribute, r, float(lam), int(extract),
                                                      DTYPES[odt], p, dev), "filter_as")
        return self._shape(a)

    def check(self, attribute: int, out=None):
        self._ensure_group(attribute)
        a, p, dev = self._out(np.float32, out)
        with self.ctx.ordered(a):
            self.ctx.check(self.ctx.lib.dcf_attribute_check(self.ctx.h, self.h, attribute, p, dev), "check")
        return self._shape(a)

    def dmp(self, attribute: int, lvec, rule="direct", out=None):
        self._ensure_group(attribute)
        lv = np.ascontiguousarray(lvec, np.float32)
        r = RULES[rule] if isinstance(rule, str) else int(rule)
        a, p, dev = self._out(np.float32, out, count=(lv.size - 1) * self.n)
        with self.ctx.ordered(a):
            self.ctx.check(self.ctx.lib.dcf_dmp(self.ctx.h, self.h, attribute, r, lv.ctypes.data, lv.size, p, dev),
                           "dmp")
        return self._shape(a, (lv.size - 1,))

    def pattern_spectrum(self, attribute: int, lvec, out=None):
        """lvec: bins including the leading 0 (read_lvec / lvec_from_values)."""
        self._ensure_group(attribute)
        lv = np.ascontiguousarray(lvec, np.float32)
        spec = out if out is not None else np.zeros(lv.size, np.float64)
        dev = int(_is_torch_cuda(spec))
        p = spec.data_ptr() if dev else spec.ctypes.data
        with self.ctx.ordered(spec):
            self.ctx.check(self.ctx.lib.dcf_pattern_spectrum(self.ctx.h, self.h, attribute, lv.ctypes.data, lv.size,
                                                             p, dev), "pattern_spectrum")
        return spec

    def pattern_spectrum2d(self, attr1: int, lvec1, attr2: int, lvec2, out=None):
        """spectrum[s2, s1] (row-major [n2, n1]), the reference's s1 + s2*n1 layout."""
        self._ensure_group(attr1)
        l1 = np.ascontiguousarray(lvec1, np.float32)
        l2 = np.ascontiguousarray(lvec2, np.float32)
        spec = out if out is not None else np.zeros((l2.size, l1.size), np.float64)
        dev = int(_is_torch_cuda(spec))
        p = spec.data_ptr() if dev else spec.ctypes.data
        with self.ctx.ordered(spec):
            self.ctx.check(self.ctx.lib.dcf_pattern_spectrum2d(self.ctx.h, self.h, attr1, l1.ctypes.data, l1.size,
                                                               attr2, l2.ctypes.data, l2.size, p, dev),
                           "pattern_spectrum2d")
        return spec

    # -- adjoint -------------------------------------------------------------
    def adjoint(self, grad_filtered=None, filter_attr: int = -1, lam: float = 0.0, grad_spectrum=None,
                spectrum=None, out=None):
        """d loss / d pixels of loss = sum(grad_filtered * filter(filter_attr, lam, "direct"))
        + sum(grad_spectrum * pattern_spectrum2d(*spectrum)), this tree held fixed
        (float32 max-trees).  grad_spectrum has the [n2, n1] layout of pattern_spectrum2d."""
        ops, keep = make_ops(filter_attr, lam, spectrum)
        dev = int(out is not None and _is_torch_cuda(out))

        def ptr(x, dt):
            if x is None:
                return None, None
            if dev:
                return x, x.data_ptr()
            a = np.ascontiguousarray(x, dt)
            return a, a.ctypes.data
        v, vp = ptr(grad_filtered, np.float32)
        w, wp = ptr(grad_spectrum, np.float64)
        a, p, _ = self._out(np.float32, out)
        with self.ctx.ordered(a, grad_filtered, grad_spectrum):
            self.ctx.check(self.ctx.lib.dcf_tree_adjoint(self.ctx.h, self.h, C.byref(ops), vp, wp, p, dev),
                           "adjoint")
        return self._shape(a)


class Batch:
    """Many 2-D cutouts built, filtered and binned together (dcf_batch)."""

    def __init__(self, ctx: Context, shapes, dtype, connectivity, attribute, pixdim):
        self.ctx = ctx
        self.shapes = [(int(h), int(w)) for h, w in shapes]
        self.dtype = np.dtype(dtype)
        hs = np.array([h for h, _ in self.shapes], np.uint32)
        ws = np.array([w for _, w in self.shapes], np.uint32)
        sizes = hs.astype(np.int64) * ws
        self.offsets = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
        self.n = int(sizes.sum())
        self.count = len(self.shapes)
        pd = (C.c_float * 3)(*pixdim)
        hnd = C.c_void_p()
        ctx.check(ctx.lib.dcf_batch_create(ctx.h, self.count, ws.ctypes.data, hs.ctypes.data, DTYPES[self.dtype],
                                           connectivity, attribute, pd, C.byref(hnd)), "dcf_batch_create")
        self.h = hnd
        self.attribute = attribute
        self._keep = None

    def close(self):
        if getattr(self, "h", None) and not _exiting:
            self.ctx.lib.dcf_batch_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def concat(self, cutouts) -> np.ndarray:
        """Concatenate host cutouts (each (H, W)) in the batch's pixel order."""
        return np.concatenate([np.ascontiguousarray(c, self.dtype).ravel() for c in cutouts])

    def split(self, flat):
        """Per-cutout (H, W) views of a concatenated per-pixel array."""
        return [flat[o:o + h * w].reshape(h, w) for o, (h, w) in zip(self.offsets, self.shapes)]

    def _pixels(self, pixels):
        if _is_torch_cuda(pixels):
            return pixels.data_ptr(), 1
        a = np.ascontiguousarray(pixels, self.dtype).ravel()
        if a.size != self.n:
            raise ValueError(f"expected {self.n} pixels, got {a.size}")
        self._keep = a
        return a.ctypes.data, 0

    def info(self):
        n, m, g = C.c_uint64(), C.c_uint64(), C.c_uint64()
        sch = (C.c_int * 6)()
        self.ctx.check(self.ctx.lib.dcf_batch_info(self.h, C.byref(n), C.byref(m), sch, C.byref(g)), "batch_info")
        return {"pixels": n.value, "nodes": m.value, "tile": (sch[0], sch[1]), "ctas_per_sm": sch[2],
                "chunk": sch[3], "seam_buckets": sch[4], "up_steps": sch[5], "graph_kernels": g.value}

    def set_schedule(self, tile=(64, 64), ctas_per_sm=0, chunk=1):
        self.ctx.check(self.ctx.lib.dcf_batch_set_schedule(self.ctx.h, self.h, tile[0], tile[1], ctas_per_sm, chunk),
                       "set_schedule")

    def set_merge(self, seam_buckets: int = 16, up_steps: int = 2048):
        self.ctx.check(self.ctx.lib.dcf_batch_set_merge(self.ctx.h, self.h, seam_buckets, up_steps), "set_merge")

    def autotune(self, pixels, repeats: int = 3) -> float:
        p, dev = self._pixels(pixels)
        ms = C.c_double()
        with self.ctx.ordered(pixels):
            self.ctx.check(self.ctx.lib.dcf_batch_autotune(self.ctx.h, self.h, p, dev, repeats, C.byref(ms)),
                           "autotune")
        return ms.value

    def run(self, pixels, filter_attr: int = -1, lam: float = 0.0, spectrum=None, use_graph: bool = True,
            filtered=None, spectra=None, want_filtered: bool = True, want_spectra: bool = True):
        """Build all trees, then filter and/or bin.  pixels: host array (concatenated or
        a list of cutouts) or a CUDA tensor of N elements.  Outputs go to `filtered` /
        `spectra` when given (CUDA tensors: device outputs), else new host arrays.
        Returns (filtered[N] or None, spectra[count, n2, n1] or None)."""
        if isinstance(pixels, (list, tuple)):
            pixels = self.concat(pixels)
        p, pdev = self._pixels(pixels)
        ops, keep = make_ops(filter_attr, lam, spectrum, use_graph)
        odev = int((filtered is not None and _is_torch_cuda(filtered)) or
                   (spectra is not None and _is_torch_cuda(spectra)))
        f = s = None
        if filter_attr >= 0 and want_filtered:
            f = filtered if filtered is not None else np.empty(self.n, np.float32)
        if spectrum is not None and want_spectra:
            s = spectra if spectra is not None else np.empty((self.count, ops.n2, ops.n1), np.float64)
        fp = (f.data_ptr() if odev else f.ctypes.data) if f is not None else None
        sp = (s.data_ptr() if odev else s.ctypes.data) if s is not None else None
        with self.ctx.ordered(pixels, f, s):
            self.ctx.check(self.ctx.lib.dcf_batch_run(self.ctx.h, self.h, p, pdev, C.byref(ops), fp, sp, odev),
                           "batch_run")
        self._ops_keep = keep
        return f, s

    def parent(self, out=None):
        """Canonical parents, as indices inside each cutout (concatenated)."""
        a = out if out is not None else np.empty(self.n, np.int64)
        dev = int(_is_torch_cuda(a))
        with self.ctx.ordered(a):
            self.ctx.check(self.ctx.lib.dcf_batch_parent(self.ctx.h, self.h, a.data_ptr() if dev else a.ctypes.data,
                                                         dev), "batch_parent")
        return a

    def node_attribute(self, attribute: int, out=None):
        a = out if out is not None else np.empty(self.n, np.float64)
        dev = int(_is_torch_cuda(a))
        with self.ctx.ordered(a):
            self.ctx.check(self.ctx.lib.dcf_batch_node_attribute(self.ctx.h, self.h, attribute,
                                                                 a.data_ptr() if dev else a.ctypes.data, dev),
                           "batch_node_attribute")
        return a

    def adjoint(self, grad_filtered=None, grad_spectra=None, out=None):
        """d loss / d pixels for the last run's operations (trees held fixed)."""
        dev = int(out is not None and _is_torch_cuda(out))
        if dev:
            vp = grad_filtered.data_ptr() if grad_filtered is not None else None
            wp = grad_spectra.data_ptr() if grad_spectra is not None else None
            g = out
            gp = out.data_ptr()
        else:
            v = None if grad_filtered is None else np.ascontiguousarray(grad_filtered, np.float32).ravel()
            w = None if grad_spectra is None else np.ascontiguousarray(grad_spectra, np.float64).ravel()
            vp = v.ctypes.data if v is not None else None
            wp = w.ctypes.data if w is not None else None
            g = np.empty(self.n, np.float32)
            gp = g.ctypes.data
        with self.ctx.ordered(g, grad_filtered, grad_spectra):
            self.ctx.check(self.ctx.lib.dcf_batch_adjoint(self.ctx.h, self.h, vp, wp, gp, dev), "batch_adjoint")
        return g
