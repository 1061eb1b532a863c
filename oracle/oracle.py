"""CPU oracle wrappers (TEST INFRASTRUCTURE ONLY).

Two libraries, both built by ``oracle/Makefile`` into ``oracle/_ref/``:

* ``libdcfref.so``   -- the reference's own hot-path C sources (flood.c,
  attributes.c, filtering.c, pattern.c, operation.c, ...) compiled unmodified
  with a single-rank mpi.h stub.  It only builds where the reference checkout
  exists, so it is used by CPU tests here to pin ``libdcforacle.so``.
* ``libdcforacle.so`` -- ``oracle/dcf_oracle.c``, a CPU restatement of the same
  algorithms in this project's own code.  It builds anywhere (gcc only) and is
  the checker that GPU parity tests and ``bench.py``'s CPU baseline use.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (its CPU-baseline
leg) may import this module.  The product never routes through it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SO = os.path.join(HERE, "_ref", "libdcfref.so")
PORT_SO = os.path.join(HERE, "_ref", "libdcforacle.so")

# filter rules (filtering.c:271-277) and operation names (operation.c:110-211)
RULES = {"direct": 0, "min": 1, "max": 2, "subtractive": 3}


# The reference checkout the recipes compile from and CPU tests compare with:
# $DCF_REFERENCE_DIR, else the build container's checkout location.  GPU machines have
# no checkout; there reference_dir() is None and only the committed fixtures pin
# the restatement.
_DEFAULT_REFERENCE_DIR = "/root/reference"


def reference_dir():
    """Path of the reference checkout, or None when it is absent."""
    d = os.environ.get("DCF_REFERENCE_DIR") or _DEFAULT_REFERENCE_DIR
    return d if os.path.exists(os.path.join(d, "src", "sources", "flood.c")) else None


def build(ref: bool = False) -> None:
    """Compile the oracle port (and, when asked and present, the reference)."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    if ref and reference_dir():
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REFSRC=" + os.path.join(reference_dir(), "src")],
                       check=True)


def write_lvec(values, path=None) -> str:
    """Write a lambda-vector file in the reference's format (lambdavec.c:35-84)."""
    if path is None:
        fd, path = tempfile.mkstemp(suffix=".txt", prefix="lvec_")
        os.close(fd)
    with open(path, "w") as f:
        f.write("#LambdaVector file. Keep this exact line in all similar lambda vector files\n")
        for v in values:
            f.write(repr(float(v)) + "\n")
    return path


def reference_lvec(values, imscale: float = 1.0) -> np.ndarray:
    """The bins lambda_vector_read produces: [0, l1/imscale, ...] as float32."""
    out = [np.float32(0.0)]
    for v in values:
        out.append(np.float32(np.float64(np.float32(v)) / imscale))
    return np.array(out, dtype=np.float32)


class Reference:
    """ctypes view of oracle/_ref/libdcfref.so (the reference's own code)."""

    def __init__(self, path: str = REF_SO):
        if "OMP_STACKSIZE" not in os.environ:
            # the subtractive rule keeps two g_max_levels-long arrays on the stack
            os.environ["OMP_STACKSIZE"] = "1G"
        self.lib = C.CDLL(path)
        L = self.lib
        L.dcfref_load.restype = C.c_int
        L.dcfref_load.argtypes = [C.c_void_p, C.c_ulong, C.c_ulong, C.c_ulong, C.c_int, C.c_int,
                                  C.c_int, C.c_float, C.c_float, C.c_float]
        L.dcfref_op.restype = C.c_long
        L.dcfref_op.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_char_p,
                                C.c_double, C.c_char_p, C.c_double, C.c_void_p, C.c_size_t]
        L.dcfref_parent.argtypes = [C.c_void_p]
        L.dcfref_gval.argtypes = [C.c_void_p]
        L.dcfref_max_gval.restype = C.c_float
        L.dcfref_node_attr.argtypes = [C.c_int, C.c_int, C.c_void_p]
        L.dcfref_aux.restype = C.c_long
        L.dcfref_aux.argtypes = [C.c_void_p, C.c_size_t]
        L.dcfref_time_build.restype = C.c_double
        L.dcfref_time_op.restype = C.c_double
        L.dcfref_pattern2d_ext.argtypes = [C.c_int, C.c_char_p, C.c_double, C.c_int, C.c_char_p,
                                           C.c_double, C.c_void_p]
        self.n = 0

    def load(self, img: np.ndarray, conn: int, tree: str = "max", threads: int = 1,
             pixdim=(1.0, 1.0, 1.0)) -> int:
        img = np.ascontiguousarray(img, dtype=np.float32)
        d, h, w = (1,) + img.shape if img.ndim == 2 else img.shape
        self._img = img
        self.shape = img.shape
        self.n = img.size
        return self.lib.dcfref_load(img.ctypes.data, w, h, d, conn, int(tree == "min"), threads,
                                    *[float(p) for p in pixdim])

    def _op(self, name, attr, attr2=0, rule=0, lam=0.0, lvec1=None, s1=1.0, lvec2=None, s2=1.0,
            out=None):
        nb = out.nbytes if out is not None else 0
        ptr = out.ctypes.data if out is not None else None
        r = self.lib.dcfref_op(name.encode(), attr, attr2, rule, lam,
                               lvec1.encode() if lvec1 else None, s1,
                               lvec2.encode() if lvec2 else None, s2, ptr, nb)
        if r < 0:
            raise RuntimeError(f"reference op {name} failed")
        return r

    def filter(self, attr: int, lam: float, rule: int = 0, extract: bool = False) -> np.ndarray:
        out = np.empty(self.n, np.float32)
        self._op("extract" if extract else "filter", attr, 0, rule, lam, out=out)
        return out.reshape(self.shape)

    def check(self, attr: int) -> np.ndarray:
        out = np.empty(self.n, np.float32)
        self._op("check", attr, out=out)
        return out.reshape(self.shape)

    def dmp(self, attr: int, lvec, rule: int = 0, imscale: float = 1.0) -> np.ndarray:
        p = write_lvec(lvec)
        try:
            out = np.empty((len(lvec)) * self.n, np.float32)
            self._op("dmp", attr, 0, rule, 0.0, p, imscale, out=out)
        finally:
            os.unlink(p)
        return out.reshape((len(lvec),) + self.shape)

    def pattern(self, attr: int, lvec, imscale: float = 1.0) -> np.ndarray:
        p = write_lvec(lvec)
        try:
            out = np.empty(len(lvec) + 1, np.float64)
            self._op("pattern", attr, 0, 0, 0.0, p, imscale, out=out)
        finally:
            os.unlink(p)
        return out

    def pattern2d(self, a1: int, lvec1, a2: int, lvec2, s1=1.0, s2=1.0) -> np.ndarray:
        p1, p2 = write_lvec(lvec1), write_lvec(lvec2)
        n1, n2 = len(lvec1) + 1, len(lvec2) + 1
        try:
            out = np.zeros(n1 * n2, np.float64)
            if a1 == 18 or a2 == 18:
                # make sure group-1 data is current, then use the harness' extension
                self._op("check", 1, out=np.empty(self.n, np.float32))
                r = self.lib.dcfref_pattern2d_ext(a1, p1.encode(), s1, a2, p2.encode(), s2,
                                                  out.ctypes.data)
                if r != 0:
                    raise RuntimeError("pattern2d_ext failed")
            else:
                self._op("pattern2D", a1, a2, 0, 0.0, p1, s1, p2, s2, out=out)
        finally:
            os.unlink(p1)
            os.unlink(p2)
        return out.reshape(n2, n1)

    def csl(self, attr: int, lvec, imscale: float = 1.0):
        """perform_csl (operation.c:31): (contrast, scale, luminance) images."""
        p = write_lvec(lvec)
        try:
            out = np.empty(3 * self.n, np.float32)
            self._op("csl", attr, 0, 0, 0.0, p, imscale, out=out)
        finally:
            os.unlink(p)
        return out[:self.n].copy(), out[self.n:2 * self.n].copy(), out[2 * self.n:].copy()

    def parent(self) -> np.ndarray:
        out = np.empty(self.n, np.int64)
        if self.lib.dcfref_parent(out.ctypes.data) != 0:
            raise RuntimeError("no tree")
        return out

    def gval(self) -> np.ndarray:
        out = np.empty(self.n, np.float32)
        self.lib.dcfref_gval(out.ctypes.data)
        return out

    def node_attr(self, attr: int, area: bool = False) -> np.ndarray:
        out = np.empty(self.n, np.float64)
        r = self.lib.dcfref_node_attr(attr, int(area), out.ctypes.data)
        if r != 0:
            raise RuntimeError(f"node_attr failed ({r})")
        return out

    def times(self):
        return self.lib.dcfref_time_build(), self.lib.dcfref_time_op()


def canonical_parent(parent: np.ndarray, gval: np.ndarray) -> np.ndarray:
    """Map a parent array to canonical form: every pixel -> min-index pixel of its
    node; every node representative -> representative of its parent node; root -> -1.

    The sequential reference already produces this form (its level root is the
    lowest-rank pixel of a node's flat zone, i.e. the lowest index); OpenMP builds
    with >1 thread may pick other representatives, so tests compare after this map.
    """
    n = parent.size
    par = parent.astype(np.int64).copy()
    lr = np.arange(n, dtype=np.int64)
    # level root of each pixel: follow parents while the grey level is equal
    cur = np.arange(n, dtype=np.int64)
    for _ in range(64):
        p = par[cur]
        step = (p >= 0) & (gval[np.maximum(p, 0)] == gval[cur])
        if not step.any():
            break
        cur = np.where(step, p, cur)
    else:
        raise RuntimeError("flat-zone chains too deep for canonical_parent")
    lr = cur
    # min index per node
    rep = np.full(n, n, dtype=np.int64)
    np.minimum.at(rep, lr, np.arange(n, dtype=np.int64))
    canon = rep[lr]
    out = canon.copy()
    is_rep = canon == np.arange(n)
    pl = par[lr]
    out[is_rep] = np.where(pl[is_rep] >= 0, canon[np.maximum(pl[is_rep], 0)], -1)
    return out


class Port:
    """ctypes view of oracle/_ref/libdcforacle.so (this project's CPU restatement).

    Same method surface as :class:`Reference`, so tests can swap one for the other.
    """

    def __init__(self, path: str = PORT_SO, threads: int = 1):
        self.lib = C.CDLL(path)
        L = self.lib
        L.dco_create.restype = C.c_void_p
        L.dco_create.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_uint64, C.c_int, C.c_int,
                                 C.c_int, C.c_float, C.c_float, C.c_float]
        L.dco_destroy.argtypes = [C.c_void_p]
        L.dco_connectivity.argtypes = [C.c_void_p]
        L.dco_max_gval.argtypes = [C.c_void_p]
        L.dco_max_gval.restype = C.c_float
        L.dco_prepare.argtypes = [C.c_void_p, C.c_int]
        L.dco_parent.argtypes = [C.c_void_p, C.c_void_p]
        L.dco_gval.argtypes = [C.c_void_p, C.c_void_p]
        L.dco_node_attr.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        L.dco_filter.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_int, C.c_void_p]
        L.dco_check.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.dco_pattern.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p]
        L.dco_pattern2d.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                    C.c_int, C.c_void_p]
        L.dco_sym_eig2.argtypes = [C.c_void_p, C.c_void_p]
        L.dco_sym_eig3.argtypes = [C.c_void_p, C.c_void_p]
        self.t = None
        self.threads = threads
        self.n = 0

    def __del__(self):
        if getattr(self, "t", None):
            self.lib.dco_destroy(self.t)
            self.t = None

    def load(self, img: np.ndarray, conn: int, tree: str = "max", threads: int | None = None,
             pixdim=(1.0, 1.0, 1.0)) -> int:
        if self.t:
            self.lib.dco_destroy(self.t)
        img = np.ascontiguousarray(img, dtype=np.float32)
        d, h, w = (1,) + img.shape if img.ndim == 2 else img.shape
        self._img = img
        self.shape = img.shape
        self.n = img.size
        nt = threads if threads is not None else self.threads
        self.t = self.lib.dco_create(img.ctypes.data, w, h, d, conn, int(tree == "min"), nt,
                                     *[float(p) for p in pixdim])
        return self.lib.dco_connectivity(self.t)

    def prepare(self, attr: int) -> None:
        if self.lib.dco_prepare(self.t, attr) != 0:
            raise RuntimeError("prepare failed")

    def filter(self, attr: int, lam: float, rule: int = 0, extract: bool = False) -> np.ndarray:
        out = np.empty(self.n, np.float32)
        if self.lib.dco_filter(self.t, attr, rule, lam, int(extract), out.ctypes.data) != 0:
            raise RuntimeError("filter failed")
        return out.reshape(self.shape)

    def check(self, attr: int) -> np.ndarray:
        out = np.empty(self.n, np.float32)
        if self.lib.dco_check(self.t, attr, out.ctypes.data) != 0:
            raise RuntimeError("check failed")
        return out.reshape(self.shape)

    def pattern(self, attr: int, lvec, imscale: float = 1.0) -> np.ndarray:
        lv = reference_lvec(lvec, imscale)
        out = np.zeros(lv.size, np.float64)
        if self.lib.dco_pattern(self.t, attr, lv.ctypes.data, lv.size, out.ctypes.data) != 0:
            raise RuntimeError("pattern failed")
        return out

    def pattern2d(self, a1: int, lvec1, a2: int, lvec2, s1=1.0, s2=1.0) -> np.ndarray:
        l1, l2 = reference_lvec(lvec1, s1), reference_lvec(lvec2, s2)
        out = np.zeros(l1.size * l2.size, np.float64)
        r = self.lib.dco_pattern2d(self.t, a1, l1.ctypes.data, l1.size, a2, l2.ctypes.data, l2.size,
                                   out.ctypes.data)
        if r != 0:
            raise RuntimeError(f"pattern2d failed ({r})")
        return out.reshape(l2.size, l1.size)

    def parent(self) -> np.ndarray:
        out = np.empty(self.n, np.int64)
        if self.lib.dco_parent(self.t, out.ctypes.data) != 0:
            raise RuntimeError("no tree")
        return out

    def gval(self) -> np.ndarray:
        out = np.empty(self.n, np.float32)
        self.lib.dco_gval(self.t, out.ctypes.data)
        return out

    def node_attr(self, attr: int, area: bool = False) -> np.ndarray:
        self.prepare(attr)
        out = np.empty(self.n, np.float64)
        if self.lib.dco_node_attr(self.t, attr, int(area), out.ctypes.data) != 0:
            raise RuntimeError("node_attr failed")
        return out


def find_scale(lvec, values) -> np.ndarray:
    """The reference's bin search (pattern.c:7-24) over many values: the last bin
    whose lambda is <= the value (the bisection itself, so NaN lands where it does
    in C: bin 0)."""
    lv = np.asarray(lvec, np.float32).astype(np.float64)
    v = np.asarray(values, np.float64)
    n = lv.size
    upper = np.full(v.shape, n - 1, np.int64)
    lower = np.zeros(v.shape, np.int64)
    top = v >= lv[n - 1]
    mid = (upper + lower) // 2
    active = ~top & (mid != lower)
    while active.any():
        ge = v >= lv[mid]
        lower = np.where(active & ge, mid, lower)
        upper = np.where(active & ~ge, mid, upper)
        mid = (upper + lower) // 2
        active = active & (mid != lower)
    return np.where(top, n - 1, lower)


def adjoint_fp64(parent, gval, v=None, filter_values=None, lam=0.0, w=None, area=None, bin1=None, lvec1=None,
                 bin2=None, lvec2=None) -> np.ndarray:
    """FP64 CPU adjoint of sum(v * filtered) + sum(w * spectrum) with the tree fixed.

    parent: canonical parent array (pixel -> level root, level root -> parent's
    level root, root -> -1), e.g. from the reference's flood.  Filter: the direct
    rule of filtering.c:102-153 -- a pixel takes the level of its nearest
    ancestor-or-self node whose attribute (filter_values, per level root) is >=
    lam, or 0.  Spectrum: pattern.c:110-203 -- every level root u adds
    (level(u) - level(parent(u))) * area(u) to bin [find_scale(bin2(u)),
    find_scale(bin1(u))] of w's [n2, n1] layout.  Both are linear in the levels,
    and a node's level is its level root's pixel value.
    """
    par = np.asarray(parent, np.int64)
    g = np.asarray(gval, np.float64)
    n = par.size
    idx = np.arange(n)
    isroot = (par < 0) | (g[np.maximum(par, 0)] != g)
    node = np.where(isroot, idx, par)
    grad = np.zeros(n, np.float64)
    roots = idx[isroot]
    if v is not None:
        keep = np.zeros(n, bool)
        keep[roots] = np.asarray(filter_values, np.float64)[roots] >= lam
        target = np.full(n, -1, np.int64)
        for u in roots[np.argsort(g[roots], kind="stable")]:  # parents before children
            if keep[u]:
                target[u] = u
            elif par[u] >= 0:
                target[u] = target[par[u]]
        t = target[node]
        ok = t >= 0
        np.add.at(grad, t[ok], np.asarray(v, np.float64).ravel()[ok])
    if w is not None:
        w2 = np.asarray(w, np.float64)
        s1 = find_scale(lvec1, np.asarray(bin1, np.float64)[roots])
        s2 = find_scale(lvec2, np.asarray(bin2, np.float64)[roots]) if w2.shape[0] > 1 else np.zeros_like(s1)
        c = w2[s2, s1] * np.asarray(area, np.float64)[roots]
        np.add.at(grad, roots, c)
        pr = par[roots]
        has = pr >= 0
        np.add.at(grad, pr[has], -c[has])
    return grad
