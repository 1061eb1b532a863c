"""CPU tests: the oracle restatement against the reference's own golden fixtures,
its synthetic reference outputs, and (when the checkout exists) the compiled
reference itself."""
import os

import numpy as np
import pytest

from oracle import oracle

REF_DIR = oracle.reference_dir()
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_port_lena_filters(port_lib, lena):
    p = port_lib.Port()
    p.load(lena["lena"].astype(np.float32), 4)
    assert np.array_equal(p.filter(0, 200.0).astype(np.uint8), lena["gt_area_200"])
    assert np.array_equal(p.filter(17, 0.2).astype(np.uint8), lena["gt_ncomp_0_2"])


def test_port_lena_checks(port_lib, lena):
    p = port_lib.Port()
    p.load(lena["lena"].astype(np.float32), 4)
    assert np.array_equal(p.check(0), lena["check_area_c4"])
    assert np.array_equal(p.check(17), lena["check_ncomp_c4"])
    p.load(lena["lena"].astype(np.float32), 8)
    assert np.array_equal(p.check(0), lena["check_area_c8"])


def test_port_lena_tree(port_lib, lena):
    p = port_lib.Port()
    p.load(lena["lena"].astype(np.float32), 4)
    p.prepare(0)
    par, g = p.parent(), p.gval()
    roots = np.nonzero((par < 0) | (g[np.maximum(par, 0)] != g))[0]
    assert np.array_equal(roots, lena["tree_index"])
    assert np.array_equal(par[roots], lena["tree_parent"])
    area = p.node_attr(0)[roots]
    assert np.array_equal(area.astype(np.int64), lena["tree_area"])


def test_port_area_spectrum_sums_to_grey_total(port_lib, lena):
    # docs/source/examples.rst:351: the area spectrum (background included) sums to sum(gray)
    p = port_lib.Port()
    img = lena["lena"].astype(np.float32)
    p.load(img, 4)
    s = p.pattern(0, [100, 1000, 10000, 50000, 100000, 150000])
    assert s.sum() == img.astype(np.float64).sum()


@pytest.mark.parametrize("name", ["u8_2d_c4_max", "u8_2d_c8_min", "u16_2d_c8_max", "f32_2d_c4_max", "u8_3d_c6_max",
                                  "u16_3d_c26_min", "f32_3d_c26_max"])
def test_port_synthetic_reference(port_lib, synthetic, name):
    c = synthetic[name]
    p = port_lib.Port()
    p.load(c["img"].astype(np.float32), int(c["conn"]), c["tree"].item().decode())
    p.prepare(0)
    assert np.array_equal(p.parent(), c["parent"])
    assert np.array_equal(p.node_attr(0), c["area"], equal_nan=True)
    for rule in range(4):
        assert np.array_equal(p.filter(0, 12.0, rule), c[f"filter_area_r{rule}"]), rule
    assert np.array_equal(p.filter(0, 12.0, 0, extract=True), c["extract_area"])
    assert np.array_equal(p.pattern(0, [2, 5, 10, 50, 200]), c["pattern_area"])
    for a in range(1, 18):
        assert np.array_equal(p.node_attr(a), c[f"attr{a}"], equal_nan=True), a
    for rule in range(3):
        assert np.array_equal(p.filter(17, 0.3, rule), c[f"filter_ncomp_r{rule}"]), rule
    assert np.array_equal(p.pattern2d(14, [1.2, 2, 4], 0, [2, 5, 10, 50, 200]), c["pattern2d_elong_area"])


def test_canonical_parent_is_identity_on_sequential_trees(port_lib, synthetic):
    c = synthetic["u16_2d_c8_max"]
    p = port_lib.Port()
    p.load(c["img"].astype(np.float32), 8)
    p.prepare(0)
    par, g = p.parent(), p.gval()
    assert np.array_equal(oracle.canonical_parent(par, g), par)


def test_port_threads_agree_after_canonicalisation(port_lib, synthetic):
    c = synthetic["u16_2d_c8_max"]
    one, four = port_lib.Port(), port_lib.Port()
    img = c["img"].astype(np.float32)
    one.load(img, 8, threads=1)
    four.load(img, 8, threads=4)
    one.prepare(0)
    four.prepare(0)
    assert np.array_equal(oracle.canonical_parent(four.parent(), four.gval()), one.parent())
    assert np.array_equal(four.filter(0, 30.0), one.filter(0, 30.0))
    assert np.array_equal(four.pattern(0, [5, 20, 100]), one.pattern(0, [5, 20, 100]))


@pytest.mark.parametrize("tree", ["max", "min"])
def test_port_threaded_filters_agree_across_slab_seams(port_lib, tree):
    # The filter threads stop at nodes other threads resolved and copy their value;
    # on smooth images whose level components cross every slab seam the threaded
    # rules 0, 1 and 3 must equal the single-threaded ones (the copy is published
    # with release/acquire ordering, which weakly ordered hosts need)
    rng = np.random.default_rng(11)
    n = 384
    f = np.fft.rfft2(rng.standard_normal((n, n)))
    k2 = np.fft.fftfreq(n)[:, None] ** 2 + np.fft.rfftfreq(n)[None, :] ** 2
    s = np.fft.irfft2(f * np.exp(-k2 * (n / 24.0) ** 2), (n, n))
    img = ((s - s.min()) / (s.max() - s.min()) * 40000).astype(np.uint16).astype(np.float32)
    one, many = port_lib.Port(threads=1), port_lib.Port(threads=8)
    one.load(img, 8, tree, threads=1)
    many.load(img, 8, tree, threads=8)
    for rule in (0, 1, 3):
        for lam in (50.0, 2000.0):
            assert np.array_equal(many.filter(0, lam, rule), one.filter(0, lam, rule)), (rule, lam)


def test_eigen_restatement_diagonal_exact(port_lib):
    import ctypes as C
    p = port_lib.Port()
    m = np.array([1 / 3, 0.0, 0.0, 1 / 12], np.float64)
    ev = np.zeros(2)
    p.lib.dco_sym_eig2(m.ctypes.data, ev.ctypes.data)
    assert ev[1] / ev[0] == 4.0


@pytest.mark.reference
@pytest.mark.skipif(REF_DIR is None, reason="reference checkout not present")
def test_port_matches_compiled_reference_random():
    oracle.build(ref=True)
    ref, port = oracle.Reference(), oracle.Port()
    rng = np.random.default_rng(7)
    for shape, conn, tree, q in [((40, 33), 4, "max", 30), ((31, 45), 8, "min", 1000), ((6, 9, 7), 6, "max", 20),
                                 ((5, 8, 9), 26, "min", 0)]:
        img = rng.random(shape).astype(np.float32)
        if q:
            img = np.rint(img * q).astype(np.float32)
        ref.load(img, conn, tree)
        port.load(img, conn, tree)
        for attr, lam in [(0, 9.0), (17, 0.25), (14, 1.5), (3, 4.0)]:
            for rule in range(4):
                assert np.array_equal(ref.filter(attr, lam, rule), port.filter(attr, lam, rule)), (attr, rule)
        assert np.array_equal(ref.parent(), port.parent())
        assert np.array_equal(ref.pattern2d(16, [0.9, 1.1, 1.5], 0, [3, 9, 27]),
                              port.pattern2d(16, [0.9, 1.1, 1.5], 0, [3, 9, 27]))


@pytest.mark.reference
def test_golden_fixtures_regenerate_identically(tmp_path):
    # the committed fixtures are exactly what tests/golden/make_golden.py makes from
    # the reference checkout and the reference compiled from it
    if REF_DIR is None:
        pytest.skip("reference checkout absent")
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    mg.main(REF_DIR, str(tmp_path))
    for name in ("lena_fixtures.npz", "synthetic_reference.npz"):
        want, got = np.load(os.path.join(GOLDEN, name)), np.load(str(tmp_path / name))
        assert sorted(want.files) == sorted(got.files), name
        for k in want.files:
            assert np.array_equal(want[k], got[k], equal_nan=want[k].dtype.kind == "f"), (name, k)
