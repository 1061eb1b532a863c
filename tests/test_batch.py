"""GPU tests of the batched cutout path (dcf_batch_*) and of the adjoint.

Every cutout of a batch must give exactly what the single-image path and the oracle
give for that cutout alone: canonical parents and filtered images bit-exact,
spectra bit-exact for integer images and within 1e-9 relative for float images
(float dh * area terms summed in a different order), attributes likewise.  The
adjoint is checked against the FP64 CPU adjoint computed over the oracle's parent
array (1e-5 relative) and against central finite differences of the GPU forward on
dyadic inputs, where they are exact.
"""
import numpy as np
import pytest

import disccofan_gb300 as dcf
from oracle import oracle

pytestmark = pytest.mark.gpu

LV1 = [2.0, 5.0, 10.0, 30.0, 100.0, 400.0]   # inertia trace (13) bins
LV2 = [2.0, 8.0, 32.0, 128.0, 512.0]         # area bins
SPEC_TOL = 1e-9


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def cutout(shape, seed, dtype):
    rng = np.random.default_rng(seed)
    base = rng.normal(size=shape)
    k = np.ones(3) / 3.0
    for ax in range(2):
        base = np.apply_along_axis(lambda r: np.convolve(np.pad(r, 1, mode="edge"), k, mode="valid"), ax, base)
    h, w = shape
    yy, xx = np.mgrid[0:h, 0:w]
    for _ in range(int(rng.integers(1, 6))):
        cy, cx, s = rng.uniform(0, h), rng.uniform(0, w), rng.uniform(1, 4)
        base += rng.uniform(1, 3) * np.exp(-((yy - cy) ** 2 + (xx - cx) ** 2) / (2 * s * s))
    if dtype == np.uint16:
        return np.clip(np.rint((base - base.min()) * 300), 0, 65535).astype(np.uint16)
    return base.astype(np.float32)


def random_shapes(n, seed, lo=2, hi=150):
    rng = np.random.default_rng(seed)
    return [(int(rng.integers(lo, hi)), int(rng.integers(lo, hi))) for _ in range(n)]


def spec_ops():
    return (13, dcf.lvec_from_values(LV1), 0, dcf.lvec_from_values(LV2))


def check_against_port(batch, cuts, filtered, spectra, conn, lam, exact_spec):
    par = batch.split(batch.parent())
    filt = batch.split(filtered)
    trace = batch.split(batch.node_attribute(13))
    port = oracle.Port()
    for i, c in enumerate(cuts):
        port.load(c.astype(np.float32), conn, "max")
        port.prepare(13)
        pp = port.parent().reshape(c.shape)
        assert np.array_equal(par[i], pp), f"parent of cutout {i} {c.shape}"
        assert np.array_equal(filt[i], port.filter(0, lam, 0)), f"filtered cutout {i}"
        ref_t = port.node_attr(13).reshape(c.shape)
        np.testing.assert_allclose(trace[i], ref_t, rtol=1e-12, equal_nan=True)
        ref_s = port.pattern2d(13, LV1, 0, LV2)
        if exact_spec:
            assert np.array_equal(spectra[i], ref_s), f"spectrum of cutout {i}"
        else:
            np.testing.assert_allclose(spectra[i], ref_s, rtol=SPEC_TOL, atol=SPEC_TOL * np.abs(ref_s).max())


@pytest.mark.parametrize("dtype,conn", [(np.float32, 8), (np.float32, 4), (np.uint16, 8)])
def test_batch_matches_oracle_in_every_mode(dtype, conn):
    _torch()
    ctx = dcf.Context(0)
    shapes = random_shapes(11, 7 + conn)
    cuts = [cutout(s, 50 + i, dtype) for i, s in enumerate(shapes)]
    b = ctx.batch(shapes, dtype, connectivity=conn, attribute=13)
    pix = b.concat(cuts)
    lam = 20.0
    results = []
    for use_graph in (False, True, True, True):  # exact, learn, record graph, replay
        f, s = b.run(pix, filter_attr=0, lam=lam, spectrum=spec_ops(), use_graph=use_graph)
        results.append((f, s))
    assert b.info()["graph_kernels"] > 0
    for f, s in results[1:]:
        assert np.array_equal(f, results[0][0])
        if dtype == np.uint16:
            assert np.array_equal(s, results[0][1])
        else:
            np.testing.assert_allclose(s, results[0][1], rtol=1e-12, atol=1e-12 * np.abs(s).max())
    check_against_port(b, cuts, results[-1][0], results[-1][1], conn, lam, dtype == np.uint16)
    b.close()
    ctx.close()


def test_batch_schedules_agree():
    _torch()
    ctx = dcf.Context(0)
    shapes = random_shapes(9, 3, 2, 300)
    cuts = [cutout(s, 80 + i, np.uint16) for i, s in enumerate(shapes)]
    b = ctx.batch(shapes, np.uint16, connectivity=8, attribute=13)
    pix = b.concat(cuts)
    first = None
    # tile shape, CTAs per SM, queue chunk, seam buckets, bottom-up steps
    for tile, ctas, chunk, buckets, up in (((64, 64), 0, 1, 16, 2048), ((32, 32), 1, 4, 0, 7),
                                           ((16, 64), 2, 2, 64, 100000), ((128, 16), 0, 8, 3, 2048),
                                           ((64, 32), 3, 1, 256, 0)):
        b.set_schedule(tile, ctas, chunk)
        b.set_merge(seam_buckets=buckets, up_steps=up)
        info = b.info()
        assert info["tile"] == tile and info["chunk"] == chunk
        assert info["seam_buckets"] == buckets and info["up_steps"] == up
        f, s = b.run(pix, filter_attr=0, lam=50.0, spectrum=spec_ops(), use_graph=False)
        par = b.parent()
        if first is None:
            first = (f, s, par)
        else:
            assert np.array_equal(par, first[2]), tile
            assert np.array_equal(f, first[0]), tile
            assert np.array_equal(s, first[1]), tile
    b.close()
    ctx.close()


def test_batch_autotune_then_run():
    _torch()
    ctx = dcf.Context(0)
    shapes = random_shapes(24, 5, 30, 400)
    cuts = [cutout(s, 200 + i, np.float32) for i, s in enumerate(shapes)]
    b = ctx.batch(shapes, np.float32, connectivity=8, attribute=13)
    pix = b.concat(cuts)
    f0, s0 = b.run(pix, filter_attr=0, lam=30.0, spectrum=spec_ops(), use_graph=False)
    ms = b.autotune(pix, repeats=2)
    assert ms > 0
    info = b.info()
    assert info["tile"][0] * info["tile"][1] <= 4096 and info["ctas_per_sm"] >= 1
    f1, s1 = b.run(pix, filter_attr=0, lam=30.0, spectrum=spec_ops(), use_graph=True)
    f2, s2 = b.run(pix, filter_attr=0, lam=30.0, spectrum=spec_ops(), use_graph=True)
    for f, s in ((f1, s1), (f2, s2)):
        assert np.array_equal(f, f0)
        np.testing.assert_allclose(s, s0, rtol=1e-12, atol=1e-12 * np.abs(s0).max())
    b.close()
    ctx.close()


def test_batch_thin_cutouts_match_single_image_path():
    # one-pixel-thin images are compared with the single-image GPU path (the
    # reference itself double-counts areas on them)
    _torch()
    ctx = dcf.Context(0)
    shapes = [(1, 50), (50, 1), (1, 1), (2, 2), (3, 70), (70, 3)]
    cuts = [cutout(s, 300 + i, np.float32) if min(s) > 1 else
            np.random.default_rng(i).normal(size=s).astype(np.float32) for i, s in enumerate(shapes)]
    b = ctx.batch(shapes, np.float32, connectivity=8, attribute=13)
    f, s = b.run(b.concat(cuts), filter_attr=0, lam=3.0, spectrum=spec_ops(), use_graph=False)
    par, filt, area = b.split(b.parent()), b.split(f), b.split(b.node_attribute(0))
    for i, c in enumerate(cuts):
        t = ctx.build(c, connectivity=8, tree_type="max", attribute=13)
        assert np.array_equal(par[i].ravel(), t.parent())
        assert np.array_equal(filt[i], t.filter(0, 3.0, "direct"))
        np.testing.assert_array_equal(area[i].ravel(), t.node_attribute(0))
        ts = t.pattern_spectrum2d(13, dcf.lvec_from_values(LV1), 0, dcf.lvec_from_values(LV2))
        np.testing.assert_allclose(s[i], ts, rtol=1e-12, atol=1e-12 * max(np.abs(ts).max(), 1.0))
        t.close()
    b.close()
    ctx.close()


def test_batch_graph_capacity_overflow_reruns_exactly():
    # a constant cutout leaves no nodes for pointer jumping (capacity = minimum);
    # a ramp is one chain of 262,144 nodes, far beyond it: the graph run must be
    # detected, redone without the graph and give the single-image results
    _torch()
    ctx = dcf.Context(0)
    b = ctx.batch([(512, 512)], np.float32, connectivity=4, attribute=13)
    flat = np.zeros(512 * 512, np.float32)
    b.run(flat, filter_attr=0, lam=64.0, spectrum=spec_ops(), use_graph=True)
    ramp = np.arange(512 * 512, dtype=np.float32) / 7.0
    f, s = b.run(ramp, filter_attr=0, lam=64.0, spectrum=spec_ops(), use_graph=True)
    t = ctx.build(ramp.reshape(512, 512), connectivity=4, tree_type="max", attribute=13)
    assert np.array_equal(b.parent(), t.parent())
    assert np.array_equal(f, t.filter(0, 64.0, "direct").ravel())
    ts = t.pattern_spectrum2d(13, dcf.lvec_from_values(LV1), 0, dcf.lvec_from_values(LV2))
    np.testing.assert_allclose(s[0], ts, rtol=1e-12)
    # and a graph recorded with the grown capacity now covers the ramp
    f2, s2 = b.run(ramp, filter_attr=0, lam=64.0, spectrum=spec_ops(), use_graph=True)
    f3, s3 = b.run(ramp, filter_attr=0, lam=64.0, spectrum=spec_ops(), use_graph=True)
    assert np.array_equal(f2, f) and np.array_equal(f3, f)
    t.close()
    b.close()
    ctx.close()


def test_batch_errors():
    _torch()
    ctx = dcf.Context(0)
    with pytest.raises(dcf.DcfError) as e:
        ctx.batch([(10, 10)], np.float32, connectivity=6)
    assert e.value.status == 1
    b = ctx.batch([(10, 12), (7, 9)], np.float32, connectivity=8, attribute=13)
    with pytest.raises(dcf.DcfError) as e:
        b.adjoint(np.zeros(b.n, np.float32))
    assert e.value.status == 6
    pix = np.ones(b.n, np.float32)
    pix[5] = np.nan
    with pytest.raises(dcf.DcfError) as e:
        b.run(pix, filter_attr=0, lam=1.0)
    assert e.value.status == 5
    with pytest.raises(dcf.DcfError) as e:  # attribute 3 (x extent) is not in group 4
        b.run(np.ones(b.n, np.float32), filter_attr=3, lam=1.0)
    assert e.value.status == 1
    with pytest.raises(dcf.DcfError):
        b.set_schedule((128, 64))
    b.close()
    u = ctx.batch([(10, 10)], np.uint16, connectivity=8, attribute=13)
    u.run(np.ones(100, np.uint16), filter_attr=0, lam=1.0)
    with pytest.raises(dcf.DcfError) as e:
        u.adjoint(np.zeros(100, np.float32))
    assert e.value.status == 8
    u.close()
    ctx.close()


# ---------------------------------------------------------------------------
# adjoint
# ---------------------------------------------------------------------------
ADJ_LAM = 8.0
ADJ_LV1 = [1.2, 1.5, 2.0, 3.0, 5.0]     # elongation (14)
ADJ_LV2 = [2.0, 4.0, 8.0, 16.0, 64.0]   # area
STEP = 1.0 / 4096


def dyadic(shape, seed):
    """Distinct values k/1024 ordered like smoothed noise (exact under +-1/4096)."""
    rng = np.random.default_rng(seed)
    base = rng.normal(size=shape)
    k = np.ones(3) / 3.0
    for ax in range(2):
        base = np.apply_along_axis(lambda r: np.convolve(np.pad(r, 1, mode="edge"), k, mode="valid"), ax, base)
    base += 0.05 * rng.normal(size=shape)
    ranks = np.empty(base.size, np.int64)
    ranks[np.argsort(base.ravel(), kind="stable")] = np.arange(base.size)
    return (ranks.reshape(shape) / 1024.0).astype(np.float32)


def adj_spec():
    return (14, dcf.lvec_from_values(ADJ_LV1), 0, dcf.lvec_from_values(ADJ_LV2))


def loss(b, pix, v, w):
    f, s = b.run(pix, filter_attr=0, lam=ADJ_LAM, spectrum=adj_spec(), use_graph=False)
    return float((v * f.astype(np.float64)).sum() + (w * s).sum())


def test_batch_adjoint_matches_fp64_oracle_and_finite_differences():
    _torch()
    ctx = dcf.Context(0)
    shapes = random_shapes(5, 11, 12, 70)
    cuts = [dyadic(s, 400 + i) for i, s in enumerate(shapes)]
    b = ctx.batch(shapes, np.float32, connectivity=8, attribute=14)
    pix = b.concat(cuts)
    rng = np.random.default_rng(9)
    v = rng.normal(size=b.n)
    w = rng.normal(size=(b.count, len(ADJ_LV2) + 1, len(ADJ_LV1) + 1))
    b.run(pix, filter_attr=0, lam=ADJ_LAM, spectrum=adj_spec(), use_graph=False)
    grad = b.adjoint(v.astype(np.float32), w).astype(np.float64)
    # FP64 CPU adjoint over the oracle's parent array, cutout by cutout
    port = oracle.Port()
    l1, l2 = oracle.reference_lvec(ADJ_LV1), oracle.reference_lvec(ADJ_LV2)
    vv = b.split(v.astype(np.float32).astype(np.float64))
    for i, c in enumerate(cuts):
        port.load(c, 8, "max")
        port.prepare(14)
        ref = oracle.adjoint_fp64(port.parent(), port.gval(), v=vv[i].ravel(), filter_values=port.node_attr(0),
                                  lam=ADJ_LAM, w=w[i], area=port.node_attr(14, area=True), bin1=port.node_attr(14),
                                  lvec1=l1, bin2=port.node_attr(14, area=True), lvec2=l2)
        got = b.split(grad)[i].ravel()
        scale = np.abs(ref).max()
        np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-5 * scale)
    # central finite differences of the GPU forward along random directions
    for trial in range(4):
        d = rng.integers(-1, 2, size=b.n).astype(np.float64)
        fd = (loss(b, (pix + STEP * d).astype(np.float32), v.astype(np.float32).astype(np.float64), w) -
              loss(b, (pix - STEP * d).astype(np.float32), v.astype(np.float32).astype(np.float64), w)) / (2 * STEP)
        assert fd == pytest.approx(float((grad * d).sum()), rel=1e-5)
    b.close()
    ctx.close()


def test_autograd_function_and_tree_adjoint():
    torch = _torch()
    from disccofan_gb300.autograd import filter_and_spectrum
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        ctx = dcf.Context(0, stream=stream.cuda_stream)
        imgs = np.stack([dyadic((48, 40), 500 + i) for i in range(3)])
        b = ctx.batch([(48, 40)] * 3, np.float32, connectivity=8, attribute=14)
        x = torch.tensor(imgs, device="cuda", requires_grad=True)
        rng = np.random.default_rng(4)
        v = torch.tensor(rng.normal(size=imgs.shape), dtype=torch.float32, device="cuda")
        w = torch.tensor(rng.normal(size=(3, len(ADJ_LV2) + 1, len(ADJ_LV1) + 1)), dtype=torch.float64,
                         device="cuda")
        for use_graph in (False, True, True):
            x.grad = None
            filtered, spectra = filter_and_spectrum(b, x, 0, ADJ_LAM, adj_spec(), use_graph=use_graph)
            total = (v * filtered).sum(dtype=torch.float64) + (w * spectra).sum()
            total.backward()
            stream.synchronize()
            g = x.grad.detach().cpu().numpy()
            # the same as the explicit adjoint call
            b.run(imgs.ravel(), filter_attr=0, lam=ADJ_LAM, spectrum=adj_spec(), use_graph=False)
            ref = b.adjoint(v.cpu().numpy().ravel(), w.cpu().numpy()).reshape(imgs.shape)
            np.testing.assert_allclose(g, ref, rtol=1e-6, atol=1e-6 * np.abs(ref).max())
        # the single-tree adjoint on the first image
        t = ctx.build(imgs[0], connectivity=8, tree_type="max", attribute=14)
        gt = t.adjoint(v[0].cpu().numpy(), 0, ADJ_LAM, w[0].cpu().numpy(), adj_spec())
        np.testing.assert_allclose(gt, ref[0], rtol=1e-6, atol=1e-6 * np.abs(ref[0]).max())
        t.close()
        b.close()
        ctx.close()
