"""GPU parity on the benchmark's own workloads, generated exactly as bench.py makes
them, against the CPU oracle.

* 16384^2 uint16 log-normal field with 1e5 sources (the headline image): two crops,
  one tile-aligned and one ragged, as max- and min-trees, 8-connectivity, extent
  group.  Parents, the area and bounding-box attributes (0-4) and the bounding-box
  elongation (18) per node, the direct area opening at 1000 and the 21 x 21
  elongation x area spectrum on the headline's own bins are compared bit-exactly
  (u16 levels: every dh * area term is an exact integer).
* 4096 float32 cutouts of 64-1024 px a side: 24 of them -- the four largest and 20
  drawn at random -- through one batch with the CUDA graph, 8-connectivity, inertia
  group: parents and the area opening bit-exact, the 25 x 25 inertia-trace x area
  spectra within 1e-9 relative (float dh * area terms summed in another order).
* 256 float32 512^2 images with distinct values: the first three through the
  autograd Function (forward, then backward with the trees rebuilt); the gradient
  within 1e-5 relative of the FP64 CPU adjoint over the oracle's parent array.
"""
import numpy as np
import pytest

import bench
import disccofan_gb300 as dcf
from oracle import oracle

pytestmark = pytest.mark.gpu

SIDE = 16384
SPEC_RTOL = 1e-9
GRAD_RTOL = 1e-5


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def headline_image():
    _torch()
    img = bench.make_image(SIDE)
    yield img
    del img


# (y0, x0, height, width): tile-aligned, then ragged at both ends
CROPS = [(0, 0, 2048, 2048), (9001, 3333, 1531, 2600)]


@pytest.mark.parametrize("crop", CROPS)
def test_headline_crop_matches_oracle(headline_image, crop):
    y0, x0, h, w = crop
    dev = headline_image[y0:y0 + h, x0:x0 + w].contiguous()
    host = dev.cpu().numpy()
    l_elong, l_area = bench.lvecs(SIDE * SIDE)
    v_elong, v_area = list(np.geomspace(1, 16384, 20)), list(np.geomspace(1, SIDE * SIDE, 20))
    ctx = dcf.Context(0)
    port = oracle.Port()
    for tt in ("max", "min"):
        t = ctx.build(dev, connectivity=8, tree_type=tt, attribute=18)
        port.load(host.astype(np.float32), 8, tt)
        port.prepare(18)
        assert np.array_equal(t.parent(), port.parent()), tt
        assert t.info()["nodes"] == int(np.count_nonzero(~np.isnan(port.node_attr(0)))), tt
        for a in (0, 1, 2, 3, 4, 18):
            assert np.array_equal(t.node_attribute(a), port.node_attr(a), equal_nan=True), (tt, a)
        assert np.array_equal(t.filter(0, 1000.0, "direct"), port.filter(0, 1000.0, 0)), tt
        got = t.pattern_spectrum2d(18, l_elong, 0, l_area)
        want = port.pattern2d(18, v_elong, 0, v_area)
        assert np.array_equal(got, want), tt
        # the spectrum of a max-tree adds up to the grey-level sum (examples.rst:351)
        if tt == "max":
            assert got.sum() == float(host.astype(np.int64).sum())
        t.close()
    ctx.close()


def test_batched_cutouts_at_configured_sizes_match_oracle():
    torch = _torch()
    shapes, pix = bench.make_cutouts(4096)
    sizes = np.array([h * w for h, w in shapes])
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    rng = np.random.default_rng(11)
    largest = list(np.argsort(sizes)[-4:])
    rest = [int(i) for i in rng.choice(np.setdiff1d(np.arange(len(shapes)), largest), 20, replace=False)]
    pick = [int(i) for i in largest] + rest
    sub_shapes = [shapes[i] for i in pick]
    sub = torch.cat([pix[offs[i]:offs[i] + sizes[i]] for i in pick])
    v_tr, v_ar = list(np.geomspace(1, 1e11, 24)), list(np.geomspace(1, 1 << 20, 24))
    spec = (13, dcf.lvec_from_values(v_tr), 0, dcf.lvec_from_values(v_ar))
    lam = 100.0
    ctx = dcf.Context(0)
    b = ctx.batch(sub_shapes, np.float32, connectivity=8, attribute=13)
    filtered = torch.empty(b.n, dtype=torch.float32, device="cuda")
    spectra = torch.empty((b.count, 25, 25), dtype=torch.float64, device="cuda")
    for _ in range(3):  # learn the capacity, record the graph, replay it
        b.run(sub, filter_attr=0, lam=lam, spectrum=spec, use_graph=True, filtered=filtered, spectra=spectra)
    assert b.info()["graph_kernels"] > 0
    par = b.split(b.parent())
    filt = b.split(filtered.cpu().numpy())
    specs = spectra.cpu().numpy()
    host = sub.cpu().numpy()
    port = oracle.Port()
    o = 0
    for i, (h, w) in enumerate(sub_shapes):
        c = host[o:o + h * w].reshape(h, w)
        o += h * w
        port.load(c, 8, "max")
        port.prepare(13)
        assert np.array_equal(par[i].ravel(), port.parent()), f"parent of cutout {pick[i]} {c.shape}"
        assert np.array_equal(filt[i], port.filter(0, lam, 0)), f"filtered cutout {pick[i]}"
        want = port.pattern2d(13, v_tr, 0, v_ar)
        np.testing.assert_allclose(specs[i], want, rtol=SPEC_RTOL, atol=SPEC_RTOL * np.abs(want).max(),
                                   err_msg=f"spectrum of cutout {pick[i]}")
    b.close()
    ctx.close()


def test_differentiable_images_at_configured_size_match_fp64_adjoint():
    torch = _torch()
    from disccofan_gb300.autograd import filter_and_spectrum
    count, size, lam = 3, 512, 64.0
    x = bench.make_distinct_images(count, size)
    torch.cuda.synchronize()  # made on the default stream, used on another below
    v_el, v_ar = list(np.geomspace(1, 100, 16)), list(np.geomspace(1, size * size, 16))
    spec = (14, dcf.lvec_from_values(v_el), 0, dcf.lvec_from_values(v_ar))
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        ctx = dcf.Context(0, stream=stream.cuda_stream)
        b = ctx.batch([(size, size)] * count, np.float32, connectivity=8, attribute=14)
        rng = np.random.default_rng(6)
        v = torch.from_numpy(rng.standard_normal((count, size, size), dtype=np.float32)).cuda()
        w = torch.from_numpy(rng.standard_normal((count, 17, 17))).cuda()
        xg = x.clone().requires_grad_(True)
        f, s = filter_and_spectrum(b, xg, 0, lam, spec)
        ((v * f).sum(dtype=torch.float64) + (w * s).sum()).backward()
        stream.synchronize()
        grad = xg.grad.detach().cpu().numpy().astype(np.float64)
        b.close()
        ctx.close()
    l1, l2 = oracle.reference_lvec(v_el), oracle.reference_lvec(v_ar)
    port = oracle.Port()
    imgs = x.cpu().numpy()
    vv, ww = v.cpu().numpy().astype(np.float64), w.cpu().numpy()
    for i in range(count):
        port.load(imgs[i], 8, "max")
        port.prepare(14)
        ref = oracle.adjoint_fp64(port.parent(), port.gval(), v=vv[i].ravel(), filter_values=port.node_attr(0),
                                  lam=lam, w=ww[i], area=port.node_attr(14, area=True), bin1=port.node_attr(14),
                                  lvec1=l1, bin2=port.node_attr(14, area=True), lvec2=l2)
        np.testing.assert_allclose(grad[i].ravel(), ref, rtol=GRAD_RTOL, atol=GRAD_RTOL * np.abs(ref).max(),
                                   err_msg=f"image {i}")
