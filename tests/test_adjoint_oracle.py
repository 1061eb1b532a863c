"""CPU tests of the FP64 adjoint oracle (oracle.adjoint_fp64).

The oracle adjoint is pinned against central finite differences of the oracle's own
forward (the restated direct filter and 2-D pattern spectrum).  Pixel values are
distinct multiples of 1/1024 and the step is 1/4096, below half the smallest level
gap, so the tree does not change and every level difference, and hence every
spectrum term, is exact in float and double: the finite differences are exact.
"""
import numpy as np
import pytest

from oracle import oracle

LAM = 8.0
A1, A2 = 14, 0                          # elongation x area (group 4)
LV1 = [1.2, 1.5, 2.0, 3.0, 5.0]
LV2 = [2.0, 4.0, 8.0, 16.0, 64.0]
STEP = 1.0 / 4096


def dyadic_image(shape, seed):
    """Distinct values k/1024 ordered like smoothed noise (k a permutation of 0..N-1)."""
    rng = np.random.default_rng(seed)
    base = rng.normal(size=shape)
    k = np.ones(3) / 3.0
    for ax in range(2):
        base = np.apply_along_axis(lambda r: np.convolve(np.pad(r, 1, mode="edge"), k, mode="valid"), ax, base)
    base += 0.05 * rng.normal(size=shape)
    ranks = np.empty(base.size, np.int64)
    ranks[np.argsort(base.ravel(), kind="stable")] = np.arange(base.size)
    return (ranks.reshape(shape) / 1024.0).astype(np.float32)


def forward_loss(port, img, v, w):
    port.load(img, 8, "max")
    f = port.filter(0, LAM, 0).astype(np.float64)
    s = port.pattern2d(A1, LV1, A2, LV2)
    return float((v * f).sum() + (w * s).sum())


def oracle_grad(port, img, v, w):
    port.load(img, 8, "max")
    port.prepare(A1)
    par, g = port.parent(), port.gval()
    area_f = port.node_attr(0)
    elong = port.node_attr(A1)
    area_g4 = port.node_attr(A1, area=True)
    l1, l2 = oracle.reference_lvec(LV1), oracle.reference_lvec(LV2)
    return oracle.adjoint_fp64(par, g, v=v.ravel(), filter_values=area_f, lam=LAM, w=w, area=area_g4, bin1=elong,
                               lvec1=l1, bin2=area_g4, lvec2=l2)


@pytest.mark.parametrize("shape,seed", [((24, 20), 1), ((17, 31), 2)])
def test_oracle_adjoint_matches_finite_differences(port_lib, shape, seed):
    port = port_lib.Port()
    img = dyadic_image(shape, seed)
    rng = np.random.default_rng(100 + seed)
    v = rng.normal(size=shape)
    w = rng.normal(size=(len(LV2) + 1, len(LV1) + 1))
    grad = oracle_grad(port, img, v, w).reshape(shape)
    # directional derivatives along random sign patterns, plus single pixels
    for trial in range(6):
        d = rng.integers(-1, 2, size=shape).astype(np.float64)
        xp = (img + STEP * d).astype(np.float32)
        xm = (img - STEP * d).astype(np.float32)
        assert np.array_equal(xp.astype(np.float64) - img, STEP * d)  # exact perturbation
        fd = (forward_loss(port, xp, v, w) - forward_loss(port, xm, v, w)) / (2 * STEP)
        assert fd == pytest.approx(float((grad * d).sum()), rel=1e-12, abs=1e-9)
    for flat in rng.choice(img.size, 5, replace=False):
        d = np.zeros(img.size)
        d[flat] = 1.0
        d = d.reshape(shape)
        fd = (forward_loss(port, (img + STEP * d).astype(np.float32), v, w) -
              forward_loss(port, (img - STEP * d).astype(np.float32), v, w)) / (2 * STEP)
        assert fd == pytest.approx(grad.ravel()[flat], rel=1e-12, abs=1e-9)


def test_find_scale_matches_bisection():
    lv = oracle.reference_lvec([1.0, 2.0, 4.0, 8.0])
    vals = np.array([-1.0, 0.0, 0.5, 1.0, 1.5, 2.0, 7.9, 8.0, 100.0, np.nan])
    assert list(oracle.find_scale(lv, vals)) == [0, 0, 0, 1, 1, 2, 3, 4, 4, 0]
