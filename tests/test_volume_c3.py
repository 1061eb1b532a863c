"""GPU parity on 3-D float volumes shaped like the reference's 3-D use: a log-normal
density field (unit Gaussian noise blurred with sigma = 6 voxels, standardised to
mean 0 and std 1.5, exponentiated), 6-connected max-tree with the inertia group,
direct filter keeping non-compactness >= 2.0, and the 2-D pattern spectrum of
non-compactness (17) x volume (0) on 16 log-spaced thresholds each.

Against the CPU oracle: parents and the filtered volume bit-exact; node attributes
and spectrum within 1e-9 relative (the volumes are float, so grey-weighted sums and
dh * volume terms are summed in a different order; non-compactness of 3-D nodes
divides by pow(volume, 5/3), evaluated to within an ulp of glibc).  The smaller
volume also covers the operations built from the filter: extract, the differential
morphological profile and the attribute check.

The 512^3 case needs about 4.5 minutes of single-threaded oracle time and 21 GB of
host memory, so it runs only with DCF_LARGE_TESTS=1.
"""
import os

import numpy as np
import pytest

import disccofan_gb300 as dcf
from oracle import oracle

pytestmark = pytest.mark.gpu

LV_NCOMP = list(np.geomspace(0.3, 30.0, 16))
RTOL = 1e-9


def lognormal_volume(n, seed=3, sigma=6.0):
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal((n, n, n))
    f = np.fft.fftfreq(n)
    g = np.exp(-2.0 * np.pi ** 2 * sigma ** 2 * (f[:, None, None] ** 2 + f[None, :, None] ** 2 + f[None, None, :] ** 2))
    field = np.fft.ifftn(np.fft.fftn(noise) * g).real
    field = (field - field.mean()) / field.std() * 1.5
    return np.exp(field).astype(np.float32)


@pytest.mark.parametrize("n", [64, 256])
def test_lognormal_volume_against_oracle(ctx, n):
    vol = lognormal_volume(n)
    # one oracle thread: with several, like the reference under OpenMP, level roots
    # inside flat zones (float32 ties) are not the canonical lowest index
    port = oracle.Port(threads=1)
    port.load(vol, 6, "max")
    port.prepare(17)
    t = ctx.build(vol, connectivity=6, tree_type="max", attribute=17)
    assert np.array_equal(t.parent(), port.parent())
    assert np.array_equal(t.filter(17, 2.0, "direct"), port.filter(17, 2.0, 0))
    for a in (0, 13, 14, 15, 16, 17):
        got, want = t.node_attribute(a), port.node_attr(a)
        if a == 0:
            assert np.array_equal(got, want, equal_nan=True)
        else:
            np.testing.assert_allclose(got, want, rtol=RTOL, atol=0, equal_nan=True, err_msg=str(a))
    lv_vol = list(np.geomspace(1.0, float(n) ** 3, 16))
    spec = t.pattern_spectrum2d(17, dcf.lvec_from_values(LV_NCOMP), 0, dcf.lvec_from_values(lv_vol))
    want = port.pattern2d(17, LV_NCOMP, 0, lv_vol)
    np.testing.assert_allclose(spec, want, rtol=RTOL, atol=RTOL * np.abs(want).max())
    if n == 64:
        # operations built from the filter (operation.c): extract, DMP, check
        assert np.array_equal(t.filter(17, 2.0, "direct", extract=True), port.filter(17, 2.0, 0, extract=True))
        lv = dcf.lvec_from_values([0.5, 1.0, 2.0, 4.0])
        dmp = t.dmp(17, lv, "direct")
        for i, lam in enumerate(lv[1:]):
            assert np.array_equal(dmp[i], port.filter(17, float(lam), 0, extract=True)), float(lam)
        np.testing.assert_allclose(t.check(17), port.check(17), rtol=1e-6, atol=0)
    t.close()


@pytest.mark.skipif(os.environ.get("DCF_LARGE_TESTS") != "1",
                    reason="512^3 oracle run: about 4.5 min on one core and 21 GB; set DCF_LARGE_TESTS=1")
def test_lognormal_volume_512_against_oracle(ctx):
    n = 512
    vol = lognormal_volume(n)
    port = oracle.Port(threads=1)
    port.load(vol, 6, "max")
    port.prepare(17)
    t = ctx.build(vol, connectivity=6, tree_type="max", attribute=17)
    assert np.array_equal(t.parent(), port.parent())
    assert np.array_equal(t.filter(17, 2.0, "direct"), port.filter(17, 2.0, 0))
    assert np.array_equal(t.node_attribute(0), port.node_attr(0), equal_nan=True)
    np.testing.assert_allclose(t.node_attribute(17), port.node_attr(17), rtol=RTOL, atol=0, equal_nan=True)
    lv_vol = list(np.geomspace(1.0, float(n) ** 3, 16))
    spec = t.pattern_spectrum2d(17, dcf.lvec_from_values(LV_NCOMP), 0, dcf.lvec_from_values(lv_vol))
    want = port.pattern2d(17, LV_NCOMP, 0, lv_vol)
    np.testing.assert_allclose(spec, want, rtol=RTOL, atol=RTOL * np.abs(want).max())
    t.close()
