"""The C1 parity case at its full size: a 1024 x 1024 uint8 image (unit Gaussian
noise, seed 1, blurred with sigma = 4 px, scaled to 0..200, plus 300 Gaussian
point sources of sigma U(1, 3) px and peak U(50, 55), clipped to 255 and rounded),
max-tree, 4-connectivity, area attribute, subtractive rule, lambda = 100.

The filtered image is compared with the oracle bit for bit: u8 levels make every
subtractive sum an exact integer.  Parents and areas are compared as well."""
import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu


def c1_image(size=1024, seed=1):
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal((size, size))
    f = np.fft.fftfreq(size)
    g = np.exp(-2.0 * np.pi ** 2 * 16.0 * (f[:, None] ** 2 + f[None, :] ** 2))
    field = np.fft.ifft2(np.fft.fft2(noise) * g).real
    field = (field - field.min()) / (field.max() - field.min()) * 200.0
    yy, xx = np.mgrid[0:size, 0:size]
    for cx, cy, s, pk in zip(rng.uniform(0, size, 300), rng.uniform(0, size, 300), rng.uniform(1, 3, 300),
                             rng.uniform(50, 55, 300)):
        x0, x1 = max(int(cx) - 12, 0), min(int(cx) + 13, size)
        y0, y1 = max(int(cy) - 12, 0), min(int(cy) + 13, size)
        d2 = (xx[y0:y1, x0:x1] - cx) ** 2 + (yy[y0:y1, x0:x1] - cy) ** 2
        field[y0:y1, x0:x1] += pk * np.exp(-d2 / (2.0 * s * s))
    return np.rint(np.clip(field, 0, 255)).astype(np.uint8)


def test_c1_subtractive_area_opening_matches_oracle(ctx):
    img = c1_image()
    port = oracle.Port()
    port.load(img.astype(np.float32), 4, "max")
    port.prepare(0)
    t = ctx.build(img, connectivity=4, tree_type="max", attribute=0)
    assert np.array_equal(t.parent(), port.parent())
    assert np.array_equal(t.node_attribute(0), port.node_attr(0), equal_nan=True)
    got = t.filter(0, 100.0, "subtractive")
    want = port.filter(0, 100.0, 3)
    assert np.array_equal(got, want)
    t.close()
