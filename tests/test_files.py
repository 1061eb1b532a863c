"""File formats next to the path (CPU): the FITS reader against the reference's
own FITS fixtures (when the reference checkout is present) and against FITS files
written here for every supported BITPIX, with BZERO/BSCALE scaling."""
import os

import numpy as np
import pytest

import disccofan_gb300 as dcf

REF_CHECKIMG = "/root/reference/tests/checkimg"


def write_fits(path, arr, bitpix, bzero=None, bscale=None):
    cards = ["SIMPLE  = %20s" % "T", "BITPIX  = %20d" % bitpix, "NAXIS   = %20d" % arr.ndim]
    for i, n in enumerate(arr.shape[::-1]):
        cards.append("NAXIS%-3d= %20d" % (i + 1, n))
    if bzero is not None:
        cards.append("BZERO   = %20s" % repr(float(bzero)))
    if bscale is not None:
        cards.append("BSCALE  = %20s" % repr(float(bscale)))
    cards.append("END")
    hdr = "".join(c.ljust(80) for c in cards)
    hdr = hdr.ljust((len(hdr) + 2879) // 2880 * 2880)
    dt = {8: ">u1", 16: ">i2", 32: ">i4", -32: ">f4", -64: ">f8"}[bitpix]
    data = np.ascontiguousarray(arr).astype(dt).tobytes()
    data += b"\0" * ((-len(data)) % 2880)
    with open(path, "wb") as f:
        f.write(hdr.encode("ascii") + data)


@pytest.mark.parametrize("bitpix", [8, 16, 32, -32, -64])
def test_fits_roundtrip(tmp_path, bitpix):
    rng = np.random.default_rng(bitpix + 100)
    shape = (3, 5, 7) if bitpix == 32 else (13, 17)
    if bitpix == 8:
        raw = rng.integers(0, 256, shape)
    elif bitpix == 16:
        raw = rng.integers(-32768, 32768, shape)
    elif bitpix == 32:
        raw = rng.integers(-2**31, 2**31, shape)
    else:
        raw = rng.standard_normal(shape)
    bzero, bscale = (32768.0, None) if bitpix == 16 else ((None, 0.5) if bitpix == 32 else (None, None))
    p = str(tmp_path / f"img{bitpix}.fits")
    write_fits(p, raw, bitpix, bzero, bscale)
    got = dcf.read_fits(p)
    want = (raw.astype(np.float64) if bitpix > 0 else raw.astype(">f4" if bitpix == -32 else ">f8").astype(np.float64))
    want = (bzero or 0.0) + (bscale or 1.0) * want
    assert got.shape == shape
    assert np.array_equal(got, want.astype(np.float32))


def test_fits_errors(tmp_path):
    with pytest.raises(dcf.DcfError) as e:
        dcf.read_fits(str(tmp_path / "missing.fits"))
    assert e.value.status == 7
    p = str(tmp_path / "bad.fits")
    write_fits(p, np.zeros((2, 2)), 8)
    with open(p, "r+b") as f:  # BITPIX 12 is not a FITS type
        f.seek(80)
        f.write(("BITPIX  = %20d" % 12).ljust(80).encode())
    with pytest.raises(dcf.DcfError) as e:
        dcf.read_fits(p)
    assert e.value.status == 8


@pytest.mark.skipif(not os.path.isdir(REF_CHECKIMG), reason="reference checkout not present")
def test_fits_reads_reference_fixtures(lena):
    img = dcf.read_fits(os.path.join(REF_CHECKIMG, "lena512.fits"))
    assert np.array_equal(img, lena["lena"].astype(np.float32))
    for name, key in (("GT_2D_check_area.fits", "check_area_c4"), ("GT_2D_check_area_8.fits", "check_area_c8"),
                      ("GT_2D_check_ncomp.fits", "check_ncomp_c4")):
        assert np.array_equal(dcf.read_fits(os.path.join(REF_CHECKIMG, name)), lena[key]), name
