"""File formats next to the path (CPU): the FITS reader against the reference's
own FITS fixtures (when the reference checkout is present) and against FITS files
written here for every supported BITPIX, with BZERO/BSCALE scaling."""
import os

import numpy as np
import pytest

import disccofan_gb300 as dcf

from oracle import oracle

REF_CHECKIMG = os.path.join(oracle.reference_dir() or "", "tests", "checkimg")


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


@pytest.mark.parametrize("kind", ["u8", "u16", "u32", "f32"])
def test_fits_raw_matches_float_read(tmp_path, kind):
    # the raw read gives the file's unsigned / float pixels, equal to the float read
    # once converted (u32 with the same round-to-nearest as the tree build)
    rng = np.random.default_rng(len(kind) + ord(kind[1]))
    shape = (2, 9, 11) if kind == "u32" else (19, 23)
    if kind == "u8":
        want, bitpix, bzero, stored = rng.integers(0, 256, shape).astype(np.uint8), 8, None, None
    elif kind == "u16":
        want, bitpix, bzero = rng.integers(0, 65536, shape).astype(np.uint16), 16, 32768.0
        stored = want.astype(np.int64) - 32768
    elif kind == "u32":
        want, bitpix, bzero = rng.integers(0, 2**32, shape, dtype=np.uint64).astype(np.uint32), 32, 2147483648.0
        stored = want.astype(np.int64) - 2**31
    else:
        want, bitpix, bzero, stored = rng.standard_normal(shape).astype(np.float32), -32, None, None
    p = str(tmp_path / f"raw_{kind}.fits")
    write_fits(p, want if stored is None else stored, bitpix, bzero)
    got = dcf.read_fits_raw(p)
    assert got.dtype == want.dtype and got.shape == shape
    assert np.array_equal(got, want)
    assert np.array_equal(got.astype(np.float32), dcf.read_fits(p))


def test_fits_raw_refuses_other_scalings(tmp_path):
    p = str(tmp_path / "signed16.fits")
    write_fits(p, np.arange(-6, 6).reshape(3, 4), 16)        # signed 16-bit: no BZERO
    with pytest.raises(dcf.DcfError) as e:
        dcf.read_fits_raw(p)
    assert e.value.status == 8
    q = str(tmp_path / "scaled.fits")
    write_fits(q, np.arange(12).reshape(3, 4), 8, bscale=2.0)
    with pytest.raises(dcf.DcfError) as e:
        dcf.read_fits_raw(q)
    assert e.value.status == 8
    assert np.array_equal(dcf.read_fits(q), 2.0 * np.arange(12, dtype=np.float32).reshape(3, 4))
