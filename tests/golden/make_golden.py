"""Regenerate the golden fixtures in tests/golden/ (run in a container that has
the reference checkout; the GPU machine never runs this).

Sources:
  * The reference's own test fixtures (tests/checkimg/ of sgazagnes/disccofan):
    input_image.png, GT_area_200.png, GT_ncomp_0.2.png, GT_2D_check_area.fits,
    GT_2D_check_area_8.fits, GT_2D_check_ncomp.fits and the parent/area columns of
    GT_tree.txt.  They are decoded here (PNG via zlib, FITS via its 2880-byte
    header blocks) and stored in the reference's pixel order: FreeImage reads
    scanlines bottom-up, so PNG rows are flipped; FITS rows are stored as-is.
  * Outputs of the reference's own code (oracle/_ref/libdcfref.so) on small seeded
    synthetic inputs, covering what the reference's fixtures leave unpinned:
    3-D 6/26-connectivity, min/max/subtractive rules, 16-bit/float inputs,
    min-trees, spectra, the extent/mean/wmean/inertia groups.

Usage:  python tests/golden/make_golden.py [/path/to/reference]
"""
from __future__ import annotations

import hashlib
import os
import struct
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402


def read_png_gray8(path: str) -> np.ndarray:
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    i, idat, hdr = 8, b"", None
    while i < len(data):
        (ln,) = struct.unpack(">I", data[i:i + 4])
        typ = data[i + 4:i + 8]
        body = data[i + 8:i + 8 + ln]
        if typ == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif typ == b"IDAT":
            idat += body
        i += 12 + ln
    w, h, depth, ctype, _, _, interlace = hdr
    assert depth == 8 and interlace == 0
    ch = {0: 1, 2: 3, 4: 2, 6: 4}[ctype]
    raw = zlib.decompress(idat)
    stride = w * ch
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    pos = 0
    for y in range(h):
        f = raw[pos]
        line = np.frombuffer(raw, np.uint8, stride, pos + 1).astype(np.int32)
        pos += 1 + stride
        cur = np.zeros(stride, np.int32)
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 255
        else:
            for x in range(stride):
                a = cur[x - ch] if x >= ch else 0
                b = prev[x]
                c = prev[x - ch] if x >= ch else 0
                if f == 1:
                    pr = a
                elif f == 3:
                    pr = (a + b) >> 1
                else:
                    p = a + b - c
                    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                    pr = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[x] = (line[x] + pr) & 255
        out[y] = cur
        prev = cur
    img = out.reshape(h, w, ch)
    if ch >= 3:
        raise ValueError("colour PNG not expected")
    return img[:, :, 0]


def read_fits(path: str) -> np.ndarray:
    data = open(path, "rb").read()
    hdr, pos = {}, 0
    while True:
        block = data[pos:pos + 2880]
        pos += 2880
        done = False
        for k in range(36):
            card = block[k * 80:(k + 1) * 80].decode("ascii", "replace")
            key = card[:8].strip()
            if key == "END":
                done = True
                break
            if card[8:10] == "= ":
                hdr[key] = card[10:].split("/")[0].strip()
        if done:
            break
    bitpix, naxis = int(hdr["BITPIX"]), int(hdr["NAXIS"])
    dims = [int(hdr[f"NAXIS{i + 1}"]) for i in range(naxis)]
    dt = {8: ">u1", 16: ">i2", 32: ">i4", -32: ">f4", -64: ">f8"}[bitpix]
    n = int(np.prod(dims))
    arr = np.frombuffer(data, dt, n, pos).astype(dt[1:])
    return arr.reshape(dims[::-1])


def synth(seed: int, shape, kind: str) -> np.ndarray:
    """Small seeded test images: smooth field + sources, quantised per kind."""
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(shape)
    # separable box blur (a few passes ~ Gaussian)
    for ax in range(len(shape)):
        for _ in range(2):
            x = (np.roll(x, 1, ax) + x + np.roll(x, -1, ax)) / 3.0
    x = (x - x.min()) / (x.max() - x.min() + 1e-12)
    if kind == "u8":
        return np.rint(x * 40).astype(np.uint8)          # few levels: large flat zones
    if kind == "u16":
        return np.rint(x * 3000).astype(np.uint16)
    if kind == "f32":
        return (x + 1e-3 * rng.standard_normal(shape)).astype(np.float32)
    raise ValueError(kind)


CASES = [
    # name, seed, shape, dtype, conn, tree
    ("u8_2d_c4_max", 11, (37, 53), "u8", 4, "max"),
    ("u8_2d_c8_min", 12, (41, 29), "u8", 8, "min"),
    ("u16_2d_c8_max", 13, (64, 96), "u16", 8, "max"),
    ("f32_2d_c4_max", 14, (48, 40), "f32", 4, "max"),
    ("u8_3d_c6_max", 15, (9, 13, 11), "u8", 6, "max"),
    ("u16_3d_c26_min", 16, (8, 10, 12), "u16", 26, "min"),
    ("f32_3d_c26_max", 17, (7, 9, 8), "f32", 26, "max"),
]


def reference_case(ref: oracle.Reference, img: np.ndarray, conn: int, tree: str) -> dict:
    out = {"img": img, "conn": np.int64(conn), "tree": np.bytes_(tree)}
    ref.load(img.astype(np.float32), conn, tree)
    ref.check(0)
    out["parent"] = ref.parent()
    out["area"] = ref.node_attr(0)
    for rule in range(4):
        out[f"filter_area_r{rule}"] = ref.filter(0, 12.0, rule)
    out["extract_area"] = ref.filter(0, 12.0, 0, extract=True)
    lv = [2, 5, 10, 50, 200]
    out["pattern_area"] = ref.pattern(0, lv)
    ref.check(1)
    for a in (1, 2, 3, 4, 5):
        out[f"attr{a}"] = ref.node_attr(a)
    ref.check(6)
    for a in (6, 7, 8):
        out[f"attr{a}"] = ref.node_attr(a)
    ref.check(9)
    for a in (9, 10, 11, 12):
        out[f"attr{a}"] = ref.node_attr(a)
    ref.check(13)
    for a in range(13, 18):
        out[f"attr{a}"] = ref.node_attr(a)
    out["filter_ncomp_r0"] = ref.filter(17, 0.3, 0)
    out["filter_ncomp_r1"] = ref.filter(17, 0.3, 1)
    out["filter_ncomp_r2"] = ref.filter(17, 0.3, 2)
    out["pattern2d_elong_area"] = ref.pattern2d(14, [1.2, 2, 4], 0, lv)
    # CSL segmentation (perform_csl): on elongation (inertia group is current) and,
    # after re-flooding group 0, on area
    out["csl_elong"] = np.stack(ref.csl(14, [1.2, 2, 4]))
    ref.check(0)
    out["csl_area"] = np.stack(ref.csl(0, lv))
    return out


def main(refdir: str | None = None, outdir: str = HERE) -> None:
    refdir = refdir or oracle.reference_dir()
    if refdir is None:
        raise SystemExit("reference checkout not found (set DCF_REFERENCE_DIR)")
    ck = os.path.join(refdir, "tests", "checkimg")
    lena = np.flipud(read_png_gray8(os.path.join(ck, "input_image.png"))).copy()
    gt_area = np.flipud(read_png_gray8(os.path.join(ck, "GT_area_200.png"))).copy()
    gt_ncomp = np.flipud(read_png_gray8(os.path.join(ck, "GT_ncomp_0.2.png"))).copy()
    chk_area = read_fits(os.path.join(ck, "GT_2D_check_area.fits")).astype(np.float32)
    chk_area8 = read_fits(os.path.join(ck, "GT_2D_check_area_8.fits")).astype(np.float32)
    chk_ncomp = read_fits(os.path.join(ck, "GT_2D_check_ncomp.fits")).astype(np.float32)
    lena_fits = read_fits(os.path.join(ck, "lena512.fits")).astype(np.uint8)
    assert np.array_equal(lena_fits, lena), "input_image.png (flipped) != lena512.fits"
    # trailing newlines normalised to one (the fixture ends with an extra blank line
    # that write_tree itself does not print)
    tree_bytes = open(os.path.join(ck, "GT_tree.txt"), "rb").read().rstrip(b"\n") + b"\n"
    tree_lines = tree_bytes.split(b"\n")
    idx, par, area = [], [], []
    with open(os.path.join(ck, "GT_tree.txt")) as f:
        next(f)
        for line in f:
            if not line.strip():
                continue
            c = line.split(",")
            idx.append(int(c[0]))
            par.append(int(c[5]))
            area.append(int(c[7]))
    with open(os.path.join(refdir, "tests", "lvec.txt")) as f:
        next(f)
        lvec_txt = [float(v) for v in f.read().split()]
    oracle.build(ref=True)
    lref = oracle.Reference()
    lref.load(lena.astype(np.float32), 4, "max")
    lref.check(0)
    csl_lena = lref.csl(0, lvec_txt)
    del lref
    np.savez_compressed(
        os.path.join(outdir, "lena_fixtures.npz"),
        lena=lena, gt_area_200=gt_area, gt_ncomp_0_2=gt_ncomp,
        check_area_c4=chk_area, check_area_c8=chk_area8, check_ncomp_c4=chk_ncomp,
        tree_index=np.array(idx, np.int64), tree_parent=np.array(par, np.int64),
        tree_area=np.array(area, np.int64),
        # the whole tree file, for the end-to-end check of the tree export: its
        # SHA-256, length and a few lines (header, first rows, last rows)
        tree_txt_sha256=np.frombuffer(hashlib.sha256(tree_bytes).digest(), np.uint8),
        tree_txt_bytes=np.int64(len(tree_bytes)),
        tree_txt_sample=np.array([l.decode() for l in tree_lines[:4] + tree_lines[-3:-1]]),
        # CSL segmentation of the fixture image, area attribute, lambdas of the
        # reference's tests/lvec.txt, 4-connectivity max-tree
        csl_lvec=np.array(lvec_txt, np.float64),
        csl_area_c4=np.stack(csl_lena))

    oracle.build(ref=True)
    ref = oracle.Reference()
    cases = {}
    for name, seed, shape, kind, conn, tree in CASES:
        img = synth(seed, shape, kind)
        res = reference_case(ref, img, conn, tree)
        for k, v in res.items():
            cases[f"{name}/{k}"] = v
    np.savez_compressed(os.path.join(outdir, "synthetic_reference.npz"), **cases)
    print("wrote", os.path.join(outdir, "lena_fixtures.npz"), "and synthetic_reference.npz")


if __name__ == "__main__":
    main(*(sys.argv[1:]))
