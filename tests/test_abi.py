"""CPU tests of the C-ABI library: it loads, exports every symbol include/*.h
declares, and its host-only entry points behave like the reference's."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols(headers=("dcf.h",)):
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f in headers:
            text = open(os.path.join(inc, f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(dcf_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    import disccofan_gb300 as dcf
    return dcf.library()


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("dcf_tree_build", "dcf_filter", "dcf_pattern_spectrum2d", "dcf_tree_parent", "dcf_lvec_read"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_lvec_read_matches_reference_semantics(tmp_path):
    import disccofan_gb300 as dcf
    p = tmp_path / "lvec.txt"
    p.write_text("#LambdaVector file. Keep this exact line in all similar lambda vector files\n"
                 "100\n1000\n10000\n50000\n100000\n150000\n\n")
    got = dcf.read_lvec(str(p), 3.0)
    want = dcf.lvec_from_values([100, 1000, 10000, 50000, 100000, 150000], 3.0)
    assert np.array_equal(got, want)
    assert got[0] == 0 and got.size == 7


def test_lvec_read_errors(tmp_path):
    import disccofan_gb300 as dcf
    with pytest.raises(dcf.DcfError):
        dcf.read_lvec(str(tmp_path / "missing.txt"))
    bad = tmp_path / "bad.txt"
    bad.write_text("1\n2\n")
    with pytest.raises(dcf.DcfError):
        dcf.read_lvec(str(bad))


def test_ctx_create_without_gpu_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    st = lib.dcf_ctx_create(0, None, C.byref(h))
    assert st != 0 and not h.value


C_CALLER = r"""
#include <stdio.h>
#include <string.h>
#include "dcf.h"

int main(int argc, char **argv)
{
    if (argc < 2) return 5;
    float lv[8];
    int n = 0;
    dcf_status s = dcf_lvec_read(argv[1], 2.0, lv, 8, &n);
    if (s != DCF_OK || n != 4 || lv[0] != 0.0f || lv[1] != 5.0f || lv[3] != 50.0f) return 1;
    if (strlen(dcf_status_string(DCF_ERR_INVALID)) == 0) return 2;
    dcf_ctx *ctx = NULL;
    s = dcf_ctx_create(0, NULL, &ctx);
    if (s == DCF_OK) {           /* a GPU is present */
        if (!ctx || dcf_ctx_destroy(ctx) != DCF_OK) return 3;
    } else if (ctx != NULL) {    /* no GPU: a clean error and no context */
        return 4;
    }
    printf("ok %d\n", n);
    return 0;
}
"""


def test_header_compiles_as_c99_and_links(tmp_path):
    import shutil
    import subprocess
    import disccofan_gb300 as dcf
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib_path = dcf.library()._name
    src = tmp_path / "caller.c"
    src.write_text(C_CALLER)
    exe = tmp_path / "caller"
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                    lib_path, f"-Wl,-rpath,{os.path.dirname(lib_path)}", "-o", str(exe)], check=True)
    lv = tmp_path / "lvec.txt"
    lv.write_text("#LambdaVector file. Keep this exact line in all similar lambda vector files\n10\n40\n100\n")
    r = subprocess.run([str(exe), str(lv)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok 4", (r.returncode, r.stdout, r.stderr)
