"""The link-compatible replacement of the reference's hot-path functions
(disccofan_gb300/csrc/dcf_refshim.c -> libdcf_refshim.so).

CPU: it builds warning-free against this repository's declarations of the
reference's layouts (include/dcf_reftypes.h) and, where the reference checkout is
present, against the reference's own headers and prototypes; the two sets of
layouts agree field by field; the C driver that calls it links.
GPU: the driver calls the seven functions the way operation.c / disccofan.c do
on the reference's lena fixture and reproduces GT_area_200 and GT_ncomp_0.2, the
area and non-compactness check images, the canonical parents, and the 1-D area
and 2-D elongation x area ("pattern2D 14, 0") spectra of the oracle.
"""
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")
PKG = os.path.join(ROOT, "disccofan_gb300")
SHIM = os.path.join(PKG, "csrc", "dcf_refshim.c")
DRIVER = os.path.join(ROOT, "tests", "refshim_driver.c")
MPI_STUB = os.path.join(ROOT, "oracle", "mpi_stub")
WARN = ["-std=gnu11", "-Wall", "-Wextra", "-Werror"]

# every field the replacement or its callers touch, per layout
LAYOUT = {
    "LambdaVec": ["num_lambdas", "lambdas"],
    "Operation": ["name", "lvec_name", "lvec_name_2D", "attribute_idx", "attribute_idx_2D", "decision_idx", "lambda",
                  "imscale", "imscale_2D", "lvec1", "lvec2"],
    "DataParams": ["dims_process", "dims_full", "pixdim", "border", "offsets", "g_max_gval", "g_min_gval"],
    "Arguments": ["interactive", "folder_run", "preprocessing", "tile_overlap", "mpi_grid", "pixel_dim", "threads",
                  "bpp", "pixel_connectivity", "include_background", "save_output", "save_tree", "num_operations",
                  "image_stats", "ope_list"],
    "AuxDataStore": ["data", "size_item", "size_alloc", "item_curr"],
    "Node": ["parent", "border_idx", "attribute", "area_copy", "gval", "gval_par", "size_init", "size_curr",
             "size_attr", "offsets", "border"],
    "AttribStruct": ["name", "short_name", "size", "group", "new_data", "init_data", "delete_data", "add_to_data",
                     "merge_data", "merge_to_data", "clone_data", "create_mpi_data", "area", "attribute"],
}


def _gcc(args, cwd=None):
    r = subprocess.run(["gcc", *args], capture_output=True, text=True, cwd=cwd)
    assert r.returncode == 0, r.stdout + r.stderr
    return r


def layout_program(path):
    lines = ["#include <stdio.h>", "#include <stddef.h>", "int main(void) {"]
    for t, fields in LAYOUT.items():
        lines.append(f'  printf("{t} %zu\\n", sizeof({t}));')
        for f in fields:
            lines.append(f'  printf("{t}.{f} %zu %zu\\n", offsetof({t}, {f}), sizeof((({t} *)0)->{f}));')
    for c in ("NUMATTR", "BOTTOM", "MAX_OPERATION_SIZE"):
        lines.append(f'  printf("{c} %d\\n", (int)({c}));')
    lines += ['  printf("value %zu idx %zu ulong %zu\\n", sizeof(value), sizeof(idx), sizeof(ulong));', "  return 0;",
              "}"]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def run_layout(tmp_path, header_args, include_line, name):
    src = tmp_path / f"{name}.c"
    layout_program(str(src))
    text = src.read_text()
    src.write_text(include_line + "\n" + text)
    exe = tmp_path / name
    _gcc([*header_args, "-std=gnu11", str(src), "-o", str(exe)])
    return subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout


def test_shim_builds_warning_free_on_own_declarations(tmp_path):
    _gcc([*WARN, "-O2", "-fPIC", "-I" + INC, "-c", SHIM, "-o", str(tmp_path / "shim.o")])
    _gcc([*WARN, "-O2", "-I" + INC, "-c", DRIVER, "-o", str(tmp_path / "driver.o")])


@pytest.mark.skipif(oracle.reference_dir() is None, reason="reference checkout not present")
def test_shim_builds_against_reference_headers(tmp_path):
    # the reference's own types.h and flood.h / filtering.h / pattern.h prototypes:
    # any signature that differs from the reference's is a compile error
    hdr = os.path.join(oracle.reference_dir(), "src", "headers")
    _gcc([*WARN, "-O2", "-fPIC", "-fopenmp", "-DDCF_REFSHIM_REFERENCE_HEADERS", "-I" + MPI_STUB, "-I" + hdr,
          "-I" + INC, "-c", SHIM, "-o", str(tmp_path / "shim_ref.o")])


@pytest.mark.skipif(oracle.reference_dir() is None, reason="reference checkout not present")
def test_declared_layouts_match_reference_types(tmp_path):
    hdr = os.path.join(oracle.reference_dir(), "src", "headers")
    ours = run_layout(tmp_path, ["-I" + INC], '#include "dcf_reftypes.h"', "ours")
    theirs = run_layout(tmp_path, ["-fopenmp", "-I" + MPI_STUB, "-I" + hdr], '#include "types.h"', "theirs")
    assert ours == theirs
    assert "Node.gval" in ours


def build_driver(out_dir):
    import disccofan_gb300 as dcf
    from disccofan_gb300 import _build
    dcf.library()
    _build.build_shim()
    exe = os.path.join(out_dir, "refshim_driver")
    _gcc([*WARN, "-O2", "-I" + INC, DRIVER, "-o", exe, "-L" + PKG, "-ldcf_refshim", "-ldcf_gb300",
          "-Wl,-rpath," + PKG])
    return exe


def test_driver_links_against_shim(tmp_path):
    assert os.path.exists(build_driver(str(tmp_path)))


def test_shim_exports_the_reference_functions(tmp_path):
    build_driver(str(tmp_path))
    out = subprocess.run(["nm", "-D", "--defined-only", os.path.join(PKG, "libdcf_refshim.so")], capture_output=True,
                         text=True, check=True).stdout
    names = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    for f in ("build_tree_with_attributes", "flood_attributes", "get_levelroot", "tree_filtering",
              "tree_attribute_check", "tree_pattern_spectrum", "tree_pattern_spectrum2d", "dcf_refshim_release"):
        assert f in names, f


@pytest.mark.gpu
def test_shim_reproduces_reference_fixtures(tmp_path, lena):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    exe = build_driver(str(tmp_path))
    img = lena["lena"].astype(np.float32)
    h, w = img.shape
    src = tmp_path / "lena.f32"
    img.tofile(str(src))
    r = subprocess.run([exe, str(src), str(w), str(h), "4", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr

    def load(name, dt):
        return np.fromfile(str(tmp_path / name), dt)

    n = h * w
    assert np.array_equal(load("filter_area_200.f32", np.float32).reshape(h, w).astype(np.uint8),
                          lena["gt_area_200"])
    assert np.array_equal(load("filter_ncomp_0.2.f32", np.float32).reshape(h, w).astype(np.uint8),
                          lena["gt_ncomp_0_2"])
    assert np.array_equal(load("check_area.f32", np.float32).reshape(h, w), lena["check_area_c4"])
    assert np.array_equal(load("check_ncomp.f32", np.float32).reshape(h, w), lena["check_ncomp_c4"])
    port = oracle.Port()
    port.load(img, 4, "max")
    port.prepare(0)
    par = load("parent.i64", np.int64)
    assert np.array_equal(par, port.parent())
    # the tree file's level roots and their parents (GT_tree.txt)
    assert np.array_equal(par[lena["tree_index"]], lena["tree_parent"])
    g = img.ravel()
    lr = load("levelroot.i64", np.int64)
    want_lr = np.where((par >= 0) & (g[np.maximum(par, 0)] == g), par, np.arange(n))
    assert np.array_equal(lr, want_lr)
    assert np.array_equal(load("pattern_area.f64", np.float64), port.pattern(0, [2, 10, 50, 200]))
    port.prepare(14)
    want2 = port.pattern2d(14, [1.5, 2, 4], 0, [2, 10, 50, 200])
    assert np.array_equal(load("pattern2d_14_0.f64", np.float64).reshape(want2.shape), want2)
