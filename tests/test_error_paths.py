"""GPU tests of the error paths the C ABI promises in place of the reference's
check_alloc -> MPI_Abort (src/sources/checks.c:4-24).

* Bounded device loops.  Every tree-merge loop has an iteration limit; when it runs
  out the kernel sets an error bit and returns (no trap, no hang), and the next
  synchronising call reports DCF_ERR_TIMEOUT.  The test lowers the limit with the
  context's DCF_MERGE_BOUND knob so that an ordinary build runs out, then checks the
  status and that the device stays usable.
* Allocation failures.  The context's DCF_FAIL_ALLOC = k knob makes its k-th device
  allocation report out-of-memory; every k up to the number of allocations a build,
  filter and spectrum make must give DCF_ERR_NOMEM, and the same context must then
  build correctly.
Both knobs are read when a context is created.
"""
import numpy as np
import pytest

import disccofan_gb300 as dcf
from oracle import oracle

pytestmark = pytest.mark.gpu

TIMEOUT, NOMEM = 4, 2


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def knob_ctx(monkeypatch, name, value):
    monkeypatch.setenv(name, str(value))
    ctx = dcf.Context(0)
    monkeypatch.delenv(name)
    return ctx


def image(seed=3, shape=(200, 230)):
    rng = np.random.default_rng(seed)
    return rng.integers(0, 5000, shape).astype(np.uint16)


def check_against_oracle(t, img, conn, tree):
    port = oracle.Port()
    port.load(img.astype(np.float32), conn, tree)
    port.prepare(0)
    assert np.array_equal(t.parent(), port.parent())
    assert np.array_equal(t.filter(0, 50.0), port.filter(0, 50.0, 0))


@pytest.mark.parametrize("conn,shape", [(8, (200, 230)), (4, (130, 300)), (6, (20, 40, 50))])
def test_merge_loop_limit_reports_timeout(monkeypatch, conn, shape):
    _torch()
    img = image(shape=shape)
    ctx = knob_ctx(monkeypatch, "DCF_MERGE_BOUND", 2)
    with pytest.raises(dcf.DcfError) as e:
        t = ctx.build(img, connectivity=conn, tree_type="max", attribute=0)
        t.parent()
    assert e.value.status == TIMEOUT
    ctx.close()
    # the device and a fresh context are unaffected
    ok = dcf.Context(0)
    check_against_oracle(ok.build(img, connectivity=conn, tree_type="max", attribute=0), img, conn, "max")
    ok.close()


def test_merge_loop_limit_reports_timeout_in_batches(monkeypatch):
    _torch()
    shapes = [(90, 70), (64, 130), (150, 40)]
    rng = np.random.default_rng(8)
    cuts = [rng.standard_normal(s).astype(np.float32) for s in shapes]
    ctx = knob_ctx(monkeypatch, "DCF_MERGE_BOUND", 2)
    b = ctx.batch(shapes, np.float32, connectivity=8, attribute=13)
    with pytest.raises(dcf.DcfError) as e:
        b.run(b.concat(cuts), filter_attr=0, lam=10.0, use_graph=False)
    assert e.value.status == TIMEOUT
    b.close()
    ctx.close()


def test_every_allocation_failure_reports_nomem(monkeypatch):
    _torch()
    img = image(shape=(150, 170))
    lv1 = dcf.lvec_from_values([1.5, 2, 4, 8])
    lv2 = dcf.lvec_from_values([4, 16, 64, 256])
    failures = 0
    for k in range(64):
        ctx = knob_ctx(monkeypatch, "DCF_FAIL_ALLOC", k)
        try:
            t = ctx.build(img, connectivity=8, tree_type="min", attribute=18)
            t.filter(0, 50.0, "subtractive")
            t.pattern_spectrum2d(18, lv1, 0, lv2)
            t.set_attribute(13)
            t.filter(14, 2.0)
        except dcf.DcfError as e:
            assert e.status == NOMEM, (k, str(e))
            failures += 1
            # one refusal only: the same context then works
            check_against_oracle(ctx.build(img, connectivity=8, tree_type="min", attribute=0), img, 8, "min")
            ctx.close()
            continue
        ctx.close()
        break
    else:
        pytest.fail("the knob never ran past the allocations of a build")
    assert failures >= 5


def test_batch_allocation_failures_report_nomem(monkeypatch):
    _torch()
    shapes = [(40, 50), (70, 33)]
    rng = np.random.default_rng(2)
    cuts = [rng.standard_normal(s).astype(np.float32) for s in shapes]
    failures = 0
    for k in range(64):
        ctx = knob_ctx(monkeypatch, "DCF_FAIL_ALLOC", k)
        b = None
        try:
            b = ctx.batch(shapes, np.float32, connectivity=8, attribute=13)
            b.run(b.concat(cuts), filter_attr=0, lam=10.0, use_graph=False)
        except dcf.DcfError as e:
            assert e.status == NOMEM, (k, str(e))
            failures += 1
            if b is not None:
                b.close()  # batches go before their context
            ctx.close()
            continue
        b.close()
        ctx.close()
        break
    else:
        pytest.fail("the knob never ran past the allocations of a batch")
    assert failures >= 5
