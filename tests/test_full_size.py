"""Full-size checks on the headline workload: a 16384 x 16384 uint16 log-normal
image with 1e5 sources (bench.make_image), max- and min-tree, 8-connectivity.

The oracle cannot build trees of 268 Mpx in test time, so this size is checked
through properties that hold for any correct component tree, all exact:

- canonical form: one root; every other pixel points to a level root of its own
  level with a lower index, and every level root to a strictly lower level;
- areas: the root's area is N and every node's area exceeds its children's;
- the node count equals the number of level roots;
- the 1-D area spectrum over one all-covering bin sums to the grey-level sum of
  the image (each pixel contributes its level once along its root path);
- the area opening (max-tree) is anti-extensive, the closing (min-tree) extensive,
  and both are idempotent: filtering the output again changes nothing.
"""
import numpy as np
import pytest

import disccofan_gb300 as dcf

pytestmark = pytest.mark.gpu

SIZE = 16384
LAMBDA = 1000.0


def check_tree(ctx, torch, img, tree_type):
    n = img.numel()
    # the extent group (the workload's attribute 18) reads areas back as exact
    # integers; group 0's readout rounds them through float, as the reference does
    t = ctx.build(img, connectivity=8, tree_type=tree_type, attribute=18)
    par = torch.empty(n, dtype=torch.int64, device="cuda")
    g = torch.empty(n, dtype=torch.float32, device="cuda")
    area = torch.empty(n, dtype=torch.float64, device="cuda")
    t.parent(out=par)
    t.gval(out=g)
    t.node_attribute(0, area=True, out=area)
    ctx.synchronize()

    idx = torch.arange(n, device="cuda")
    has_par = par >= 0
    assert int((~has_par).sum()) == 1
    pc = par.clamp(min=0)
    lr = ~has_par | (g[pc] != g)                         # level roots
    non = ~lr
    assert bool((pc[non] < idx[non]).all())             # min-index level root
    assert bool(lr[pc[non]].all())                      # ... which is a level root
    child = lr & has_par
    assert bool((g[pc[child]] < g[child]).all())        # strictly lower parent level
    assert bool((area[pc[child]] > area[child]).all())  # strictly larger parent area
    root = int(torch.nonzero(~has_par)[0])
    assert float(area[root]) == float(n)
    assert t.info()["nodes"] == int(lr.sum())

    spec = t.pattern_spectrum(0, dcf.lvec_from_values([float(n) + 1.0]))
    assert float(spec.sum()) == float(g.double().sum())

    out = torch.empty(n, dtype=torch.float32, device="cuda")
    t.filter(0, LAMBDA, "direct", out=out)
    ctx.synchronize()
    x = img.reshape(-1).float()
    if tree_type == "max":
        assert bool((out <= x).all())
    else:
        assert bool((out >= x).all())
    again_in = out.to(torch.int32).to(img.dtype).reshape(img.shape)
    torch.cuda.synchronize()
    t2 = ctx.build(again_in, connectivity=8, tree_type=tree_type, attribute=18)
    out2 = torch.empty(n, dtype=torch.float32, device="cuda")
    t2.filter(0, LAMBDA, "direct", out=out2)
    ctx.synchronize()
    assert torch.equal(out, out2)
    t2.close()
    t.close()


@pytest.mark.parametrize("tree_type", ["max", "min"])
def test_full_size_c2_properties(ctx, tree_type):
    torch = pytest.importorskip("torch")
    import bench
    if not hasattr(torch, "uint16"):
        pytest.skip("torch without uint16")
    img = bench.make_image(SIZE, seed=2)
    torch.cuda.synchronize()
    check_tree(ctx, torch, img, tree_type)
