#!/usr/bin/env python
"""Benchmark of the component-forest hot path on one GB300 (or N replicas).

Workload (default): a 16384 x 16384 uint16 image (268 Mpx) -- a seeded log-normal
field (exp of Gaussian-smoothed noise, sigma = 8 px, rescaled to 0..65535) with
1e5 injected compact sources -- processed as the reference's operation list

    ("filter", 0, 1000)  then  ("pattern2D", 18, lvec_elong, 0, lvec_area)

on BOTH its max-tree and its min-tree, 8-connectivity: tree build with the
extent attribute group (area + bounding box), direct-rule area opening
lambda = 1000, and the 2-D pattern spectrum of bounding-box elongation x area on
20 log-spaced thresholds each (21 x 21 bins with the leading 0 bin).

One step = both trees.  `value` is Mpx/s = image pixels / step time with the image
already in HBM; `e2e` is the same through the public API with the image in pinned
host memory and the filtered images + spectra read back every step.  Inputs are
537 MB (larger than the 126 MB L2), so no L2 flush is needed between steps.

`--impl reference` times the reference's CPU path: the oracle restatement of the
reference's flooding, seam merge, filter and spectrum (oracle/dcf_oracle.c, pinned
bit-exact against the reference's own code), on all host threads, on the whole
16384^2 image (--ref-reps full-size steps), plus a one-thread figure on a crop.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mpx/s tree build+filter+spectrum (% HBM roofline); fwd+adjoint/fwd time, 1 GB300"
WORKLOAD = "16384^2 u16 log-normal + 1e5 sources; max+min tree, 8-conn, area opening 1000, 2D spectrum bbox-elong x area 21x21"


_T0 = time.perf_counter()


def log(msg: str):
    """Progress on stderr (the JSON result is the only line on stdout)."""
    print(f"[bench {time.perf_counter() - _T0:8.1f}s] {msg}", file=sys.stderr, flush=True)


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def max_over_ranks(values, device):
    """Element-wise maximum of `values` over the ranks of the default process group
    (every rank gets it): the job's time is its slowest replica's."""
    import torch
    t = torch.tensor(values, dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return [float(x) for x in t]


def load_dram_profile():
    """Per-kernel DRAM bytes per launch measured by ncu on the 4096^2 crop of the
    main workload (profiles/dram_c2_4096_u16.json), or None."""
    p = os.path.join(ROOT, "profiles", "dram_c2_4096_u16.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        return json.load(f)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# synthetic input (seeded)
# ---------------------------------------------------------------------------
def make_image(size: int, seed: int = 2, n_sources: int = 100_000, device="cuda"):
    import torch
    rng = np.random.default_rng(seed)
    noise = torch.from_numpy(rng.standard_normal((size, size), dtype=np.float32)).to(device)
    fy = torch.fft.fftfreq(size, device=device)
    fx = torch.fft.rfftfreq(size, device=device)
    sigma = 8.0
    g = torch.exp(-2.0 * (np.pi ** 2) * sigma ** 2 * (fy[:, None] ** 2 + fx[None, :] ** 2))
    field = torch.fft.irfft2(torch.fft.rfft2(noise) * g, s=(size, size))
    del noise
    field = (field - field.mean()) / field.std()
    field = torch.exp(field)
    field = (field - field.min()) / (field.max() - field.min()) * 65535.0
    # compact sources: Gaussian profiles, sigma ~ U(0.7, 2) px, peak ~ U(500, 5000)
    n = int(n_sources * (size / 16384) ** 2) if size < 16384 else n_sources
    cx = torch.from_numpy(rng.uniform(0, size, n)).to(device)
    cy = torch.from_numpy(rng.uniform(0, size, n)).to(device)
    sg = torch.from_numpy(rng.uniform(0.7, 2.0, n)).to(device)
    pk = torch.from_numpy(rng.uniform(500, 5000, n)).to(device)
    r = 6
    off = torch.arange(-r, r + 1, device=device, dtype=torch.float64)
    px = torch.floor(cx)[:, None, None] + off[None, None, :]
    py = torch.floor(cy)[:, None, None] + off[None, :, None]
    d2 = (px - cx[:, None, None]) ** 2 + (py - cy[:, None, None]) ** 2
    val = pk[:, None, None] * torch.exp(-d2 / (2 * sg[:, None, None] ** 2))
    ix = px.expand_as(val).long()
    iy = py.expand_as(val).long()
    ok = (ix >= 0) & (ix < size) & (iy >= 0) & (iy < size)
    flat = (iy[ok] * size + ix[ok])
    field = field.reshape(-1).double()
    field.index_put_((flat,), val[ok], accumulate=True)
    img = torch.clamp(torch.round(field), 0, 65535).to(torch.int32).reshape(size, size)
    return img.to(torch.uint16) if hasattr(torch, "uint16") else img


def lvecs(npix: int):
    import disccofan_gb300 as dcf
    l_elong = dcf.lvec_from_values(np.geomspace(1, 16384, 20))
    l_area = dcf.lvec_from_values(np.geomspace(1, npix, 20))
    return l_elong, l_area


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            c = [x.strip() for x in ln.split(",")]
            if len(c) < 9:
                continue
            try:
                sm.append(float(c[1]))
                smax = max(smax, float(c[2]))
            except ValueError:
                continue
            for nm, v in zip(names, c[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax or None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_ours(args):
    import torch
    import disccofan_gb300 as dcf

    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    # a dedicated stream per tree: the step's max and min trees are independent, so
    # they run concurrently, one library context (stream) and one host thread each
    # (--serial-trees: one after the other on one stream); the timing events are on
    # the first stream, which joins the second at the end of the timed region
    from concurrent.futures import ThreadPoolExecutor
    concurrent = not args.serial_trees
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    stream = streams[0]
    torch.cuda.set_stream(stream)
    ctxs = [dcf.Context(local, stream=s.cuda_stream) for s in streams]
    ctx = ctxs[0]
    pool = ThreadPoolExecutor(2)
    size = args.size
    img = make_image(size, seed=2 + rank)
    npix = size * size
    l_elong, l_area = lvecs(npix)
    d_out = [torch.empty(npix, dtype=torch.float32, device="cuda") for _ in range(2)]
    d_spec = [torch.zeros((l_area.size, l_elong.size), dtype=torch.float64, device="cuda") for _ in range(2)]
    TREES = ("max", "min")

    def tree_work(k, c, src):
        with torch.cuda.stream(streams[k] if c is ctxs[k] else stream):
            t = c.build(src, connectivity=8, tree_type=TREES[k], attribute=18)
            t.filter(0, 1000.0, "direct", out=d_out[k])
            d_spec[k].zero_()
            t.pattern_spectrum2d(18, l_elong, 0, l_area, out=d_spec[k])
        return t

    def step(conc=concurrent):
        if conc:
            return [f.result() for f in [pool.submit(tree_work, k, ctxs[k], img) for k in range(2)]]
        return [tree_work(k, ctx, img) for k in range(2)]

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    for _ in range(args.warmup):
        step()
    barrier()
    info_trees = step()
    node_counts = [t.info()["nodes"] for t in info_trees]
    del info_trees
    barrier()

    # device-resident timed region
    launches0 = sum(c.launches for c in ctxs)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        ev0.record(stream)
        streams[1].wait_event(ev0)
        if concurrent:
            # each tree's thread runs its K steps back to back, with no join between
            # steps: the two trees drift out of phase, so one's latency-bound phases
            # (seam zips, walks) overlap the other's issue-bound tile build
            def tree_steps(k):
                for _ in range(args.steps):
                    t = tree_work(k, ctxs[k], img)
                    t.close()
            for f in [pool.submit(tree_steps, k) for k in range(2)]:
                f.result()
        else:
            for _ in range(args.steps):
                step()
        stream.wait_stream(streams[1])
        ev1.record(stream)
        barrier()
    ms = ev0.elapsed_time(ev1) / args.steps
    launches = sum(c.launches for c in ctxs) - launches0
    # per-kernel split: CUDA events on one stream over serial steps (the concurrent
    # steps overlap kernels of the two trees, so per-kernel times would overlap too)
    prof_steps = max(1, min(args.steps, 3))
    ctx.set_profiling(True)
    for _ in range(prof_steps):
        step(conc=False)
    prof = ctx.profile()
    ctx.set_profiling(False)
    ctx.synchronize()
    prof_ms_step = sum(v[0] for v in prof.values()) / prof_steps

    # e2e through the public API: every step copies the pinned host image to the
    # device (dcf_image_stage) -- with concurrent trees once per tree, each tree's
    # thread running its steps back to back as in the device-resident region, so one
    # tree's copies overlap the other's kernels; serially once for both trees.  The
    # filtered images come back in the input's own uint16 type (dcf_filter_as, as
    # the reference writes a 16-bit input's output) and the spectra as doubles
    h_img = torch.empty((size, size), dtype=img.dtype, pin_memory=True)
    h_img.copy_(img)
    h_img_np = h_img.numpy() if img.dtype != torch.int32 else h_img.numpy().astype(np.uint16)
    h_out = [torch.empty(npix, dtype=torch.uint16 if hasattr(torch, "uint16") else torch.int16,
                         pin_memory=True).numpy().view(np.uint16) for _ in range(2)]
    h_spec = [np.zeros((l_area.size, l_elong.size), np.float64) for _ in range(2)]

    def e2e_tree(k, c, staged):
        t = c.build(staged, connectivity=8, tree_type=TREES[k], attribute=18)
        t.filter(0, 1000.0, "direct", out=h_out[k])
        h_spec[k][:] = 0
        t.pattern_spectrum2d(18, l_elong, 0, l_area, out=h_spec[k])
        t.close()

    def e2e_step():
        staged = ctx.stage(h_img_np)
        for k in range(2):
            e2e_tree(k, ctx, staged)

    def e2e_tree_steps(k, n):
        for _ in range(n):
            e2e_tree(k, ctxs[k], ctxs[k].stage(h_img_np))

    def e2e_run(n):
        if concurrent:
            for f in [pool.submit(e2e_tree_steps, k, n) for k in range(2)]:
                f.result()
        else:
            for _ in range(n):
                e2e_step()

    e2e_run(1)
    barrier()
    e2e_steps = 0 if args.no_e2e else max(1, min(args.steps, 5))
    t0 = time.perf_counter()
    e2e_run(e2e_steps)
    barrier()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / max(e2e_steps, 1)
    h2d = (2 if concurrent else 1) * npix * img.element_size()
    d2h = 2 * (h_out[0].nbytes + h_spec[0].nbytes)

    if world > 1:
        ms, e2e_ms = max_over_ranks([ms, e2e_ms], "cuda")
    if rank != 0:
        return None

    # Roofline.  Algorithmic bytes are the compulsory I/O of one tree: the u16 image
    # in, a 4-byte parent and the u16 filtered image out, and a 12-byte record
    # (area + 2-D bounding box) per node: B_tree = N (2 + 4 + 2) + 12 M, plus 8 bytes
    # per spectrum bin.  The dominant kernel's `achieved` is B_tree / its mean
    # duration per launch (one launch per tree, the max and min trees alternating,
    # so M is their mean); `kernel_bytes` is that kernel's own minimum traffic.
    peak, peak_kind = load_peaks()
    s_in = 2
    dom, (dom_ms, dom_n) = max(prof.items(), key=lambda kv: kv[1][0])
    total_prof = sum(v[0] for v in prof.values())
    M = sum(node_counts) / 2.0
    nbins = l_area.size * l_elong.size
    B_tree = npix * (s_in + 4 + s_in) + 12 * M + 8 * nbins
    B_alg = 2 * B_tree
    kernel_bytes = {
        "tile_build": npix * (s_in + 4 + 8),        # image in; level and 64-bit node word out
        "seam_merge": None,                          # chain walks: no fixed byte count
        "canonicalise": npix * (8 + 4 + 1),         # node words in, parent and root flag out
        "attr_pixels": npix * (4 + 1) + M * 12,     # parent + root flag in, area + bbox records out
        "attr_bottom_up": M * (12 + 4 + 4),
        "filter_resolve": M * (4 + 4),
        "filter_out": npix * (4 + 4 + 2),
        "spectrum": M * (12 + 4 + 4) + 8 * nbins,
    }.get(dom)
    achieved = B_tree / (dom_ms / dom_n * 1e-3) / 1e9
    dram = load_dram_profile()
    traffic = None
    pipeline_traffic = None
    if dram:
        # DRAM bytes per pixel per launch of each kernel, from ncu on the 4096^2
        # crop of this workload, scaled by pixels (per-pixel passes; node passes
        # scale with the node count, which is proportional to the pixels here)
        scale = npix / dram["pixels"]
        if dom in dram["per_launch_bytes"]:
            traffic = round(dram["per_launch_bytes"][dom] * scale)
        pipeline_traffic = round(sum(dram["per_launch_bytes"].values()) * scale * 2)
    result = {
        "metric": METRIC,
        "value": round(world * npix / 1e6 / (ms * 1e-3), 3),
        "unit": "Mpx/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u16",
        "data": "synthetic: seeded log-normal field (numpy PCG64 seed 2, FFT Gaussian blur sigma 8) + 1e5 sources",
        "config": {"workload": WORKLOAD if size == 16384 else WORKLOAD.replace("16384", str(size)),
                   "pixels": npix, "trees_per_step": 2, "connectivity": 8, "attribute_group": "extent (area+bbox)",
                   "filter": "direct, area >= 1000", "spectrum": "2D bbox-elong(18) x area(0), 21x21",
                   "nodes_per_tree": node_counts, "l2": "inputs (537 MB) larger than L2; no flush",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "pipeline_roofline": {"alg_bytes_per_step": B_alg,
                                         "achieved_gbs": round(B_alg / (ms * 1e-3) / 1e9, 2),
                                         "frac": round(B_alg / (ms * 1e-3) / 1e9 / peak, 5),
                                         "dram_bytes_per_step": pipeline_traffic,
                                         "traffic_ratio": None if pipeline_traffic is None else
                                         round(pipeline_traffic / B_alg, 3),
                                         "dram_source": dram["source"] if dram else None},
                   "trees": ("concurrent (two contexts, two streams; each tree's K steps back to back on its own "
                             "host thread)") if concurrent else "serial (one stream)",
                   "kernel_ms_per_step": {k: round(v[0] / prof_steps, 3) for k, v in sorted(prof.items())},
                   "kernel_split": f"CUDA events on one stream over {prof_steps} serial steps "
                                   f"({prof_ms_step:.1f} ms/step of kernels)"},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 5), "traffic": traffic,
                     "traffic_source": None if traffic is None else
                     "ncu DRAM read+write of one 4096^2 launch, scaled by pixels",
                     "share": round(dom_ms / total_prof, 4) if total_prof else None,
                     "alg_bytes_per_launch": round(B_tree), "kernel_bytes": kernel_bytes,
                     "alg_bytes_basis": "per tree: N*(2 in + 4 parent + 2 filtered) + 12*M + 8*bins",
                     "peak_source": f"{peak_kind} hbm_gbs"},
        "e2e": None if args.no_e2e else {
            "value": round(world * npix / 1e6 / (e2e_ms * 1e-3), 3), "unit": "Mpx/s",
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": round(e2e_ms, 3)},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    if not args.no_cpu:
        result["cpu_baseline"] = cpu_baseline(img, args.cpu_sample, reps=1, ctx=ctx)
    del img, d_out, d_spec, h_img
    log(f"main workload: {ms:.1f} ms/step")
    if not args.no_batch:
        result["batch"] = run_batch(args, ctx, stream)
    if not args.no_adjoint:
        result["adjoint"] = run_adjoint(args, ctx, stream)
    return result


# ---------------------------------------------------------------------------
# batched cutouts: one recorded CUDA graph per step vs a loop of the plain API
# ---------------------------------------------------------------------------
def make_cutouts(count: int = 4096, seed: int = 4, device="cuda"):
    """count float32 cutouts, width and height independently log-uniform in [64, 1024]:
    unit Gaussian noise blurred with sigma = 2 px plus 1..50 Gaussian sources (sigma
    U(1, 5) px, peak U(3, 10) x the background's std).  Backgrounds are windows of
    one large blurred field.  Returns (shapes [(h, w)], concatenated pixels on device)."""
    import torch
    rng = np.random.default_rng(seed)
    ws = np.rint(np.exp(rng.uniform(np.log(64), np.log(1024), count))).astype(np.int64)
    hs = np.rint(np.exp(rng.uniform(np.log(64), np.log(1024), count))).astype(np.int64)
    F = 8192
    noise = torch.from_numpy(rng.standard_normal((F, F), dtype=np.float32)).to(device)
    fy = torch.fft.fftfreq(F, device=device)
    fx = torch.fft.rfftfreq(F, device=device)
    g = torch.exp(-2.0 * (np.pi ** 2) * 4.0 * (fy[:, None] ** 2 + fx[None, :] ** 2))
    field = torch.fft.irfft2(torch.fft.rfft2(noise) * g, s=(F, F))
    del noise
    std = float(field.std())
    sizes = hs * ws
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    pix = torch.empty(int(sizes.sum()), dtype=torch.float32, device=device)
    oy = rng.integers(0, F - hs + 1)
    ox = rng.integers(0, F - ws + 1)
    for i in range(count):
        pix[offs[i]:offs[i] + sizes[i]] = field[oy[i]:oy[i] + hs[i], ox[i]:ox[i] + ws[i]].reshape(-1)
    # sources, all cutouts at once (in chunks)
    k = rng.integers(1, 51, count)
    img = np.repeat(np.arange(count), k)
    cy = rng.uniform(0, hs[img])
    cx = rng.uniform(0, ws[img])
    sg = rng.uniform(1, 5, img.size)
    pk = rng.uniform(3, 10, img.size) * std
    r = 12

    def t(a, dt=torch.float64):
        return torch.from_numpy(np.asarray(a)).to(device=device, dtype=dt)

    off = torch.arange(-r, r + 1, device=device, dtype=torch.float64)
    for lo in range(0, img.size, 20000):
        sl = slice(lo, lo + 20000)
        tcx, tcy, tsg, tpk = t(cx[sl]), t(cy[sl]), t(sg[sl]), t(pk[sl])
        th, tw, to = t(hs[img[sl]], torch.int64), t(ws[img[sl]], torch.int64), t(offs[img[sl]], torch.int64)
        px = torch.floor(tcx)[:, None, None] + off[None, None, :]
        py = torch.floor(tcy)[:, None, None] + off[None, :, None]
        d2 = (px - tcx[:, None, None]) ** 2 + (py - tcy[:, None, None]) ** 2
        val = (tpk[:, None, None] * torch.exp(-d2 / (2 * tsg[:, None, None] ** 2))).float()
        ix, iy = px.expand_as(val).long(), py.expand_as(val).long()
        ok = (ix >= 0) & (ix < tw[:, None, None]) & (iy >= 0) & (iy < th[:, None, None])
        flat = (to[:, None, None] + iy * tw[:, None, None] + ix)[ok]
        pix.index_put_((flat,), val[ok], accumulate=True)
    return [(int(h), int(w)) for h, w in zip(hs, ws)], pix


def guarded(fn, *a):
    """A host-side baseline must not cost the run its bench line: a failure is
    reported in place of the figure."""
    try:
        return fn(*a)
    except Exception as e:  # noqa: BLE001 -- reported, not hidden
        log(f"{fn.__name__} failed: {e!r}")
        return {"error": repr(e)}


def batch_cpu_baseline(shapes, pix, count: int, threads: int | None = None):
    """The batched workload on the host: the oracle on the first `count` cutouts,
    timed two ways -- one cutout at a time on all host threads, and the cutouts
    spread over the host threads with one thread each -- and the faster reported."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import oracle
    oracle.build(ref=False)
    threads = threads or os.cpu_count() or 1
    l_tr = list(np.geomspace(1, 1e11, 24))
    l_ar = list(np.geomspace(1, 1 << 20, 24))
    npx = sum(h * w for h, w in shapes[:count])
    host = pix[:npx].to("cpu").numpy()
    views, o = [], 0
    for h, w in shapes[:count]:
        views.append(host[o:o + h * w].reshape(h, w))
        o += h * w

    def one(v, nt):
        p = oracle.Port(threads=nt)
        p.load(v, 8, "max", threads=nt)
        p.pattern2d(13, l_tr, 0, l_ar)
        del p

    t0 = time.perf_counter()
    for v in views:
        one(v, threads)
    t_all = time.perf_counter() - t0
    t0 = time.perf_counter()
    with ThreadPoolExecutor(threads) as ex:  # the oracle's C calls release the GIL
        list(ex.map(lambda v: one(v, 1), views))
    t_spread = time.perf_counter() - t0
    best = min(t_all, t_spread)
    return {"value": round(npx / 1e6 / best, 3), "unit": "Mpx/s", "cores": threads, "kind": "port",
            "sample": f"first {count} cutouts ({npx} px), max-tree 8-conn, inertia group, 2D spectrum; one "
                      f"cutout at a time on {threads} threads {t_all:.2f} s, cutouts over {threads} threads "
                      f"one each {t_spread:.2f} s; the faster"}


def run_batch(args, ctx, stream):
    """The batched workload: 4096 float32 cutouts (64..1024 a side), max-tree 8-conn,
    inertia group, 2-D spectrum inertia trace (13) x area (0) on 24 log thresholds each
    (25 x 25 bins) per cutout."""
    import torch
    import disccofan_gb300 as dcf
    log("batch: generating cutouts")
    shapes, pix = make_cutouts(args.batch_count)
    npx = pix.numel()
    log(f"batch: {len(shapes)} cutouts, {npx} pixels; autotuning")
    l_tr = dcf.lvec_from_values(np.geomspace(1, 1e11, 24))
    l_ar = dcf.lvec_from_values(np.geomspace(1, 1 << 20, 24))
    spec = (13, l_tr, 0, l_ar)
    b = ctx.batch(shapes, np.float32, connectivity=8, attribute=13)
    spectra = torch.empty((len(shapes), l_ar.size, l_tr.size), dtype=torch.float64, device="cuda")
    # the schedule is tuned on the batch itself (default), or on a sample batch of the
    # first tune_n cutouts applied to the whole batch.  A small sample misleads: its
    # seam merge is bound by the longest chain walks, the whole batch's by contention,
    # so they prefer different merge orders.
    tune_n = min(len(shapes), args.tune_sample)
    t0 = time.perf_counter()
    tune_ms = None
    if not args.no_autotune and tune_n == len(shapes):
        tune_ms = b.autotune(pix, repeats=1)
    elif not args.no_autotune:
        tb = ctx.batch(shapes[:tune_n], np.float32, connectivity=8, attribute=13)
        tune_px = sum(h * w for h, w in shapes[:tune_n])
        tune_ms = tb.autotune(pix[:tune_px], repeats=1)
        ti = tb.info()
        tb.close()
        b.set_schedule(ti["tile"], ti["ctas_per_sm"], ti["chunk"])
        b.set_merge(ti["seam_buckets"], ti["up_steps"])
    tune_s = time.perf_counter() - t0
    log(f"batch: autotuned on {tune_n} cutouts in {tune_s:.1f}s -> {b.info()}")
    for _ in range(max(args.warmup, 2)):  # learns the capacity, then records the graph
        b.run(pix, spectrum=spec, use_graph=True, spectra=spectra)
    torch.cuda.synchronize()
    steps = max(1, args.steps)
    launches0 = ctx.launches
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(steps):
        b.run(pix, spectrum=spec, use_graph=True, spectra=spectra)
    ev1.record(stream)
    torch.cuda.synchronize()
    graph_ms = ev0.elapsed_time(ev1) / steps
    graph_launches = (ctx.launches - launches0) // steps
    info = b.info()
    log(f"batch: graph {graph_ms:.1f} ms/step; looping the single-image API")
    loop_spec = torch.zeros_like(spectra)
    views = []
    o = 0
    for h, w in shapes:
        views.append(pix[o:o + h * w].view(h, w))
        o += h * w
    # the loop is timed on a bounded sample (the first loop_n cutouts) and scaled by
    # pixels, so that this arm stays within seconds
    loop_n = min(len(views), args.loop_sample)

    def loop_over(idx):
        for i in idx:
            t = ctx.build(views[i], connectivity=8, tree_type="max", attribute=13)
            t.pattern_spectrum2d(13, l_tr, 0, l_ar, out=loop_spec[i])
            t.close()

    loop_over(range(min(16, loop_n)))  # warm-up
    loop_spec.zero_()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    loop_over(range(loop_n))
    torch.cuda.synchronize()
    loop_px = sum(h * w for h, w in shapes[:loop_n])
    loop_ms = (time.perf_counter() - t0) * 1e3 * npx / loop_px
    log(f"batch: loop {loop_ms:.1f} ms/step (scaled from {loop_n} cutouts)")
    ref = loop_spec[:loop_n]
    diff = float(((spectra[:loop_n] - ref).abs().max() / ref.abs().max().clamp_min(1e-300)).item())
    b.close()
    return {"workload": f"{len(shapes)} f32 cutouts, sides log-uniform 64..1024; max-tree 8-conn, inertia group, "
                        "2D spectrum inertia-trace x area 25x25 per cutout",
            "cutouts": len(shapes), "pixels": npx, "nodes": info["nodes"],
            "graph_ms_per_step": round(graph_ms, 3), "graph_mpx_s": round(npx / 1e6 / (graph_ms * 1e-3), 2),
            "loop_ms_per_step": round(loop_ms, 3), "loop_mpx_s": round(npx / 1e6 / (loop_ms * 1e-3), 2),
            "speedup_vs_loop": round(loop_ms / graph_ms, 2), "max_rel_spectrum_diff_vs_loop": diff,
            "loop_sample": f"first {loop_n} cutouts ({loop_px} px), one pass, scaled to the batch's pixels",
            "schedule": {"tile": info["tile"], "ctas_per_sm": info["ctas_per_sm"], "chunk": info["chunk"]},
            "autotune": {"sample_cutouts": tune_n, "best_sample_build_ms": None if tune_ms is None else round(tune_ms, 3),
                         "seconds": round(tune_s, 2), "seam_buckets": info["seam_buckets"], "up_steps": info["up_steps"]},
            "graph_kernels": info["graph_kernels"], "gpu_launches_per_step": int(graph_launches), "steps": steps,
            "cpu_baseline": None if args.no_cpu else guarded(batch_cpu_baseline, shapes, pix, args.batch_cpu_sample)}


# ---------------------------------------------------------------------------
# differentiable workload: forward vs forward + adjoint (tree recomputed)
# ---------------------------------------------------------------------------
def distinct_values(im):
    """Separate exact ties of a float32 image while keeping its order: after a stable
    sort, every value not above its predecessor moves up to the next float (repeated
    until all are distinct; a 512^2 image of continuous values has a few hundred
    float32 ties and the loop ends after a few passes)."""
    import torch
    flat = im.reshape(-1)
    vals, idx = torch.sort(flat, stable=True)
    for _ in range(64):
        dup = vals[1:] <= vals[:-1]
        if not bool(dup.any()):
            break
        nxt = torch.nextafter(vals[:-1], torch.full_like(vals[:-1], float("inf")))
        vals[1:] = torch.where(dup, nxt, vals[1:])
    else:
        raise RuntimeError("could not separate tied values")
    out = torch.empty_like(flat)
    out[idx] = vals
    return out.view_as(im)


def make_distinct_images(count: int = 256, size: int = 512, seed: int = 5, device="cuda"):
    """count x size^2 float32: Gaussian blur (sigma 2) of N(0,1) plus 0.05 N(0,1) i.i.d.,
    with every image's values distinct (distinct_values)."""
    import torch
    rng = np.random.default_rng(seed)
    fy = torch.fft.fftfreq(size, device=device)
    fx = torch.fft.rfftfreq(size, device=device)
    g = torch.exp(-2.0 * (np.pi ** 2) * 4.0 * (fy[:, None] ** 2 + fx[None, :] ** 2))
    out = torch.empty((count, size, size), dtype=torch.float32, device=device)
    for i in range(count):
        a = torch.from_numpy(rng.standard_normal((size, size), dtype=np.float32)).to(device)
        e = torch.from_numpy(rng.standard_normal((size, size), dtype=np.float32)).to(device)
        im = distinct_values((torch.fft.irfft2(torch.fft.rfft2(a) * g, s=(size, size)) + 0.05 * e).float())
        assert torch.unique(im).numel() == im.numel()
        out[i] = im
    return out


def run_adjoint(args, ctx, stream):
    """256 float32 512^2 images: area opening (lambda 64, direct rule) and the 2-D
    spectrum elongation (14) x area (0) on 16 log thresholds each, then the adjoint of
    sum(w * spectra) + sum(v * filtered), w, v ~ N(0, 1), through the autograd Function
    (backward rebuilds the trees)."""
    import torch
    import disccofan_gb300 as dcf
    from disccofan_gb300.autograd import filter_and_spectrum
    count, size = args.adj_count, 512
    log("adjoint: generating images")
    x = make_distinct_images(count, size)
    log("adjoint: timing")
    l_el = dcf.lvec_from_values(np.geomspace(1, 100, 16))
    l_ar = dcf.lvec_from_values(np.geomspace(1, size * size, 16))
    spec = (14, l_el, 0, l_ar)
    b = ctx.batch([(size, size)] * count, np.float32, connectivity=8, attribute=14)
    rng = np.random.default_rng(6)
    v = torch.from_numpy(rng.standard_normal((count, size, size), dtype=np.float32)).to("cuda")
    w = torch.from_numpy(rng.standard_normal((count, l_ar.size, l_el.size))).to("cuda")
    xg = x.clone().requires_grad_(True)

    def fwd():
        with torch.no_grad():
            return filter_and_spectrum(b, x, 0, 64.0, spec)

    def fwd_adj():
        xg.grad = None
        f, s = filter_and_spectrum(b, xg, 0, 64.0, spec)
        ((v * f).sum(dtype=torch.float64) + (w * s).sum()).backward()
        return xg.grad

    def timed(fn, n):
        for _ in range(max(args.warmup, 2)):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(n):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n

    n = max(1, args.steps)
    t_fwd = timed(fwd, n)
    t_both = timed(fwd_adj, n)
    t_f = min(t_fwd, timed(fwd, n))
    b.close()
    return {"workload": f"{count} f32 {size}^2 images (distinct values); area opening 64 + 2D spectrum "
                        "elongation x area 17x17; adjoint of sum(w*spectra)+sum(v*filtered), tree recomputed",
            "fwd_ms": round(t_f, 3), "fwd_adjoint_ms": round(t_both, 3), "ratio": round(t_both / t_f, 3),
            "target_ratio": 2.5, "fwd_mpx_s": round(count * size * size / 1e6 / (t_f * 1e-3), 2), "steps": n}


# ---------------------------------------------------------------------------
# CPU baseline: the oracle restatement of the reference's path, all host threads
# ---------------------------------------------------------------------------
def oracle_step(img_f32, threads: int, npix_bins: int):
    """The main workload's step on the host: the oracle restatement of the reference's
    build, area filter and 2-D spectrum (bins of the full image), max and min tree.
    Returns (seconds, {tree: (filtered, spectrum)})."""
    from oracle import oracle
    l_el = list(np.geomspace(1, 16384, 20))
    l_ar = list(np.geomspace(1, npix_bins, 20))
    out = {}
    t0 = time.perf_counter()
    for tt in ("max", "min"):
        p = oracle.Port(threads=threads)
        p.load(img_f32, 8, tt, threads=threads)
        out[tt] = (p.filter(0, 1000.0, 0), p.pattern2d(18, l_el, 0, l_ar))
        del p
    return time.perf_counter() - t0, out


def cpu_baseline(img_dev, sample: int, reps: int = 1, threads: int | None = None, ctx=None):
    """The oracle on a sample x sample crop of the image on all host threads; with a
    context, the GPU path runs on the same crop and `parity_vs_gpu` says whether the
    filtered images and spectra of both trees are identical."""
    from oracle import oracle
    oracle.build(ref=False)
    npix_full = img_dev.shape[0] * img_dev.shape[1]
    crop = img_dev[:sample, :sample].to("cpu").numpy().astype(np.float32) if hasattr(img_dev, "to") else \
        np.asarray(img_dev[:sample, :sample], np.float32)
    threads = threads or os.cpu_count() or 1
    times, outs = [], None
    for _ in range(reps):
        secs, outs = oracle_step(crop, threads, npix_full)
        times.append(secs)
    best = min(times)
    res = {"value": round(crop.size / 1e6 / best, 3), "unit": "Mpx/s", "cores": threads, "kind": "port",
           "sample": f"{sample}x{sample} crop of the same image, max+min tree, same ops; best of {reps}",
           "seconds_per_step": round(best, 3)}
    if ctx is not None and hasattr(img_dev, "to"):
        l_elong, l_area = lvecs(npix_full)
        dev = img_dev[:sample, :sample].contiguous()
        same, detail = True, {}
        for tt in ("max", "min"):
            t = ctx.build(dev, connectivity=8, tree_type=tt, attribute=18)
            f = t.filter(0, 1000.0, "direct")
            s = t.pattern_spectrum2d(18, l_elong, 0, l_area)
            t.close()
            nf, ns = int((f != outs[tt][0]).sum()), int((s != outs[tt][1]).sum())
            same = same and nf == 0 and ns == 0
            detail[tt] = {"filtered_pixels_differing": nf, "spectrum_bins_differing": ns}
        res["parity_vs_gpu"] = bool(same)
        if not same:
            res["parity_detail"] = detail
    return res


def run_reference(args):
    rank, world, local = env_rank()
    if rank != 0:
        return None
    import torch
    from oracle import oracle
    oracle.build(ref=False)
    size = args.size
    # the same image as our arm (generated on the GPU when there is one: the FFT
    # and the sources are identical to ours), then held in host memory as the
    # reference holds every pixel, float32
    img = make_image(size, seed=2, device="cuda" if torch.cuda.is_available() else "cpu")
    img = img.to("cpu").numpy().astype(np.float32)
    threads = os.cpu_count() or 1
    # Each full-size step (both trees, ~80 s on 16 cores) is timed as a whole; the
    # --steps/--warmup counts would make this arm take half an hour, so
    # --ref-reps full-size steps are timed (default 1) with no warm-up: the
    # oracle's only warm-up effect is first-touch of its host buffers, which
    # each step pays again anyway (its trees are freed after every step)
    reps = max(1, args.ref_reps)
    times = [oracle_step(img, threads, img.size)[0] for _ in range(reps)]
    secs = statistics.median(times)
    v = round(img.size / 1e6 / secs, 3)
    # one host thread, on a 1024^2 crop (bins of the full image)
    s1 = min(1024, size)
    crop = np.ascontiguousarray(img[:s1, :s1])
    secs1 = oracle_step(crop, 1, img.size)[0]
    sample = (f"the whole {size}x{size} image, max+min tree, same ops, {threads} host threads; "
              f"{reps} full-size step(s) timed (median), not --steps")
    cb = {"value": v, "unit": "Mpx/s", "cores": threads, "kind": "port", "sample": sample,
          "seconds_per_step": round(secs, 3),
          "single_thread": {"value": round(crop.size / 1e6 / secs1, 3), "unit": "Mpx/s", "cores": 1,
                            "sample": f"{s1}x{s1} crop, max+min tree, same ops", "seconds": round(secs1, 3)}}
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "Mpx/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(secs * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u16",
            "data": "synthetic: the same seeded image as the GPU arm",
            "config": {"workload": WORKLOAD if size == 16384 else WORKLOAD.replace("16384", str(size)),
                       "sample": sample},
            "cpu_baseline": cb, "e2e": {"value": v, "unit": "Mpx/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=16384)
    ap.add_argument("--cpu-sample", type=int, default=4096)
    ap.add_argument("--ref-reps", type=int, default=1, help="--impl reference: full-size steps timed")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end pass (profiling runs)")
    ap.add_argument("--serial-trees", action="store_true",
                    help="build a step's max and min trees one after the other on one stream")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-cutout workload")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the forward+adjoint workload")
    ap.add_argument("--no-autotune", action="store_true", help="batched workload: keep the default schedule")
    ap.add_argument("--batch-count", type=int, default=4096)
    ap.add_argument("--loop-sample", type=int, default=512, help="cutouts timed through the single-image API")
    ap.add_argument("--tune-sample", type=int, default=4096, help="cutouts the batch schedule is tuned on")
    ap.add_argument("--adj-count", type=int, default=256)
    ap.add_argument("--batch-cpu-sample", type=int, default=64, help="cutouts of the batch's CPU baseline")
    args = ap.parse_args()
    res = run_reference(args) if args.impl == "reference" else run_ours(args)
    if res is not None:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
