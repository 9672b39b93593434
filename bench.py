#!/usr/bin/env python3
"""Benchmark: sRGBA8 mip-chain generation on GB300 through the C ABI.

Headline workload: one 16384x16384 sRGBA8 image of uniform random bytes,
full 15-level chain (the reference's per-dispatch schedule F6 F6 F2), inputs
resident in HBM.  A step is one full chain.  value = microseconds per chain
for the whole job (lower is better).  The base level (1 GiB) is larger than
L2, so no flush is needed between steps of the headline loop.

Also reported (key "extra"): 4096^2, 4095^2, 4094^2, 1920x1080 and 2048^2
chains, L2-flushed and warm; the roofline of the dominant kernel; the CPU
baseline (a port of the reference's cpuGenerateMipmaps_sRGBA); an end-to-end
number with host buffers (H2D copy of the base level and D2H copy of the
generated levels inside the timed region).

--impl reference times the reference's CPU implementation of this path on
the host cores (its restatement in oracle/, since the reference itself cannot
be built on every host) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import socket
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

HEADLINE = (16384, 16384)
CONFIGS = [(4096, 4096), (4095, 4095), (4094, 4094), (1920, 1080), (2048, 2048),
           # the reference's other published sizes (1440p, 4k, the all-3x3 2047^2)
           (2560, 1440), (3840, 2160), (2047, 2047)]
L2_FLUSH_BYTES = 512 << 20


def algorithmic_bytes(w: int, h: int, bpp: int = 4, first: int = 0, last: int | None = None) -> int:
    """One read of level `first` plus one write of levels first+1..last."""
    from vk_compute_mipmaps_gb300.pyramid import level_sizes
    sizes = level_sizes(w, h)
    last = len(sizes) - 1 if last is None else last
    lw, lh = sizes[first]
    return bpp * (lw * lh + sum(a * b for a, b in sizes[first + 1:last + 1]))


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel_key: str):
    """Per-launch DRAM bytes of a kernel from the committed ncu summary, if any."""
    p = ROOT / "profiles" / "dram_traffic.json"
    if not p.exists():
        return None
    d = json.loads(p.read_text())
    return d.get(kernel_key)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during a timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        import torch
        try:
            u = str(torch.cuda.get_device_properties(device).uuid)
            self.gpu = u if u.startswith("GPU-") else f"GPU-{u}"
        except Exception:
            vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
            self.gpu = vis.split(",")[device.index or 0] if vis else str(device.index or 0)
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.proc or not self.file:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        rows = [r.split(",") for r in Path(self.file.name).read_text().splitlines() if r.strip()]
        os.unlink(self.file.name)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        sm, smax, reasons = [], [], set()
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except ValueError:
                continue
            for name, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# GPU side

def make_chain(w, h, dev, seed=1234):
    import torch
    import vk_compute_mipmaps_gb300 as V
    chain = V.MipChain(w, h, V.PRESET_SRGBA8, device=dev)
    g = torch.Generator(device=dev).manual_seed(seed)
    chain.storage[:chain.offsets[1]].copy_(
        torch.randint(0, 256, (chain.offsets[1],), generator=g, device=dev, dtype=torch.uint8))
    return chain


class Runner:
    """Records one chain's dispatches once per call and launches them on `stream`."""

    def __init__(self, chain, stream, mip_levels=0, flags=0):
        import vk_compute_mipmaps_gb300 as V
        self.V = V
        self.chain, self.stream, self.mips, self.flags = chain, stream, mip_levels, flags
        self.pipes = V.Pipelines(V.PRESET_SRGBA8)
        self.cmd = V.Cmd(flags)
        self.image = chain.image()

        self.lib = V._native.load()
        self.args = (self.cmd.handle, stream.cuda_stream, self.pipes.struct, ctypes.byref(self.image), mip_levels)

    def __call__(self):
        rc = self.lib.nvproPyramidGenerate(*self.args)
        if rc:
            self.V._native.check(rc, "nvproPyramidGenerate")
        return self.lib.nvproPyramidCmdLaunchCount(self.args[0])


CLOCK_WINDOW_S = 0.6


def keep_busy(fn, seconds):
    """Run `fn` back to back (untimed) for about `seconds` of wall time."""
    import torch
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        for _ in range(8):
            fn()
        torch.cuda.synchronize()


def time_loop(fn, stream, steps, warmup, flush=None):
    """Per-step device times (ms) with CUDA events on `stream`."""
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    times = []
    for _ in range(steps):
        if flush is not None:
            flush.zero_()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        fn()
        e.record(stream)
        times.append((s, e))
    torch.cuda.synchronize()
    return [s.elapsed_time(e) for s, e in times]


def bench_config(w, h, dev, stream, flush, steps, content="random"):
    chain = make_chain(w, h, dev)
    if content == "smooth":
        import torch
        from vk_compute_mipmaps_gb300.workloads import smooth_field
        base = torch.from_numpy(smooth_field(w, h, seed=w * 31 + h).reshape(-1))
        chain.storage[:chain.offsets[1]].copy_(base)
    run = Runner(chain, stream)
    with __import__("torch").cuda.stream(stream):
        cold = time_loop(run, stream, steps, 3, flush=flush)
        warm = time_loop(run, stream, steps, 3)
    nbytes = algorithmic_bytes(w, h)
    peak, _ = measured_peak()
    out = {}
    for name, ts in (("l2_flushed", cold), ("warm", warm)):
        us = statistics.median(ts) * 1e3
        out[name] = {"us_per_chain": round(us, 2), "us_min": round(min(ts) * 1e3, 2),
                     "GBps": round(nbytes / (us * 1e-6) / 1e9, 1),
                     "frac_of_hbm_peak": round(nbytes / (us * 1e-6) / 1e9 / peak, 4)}
    out["launches_per_chain"] = run()
    out["algorithmic_bytes"] = nbytes
    if w >= 2 and h >= 2:  # the speed-of-light probe on the same chain (the reference's "baseline")
        import vk_compute_mipmaps_gb300 as V
        img = chain.image()
        lib = V._native.load()
        probe = lambda: V._native.check(  # noqa: E731
            lib.nvproPyramidSpeedOfLightProbe(stream.cuda_stream, ctypes.byref(img), 0), "probe")
        with __import__("torch").cuda.stream(stream):
            pt = time_loop(probe, stream, steps, 3, flush=flush)
        out["probe_l2_flushed_us"] = round(statistics.median(pt) * 1e3, 2)
    del chain
    return out


def bench_premultiply(dev, stream, steps, w=16384, h=16384):
    """The premultiplied-alpha staging pass over a 16384^2 sRGBA8 image in
    place (1 GiB read + 1 GiB written; larger than L2), device-timed."""
    import torch
    import vk_compute_mipmaps_gb300 as V
    g = torch.Generator(device=dev).manual_seed(77)
    img = torch.randint(0, 256, (h, w, 4), generator=g, device=dev, dtype=torch.uint8)
    with torch.cuda.stream(stream):
        ts = time_loop(lambda: V.premultiply_alpha(img, stream=stream.cuda_stream), stream, steps, 3)
    us = statistics.median(ts) * 1e3
    nbytes = 2 * w * h * 4
    peak, _ = measured_peak()
    del img
    torch.cuda.empty_cache()
    return {"image": f"{w}x{h}", "us": round(us, 1), "GBps": round(nbytes / (us * 1e-6) / 1e9, 1),
            "frac_of_hbm_peak": round(nbytes / (us * 1e-6) / 1e9 / peak, 4), "bytes": nbytes}


def bench_batch(dev, stream, flush, steps, rank=0, world=1):
    """256 sRGBA8 images (sides log-uniform in [17, 4096], aspect in [1/4, 4],
    seed 2024) in one buffer: one batch launch (autotuned, CUDA graph) against
    256 per-image nvproPyramidGenerate calls, both device-timed, L2 flushed.
    With several ranks the 256 images are split by image (shard_by_image):
    each rank launches a batch of its share, and the job's time is the max
    over ranks (no data is exchanged)."""
    import torch
    import vk_compute_mipmaps_gb300 as V
    from vk_compute_mipmaps_gb300.workloads import batch_sizes, chain_bytes, shard_by_image
    peak, _ = measured_peak()
    all_sizes = batch_sizes(256)
    sizes = [all_sizes[i] for i in shard_by_image(all_sizes, rank, world)]
    storage, chains = V.pack_chains(sizes, device=dev)
    g = torch.Generator(device=dev).manual_seed(2024)
    storage.copy_(torch.randint(0, 256, (storage.numel(),), generator=g, device=dev, dtype=torch.uint8))
    nbytes = sum(chain_bytes(w, h) for w, h in all_sizes)
    with torch.cuda.stream(stream):
        batch = V.Batch(V.BATCH_AUTOTUNE | V.BATCH_GRAPH)
        batch.build(chains, stream=stream.cuda_stream)
        barrier(world)
        tb = time_loop(lambda: batch.launch(stream.cuda_stream), stream, steps, 3, flush=flush)
        barrier(world)
        tp = time_loop(lambda: [V.generate(c, stream=stream.cuda_stream) for c in chains], stream,
                       max(3, steps // 4), 3, flush=flush)
    b_us = max_over_ranks(statistics.median(tb) * 1e3, world)
    p_us = max_over_ranks(statistics.median(tp) * 1e3, world)
    sizes = all_sizes
    info = batch.info()
    batch.close()
    del storage, chains
    torch.cuda.empty_cache()
    return {"images": len(sizes), "batch_us": round(b_us, 1), "plain_us": round(p_us, 1),
            "batch_images_per_s": round(len(sizes) / (b_us * 1e-6), 1),
            "plain_images_per_s": round(len(sizes) / (p_us * 1e-6), 1),
            "speedup_vs_plain": round(p_us / b_us, 3), "algorithmic_bytes": nbytes,
            "batch_frac_of_hbm_peak": round(nbytes / (b_us * 1e-6) / 1e9 / peak, 4),
            "phases": info["phaseCount"], "jobs": info["jobCount"], "strip_band": info["stripBand"],
            "fast_region_rows": info["fastRegionRows"], "threads_per_cta": info["threadsPerCta"],
            "tuning": "autotuned" + (" (cached)" if info["fromCache"] else " (timed at build)"),
            "launches_per_batch": 1, "ranks": world,
            "split": "by image across ranks, max of the ranks' times" if world > 1 else "one GPU"}


def level_errors_fp64(levels, base):
    """Per-level max |error| / max |FP64 value| of a power-of-two float
    pyramid, against FP64 block means of the base (the fast pipeline's 2x2
    box in exact arithmetic: level k is the mean of each 2^k x 2^k block)."""
    import torch
    errs = []
    b = base[0].double() if base.dim() == 4 else base.double()
    H, W = b.shape[0], b.shape[1]
    for k, lv in enumerate(levels, start=1):
        s = 1 << k
        hk, wk = max(H >> k, 1), max(W >> k, 1)
        ref = torch.zeros((hk, wk, 4), dtype=torch.float64, device=b.device)
        rows = max(1, (1 << 22) // (W * s))  # a few M texels of the base at a time
        for r0 in range(0, hk, rows):
            r1 = min(hk, r0 + rows)
            blk = b[r0 * s:r1 * s].reshape(r1 - r0, s, wk, s, 4)
            ref[r0:r1] = blk.mean(dim=(1, 3))
        got = (lv[0] if lv.dim() == 4 else lv).double()
        errs.append(float((got - ref).abs().max() / ref.abs().max()))
        del ref
    return errs


def bench_float_adjoint(dev, stream, flush, steps):
    """Linear float pyramids (RGBA32F, RGBA16F storage with FP32 arithmetic).

    * 8 x 2048^2 x 4 FP32, uniform [0, 1): forward, and forward + backward
      through the torch.autograd.Function with N(0, 1) upstream gradients on
      every level;
    * 1023 x 777 x 4 FP32 (three-tap kernels on every level): forward + backward;
    * 16384^2 x 4 FP32 and FP16, log-normal(0, 1): forward and the adjoint
      with N(0, 1) gradients on all 15 levels, %HBM, and the forward's
      per-level error against FP64.
    Algorithmic bytes: forward = base read + levels written; adjoint =
    upstream gradients read + base gradient written."""
    import torch
    from vk_compute_mipmaps_gb300 import autograd as A
    from vk_compute_mipmaps_gb300.pyramid import level_sizes
    peak, _ = measured_peak()
    out = {}
    g = torch.Generator(device=dev).manual_seed(11)

    def fwd_bwd_autograd(B, H, W):
        base = torch.rand((B, H, W, 4), generator=g, device=dev).requires_grad_(True)
        ups = [torch.randn((B, h, w, 4), generator=g, device=dev) for w, h in level_sizes(W, H)]

        def fwd():
            with torch.no_grad():
                A.pyramid(base)

        def both_outputs():  # upstream gradients on the Function's outputs, levels 1..n-1
            base.grad = None
            torch.autograd.backward(A.pyramid(base), ups[1:])

        def both_all():  # on every level 0..n-1: level 0 is an alias of the base (with_base)
            base.grad = None
            torch.autograd.backward(A.pyramid(base, with_base=True), ups)

        # the same work through the C ABI directly (one strided call each way, no autograd engine)
        det = base.detach()

        def fwd_c():
            A.forward_levels(det)

        def both_c():
            A.forward_levels(det)
            A.adjoint([None] + ups[1:], (B, H, W, 4), torch.float32, dev)

        with torch.cuda.stream(stream):
            tf = time_loop(fwd, stream, steps, 3, flush=flush)
            to = time_loop(both_outputs, stream, steps, 3, flush=flush)
            ta = time_loop(both_all, stream, steps, 3, flush=flush)
            tfc = time_loop(fwd_c, stream, steps, 3, flush=flush)
            tbc = time_loop(both_c, stream, steps, 3, flush=flush)
            # the same autograd steps captured in CUDA graphs (the usual cure for
            # a host-bound training step): replays carry no host work
            gf, gb = torch.cuda.CUDAGraph(), torch.cuda.CUDAGraph()
            with torch.cuda.graph(gf, stream=stream):
                fwd()
            base.grad = None
            with torch.cuda.graph(gb, stream=stream):
                torch.autograd.backward(A.pyramid(base), ups[1:])
            tgf = time_loop(gf.replay, stream, steps, 3, flush=flush)
            tgb = time_loop(gb.replay, stream, steps, 3, flush=flush)
            del gf, gb
            base.grad = None
        f_us, o_us, a_us = (statistics.median(t) * 1e3 for t in (tf, to, ta))
        fc_us, bc_us = statistics.median(tfc) * 1e3, statistics.median(tbc) * 1e3
        gf_us, gb_us = statistics.median(tgf) * 1e3, statistics.median(tgb) * 1e3
        res = {"forward_us": round(f_us, 2),
               "fwd_plus_bwd_us": round(o_us, 2), "fwd_plus_bwd_over_fwd": round(o_us / f_us, 3),
               "fwd_plus_bwd_all_levels_us": round(a_us, 2),
               "fwd_plus_bwd_all_levels_over_fwd": round(a_us / f_us, 3),
               "c_abi_forward_us": round(fc_us, 2), "c_abi_fwd_plus_bwd_us": round(bc_us, 2),
               "c_abi_fwd_plus_bwd_over_fwd": round(bc_us / fc_us, 3),
               "graphed_forward_us": round(gf_us, 2), "graphed_fwd_plus_bwd_us": round(gb_us, 2),
               "graphed_fwd_plus_bwd_over_fwd": round(gb_us / gf_us, 3),
               "path": "torch.autograd.Function (one strided launch per dispatch each way); c_abi_*: the "
                       "same strided calls without the autograd engine; graphed_*: the autograd steps "
                       "captured in a CUDA graph and replayed",
               "note": "all_levels adds N(0,1) on level 0: the backward then reads the level-0 gradient "
                       "too, 1.75x the forward's bytes"}
        return res

    out["fp32_8x2048x2048"] = fwd_bwd_autograd(8, 2048, 2048)
    out["fp32_1023x777"] = fwd_bwd_autograd(1, 777, 1023)

    for name, dt in (("fp32_16384x16384", torch.float32), ("fp16_16384x16384", torch.float16)):
        S = 16384
        base = torch.empty((1, S, S, 4), device=dev).log_normal_(0.0, 1.0, generator=g).to(dt)
        sizes = level_sizes(S, S)
        ups = [torch.randn((1, h, w, 4), generator=g, device=dev).to(dt) for w, h in sizes]
        esz = base.element_size() * 4
        base_bytes = S * S * esz
        lvl_bytes = sum(w * h for w, h in sizes[1:]) * esz
        with torch.cuda.stream(stream):
            tf = time_loop(lambda: A.forward_levels(base), stream, steps, 3, flush=flush)
            tb = time_loop(lambda: A.adjoint(ups, tuple(base.shape), dt, dev), stream, steps, 3, flush=flush)
        f_us, b_us = statistics.median(tf) * 1e3, statistics.median(tb) * 1e3
        f_bytes = base_bytes + lvl_bytes
        b_bytes = base_bytes + lvl_bytes + base_bytes  # all 15 upstream levels read, base gradient written
        levels = A.forward_levels(base)
        torch.cuda.synchronize()
        errs = level_errors_fp64(levels, base)
        out[name] = {"forward_us": round(f_us, 2), "adjoint_us": round(b_us, 2),
                     "forward_frac_of_hbm_peak": round(f_bytes / (f_us * 1e-6) / 1e9 / peak, 4),
                     "adjoint_frac_of_hbm_peak": round(b_bytes / (b_us * 1e-6) / 1e9 / peak, 4),
                     "forward_algorithmic_bytes": f_bytes, "adjoint_algorithmic_bytes": b_bytes,
                     "values": "log-normal(0, 1)",
                     "forward_max_rel_err_vs_fp64_per_level": [float(f"{e:.3g}") for e in errs]}
        del base, ups, levels
        torch.cuda.empty_cache()
    return out


def cpu_baseline_sample(threads: int, reps: int = 1):
    """The restated reference CPU generator on `threads` host threads, one
    4096^2 image per thread (as the reference benchmark runs one image per
    thread, demo_app/mipmaps_app.cpp:642-654).  Returns us per 16384^2-chain
    equivalent (16 x 4096^2 = the 16384^2 base in texels)."""
    import numpy as np
    sys.path.insert(0, str(ROOT / "tests"))
    import _oracle as O
    w = h = 4096
    bases = [np.random.default_rng(i).integers(0, 256, (h, w, 4), dtype=np.uint8) for i in range(threads)]
    bufs = [O.packed_from_base(1, b) for b in bases]
    lib = O.orc()

    def work(buf):
        for _ in range(reps):
            lib.orc_refcpu_srgba8(w, h, buf.ctypes.data_as(O.POINTER(O.c_uint8)))

    t0 = time.perf_counter()
    ths = [threading.Thread(target=work, args=(b,)) for b in bufs]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    dt = time.perf_counter() - t0
    chains_4096 = threads * reps
    scale = algorithmic_bytes(*HEADLINE) / algorithmic_bytes(w, h)
    us_per_16384 = dt / chains_4096 * scale * 1e6
    return us_per_16384, dt, f"{chains_4096} x 4096^2 chains on {threads} threads ({dt:.2f} s), scaled by bytes"


def cpu_detail_sample(threads: int):
    """The CPU figures beside the headline baseline: one 4096^2 chain on one
    thread with the restated reference generator and with the oracle (shader
    semantics, reference schedule), and the 256-image benchmark batch over
    `threads` threads (one image per thread at a time, as the reference
    benchmark hands out images)."""
    import numpy as np
    sys.path.insert(0, str(ROOT / "tests"))
    import _oracle as O
    from vk_compute_mipmaps_gb300.workloads import batch_sizes
    lib = O.orc()
    base = np.random.default_rng(0).integers(0, 256, (4096, 4096, 4), dtype=np.uint8)
    buf = O.packed_from_base(1, base)
    t0 = time.perf_counter()
    lib.orc_refcpu_srgba8(4096, 4096, buf.ctypes.data_as(O.POINTER(O.c_uint8)))
    ref_1t = time.perf_counter() - t0
    buf = O.packed_from_base(1, base)
    t0 = time.perf_counter()
    O.run(1, 4096, 4096, buf)
    orc_1t = time.perf_counter() - t0
    sizes = batch_sizes(256)
    rng = np.random.default_rng(2024)
    bufs = [O.packed_from_base(1, rng.integers(0, 256, (h, w, 4), dtype=np.uint8)) for w, h in sizes]
    order = sorted(range(len(sizes)), key=lambda i: -sizes[i][0] * sizes[i][1])  # largest first
    lock = threading.Lock()

    def work():
        while True:
            with lock:
                if not order:
                    return
                i = order.pop(0)
            w, h = sizes[i]
            lib.orc_refcpu_srgba8(w, h, bufs[i].ctypes.data_as(O.POINTER(O.c_uint8)))

    t0 = time.perf_counter()
    ths = [threading.Thread(target=work) for _ in range(threads)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    batch_s = time.perf_counter() - t0
    return {"single_thread_us_per_4096_chain": round(ref_1t * 1e6, 1),
            "oracle_single_thread_us_per_4096_chain": round(orc_1t * 1e6, 1),
            "batch_256_images_per_s": round(len(sizes) / batch_s, 1), "batch_256_threads": threads}


def run_ours(args, rank, world):
    import torch
    import vk_compute_mipmaps_gb300 as V
    local = int(os.environ.get("LOCAL_RANK", 0))
    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(dev)
    peak, peak_kind = measured_peak()
    w, h = map(int, args.image.lower().split("x"))

    chain = make_chain(w, h, dev)
    levels = len(chain.offsets) - 1
    run = Runner(chain, stream)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            run()
        torch.cuda.synchronize()
        launches = 0
        # nvidia-smi samples every 100 ms, longer than the timed steps take:
        # the sampler runs over untimed chains for CLOCK_WINDOW_S before and
        # after the timed steps, the same load, so the clocks are those the
        # timed steps ran at.
        with ClockSampler(dev) as clk:
            keep_busy(run, CLOCK_WINDOW_S)
            barrier(world)
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            for _ in range(args.steps):
                launches += run()
            e.record(stream)
            torch.cuda.synchronize()
            keep_busy(run, CLOCK_WINDOW_S)
        ms = s.elapsed_time(e)
    ms = max_over_ranks(ms, world)
    ms_per_step = ms / args.steps
    us_per_chain = ms_per_step * 1e3 / world  # whole job: world chains per step
    chain_bytes = algorithmic_bytes(w, h)

    # Dominant kernel: the first launch of the chain.  If the chain is one
    # launch (tail fused), that launch is the chain; otherwise time the first
    # dispatch alone (mipLevels = 7: the F6 over level 0).
    launches_per_chain = run()
    if launches_per_chain == 1:
        kruns, kbytes, kname = run, chain_bytes, "fast_tma_f6_fused_tail"
    else:
        kruns = Runner(chain, stream, mip_levels=7)
        kbytes, kname = algorithmic_bytes(w, h, last=6), "fast_f6_level0"
    with torch.cuda.stream(stream):
        kt = time_loop(kruns, stream, max(20, min(args.steps, 200)), 3)
    k_ms = statistics.mean(kt)
    achieved = kbytes / (k_ms * 1e-3) / 1e9
    traffic = ncu_traffic(kname)

    extra = {"chain_GBps": round(chain_bytes / (ms_per_step * 1e-3) / 1e9, 1),
             "chain_frac_of_hbm_peak": round(chain_bytes / (ms_per_step * 1e-3) / 1e9 / peak, 4),
             "chain_algorithmic_bytes": chain_bytes, "launches_per_chain": launches_per_chain}
    # Speed-of-light probe: one launch with the chain's traffic and no
    # filtering (levels 1.. get non-pyramid values; the base is untouched).
    img = chain.image()
    probe = lambda: V._native.check(  # noqa: E731
        V._native.load().nvproPyramidSpeedOfLightProbe(stream.cuda_stream, ctypes.byref(img), 0), "probe")
    with torch.cuda.stream(stream):
        pt = time_loop(probe, stream, max(20, min(args.steps, 200)), 3)
    probe_us = statistics.mean(pt) * 1e3
    extra["speed_of_light_probe"] = {
        "us": round(probe_us, 2), "frac_of_hbm_peak": round(chain_bytes / (probe_us * 1e-6) / 1e9 / peak, 4),
        "chain_over_probe": round(us_per_chain / probe_us, 3)}
    e2e = None
    cpu = None
    if rank == 0 and not args.no_e2e:
        # End to end through the public API with host buffers.
        base_host = torch.empty(chain.offsets[1], dtype=torch.uint8, pin_memory=True)
        base_host.copy_(chain.storage[:chain.offsets[1]])
        out_host = torch.empty(chain.offsets[-1] - chain.offsets[1], dtype=torch.uint8, pin_memory=True)

        def e2e_step():  # the public host-memory entry point: banded copies overlapped with the chain
            V.generate_from_host(chain, base_host, out_host, stream=stream.cuda_stream)

        n_e2e = max(3, min(args.steps, 20))
        with torch.cuda.stream(stream):
            et = time_loop(e2e_step, stream, n_e2e, 2)
        e2e_us = statistics.mean(et) * 1e3
        e2e = {"value": round(e2e_us, 2), "unit": "us", "h2d_bytes_per_step": base_host.numel(),
               "d2h_bytes_per_step": out_host.numel(), "steps": n_e2e}
        del base_host, out_host
    if not args.no_extra:  # every rank: its share of the batch
        flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
        del chain
        torch.cuda.empty_cache()
        extra["batch_256"] = bench_batch(dev, stream, flush, max(5, min(args.steps, 20)), rank, world)
    if rank == 0:
        if not args.no_extra:
            for cw, ch in CONFIGS:
                # 2048^2: uniform random bytes; the others: a smooth seeded field with radial alpha
                content = "random" if (cw, ch) == (2048, 2048) else "smooth"
                extra[f"{cw}x{ch}"] = bench_config(cw, ch, dev, stream, flush, max(10, min(args.steps, 100)),
                                                   content)
                extra[f"{cw}x{ch}"]["content"] = content
            extra["premultiply_staging"] = bench_premultiply(dev, stream, max(5, min(args.steps, 20)))
            extra["float_adjoint"] = bench_float_adjoint(dev, stream, flush, max(5, min(args.steps, 20)))
            del flush
        if not args.no_cpu:
            threads = os.cpu_count() or 1
            us, dt, sample = cpu_baseline_sample(threads)
            cpu = {"value": round(us, 1), "unit": "us per 16384^2 chain", "cores": threads, "kind": "port",
                   "sample": sample}
            cpu.update(cpu_detail_sample(threads))

    line = {
        "metric": f"srgba8_{w}x{h}_full_chain_us",
        "value": round(us_per_chain, 2),
        "unit": "us",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_per_step, 5),
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u8",
        "data": "synthetic: uniform random bytes (torch.Generator seed 1234)",
        "config": headline_config(w, h, levels, world),
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
                     "algorithmic_bytes_per_launch": kbytes, "launch_us": round(k_ms * 1e3, 2),
                     "peak_kind": peak_kind},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "extra": extra,
    }
    if rank == 0:
        print(json.dumps(line))


def headline_config(w, h, levels, world):
    """The `config` of the bench line, the same for both arms."""
    return {"workload": f"sRGBA8 {w}x{h} full chain, reference dispatch schedule",
            "image": f"{w}x{h}", "preset": "srgba8", "levels": levels,
            "l2": "inputs larger than L2 (1 GiB base level)",
            "parallelism": f"replicas x{world}"}


def run_reference(args, rank, world):
    """The reference's CPU generator (restated in oracle/) on all host cores."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_baseline_sample(threads)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        us, dt, sample = cpu_baseline_sample(threads)
        vals.append(us)
    total = time.perf_counter() - t0
    v = statistics.mean(vals)
    line = {
        "impl": "reference",
        "metric": "srgba8_16384x16384_full_chain_us",
        "value": round(v, 1),
        "unit": "us",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(total / args.steps * 1e3, 3),
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u8",
        "data": "synthetic: uniform random bytes",
        "config": headline_config(*HEADLINE, 15, world),
        "cpu_baseline": {"value": round(v, 1), "unit": "us", "cores": threads, "kind": "port",
                         "sample": sample + "; cpuGenerateMipmaps_sRGBA restated (oracle/pyr_oracle.cpp), "
                                            "bit-exact to the reference build"},
        "e2e": {"value": round(v, 1), "unit": "us", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_profile(spec: str, reps: int):
    """Run one workload `reps` times on cuda:0 without timing (for profilers)."""
    import torch
    import vk_compute_mipmaps_gb300 as V
    dev = torch.device("cuda:0")
    if spec == "batch256":
        from vk_compute_mipmaps_gb300.workloads import batch_sizes
        storage, chains = V.pack_chains(batch_sizes(256), device=dev)
        g = torch.Generator(device=dev).manual_seed(2024)
        storage.copy_(torch.randint(0, 256, (storage.numel(),), generator=g, device=dev, dtype=torch.uint8))
        batch = V.Batch(0)
        batch.build(chains)
        for _ in range(reps):
            batch.launch()
        torch.cuda.synchronize()
        batch.device_status()
    elif spec.startswith("chain:"):
        parts = spec.split(":")
        w, h = map(int, parts[1].lower().split("x"))
        mips = int(parts[2]) if len(parts) > 2 else 0
        chain = make_chain(w, h, dev)
        for _ in range(reps):
            V.generate(chain, mip_levels=mips)
        torch.cuda.synchronize()
    elif spec.startswith("adjoint:"):
        from vk_compute_mipmaps_gb300 import autograd as A
        from vk_compute_mipmaps_gb300.pyramid import level_sizes
        _, size, dtype = spec.split(":")
        w, h = map(int, size.lower().split("x"))
        dt = {"fp32": torch.float32, "fp16": torch.float16}[dtype]
        g = torch.Generator(device=dev).manual_seed(11)
        ups = [torch.randn((1, lh, lw, 4), generator=g, device=dev).to(dt) for lw, lh in level_sizes(w, h)]
        for _ in range(reps):
            A.adjoint(ups, (1, h, w, 4), dt, dev)
        torch.cuda.synchronize()
    elif spec.startswith("premultiply:"):
        w, h = map(int, spec.split(":")[1].lower().split("x"))
        img = torch.randint(0, 256, (h, w, 4), generator=torch.Generator(device=dev).manual_seed(77), device=dev,
                            dtype=torch.uint8)
        for _ in range(reps):
            V.premultiply_alpha(img)
        torch.cuda.synchronize()
    else:
        raise SystemExit(f"unknown --profile workload {spec!r}")
    print(f"profile workload {spec}: {reps} runs done")


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-extra", action="store_true", help="skip the other image sizes")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end (host buffer) measurement")
    ap.add_argument("--image", default="16384x16384", help="headline image WxH (smaller for profiling runs)")
    ap.add_argument("--profile", default=None,
                    help="run one workload --steps times and exit (for ncu): chain:WxH[:mipLevels], batch256 "
                         "or adjoint:WxH:fp32|fp16")
    args = ap.parse_args(argv)
    if args.profile:
        run_profile(args.profile, args.steps)
        return
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # No launcher: start one rank per GPU (replicas, see run_ours) the way
        # the multi-GPU contract does, on this host.
        with socket.socket() as sk:
            sk.bind(("127.0.0.1", 0))
            port = sk.getsockname()[1]
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
               "--master-addr", "127.0.0.1", f"--master-port={port}", str(Path(__file__).resolve()),
               *(sys.argv[1:] if argv is None else argv)]
        raise SystemExit(subprocess.call(cmd))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "gloo" if args.impl == "reference" else "nccl"
        dist.init_process_group(backend)
    try:
        if args.impl == "reference":
            run_reference(args, rank, world)
        else:
            run_ours(args, rank, world)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
