"""Batches (nvproPyramidBatch*): one persistent launch for many sRGBA8 images
of any sizes; the bytes of every image equal a per-image
nvproPyramidGenerate, and the oracle's for small images."""
from pathlib import Path

import numpy as np
import pytest

import _oracle as O
from vk_compute_mipmaps_gb300 import _native as N
from vk_compute_mipmaps_gb300 import pyramid as P
from vk_compute_mipmaps_gb300.workloads import batch_sizes

pytestmark = pytest.mark.gpu

SENTINEL = 0xA7

# every schedule shape: 1xN, Nx1, odd/even mixes (all strip variants), fast
# dispatches of 1..6 levels, the fast pipeline re-entering (2052), tiny levels
MIXED = [(1, 1), (2, 1), (1, 2), (1, 37), (37, 1), (3, 3), (4, 4), (5, 7), (8, 8), (17, 17), (17, 33), (33, 17),
         (64, 64), (65, 63), (96, 40), (127, 129), (128, 128), (256, 255), (300, 201), (301, 202), (302, 203),
         (303, 200), (640, 384), (513, 512), (1000, 3), (3, 1000), (1920, 1080), (2052, 2052), (1023, 777),
         (4096, 64), (4095, 63), (2047, 2049)]


def fill_random(chains, seed):
    import torch
    g = torch.Generator(device=chains[0].storage.device).manual_seed(seed)
    for c in chains:
        c.storage.fill_(SENTINEL)
        n = c.offsets[1]
        c.storage[:n].copy_(torch.randint(0, 256, (n,), generator=g, device=c.storage.device, dtype=torch.uint8))


def per_image_reference(chains):
    """Each chain generated alone by nvproPyramidGenerate on a copy."""
    import torch
    out = []
    for c in chains:
        ref = P.MipChain(c.width, c.height, N.PRESET_SRGBA8, device=c.storage.device,
                         storage=c.storage.clone())
        P.generate(ref)
        out.append(ref)
    torch.cuda.synchronize()
    return out


def check_equal(chains, refs):
    import torch
    for c, r in zip(chains, refs):
        if not torch.equal(c.storage, r.storage):
            for k in range(1, c.levels):
                a, b = c.level(k), r.level(k)
                if not torch.equal(a, b):
                    bad = (a != b).any(-1).nonzero()
                    y, x = bad[0].tolist()
                    raise AssertionError(f"{c.width}x{c.height} level {k}: {bad.shape[0]} texels differ, first "
                                         f"({x}, {y}) got {a[y, x].tolist()} want {b[y, x].tolist()}")


@pytest.mark.parametrize("flags", [0, N.BATCH_GRAPH])
def test_batch_mixed_sizes_equal_per_image(cuda, flags):
    import torch
    _, chains = P.pack_chains(MIXED, device=cuda)
    fill_random(chains, 11)
    refs = per_image_reference(chains)
    b = P.Batch(flags)
    b.build(chains)
    for _ in range(2):  # a second launch rewrites the same bytes
        b.launch()
        torch.cuda.synchronize()
        check_equal(chains, refs)
    b.device_status()
    info = b.info()
    assert info["imageCount"] == len(MIXED) and info["graph"] == (1 if flags else 0)
    assert info["phaseCount"] == max(len(O.default_schedule(w, h)) for w, h in MIXED)


def test_batch_small_images_equal_oracle(cuda):
    import torch
    sizes = [(w, h) for w, h in MIXED if w * h <= 300 * 300]
    _, chains = P.pack_chains(sizes, device=cuda)
    fill_random(chains, 12)
    b = P.Batch()
    b.build(chains)
    b.launch()
    torch.cuda.synchronize()
    for c in chains:
        base = c.level(0).cpu().numpy()
        mips = c.levels
        off = O.offsets(c.width, c.height, mips, 4)
        want = np.full(off[-1], SENTINEL, np.uint8)
        want[:off[1]] = base.reshape(-1)
        O.run(N.PRESET_SRGBA8, c.width, c.height, want, None, mips)
        assert np.array_equal(c.storage.cpu().numpy(), want), f"{c.width}x{c.height}"


def test_batch_256_synthetic_equal_per_image(cuda):
    """The benchmark's batch: 256 images, sides log-uniform in [17, 4096]."""
    import torch
    _, chains = P.pack_chains(batch_sizes(256), device=cuda)
    fill_random(chains, 13)
    refs = per_image_reference(chains)
    b = P.Batch(N.BATCH_GRAPH)
    b.build(chains)
    b.launch()
    torch.cuda.synchronize()
    check_equal(chains, refs)
    b.device_status()


@pytest.mark.parametrize("band,rows,threads", [(4, 16, 256), (32, 32, 384), (8, 64, 256), (16, 16, 384)])
def test_batch_shapes_equal_per_image(cuda, band, rows, threads):
    """Every launch shape the autotuner can choose (strip band, fast-region
    rows, threads per CTA) writes the bytes of per-image generation."""
    import torch
    _, chains = P.pack_chains(MIXED, device=cuda)
    fill_random(chains, 21)
    refs = per_image_reference(chains)
    b = P.Batch()
    b.set_tuning(band, rows, threads)
    b.build(chains)
    info = b.info()
    assert (info["stripBand"], info["fastRegionRows"], info["threadsPerCta"]) == (band, rows, threads)
    b.launch()
    torch.cuda.synchronize()
    check_equal(chains, refs)
    b.device_status()


_SECOND_PROCESS = """
import json, sys
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[1] + "/tests")
import torch
from vk_compute_mipmaps_gb300 import _native as N
from vk_compute_mipmaps_gb300 import pyramid as P
from vk_compute_mipmaps_gb300.workloads import batch_sizes
import test_batch_gpu as T
_, chains = P.pack_chains(batch_sizes(24, seed=5, hi=1024), device="cuda")
T.fill_random(chains, 15)
refs = T.per_image_reference(chains)
b = P.Batch(N.BATCH_AUTOTUNE)
b.build(chains)
b.launch()
torch.cuda.synchronize()
T.check_equal(chains, refs)
print(json.dumps(b.info()))
"""


def test_batch_autotune_cached_per_size_class(cuda, repo_tmp, monkeypatch):
    """The autotuner times its candidates once per size class; later builds
    of the class take the cached shape from memory, and a new process takes
    it from the cache file without timing -- all writing per-image bytes."""
    import json
    import subprocess
    import sys

    import torch
    monkeypatch.setenv("NVPRO_PYRAMID_CACHE_DIR", str(repo_tmp))
    sizes = batch_sizes(24, seed=5, hi=1024)
    _, chains = P.pack_chains(sizes, device=cuda)
    fill_random(chains, 14)
    refs = per_image_reference(chains)
    b1 = P.Batch(N.BATCH_AUTOTUNE | N.BATCH_RETUNE)
    b1.build(chains)
    i1 = b1.info()
    assert i1["autotuned"] == 1 and i1["fromCache"] == 0
    assert i1["stripBand"] in (4, 8, 16, 32) and i1["fastRegionRows"] in (16, 32, 64)
    assert i1["threadsPerCta"] in (256, 384)
    b1.launch()
    torch.cuda.synchronize()
    check_equal(chains, refs)
    b2 = P.Batch(N.BATCH_AUTOTUNE | N.BATCH_GRAPH)
    b2.build(chains)  # same size class: the cached choice, no timing
    i2 = b2.info()
    shape = ("stripBand", "fastRegionRows", "threadsPerCta")
    assert i2["fromCache"] == 1 and i2["fromDisk"] == 0 and all(i2[k] == i1[k] for k in shape)
    lines = (repo_tmp / "batch_tuning.txt").read_text().splitlines()
    # "<size class> <strip band> <fast-region rows> <warps per CTA>"
    assert lines and lines[-1].split()[1:] == [str(i1["stripBand"]), str(i1["fastRegionRows"]),
                                               str(i1["threadsPerCta"] // 32)]
    res = subprocess.run([sys.executable, "-c", _SECOND_PROCESS, str(Path(__file__).resolve().parents[1])],
                         capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-3000:]
    i3 = json.loads(res.stdout.strip().splitlines()[-1])
    assert i3["fromDisk"] == 1 and i3["fromCache"] == 1 and all(i3[k] == i1[k] for k in shape)


def test_batch_empty_and_errors(cuda, native):
    import ctypes
    b = P.Batch()
    b.build([])
    b.launch()
    assert b.info()["phaseCount"] == 0
    h = ctypes.c_void_p()
    assert native.nvproPyramidCreateBatch(N.PRESET_RGBA32F, 0, ctypes.byref(h)) == N.ERROR_UNSUPPORTED
    assert native.nvproPyramidCreateBatch(N.PRESET_SRGBA8, 0x100, ctypes.byref(h)) == N.ERROR_INVALID_ARGUMENT
    b2 = P.Batch()
    assert native.nvproPyramidBatchLaunch(b2.handle, None) == N.ERROR_INVALID_STATE
