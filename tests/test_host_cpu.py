"""Host-side logic without a GPU: the bench's multi-rank helpers as two gloo
ranks, the synthetic batch workload, and the adjoint workspace rule."""
import ctypes
import os
import socket

import numpy as np
import pytest

import _oracle as O
from vk_compute_mipmaps_gb300 import pyramid as P
from vk_compute_mipmaps_gb300.workloads import batch_sizes, chain_bytes


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(world)
        out[rank] = bench.max_over_ranks(1.5 + rank * 10.0, world)
        bench.barrier(world)
    finally:
        dist.destroy_process_group()


def test_bench_rank_helpers_gloo_world_2():
    """Each rank times its own replica; the job's time is the max over ranks."""
    import torch.multiprocessing as mp
    world, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        assert dict(out) == {0: 11.5, 1: 11.5}


def _shard_rank_main(rank, world, port, out):
    import hashlib

    import torch.distributed as dist

    from vk_compute_mipmaps_gb300.workloads import shard_by_image
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sizes = batch_sizes(24, seed=9, lo=3, hi=96)
        rng = np.random.default_rng(31)
        bases = [rng.integers(0, 256, (h, w, 4), dtype=np.uint8) for w, h in sizes]

        def digest(i):  # the pyramid of image i (the oracle stands in for a GPU)
            return hashlib.sha256(O.pyramid(1, bases[i]).tobytes()).hexdigest()

        mine = shard_by_image(sizes, rank, world)
        gathered = [None] * world
        dist.all_gather_object(gathered, {i: digest(i) for i in mine})
        if rank == 0:
            out["shares"] = [sorted(g) for g in gathered]
            out["merged"] = {k: v for g in gathered for k, v in g.items()}
            out["single"] = {i: digest(i) for i in range(len(sizes))}
            out["bytes"] = [sum(chain_bytes(*sizes[i]) for i in g) for g in gathered]
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_batch_split_by_image_gloo_world_2():
    """Two ranks split a batch by image with no exchange: the shares are
    disjoint, cover every image, carry about the same bytes, and each rank's
    pyramids equal those of one process generating the whole batch."""
    import torch.multiprocessing as mp
    world, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_shard_rank_main, args=(world, port, out), nprocs=world, join=True)
        shares = out["shares"]
        assert sorted(shares[0] + shares[1]) == list(range(24)) and not set(shares[0]) & set(shares[1])
        assert out["merged"] == out["single"]
        b0, b1 = out["bytes"]
        assert abs(b0 - b1) <= max(b0, b1) * 0.25


def test_bench_gpus_flag_launches_ranks():
    """`bench.py --gpus 2` without a launcher starts two ranks itself; the
    CPU reference arm then prints one line with n_gpus 2 from rank 0."""
    import json
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    res = subprocess.run([sys.executable, str(root / "bench.py"), "--impl", "reference", "--gpus", "2",
                          "--steps", "1", "--warmup", "0"], capture_output=True, text=True, env=env, timeout=600,
                         cwd=root)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [json.loads(ln) for ln in res.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, res.stdout
    assert lines[0]["n_gpus"] == 2 and lines[0]["impl"] == "reference"
    # the reference arm reports the GPU arm's workload: same metric and config
    sys.path.insert(0, str(root))
    import bench
    assert lines[0]["metric"] == f"srgba8_{bench.HEADLINE[0]}x{bench.HEADLINE[1]}_full_chain_us"
    assert lines[0]["config"] == bench.headline_config(*bench.HEADLINE, 15, 2)
    assert lines[0]["higher_is_better"] is False and lines[0]["unit"] == "us"


def test_batch_workload_is_seeded_and_mixed():
    a, b = batch_sizes(256), batch_sizes(256)
    assert a == b and len(a) == 256
    w = np.array([s[0] for s in a])
    h = np.array([s[1] for s in a])
    assert w.max() <= 4096 and h.max() <= 4096 and min(w.min(), h.min()) >= 1
    side = np.sqrt(w * h)
    assert side.min() >= 8 and side.max() <= 4096
    assert 0.3 < np.mean(w % 2) < 0.7 and 0.3 < np.mean(h % 2) < 0.7  # about half odd
    assert np.mean((w % 4 == 0) & (h % 4 == 0)) < 0.2  # most chains start with a general dispatch
    assert batch_sizes(16, seed=3) != batch_sizes(16, seed=4)


@pytest.mark.parametrize("w,h", [(1, 1), (17, 33), (640, 384), (4095, 4095), (2052, 2052)])
def test_chain_bytes_matches_packed_layout(w, h):
    assert chain_bytes(w, h) == O.offsets(w, h, O.full_levels(w, h), 4)[-1]


def _workspace_rule(w, h, mips=0):
    """Bytes of FP32 h of every dispatch's input level above 0 and of the
    middle level of two-level general dispatches (the adjoint's workspace)."""
    mips = mips or P.full_level_count(w, h)
    need = set()
    for fast, pc, _groups in O.default_schedule(w, h, mips):
        level, count = pc >> 5, pc & 31
        if level > 0:
            need.add(level)
        if not fast and count == 2:
            need.add(level + 1)
    sizes = P.level_sizes(w, h, mips)
    return sum(sizes[k][0] * sizes[k][1] * 16 for k in need)


@pytest.mark.parametrize("w,h,mips", [(1, 1, 0), (2, 1, 0), (64, 64, 0), (1023, 777, 0), (2048, 2048, 0),
                                      (4095, 4094, 0), (1920, 1080, 0), (2052, 2052, 0), (640, 384, 4)])
def test_adjoint_workspace_bytes(native, w, h, mips):
    assert native.nvproPyramidAdjointWorkspaceBytes(w, h, mips) == _workspace_rule(w, h, mips)


def test_write_levels_tga_round_trip(native, repo_tmp):
    """writeMipmapsTga naming (include/mipmap_storage.hpp:436-479) and TGA
    contents, read back through nvproPyramidReadTga."""
    import numpy as np

    import _oracle as O
    import vk_compute_mipmaps_gb300 as V
    w, h = 37, 20
    base = np.random.default_rng(3).integers(0, 256, (h, w, 4), dtype=np.uint8)
    packed = O.pyramid(1, base)
    levels = O.full_levels(w, h)
    off = O.offsets(w, h, levels, 4)
    for name, stem, ext in (("mips.tga", "mips.", ".tga"), ("noext", "noext", "")):
        path = repo_tmp / name
        assert native.nvproPyramidWriteLevelsTga(str(path).encode(), packed.ctypes.data, w, h, 0) == 0
        for k in range(levels):
            f = path if k == 0 else repo_tmp / f"{stem}{k}{ext}"
            lw, lh = max(w >> k, 1), max(h >> k, 1)
            raw = f.read_bytes()
            assert len(raw) == 18 + lw * lh * 4
            assert raw[2] == 2 and raw[16] == 32 and raw[17] == 0x28  # uncompressed, 32 bpp, top-left
            want = packed[off[k]:off[k + 1]].reshape(lh, lw, 4)
            assert np.array_equal(V.read_tga(str(f)), want), (name, k)
    V.write_tga(str(repo_tmp / "one.tga"), base)
    assert np.array_equal(V.read_tga(str(repo_tmp / "one.tga")), base)


def test_read_tga_rle_bottom_up_24bit(native, repo_tmp):
    import numpy as np

    import vk_compute_mipmaps_gb300 as V
    from vk_compute_mipmaps_gb300 import _native as N
    # 3x2, type 10 (RLE), 24 bpp, bottom-left origin: bottom row = a run of
    # three (10, 20, 30) pixels; top row = raw packet of three pixels
    hdr = bytes([0, 0, 10] + [0] * 9 + [3, 0, 2, 0, 24, 0])
    body = bytes([0x82, 30, 20, 10, 0x02, 3, 2, 1, 6, 5, 4, 9, 8, 7])
    (repo_tmp / "rle.tga").write_bytes(hdr + body)
    got = V.read_tga(str(repo_tmp / "rle.tga"))
    want = np.array([[[1, 2, 3, 255], [4, 5, 6, 255], [7, 8, 9, 255]],
                     [[10, 20, 30, 255]] * 3], np.uint8)
    assert np.array_equal(got, want)
    (repo_tmp / "cmap.tga").write_bytes(bytes([0, 1, 1] + [0] * 15))
    w, h = ctypes.c_uint32(), ctypes.c_uint32()
    assert native.nvproPyramidReadTga(str(repo_tmp / "cmap.tga").encode(), None, 0, ctypes.byref(w),
                                      ctypes.byref(h)) == N.ERROR_UNSUPPORTED
    assert native.nvproPyramidReadTga(str(repo_tmp / "missing.tga").encode(), None, 0, ctypes.byref(w),
                                      ctypes.byref(h)) == N.ERROR_IO
    (repo_tmp / "short.tga").write_bytes(hdr + body[:5])
    buf = np.empty(24, np.uint8)
    assert native.nvproPyramidReadTga(str(repo_tmp / "short.tga").encode(), buf.ctypes.data, 24, ctypes.byref(w),
                                      ctypes.byref(h)) == N.ERROR_IO


@pytest.mark.parametrize("w,h", [(16384, 16384), (1920, 1080), (2052, 2052), (2048, 512), (4095, 4095), (64, 64),
                                 (12, 8), (96, 40), (4096, 64)])
def test_host_upload_band_plan(w, h):
    """generate_from_host's plan: the first dispatch it bands is the default
    schedule's first dispatch, and the band sub-images point at the rows of
    every level the band's dispatch writes."""
    from vk_compute_mipmaps_gb300 import pyramid as P
    sched = O.default_schedule(w, h)
    levels = O.full_levels(w, h)
    n = P._first_fast_levels(w, h, levels)
    first_fast, first_pc, _ = sched[0]
    assert n == ((first_pc & 31) if first_fast else 0), (w, h)
    if not n:
        return
    chain = P.MipChain(w, h, device="cpu")
    base = chain.storage.data_ptr()
    unit = 1 << n
    rows = max(unit, (h // 4) // unit * unit)
    for r0 in range(0, h, rows):
        band = min(rows, h - r0)
        img = P._sub_image(chain, 0, n + 1, r0, band)
        assert (img.width, img.height, img.levelCount) == (w, band, n + 1)
        for k in range(n + 1):
            lw = max(w >> k, 1)
            assert img.levels[k] == base + chain.offsets[k] + (r0 >> k) * lw * 4
            assert img.rowPitchBytes[k] == lw * 4
        assert r0 % unit == 0 and (band % unit == 0 or r0 + band == h)
