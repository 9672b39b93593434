"""Host-side logic without a GPU: the bench's multi-rank helpers as two gloo
ranks, the synthetic batch workload, and the adjoint workspace rule."""
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
