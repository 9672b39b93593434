"""Failure detection on the GPU without a fault: every device-side wait of the
library is bounded (a timer / poll limit) and reports through an error flag.
A test kernel makes each kind of wait run out (an mbarrier phase that nothing
completes; a grid barrier that nothing releases); the host must read
NVPRO_PYRAMID_ERROR_TIMEOUT, the context must stay usable, and the same
command object must produce correct chains afterwards.
"""
import ctypes
import time

import numpy as np
import pytest

import _oracle as O
from vk_compute_mipmaps_gb300 import _native as N
from vk_compute_mipmaps_gb300 import pyramid as P

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", [0, 1], ids=["mbarrier", "grid_barrier"])
def test_bounded_wait_runs_out_and_is_reported(cuda, kind):
    import torch
    lib = N.load()
    stream = torch.cuda.current_stream(cuda).cuda_stream
    cmd = P.Cmd(0)
    cmd.begin(stream)
    t0 = time.monotonic()
    N.check(lib.nvproPyramidDebugForceWaitTimeout(cmd.handle, kind), "force timeout")
    assert lib.nvproPyramidCmdDeviceStatus(cmd.handle) == N.ERROR_TIMEOUT
    elapsed = time.monotonic() - t0
    assert 0.2 < elapsed < 20, elapsed  # the wait's own limit ended it
    assert lib.nvproPyramidCmdDeviceStatus(cmd.handle) == N.SUCCESS  # reported once, counters reset
    # the context and the command's counters work: the fast kernel with its
    # fused tail (counter) and the general chain (grid barrier)
    pipes = P.Pipelines(N.PRESET_SRGBA8)
    for w, h in ((4096, 4096), (4095, 4095)):
        base = np.random.default_rng(w).integers(0, 256, (h, w, 4), dtype=np.uint8)
        chain = P.MipChain(w, h, N.PRESET_SRGBA8, device=cuda)
        chain.level(0).copy_(torch.from_numpy(base))
        P.generate(chain, stream=stream, pipelines=pipes, cmd=cmd)
        assert lib.nvproPyramidCmdDeviceStatus(cmd.handle) == N.SUCCESS
        assert np.array_equal(chain.storage.cpu().numpy(), O.pyramid(1, base)), (w, h)


@pytest.mark.parametrize("kind", [0, 1], ids=["mbarrier", "grid_barrier"])
def test_no_alloc_path_reports_a_timeout(cuda, kind):
    """The allocation-free entry point keeps a timed-out wait in its fixed
    array until nvproPyramidNoAllocDeviceStatus reads it (a later call does
    not erase it), reports it once, and the next chain is correct."""
    import torch
    lib = N.load()
    stream = torch.cuda.current_stream(cuda).cuda_stream
    assert lib.nvproPyramidNoAllocDeviceStatus(stream) == N.SUCCESS  # nothing pending from earlier tests
    N.check(lib.nvproPyramidDebugNoAllocForceWaitTimeout(stream, kind), "force timeout")
    w, h = 4095, 4095  # a general run (grid barrier) after the timed-out wait, before the query
    base = np.random.default_rng(kind + 5).integers(0, 256, (h, w, 4), dtype=np.uint8)
    chain = P.MipChain(w, h, N.PRESET_SRGBA8, device=cuda)
    chain.level(0).copy_(torch.from_numpy(base))
    img = chain.image()
    N.check(lib.nvproPyramidGenerateNoAlloc(stream, N.PRESET_SRGBA8, ctypes.byref(img), 0), "no-alloc chain")
    assert lib.nvproPyramidNoAllocDeviceStatus(stream) == N.ERROR_TIMEOUT
    assert lib.nvproPyramidNoAllocDeviceStatus(stream) == N.SUCCESS
    for w, h in ((4096, 4096), (4095, 4095)):
        base = np.random.default_rng(w + kind).integers(0, 256, (h, w, 4), dtype=np.uint8)
        chain = P.MipChain(w, h, N.PRESET_SRGBA8, device=cuda)
        chain.level(0).copy_(torch.from_numpy(base))
        img = chain.image()
        N.check(lib.nvproPyramidGenerateNoAlloc(stream, N.PRESET_SRGBA8, ctypes.byref(img), 0), "no-alloc chain")
        assert lib.nvproPyramidNoAllocDeviceStatus(stream) == N.SUCCESS
        assert np.array_equal(chain.storage.cpu().numpy(), O.pyramid(1, base)), (w, h)


def test_fast_kernel_counter_survives_a_give_up_without_a_query(cuda):
    """A CTA of the fast kernel that gives up still arrives on the kernel's
    last-CTA counter (marked as failed): the failed launch skips its fused
    tail, and the next launch on the same command -- with no status query in
    between -- runs its tail on a clean counter and is correct."""
    import torch
    lib = N.load()
    stream = torch.cuda.current_stream(cuda).cuda_stream
    cmd = P.Cmd(0)
    pipes = P.Pipelines(N.PRESET_SRGBA8)
    w = h = 4096  # F6 over level 0 with the F6 of the 64x64 level 6 in its tail: one launch
    bases = [np.random.default_rng(s).integers(0, 256, (h, w, 4), dtype=np.uint8) for s in (21, 22)]
    chains = []
    for i, base in enumerate(bases):
        chain = P.MipChain(w, h, N.PRESET_SRGBA8, device=cuda)
        chain.storage.fill_(0xA7)
        chain.level(0).copy_(torch.from_numpy(base))
        cmd.begin(stream)
        if i == 0:
            N.check(lib.nvproPyramidDebugForceWaitTimeout(cmd.handle, 2), "simulated give-up")
        cmd.bind_image(chain.image())
        P.cmd_pyramid_dispatch(cmd, pipes, w, h)
        cmd.end()
        assert cmd.launch_count == 1
        chains.append(chain)
    torch.cuda.synchronize()
    want = [O.pyramid(1, b) for b in bases]
    first = chains[0].storage.cpu().numpy()
    off = O.offsets(w, h, 13, 4)
    assert not np.array_equal(first, want[0])                     # CTA 0's regions were not written
    assert np.all(first[off[7]:] == 0xA7)                         # and the tail (levels 7..12) was skipped
    assert np.array_equal(chains[1].storage.cpu().numpy(), want[1])  # the next launch is whole
    assert lib.nvproPyramidCmdDeviceStatus(cmd.handle) == N.ERROR_TIMEOUT
    assert lib.nvproPyramidCmdDeviceStatus(cmd.handle) == N.SUCCESS
