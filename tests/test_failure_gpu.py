"""Failure detection on the GPU without a fault: every device-side wait of the
library is bounded (a timer / poll limit) and reports through an error flag.
A test kernel makes each kind of wait run out (an mbarrier phase that nothing
completes; a grid barrier that nothing releases); the host must read
NVPRO_PYRAMID_ERROR_TIMEOUT, the context must stay usable, and the same
command object must produce correct chains afterwards.
"""
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
