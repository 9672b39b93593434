"""GPU parity of the linear blit and the demo's "generalblit" mode
(demo_app/mipmap_pipelines.cpp:350-452: the fast pipeline where the sizes
allow it, vkCmdBlitImage with VK_FILTER_LINEAR otherwise), against the
oracle's restatement with the same pinned FP32 filter, for every preset.
"""
import numpy as np
import pytest

import _oracle as O
from vk_compute_mipmaps_gb300 import _native as N
from vk_compute_mipmaps_gb300 import pyramid as P

pytestmark = pytest.mark.gpu

SENTINEL = 0xA7
SIZES = [(1920, 1080), (4095, 4095), (2052, 2052), (1023, 777), (5, 3), (3, 3), (1, 9), (9, 1), (2047, 2), (97, 64)]


def base_of(preset, w, h, seed):
    rng = np.random.default_rng(seed)
    if preset == N.PRESET_SRGBA8:
        return rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    return rng.random((h, w, 4)).astype(np.float32 if preset == N.PRESET_RGBA32F else np.float16)


def run_gpu(cuda, preset, base, flags=0):
    import torch
    h, w = base.shape[:2]
    chain = P.MipChain(w, h, preset, device=cuda)
    chain.storage.fill_(SENTINEL)
    chain.storage[:chain.offsets[1]].copy_(torch.from_numpy(np.ascontiguousarray(base).view(np.uint8).reshape(-1)))
    cmd, pipes = P.Cmd(flags), P.Pipelines(preset)
    cmd.begin(torch.cuda.current_stream(cuda).cuda_stream)
    cmd.bind_image(chain.image())
    P.cmd_pyramid_dispatch(cmd, pipes, w, h, 0, general=P.blit_general_dispatcher())
    cmd.end()
    torch.cuda.synchronize()
    return chain.storage.cpu().numpy(), cmd.records()


@pytest.mark.parametrize("flags", [0, N.CMD_PORTABLE_KERNELS])
@pytest.mark.parametrize("w,h", SIZES)
def test_general_blit_mode_srgba8(cuda, w, h, flags):
    base = base_of(N.PRESET_SRGBA8, w, h, w * 7 + h)
    got, recs = run_gpu(cuda, N.PRESET_SRGBA8, base, flags)
    sched = O.fast_or_blit_schedule(w, h)
    assert sum(r["isBlit"] for r in recs) == sum(f == 2 for f, _, _ in sched)
    off = O.offsets(w, h, O.full_levels(w, h), 4)
    want = np.full(off[-1], SENTINEL, np.uint8)
    want[:off[1]] = base.reshape(-1)
    O.run(1, w, h, want, sched)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("preset", [N.PRESET_RGBA32F, N.PRESET_RGBA16F])
@pytest.mark.parametrize("w,h", [(1920, 1080), (5, 3), (1023, 777)])
def test_general_blit_mode_float(cuda, preset, w, h):
    base = base_of(preset, w, h, w + h)
    got, _ = run_gpu(cuda, preset, base)
    off = O.offsets(w, h, O.full_levels(w, h), O.BPP[preset])
    want = np.full(off[-1], SENTINEL, np.uint8)
    want[:off[1]] = base.view(np.uint8).reshape(-1)
    O.run(preset, w, h, want, O.fast_or_blit_schedule(w, h))
    assert np.array_equal(got, want)


def test_blit_level_direct(cuda):
    # vkCmdBlitImage analogue on one level of an image: level 2 -> 3 only
    import torch
    w, h = 301, 77
    base = base_of(N.PRESET_SRGBA8, w, h, 5)
    levels = O.full_levels(w, h)
    off = O.offsets(w, h, levels, 4)
    packed = O.pyramid(1, base)
    chain = P.MipChain(w, h, N.PRESET_SRGBA8, device=cuda)
    chain.storage.copy_(torch.from_numpy(packed))
    chain.storage[off[3]:off[4]].fill_(SENTINEL)
    cmd, pipes = P.Cmd(0), P.Pipelines(N.PRESET_SRGBA8)
    cmd.begin(torch.cuda.current_stream(cuda).cuda_stream)
    cmd.bind_image(chain.image())
    cmd.bind_pipeline(pipes.general)
    N.check(N.load().nvproPyramidCmdBlitLevel(cmd.handle, 2))
    cmd.end()
    torch.cuda.synchronize()
    want = packed.copy()
    O.run(1, w, h, want, [(2, 2 << 5 | 1, 1)])
    assert np.array_equal(chain.storage.cpu().numpy(), want)
