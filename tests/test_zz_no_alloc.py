"""nvproPyramidGenerateNoAlloc: the entry point for callers that may not
allocate device memory (a host application that owns every allocation, or a
hot loop that must not call cudaMalloc/cudaFree).  It keeps its kernel
counters in a fixed device array of the library instead of the command
object's allocation.

Its output must equal, byte for byte, the output of the allocating entry
point (nvproPyramidGenerate) on the same input, on two calls in a row: the
second call starts from whatever the first left in the shared array.  This
file is collected last so that a failing run has already run every other test;
it also passes on its own in a fresh process.
"""
import ctypes

import pytest

from vk_compute_mipmaps_gb300 import _native as N
from vk_compute_mipmaps_gb300 import pyramid as P

pytestmark = pytest.mark.gpu

SENTINEL = 0xA7


def make_base(torch, cuda, w, h, seed):
    g = torch.Generator(device=cuda).manual_seed(seed)
    return torch.randint(0, 256, (h * w * 4,), generator=g, device=cuda, dtype=torch.uint8)


@pytest.mark.parametrize("w,h", [(4096, 4096), (16384, 2048), (2048, 2048), (1920, 1080), (2052, 2052),
                                 (255, 257), (1, 1)])
def test_no_alloc_entry_point_matches_allocating_one(cuda, native, w, h):
    import torch
    stream = torch.cuda.current_stream(cuda).cuda_stream
    pipes, cmd = P.Pipelines(N.PRESET_SRGBA8), P.Cmd()
    for call, seed in enumerate((11 * w + h, 13 * w + h)):  # two calls in a row, different inputs
        base = make_base(torch, cuda, w, h, seed)
        want = P.MipChain(w, h, N.PRESET_SRGBA8, device=cuda)
        got = P.MipChain(w, h, N.PRESET_SRGBA8, device=cuda)
        for chain in (want, got):
            chain.storage.fill_(SENTINEL)
            chain.storage[:chain.offsets[1]].copy_(base)
        img_want, img_got = want.image(), got.image()
        N.check(native.nvproPyramidGenerate(cmd.handle, stream, pipes.struct, ctypes.byref(img_want), 0),
                "nvproPyramidGenerate")
        N.check(native.nvproPyramidGenerateNoAlloc(stream, N.PRESET_SRGBA8, ctypes.byref(img_got), 0),
                "nvproPyramidGenerateNoAlloc")
        torch.cuda.synchronize()
        assert torch.equal(want.storage, got.storage), f"{w}x{h} call {call}"


def test_no_alloc_rejects_bad_arguments(cuda, native):
    import torch
    stream = torch.cuda.current_stream(cuda).cuda_stream
    chain = P.MipChain(64, 64, N.PRESET_SRGBA8, levels=3, device=cuda)
    img = chain.image()
    # more levels than the image binds
    rc = native.nvproPyramidGenerateNoAlloc(stream, N.PRESET_SRGBA8, ctypes.byref(img), 7)
    assert rc == N.ERROR_INVALID_ARGUMENT
    assert native.nvproPyramidGenerateNoAlloc(stream, 9, ctypes.byref(img), 0) == N.ERROR_UNSUPPORTED
    assert native.nvproPyramidGenerateNoAlloc(stream, N.PRESET_SRGBA8, None, 0) == N.ERROR_INVALID_ARGUMENT
    torch.cuda.synchronize()
