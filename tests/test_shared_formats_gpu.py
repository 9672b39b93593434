"""GPU parity of the shared-memory formats SRGB_SHARED / F16_SHARED
(srgba8_mipmap_preamble.glsl:60-108; the demo's srgbShared, f16Shared,
srgbSharedGeneral and f16SharedGeneral alternatives,
demo_app/pipeline_alternative.cpp:25-31): pipelines created with the config
bits, run through the C ABI on every kernel family (TMA fast kernel with its
fused tail, general chain kernel, portable kernels), bit-exact against the
oracle run with the same formats.
"""
import numpy as np
import pytest

import _oracle as O
from vk_compute_mipmaps_gb300 import _native as N
from vk_compute_mipmaps_gb300 import pyramid as P

pytestmark = pytest.mark.gpu

SENTINEL = 0xA7
FLAGS = [0, N.CMD_NO_FUSION, N.CMD_PORTABLE_KERNELS]
BITS = {O.SHARED_FP32: 0, O.SHARED_SRGB: N.CONFIG_SRGB_SHARED, O.SHARED_F16: N.CONFIG_F16_SHARED}
# schedules: F4; F4 G2; F4 G2..; F6 F2; F6 F4; F5 G..; F3 G2..; F2 G2 F6 G1; G2.. G1; G2.. G1
SIZES = [(16, 16), (48, 80), (208, 48), (256, 256), (1024, 1024), (1440, 800), (1920, 1080), (2052, 2052),
         (1023, 777), (255, 255)]


def base_image(w, h, seed):
    return np.random.default_rng(seed).integers(0, 256, (h, w, 4), dtype=np.uint8)


def gpu_run(cuda, base, fast_fmt, general_fmt, flags=0):
    import torch
    h, w = base.shape[:2]
    mips = P.full_level_count(w, h)
    chain = P.MipChain(w, h, N.PRESET_SRGBA8, mips, device=cuda)
    chain.storage.fill_(SENTINEL)
    chain.storage[:chain.offsets[1]].copy_(torch.from_numpy(base.reshape(-1).copy()))
    pipes = P.Pipelines(N.PRESET_SRGBA8, general_config=BITS[general_fmt], fast_config=BITS[fast_fmt])
    cmd = P.Cmd(flags)
    cmd.begin(torch.cuda.current_stream(cuda).cuda_stream)
    cmd.bind_image(chain.image())
    P.cmd_pyramid_dispatch(cmd, pipes, w, h, mips)
    cmd.end()
    torch.cuda.synchronize()
    return chain.storage.cpu().numpy(), cmd.launch_count


def oracle(base, fast_fmt, general_fmt):
    h, w = base.shape[:2]
    mips = O.full_levels(w, h)
    off = O.offsets(w, h, mips, 4)
    buf = np.full(off[-1], SENTINEL, np.uint8)
    buf[:off[1]] = base.reshape(-1)
    return O.run(1, w, h, buf, None, mips, fast_fmt, general_fmt)


def check(got, want, w, h, what):
    if np.array_equal(got, want):
        return
    off = O.offsets(w, h, O.full_levels(w, h), 4)
    bad = [k for k in range(len(off) - 1) if not np.array_equal(got[off[k]:off[k + 1]], want[off[k]:off[k + 1]])]
    raise AssertionError(f"{what}: levels {bad} differ")


@pytest.mark.parametrize("fmt", [O.SHARED_SRGB, O.SHARED_F16])
@pytest.mark.parametrize("flags", FLAGS)
@pytest.mark.parametrize("w,h", SIZES)
def test_shared_format_bit_exact(cuda, w, h, flags, fmt):
    base = base_image(w, h, w * 31 + h + fmt)
    got, _ = gpu_run(cuda, base, fmt, fmt, flags)
    check(got, oracle(base, fmt, fmt), w, h, f"{w}x{h} flags={flags} fmt={fmt}")


@pytest.mark.parametrize("fmt", [O.SHARED_SRGB, O.SHARED_F16])
@pytest.mark.parametrize("w,h", [(4096, 4096), (4095, 4095), (4094, 4094)])
def test_shared_format_bit_exact_large(cuda, w, h, fmt):
    base = base_image(w, h, w + fmt)
    got, launches = gpu_run(cuda, base, fmt, fmt)
    check(got, oracle(base, fmt, fmt), w, h, f"{w}x{h} fmt={fmt}")
    _, default_launches = gpu_run(cuda, base, O.SHARED_FP32, O.SHARED_FP32)
    assert launches == default_launches  # the same fused kernels as the default pipelines


@pytest.mark.parametrize("flags", [0, N.CMD_PORTABLE_KERNELS])
@pytest.mark.parametrize("w,h", [(2052, 2052), (1920, 1080), (1024, 1024)])
@pytest.mark.parametrize("fast_fmt,general_fmt", [(O.SHARED_FP32, O.SHARED_SRGB), (O.SHARED_FP32, O.SHARED_F16),
                                                  (O.SHARED_SRGB, O.SHARED_FP32), (O.SHARED_F16, O.SHARED_SRGB)])
def test_shared_format_per_pipeline(cuda, w, h, flags, fast_fmt, general_fmt):
    base = base_image(w, h, 7 * w + h)
    got, _ = gpu_run(cuda, base, fast_fmt, general_fmt, flags)
    check(got, oracle(base, fast_fmt, general_fmt), w, h, f"{w}x{h} fast={fast_fmt} general={general_fmt}")


def test_shared_formats_reach_the_kernels(cuda):
    # the variants' bytes differ from the default pipelines' (F6 F2 and G2 G2 G2 G1)
    for w, h in ((256, 256), (255, 255)):
        base = base_image(w, h, 99)
        default, _ = gpu_run(cuda, base, O.SHARED_FP32, O.SHARED_FP32)
        for fmt in (O.SHARED_SRGB, O.SHARED_F16):
            got, _ = gpu_run(cuda, base, fmt, fmt)
            assert not np.array_equal(got, default), (w, h, fmt)
