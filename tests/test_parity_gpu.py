"""GPU parity: the CUDA kernels, called through the C ABI, against the CPU
oracle on the same seeded inputs -- bit-exact for every preset.

Outputs are pre-filled with a sentinel (the reference pre-clears to magenta,
demo_app/mipmaps_app.cpp:688-705) so unwritten texels show up.  Sizes cover
every schedule branch (docs/test_images.txt: 1080p, 4094, 4095, 2052, 4096 ...)
plus 1xN, Nx1, 2^k +- 1 and tiny images.
"""
import ctypes

import numpy as np
import pytest

import _oracle as O
from vk_compute_mipmaps_gb300 import _native as N
from vk_compute_mipmaps_gb300 import pyramid as P

pytestmark = pytest.mark.gpu

SENTINEL = 0xA7

SIZES = [(1, 1), (2, 1), (1, 2), (1, 9), (9, 1), (2, 2), (3, 3), (4, 4), (5, 5), (7, 3), (8, 8), (12, 20),
         (16, 16), (17, 17), (31, 31), (32, 32), (33, 33), (63, 64), (64, 64), (65, 65), (65, 33), (96, 160),
         (127, 129), (128, 128), (255, 256), (256, 256), (257, 257), (1024, 1), (1, 1024), (1000, 3),
         (513, 512), (640, 384), (1920, 1080), (2052, 2052), (2047, 2047)]
BIG = [(4096, 4096), (4095, 4095), (4094, 4094), (2048, 2048), (3840, 2160), (2560, 1440)]
FLAGS = [0, N.CMD_NO_FUSION, N.CMD_PORTABLE_KERNELS]


def random_base(preset, w, h, seed):
    rng = np.random.default_rng(seed)
    if preset == N.PRESET_SRGBA8:
        return rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    if preset == N.PRESET_RGBA32F:
        return rng.lognormal(0.0, 1.0, (h, w, 4)).astype(np.float32)
    return rng.lognormal(0.0, 1.0, (h, w, 4)).astype(np.float16)


def oracle_bytes(preset, base, schedule, mips):
    h, w = base.shape[:2]
    off = O.offsets(w, h, mips, O.BPP[preset])
    buf = np.full(off[-1], SENTINEL, np.uint8)
    buf[:off[1]] = np.ascontiguousarray(base).view(np.uint8).reshape(-1)
    return O.run(preset, w, h, buf, schedule, mips)


def gpu_run(cuda, preset, base, flags=0, mips=0, general=None, fast=None, has_fast=True):
    """Generate on the GPU; return (packed bytes, recorded schedule, launches)."""
    import torch
    h, w = base.shape[:2]
    mips = mips or P.full_level_count(w, h)
    chain = P.MipChain(w, h, preset, mips, device=cuda)
    chain.storage.fill_(SENTINEL)
    raw = torch.from_numpy(np.ascontiguousarray(base).view(np.uint8).reshape(-1).copy())
    chain.storage[:chain.offsets[1]].copy_(raw)
    cmd = P.Cmd(flags)
    pipes = P.Pipelines(preset, fast=has_fast)
    stream = torch.cuda.current_stream(cuda).cuda_stream
    cmd.begin(stream)
    cmd.bind_image(chain.image())
    P.cmd_pyramid_dispatch(cmd, pipes, w, h, mips, general=general, fast=fast)
    cmd.end()
    torch.cuda.synchronize()
    sched = [(r["isFastPipeline"], r["pushConstant"],
              r["groupCountX"] if r["groupCountY"] and r["groupCountZ"] else 0) for r in cmd.records()]
    return chain.storage.cpu().numpy(), sched, cmd.launch_count


def assert_same(got, want, w, h, bpp, mips, what):
    if np.array_equal(got, want):
        return
    off = O.offsets(w, h, mips, bpp)
    for k in range(mips):
        a, b = got[off[k]:off[k + 1]], want[off[k]:off[k + 1]]
        if not np.array_equal(a, b):
            idx = np.nonzero(a != b)[0]
            lw = max(w >> k, 1)
            t = idx[0] // bpp
            raise AssertionError(f"{what}: level {k} differs at {len(idx)} bytes; first texel "
                                 f"({t % lw}, {t // lw}) got {a[t*bpp:(t+1)*bpp]} want {b[t*bpp:(t+1)*bpp]}")


@pytest.mark.parametrize("flags", FLAGS)
@pytest.mark.parametrize("w,h", SIZES)
def test_srgba8_bit_exact(cuda, w, h, flags):
    base = random_base(N.PRESET_SRGBA8, w, h, w * 131 + h)
    got, sched, _ = gpu_run(cuda, N.PRESET_SRGBA8, base, flags)
    mips = P.full_level_count(w, h)
    assert sched == [tuple(s) for s in O.default_schedule(w, h)]
    assert_same(got, oracle_bytes(N.PRESET_SRGBA8, base, sched, mips), w, h, 4, mips, f"{w}x{h} flags={flags}")


# Every (w mod 4, h mod 4) but (0, 0) starts with a general dispatch whose
# kernel sizes are (2|w&1, 2|h&1) on level 0 and (2|(w>>1)&1, ...) on level 1:
# all fifteen two-level strip kernels, plus strips and bands that end mid-way.
MOD4 = [(300 + a, 200 + b) for a in range(4) for b in range(4) if (a, b) != (0, 0)]


@pytest.mark.parametrize("w,h", MOD4 + [(1001, 999), (2050, 1027), (4093, 45), (45, 4093), (6, 1023)])
def test_general_strips_bit_exact(cuda, w, h):
    base = random_base(N.PRESET_SRGBA8, w, h, w * 7 + h)
    mips = P.full_level_count(w, h)
    got, sched, _ = gpu_run(cuda, N.PRESET_SRGBA8, base)
    assert_same(got, oracle_bytes(N.PRESET_SRGBA8, base, sched, mips), w, h, 4, mips, f"{w}x{h}")


@pytest.mark.parametrize("w,h", [(1001, 999), (1000, 999), (1001, 998), (1002, 1002), (3, 700), (700, 3)])
def test_general_one_level_bit_exact(cuda, w, h):
    """mipLevels = 2: a single one-level general dispatch (the four one-level strip kernels)."""
    base = random_base(N.PRESET_SRGBA8, w, h, w + 3 * h)
    got, sched, _ = gpu_run(cuda, N.PRESET_SRGBA8, base, mips=2)
    assert_same(got, oracle_bytes(N.PRESET_SRGBA8, base, sched, 2), w, h, 4, 2, f"{w}x{h} mips=2")


@pytest.mark.parametrize("w,h", BIG)
def test_srgba8_bit_exact_large(cuda, w, h):
    from vk_compute_mipmaps_gb300.workloads import smooth_field
    base = smooth_field(w, h, 5, opaque=False)
    mips = P.full_level_count(w, h)
    want = None
    for flags in FLAGS:
        got, sched, _ = gpu_run(cuda, N.PRESET_SRGBA8, base, flags)
        if want is None:
            want = oracle_bytes(N.PRESET_SRGBA8, base, sched, mips)
        assert_same(got, want, w, h, 4, mips, f"{w}x{h} flags={flags}")


@pytest.mark.parametrize("preset", [N.PRESET_RGBA32F, N.PRESET_RGBA16F])
@pytest.mark.parametrize("w,h", [(1, 1), (3, 3), (64, 64), (65, 33), (256, 256), (257, 129), (1920, 1080),
                                 (1023, 777)])
def test_float_presets_bit_exact(cuda, preset, w, h):
    base = random_base(preset, w, h, 99 + w)
    mips = P.full_level_count(w, h)
    for flags in (0, N.CMD_PORTABLE_KERNELS):
        got, sched, _ = gpu_run(cuda, preset, base, flags)
        assert_same(got, oracle_bytes(preset, base, sched, mips), w, h, O.BPP[preset], mips, f"{preset} {w}x{h}")


@pytest.mark.parametrize("w,h", [(64, 64), (193, 97), (2052, 36)])
def test_srgba8_strided_equals_per_image(cuda, w, h):
    """nvproPyramidGenerateStrided over B sRGBA8 images (portable kernels, one
    launch per dispatch) writes the bytes of per-image nvproPyramidGenerate."""
    import torch
    B = 3
    lib = N.load()
    sizes = P.level_sizes(w, h)
    g = torch.Generator(device=cuda).manual_seed(w + h)
    lv = [torch.full((B, lh, lw, 4), SENTINEL, dtype=torch.uint8, device=cuda) for lw, lh in sizes]
    lv[0].copy_(torch.randint(0, 256, lv[0].shape, generator=g, device=cuda, dtype=torch.uint8))
    img = P.make_image([t.data_ptr() for t in lv], w, h)
    strides = (ctypes.c_uint64 * N.MAX_LEVELS)(*[t[0].numel() for t in lv])
    cmd, pipes = P.Cmd(), P.Pipelines(N.PRESET_SRGBA8)
    stream = torch.cuda.current_stream(cuda).cuda_stream
    N.check(lib.nvproPyramidGenerateStrided(cmd.handle, stream, pipes.struct, ctypes.addressof(img),
                                            ctypes.addressof(strides), B, 0))
    torch.cuda.synchronize()
    for i in range(B):
        got = np.concatenate([t[i].cpu().numpy().reshape(-1) for t in lv])
        mips = len(sizes)
        want = oracle_bytes(N.PRESET_SRGBA8, lv[0][i].cpu().numpy(), [tuple(s) for s in O.default_schedule(w, h)],
                            mips)
        assert_same(got, want, w, h, 4, mips, f"strided image {i} of {w}x{h}")


def fast_variant(div, mx):
    lib = N.load()
    return P.wrap_dispatcher(lambda c, lay, pco, pipe, st: lib.nvproPyramidFastDispatch(
        c, lay, pco, pipe, ctypes.byref(st), div, mx))


def partial_general(fraction):
    """The default general dispatcher, but dispatching only part of the grid."""
    lib = N.load()

    def fn(c, lay, pco, pipe, st):
        if pipe:
            lib.nvproPyramidCmdBindPipeline(c, pipe)
        levels = min(2, st.remainingLevels)
        pc = ctypes.c_uint32(st.currentLevel << 5 | levels)
        lib.nvproPyramidCmdPushConstants(c, lay, pco, 4, ctypes.byref(pc))
        dw, dh = max(st.currentX >> levels, 1), max(st.currentY >> levels, 1)
        full = -(-dw * dh // 128) if levels == 1 else -(-dw // 8) * -(-dh // 8)
        lib.nvproPyramidCmdDispatch(c, int(full * fraction), 1, 1)
        return levels
    return P.wrap_dispatcher(fn)


def partial_fast(fraction):
    lib = N.load()

    def fn(c, lay, pco, pipe, st):
        if st.currentX % 4 or st.currentY % 4:
            return 0
        if pipe:
            lib.nvproPyramidCmdBindPipeline(c, pipe)
        x, y, n = st.currentX, st.currentY, 0
        while x % 2 == 0 and y % 2 == 0 and n < st.remainingLevels and n < 6:
            x, y, n = x // 2, y // 2, n + 1
        pc = ctypes.c_uint32(st.currentLevel << 5 | n)
        lib.nvproPyramidCmdPushConstants(c, lay, pco, 4, ctypes.byref(pc))
        per = 4096 if n > 5 else 1024
        lib.nvproPyramidCmdDispatch(c, int(-(-st.currentX * st.currentY // per) * fraction), 1, 1)
        return n
    return P.wrap_dispatcher(fn)


@pytest.mark.parametrize("case", ["levels_1_5", "levels_1_6", "general_only", "null_fast",
                                  "partial_general", "partial_fast", "null_general"])
@pytest.mark.parametrize("w,h", [(64, 64), (96, 40), (1920, 1080), (255, 257), (2052, 2052), (640, 384)])
def test_custom_dispatchers(cuda, case, w, h):
    """Dispatcher variants of demo_app/nvpro_pyramid_dispatch_alternative.cpp:41-77,
    and dispatchers that cover only part of the grid: the GPU writes exactly
    what the oracle writes for the recorded schedule (sentinel elsewhere)."""
    nul = P.wrap_dispatcher(lambda c, lay, pco, pipe, st: st.remainingLevels)
    kw = {"levels_1_5": dict(fast=fast_variant(2, 5)), "levels_1_6": dict(fast=fast_variant(2, 6)),
          "general_only": dict(has_fast=False), "null_fast": dict(fast=nul),
          "partial_general": dict(general=partial_general(0.6)), "partial_fast": dict(fast=partial_fast(0.3)),
          "null_general": dict(general=nul)}[case]
    base = random_base(N.PRESET_SRGBA8, w, h, 7 * w + h)
    mips = P.full_level_count(w, h)
    for flags in FLAGS:
        got, sched, _ = gpu_run(cuda, N.PRESET_SRGBA8, base, flags, **kw)
        assert_same(got, oracle_bytes(N.PRESET_SRGBA8, base, sched, mips), w, h, 4, mips, f"{case} {flags}")


@pytest.mark.parametrize("w,h", [(64, 64), (257, 129), (1920, 1080)])
def test_pitched_separate_levels(cuda, w, h):
    """Levels in separate allocations with padded row pitches."""
    import torch
    base = random_base(N.PRESET_SRGBA8, w, h, 3 * w + h)
    mips = P.full_level_count(w, h)
    sizes = P.level_sizes(w, h, mips)
    pitches = [((lw * 4 + 255) // 256) * 256 + 64 for lw, _ in sizes]
    bufs = [torch.full((lh * p,), SENTINEL, dtype=torch.uint8, device=cuda) for (lw, lh), p in zip(sizes, pitches)]
    bufs[0].view(h, pitches[0])[:, :w * 4].copy_(torch.from_numpy(base.reshape(h, w * 4)))
    img = P.make_image([b.data_ptr() for b in bufs], w, h, pitches)
    for flags in FLAGS:
        cmd, pipes = P.Cmd(flags), P.Pipelines()
        cmd.begin(torch.cuda.current_stream(cuda).cuda_stream)
        cmd.bind_image(img)
        P.cmd_pyramid_dispatch(cmd, pipes, w, h)
        cmd.end()
        torch.cuda.synchronize()
        want = O.pyramid(1, base)
        off = O.offsets(w, h, mips, 4)
        for k, ((lw, lh), p) in enumerate(zip(sizes, pitches)):
            got = bufs[k].view(lh, p)[:, :lw * 4].cpu().numpy().reshape(-1)
            assert np.array_equal(got, want[off[k]:off[k + 1]]), (flags, k)


def test_16384_chain_bit_exact(cuda):
    """The 16384^2 benchmark chain (schedule F6, F6, F2; seeded uniform random
    bytes as in the bench) at full size: all 15 levels byte for byte against
    the oracle, and identical bytes from every kernel path."""
    import torch
    w = h = 16384
    g = torch.Generator(device=cuda).manual_seed(1234)
    chain = P.MipChain(w, h, N.PRESET_SRGBA8, device=cuda)
    chain.storage.fill_(SENTINEL)
    chain.storage[:chain.offsets[1]].copy_(
        torch.randint(0, 256, (chain.offsets[1],), generator=g, device=cuda, dtype=torch.uint8))
    base = chain.level(0).cpu().numpy()
    want = O.pyramid(1, base)
    mips = chain.levels
    first = None
    for flags in FLAGS:
        chain.storage[chain.offsets[1]:].fill_(SENTINEL)
        P.generate(chain, flags=flags)
        torch.cuda.synchronize()
        got = chain.storage.cpu().numpy()
        assert_same(got, want, w, h, 4, mips, f"16384^2 flags={flags}")
        if first is None:
            first = got
        else:
            assert np.array_equal(first, got), flags


def test_16384_chain_srgb_shared_bit_exact(cuda):
    """16384^2 with SRGB_SHARED pipelines (the F6 dispatches hand level L+4 on
    as sRGBA8 codes) against the oracle's shared-format mode, all levels."""
    import torch
    w = h = 16384
    g = torch.Generator(device=cuda).manual_seed(4321)
    chain = P.MipChain(w, h, N.PRESET_SRGBA8, device=cuda)
    chain.storage.fill_(SENTINEL)
    chain.storage[:chain.offsets[1]].copy_(
        torch.randint(0, 256, (chain.offsets[1],), generator=g, device=cuda, dtype=torch.uint8))
    base = chain.level(0).cpu().numpy()
    pipes = P.Pipelines(N.PRESET_SRGBA8, general_config=N.CONFIG_SRGB_SHARED, fast_config=N.CONFIG_SRGB_SHARED)
    P.generate(chain, pipelines=pipes, cmd=P.Cmd(0))
    torch.cuda.synchronize()
    want = O.pyramid(1, base, fast_shared=O.SHARED_SRGB, general_shared=O.SHARED_SRGB)
    assert_same(chain.storage.cpu().numpy(), want, w, h, 4, chain.levels, "16384^2 SRGB_SHARED")


def test_back_to_back_chains_across_the_programmatic_launch_edge(cuda):
    """Two chains on one stream with no synchronisation between them, the
    second reading the first's output: chain B's level 0 is chain A's level 1
    (a view, no copy).  The fast kernel starts as a programmatic dependent
    launch and waits for the previous kernel before its first global access,
    so B sees A's finished level 1."""
    import torch
    wa = ha = 4096
    base = random_base(N.PRESET_SRGBA8, wa, ha, 77)
    a = P.MipChain(wa, ha, N.PRESET_SRGBA8, device=cuda)
    a.storage.fill_(SENTINEL)
    a.level(0).copy_(torch.from_numpy(base))
    wb, hb = wa // 2, ha // 2
    b = P.MipChain(wb, hb, N.PRESET_SRGBA8, device=cuda)
    b.storage.fill_(SENTINEL)
    b_img = P.make_image([a.storage.data_ptr() + a.offsets[1]] +
                         [b.storage.data_ptr() + o for o in b.offsets[1:-1]], wb, hb)
    lib = N.load()
    pipes, cmd_a, cmd_b = P.Pipelines(N.PRESET_SRGBA8), P.Cmd(0), P.Cmd(0)
    stream = torch.cuda.current_stream(cuda).cuda_stream
    for _ in range(3):  # repeated: A rewrites its level 1 while B's previous launch is done
        N.check(lib.nvproPyramidGenerate(cmd_a.handle, stream, pipes.struct, ctypes.byref(a.image()), 0), "A")
        N.check(lib.nvproPyramidGenerate(cmd_b.handle, stream, pipes.struct, ctypes.byref(b_img), 0), "B")
    torch.cuda.synchronize()
    want_a = O.pyramid(1, base)
    assert np.array_equal(a.storage.cpu().numpy(), want_a)
    lvl1 = O.split_levels(want_a, wa, ha, P.full_level_count(wa, ha), 4, np.uint8)[1]
    want_b = O.pyramid(1, lvl1)
    got_b = b.storage.cpu().numpy()
    off = O.offsets(wb, hb, P.full_level_count(wb, hb), 4)
    assert np.array_equal(got_b[off[1]:], want_b[off[1]:])


def test_fast_srgb_encoder_exhaustive(cuda, native):
    """The kernels' fast encoder (lg2/ex2 candidate + one threshold compare)
    equals the exact threshold count for every FP32 value in [0, 1] (the
    linear values an sRGBA8 pyramid can produce)."""
    import torch
    lo, hi = 0, int(np.float32(1.0).view(np.uint32))
    chunk = 1 << 28
    stream = torch.cuda.current_stream(cuda).cuda_stream
    for start in range(lo, hi + 1, chunk):
        bits = torch.arange(start, min(start + chunk, hi + 1), dtype=torch.int64, device=cuda).to(torch.int32)
        x = bits.view(torch.float32)
        fast = torch.empty(x.numel(), dtype=torch.uint8, device=cuda)
        exact = torch.empty_like(fast)
        N.check(native.nvproPyramidDebugSrgbEncode(stream, x.data_ptr(), fast.data_ptr(), exact.data_ptr(),
                                                   x.numel()))
        torch.cuda.synchronize()
        bad = (fast != exact).nonzero()
        assert bad.numel() == 0, f"{bad.numel()} mismatches, first x={x[bad[0]].item()!r}"
    # the GPU's exact count is the CPU oracle's
    xs = np.concatenate([np.random.default_rng(1).random(1 << 16, dtype=np.float32), O.tables()[2][:255],
                         np.ones(1, np.float32)])
    xt = torch.from_numpy(xs).to(cuda)
    fast = torch.empty(xs.size, dtype=torch.uint8, device=cuda)
    exact = torch.empty_like(fast)
    N.check(native.nvproPyramidDebugSrgbEncode(stream, xt.data_ptr(), fast.data_ptr(), exact.data_ptr(), xs.size))
    torch.cuda.synchronize()
    assert np.array_equal(exact.cpu().numpy(), O.srgb_encode_array(xs))
    assert np.array_equal(fast.cpu().numpy(), O.srgb_encode_array(xs))


def test_fast_alpha_encoder_exhaustive(cuda, native):
    """The texel encoder's alpha byte equals clamp(uint(rn(rn(a*255)+0.5))) for
    every FP32 a in [0, 1]; the GPU's scalar reference equals the oracle's."""
    import torch
    lo, hi = 0, int(np.float32(1.0).view(np.uint32))
    chunk = 1 << 28
    stream = torch.cuda.current_stream(cuda).cuda_stream
    for start in range(lo, hi + 1, chunk):
        bits = torch.arange(start, min(start + chunk, hi + 1), dtype=torch.int64, device=cuda).to(torch.int32)
        x = bits.view(torch.float32)
        fast = torch.empty(x.numel(), dtype=torch.uint8, device=cuda)
        exact = torch.empty_like(fast)
        N.check(native.nvproPyramidDebugAlphaEncode(stream, x.data_ptr(), fast.data_ptr(), exact.data_ptr(),
                                                    x.numel()))
        torch.cuda.synchronize()
        bad = (fast != exact).nonzero()
        assert bad.numel() == 0, f"{bad.numel()} mismatches, first a={x[bad[0]].item()!r}"
    # a*255+0.5 just below / at each integer, and random values: the oracle agrees
    k = np.arange(256, dtype=np.float32)
    edges = ((k + np.float32(0.5)) / np.float32(255)).astype(np.float32)
    xs = np.concatenate([np.random.default_rng(2).random(1 << 14, dtype=np.float32),
                         np.nextafter(edges, 0, dtype=np.float32), edges, np.nextafter(edges, 2, dtype=np.float32)])
    xs = np.clip(xs, 0, 1).astype(np.float32)
    xt = torch.from_numpy(xs).to(cuda)
    fast = torch.empty(xs.size, dtype=torch.uint8, device=cuda)
    exact = torch.empty_like(fast)
    N.check(native.nvproPyramidDebugAlphaEncode(stream, xt.data_ptr(), fast.data_ptr(), exact.data_ptr(), xs.size))
    torch.cuda.synchronize()
    want = np.array([O.orc().orc_alpha_encode(float(v)) for v in xs], np.uint8)
    assert np.array_equal(exact.cpu().numpy(), want)
    assert np.array_equal(fast.cpu().numpy(), want)


def test_no_device_wait_gave_up(cuda, native):
    import torch
    cmd = P.Cmd()
    chain = P.MipChain(4096, 4096, N.PRESET_SRGBA8, device=cuda)
    chain.storage.random_(0, 256)
    P.generate(chain, cmd=cmd)
    N.check(native.nvproPyramidCmdDeviceStatus(cmd.handle), "device status")
    torch.cuda.synchronize()


@pytest.mark.parametrize("w,h,bands", [(16384, 16384, 8), (1920, 1080, 8), (2052, 2052, 5), (2048, 512, 3),
                                       (4095, 4095, 8), (64, 64, 8)])
def test_generate_from_host_equals_device_path(cuda, w, h, bands):
    """Banded host copies overlapped with the chain write the bytes of
    copy-in + generate + copy-out (the fast first dispatch is tile-local)."""
    import torch
    chain = P.MipChain(w, h, N.PRESET_SRGBA8, device=cuda)
    n0 = chain.offsets[1]
    g = torch.Generator().manual_seed(w + h)
    base_host = torch.randint(0, 256, (n0,), generator=g, dtype=torch.uint8).pin_memory()
    out_host = torch.full((chain.offsets[-1] - n0,), SENTINEL, dtype=torch.uint8).pin_memory()
    P.generate_from_host(chain, base_host, out_host, bands=bands)
    torch.cuda.synchronize()
    ref = P.MipChain(w, h, N.PRESET_SRGBA8, device=cuda)
    ref.storage[:n0].copy_(base_host)
    P.generate(ref)
    torch.cuda.synchronize()
    assert torch.equal(out_host, ref.storage[n0:].cpu())
    assert torch.equal(chain.storage[:n0].cpu(), base_host)


# The reference's own correctness check (-test, demo_app/app_args.cpp:24-26;
# mipmaps_app.cpp:233-238): the GPU pyramid against cpuGenerateMipmaps_sRGBA,
# worst per-channel delta over levels >= 1, on one size per code path of
# docs/test_images.txt.  The reference reports 2 on opaque images and 4-5 with
# alpha (demo_app/rtx3090.json); seeded smooth fields stand in for its images.
@pytest.mark.parametrize("w,h", [(1920, 1080), (2560, 1440), (3840, 2160), (2052, 2052), (4094, 4094),
                                 (4095, 4095), (2047, 2047), (4096, 4096), (2048, 2048)])
def test_worst_delta_vs_reference_cpu_generator(cuda, w, h):
    from vk_compute_mipmaps_gb300.workloads import smooth_field
    for opaque, bar in ((True, 2), (False, 5)):
        base = smooth_field(w, h, w * 13 + h + opaque, opaque)
        got, _, _ = gpu_run(cuda, N.PRESET_SRGBA8, base)
        delta = O.worst_delta(got, O.refcpu(base), w, h)
        print(f"{w}x{h} {'opaque' if opaque else 'alpha'}: worst delta {delta}")
        assert delta <= bar, (w, h, opaque, delta)
