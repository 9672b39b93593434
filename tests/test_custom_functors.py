"""Custom pipelines from device-functor sets (include/nvpro_pyramid_cuda.hpp):
the reference's customisation macros (nvpro_pyramid.glsl:27-120) as C++
types.  tests/custom_functors.cu defines two sets that are no preset of the
library -- a max depth pyramid (one FP32 channel, REDUCE only) and RGBA 16-bit
unorm (REDUCE only, REDUCE2 / REDUCE4 the reference's defaults) -- compiled
against the public header like a caller's own code; the GPU results are
compared with restatements of the same semantics: numpy for the maximum
(exact, schedule-independent), the oracle's RGBA16-unorm format for the other
(bit-exact, the reference's schedule)."""
import ctypes
import subprocess
from pathlib import Path

import numpy as np
import pytest

import _oracle as O
from vk_compute_mipmaps_gb300 import _build as B
from vk_compute_mipmaps_gb300 import _native as N
from vk_compute_mipmaps_gb300 import pyramid as P

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "custom_functors.cu"
OUT = ROOT / "tests" / ".tmp" / "custom" / "libcustom_functors.so"


@pytest.fixture(scope="session")
def custom(native):
    """The functor sets built into a shared library that links the pyramid
    library (as an application's own CUDA code would)."""
    if not OUT.exists() or OUT.stat().st_mtime < max(SRC.stat().st_mtime, N.LIB_PATH.stat().st_mtime):
        OUT.parent.mkdir(parents=True, exist_ok=True)
        cmd = [B.nvcc(), *B.ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-I", str(ROOT / "include"),
               str(SRC), "-L", str(N.LIB_PATH.parent), "-lnvpro_pyramid_cuda",
               f"-Xlinker=-rpath={N.LIB_PATH.parent}", "-o", str(OUT)]
        subprocess.run(cmd, check=True, capture_output=True)
    lib = ctypes.CDLL(str(OUT))
    lib.customCreatePipelines.restype = ctypes.c_int
    lib.customCreatePipelines.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p)]
    return lib


def make_pipelines(custom, which, fast=True):
    g, f = ctypes.c_void_p(), ctypes.c_void_p()
    N.check(custom.customCreatePipelines(which, ctypes.byref(g), ctypes.byref(f) if fast else None), "custom")
    return N.NvproPyramidPipelines(g.value, f.value if fast else None, None, 0), (g, f)


def test_custom_functor_library_builds_and_exports(custom):
    """The public header instantiates for non-preset functor sets (CPU: nvcc
    cross-compiles; no kernel runs)."""
    assert hasattr(custom, "customCreatePipelines")


def max_pyramid(base: np.ndarray) -> list:
    """Maximum over each level's footprint: kernel sizes 1..3 per axis from
    the level above (kernelSizeFromInputSize_, nvpro_pyramid.glsl:557-561)."""
    levels = [base]
    while levels[-1].shape[0] > 1 or levels[-1].shape[1] > 1:
        a = levels[-1]
        h, w = a.shape
        kx, ky = (1 if w == 1 else 2 | (w & 1)), (1 if h == 1 else 2 | (h & 1))
        nh, nw = max(h >> 1, 1), max(w >> 1, 1)
        out = np.full((nh, nw), -np.inf, np.float32)
        for dy in range(ky):
            for dx in range(kx):
                out = np.maximum(out, a[dy:dy + 2 * nh:2, dx:dx + 2 * nw:2][:nh, :nw])
        levels.append(out)
    return levels


def run_custom(cuda, pipes, w, h, bpp, base_bytes):
    import torch
    preset = {4: N.PRESET_SRGBA8, 8: N.PRESET_RGBA16F}[bpp]  # only for the packed layout's texel size
    chain = P.MipChain(w, h, preset, device=cuda)
    chain.storage.fill_(0xA7)
    chain.storage[:chain.offsets[1]].copy_(torch.from_numpy(base_bytes))
    cmd = P.Cmd(0)
    img = chain.image()
    stream = torch.cuda.current_stream(cuda).cuda_stream
    N.check(N.load().nvproPyramidGenerate(cmd.handle, stream, pipes, ctypes.byref(img), 0), "generate")
    torch.cuda.synchronize()
    return chain.storage.cpu().numpy(), chain.offsets, cmd


SIZES = [(64, 64), (256, 128), (1920, 1080), (2052, 2052), (1023, 777), (4095, 63), (1, 37), (300, 201), (5, 1)]


@pytest.mark.gpu
@pytest.mark.parametrize("fast", [True, False], ids=["fast+general", "general-only"])
@pytest.mark.parametrize("w,h", SIZES)
def test_custom_max_depth_pyramid(custom, cuda, w, h, fast):
    pipes, _keep = make_pipelines(custom, 0, fast)
    base = np.random.default_rng(w * 7 + h).random((h, w), dtype=np.float32)
    got, off, cmd = run_custom(cuda, pipes, w, h, 4, base.view(np.uint8).reshape(-1))
    want = max_pyramid(base)
    for k, lv in enumerate(want):
        assert np.array_equal(got[off[k]:off[k + 1]].view(np.float32).reshape(lv.shape), lv), (w, h, k)
    recs = cmd.records()
    assert all(r["preset"] == 0x100 for r in recs)
    assert any(r["isFastPipeline"] for r in recs) == (fast and w % 4 == 0 and h % 4 == 0)


@pytest.mark.gpu
@pytest.mark.parametrize("w,h", SIZES)
def test_custom_rgba16_unorm_matches_oracle(custom, cuda, w, h):
    pipes, _keep = make_pipelines(custom, 1)
    base = np.random.default_rng(w + 13 * h).integers(0, 65536, (h, w, 4), dtype=np.uint16)
    got, off, _ = run_custom(cuda, pipes, w, h, 8, base.view(np.uint8).reshape(-1))
    want = O.pyramid(4, base)
    assert np.array_equal(got, want), (w, h)


def test_custom_pipeline_rejects_bad_arguments(native):
    pipe = ctypes.c_void_p()
    assert native.nvproPyramidCreateCustomPipeline(0, 8, None, None, ctypes.byref(pipe)) == N.ERROR_INVALID_ARGUMENT
    assert native.nvproPyramidCreateCustomPipeline(0, 0, ctypes.c_void_p(1), None, ctypes.byref(pipe)) == \
        N.ERROR_INVALID_ARGUMENT
