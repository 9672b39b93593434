"""Python mirror of the nvpro_pyramid host interface over the C ABI.

Names follow nvpro_pyramid/nvpro_pyramid_dispatch.hpp: Pipelines is
NvproPyramidPipelines, Cmd is the command buffer that nvproCmdPyramidDispatch
records into, and cmd_pyramid_dispatch is nvproCmdPyramidDispatch itself.
MipChain is a convenience for torch users: a packed device allocation in the
layout of include/mipmap_storage.hpp:53-76 (levels contiguous, each [y][x]).
"""
from __future__ import annotations

import ctypes
import threading
from typing import Callable, Optional, Sequence

from . import _native as N

PRESET_BYTES = {N.PRESET_SRGBA8: 4, N.PRESET_RGBA32F: 16, N.PRESET_RGBA16F: 8}


def full_level_count(width: int, height: int) -> int:
    """floor(log2(max(w, h))) + 1 (nvpro_pyramid_dispatch.hpp:122-132)."""
    m = 0
    while width or height:
        width >>= 1
        height >>= 1
        m += 1
    return m


def level_sizes(width: int, height: int, levels: int = 0) -> list[tuple[int, int]]:
    levels = levels or full_level_count(width, height)
    return [(max(width >> k, 1), max(height >> k, 1)) for k in range(levels)]


def packed_offsets(width: int, height: int, levels: int, bytes_per_texel: int) -> list[int]:
    """Byte offset of each level in the packed layout, plus the total size."""
    offs, o = [], 0
    for w, h in level_sizes(width, height, levels):
        offs.append(o)
        o += w * h * bytes_per_texel
    return offs + [o]


class Pipelines:
    """NvproPyramidPipelines of one preset (nvpro_pyramid_dispatch.hpp:29-35)."""

    def __init__(self, preset: int = N.PRESET_SRGBA8, fast: bool = True, general_config: int = 0,
                 fast_config: int = 0):
        """general_config / fast_config: NVPRO_PYRAMID_CONFIG_* bits of each
        pipeline (CONFIG_SRGB_SHARED, CONFIG_F16_SHARED, CONFIG_NO_BILINEAR),
        as the reference demo's per-pipeline config bits
        (demo_app/pipeline_alternative.cpp:25-32)."""
        lib = N.load()
        self.preset = preset
        self._general = ctypes.c_void_p()
        self._fast = ctypes.c_void_p()
        N.check(lib.nvproPyramidCreatePipelineEx(preset, 0, general_config, ctypes.byref(self._general)),
                "create general pipeline")
        if fast:
            N.check(lib.nvproPyramidCreatePipelineEx(preset, 1, fast_config, ctypes.byref(self._fast)),
                    "create fast pipeline")

    @property
    def struct(self) -> N.NvproPyramidPipelines:
        return N.NvproPyramidPipelines(self._general.value, self._fast.value, None, 0)

    @property
    def general(self) -> Optional[int]:
        return self._general.value

    @property
    def fast(self) -> Optional[int]:
        return self._fast.value

    def close(self) -> None:
        lib = N.load()
        for h in (self._general, self._fast):
            if h.value:
                lib.nvproPyramidDestroyPipeline(h)
                h.value = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def make_image(levels: Sequence[int], width: int, height: int,
               pitches: Optional[Sequence[int]] = None) -> N.NvproPyramidImage:
    """NvproPyramidImage from per-level device addresses (and row pitches)."""
    img = N.NvproPyramidImage()
    img.width, img.height, img.levelCount = width, height, len(levels)
    for k, ptr in enumerate(levels):
        img.levels[k] = ptr
        img.rowPitchBytes[k] = pitches[k] if pitches else 0
    return img


class Cmd:
    """Command recorder bound to a CUDA stream (VkCommandBuffer analogue)."""

    def __init__(self, flags: int = 0):
        self._lib = N.load()
        self._h = ctypes.c_void_p()
        N.check(self._lib.nvproPyramidCreateCmd(flags, ctypes.byref(self._h)), "create command")
        self._keep: list = []

    @property
    def handle(self) -> int:
        return self._h.value

    def begin(self, stream: Optional[int] = None) -> "Cmd":
        """stream: a cudaStream_t as an int (e.g. torch.cuda.current_stream().cuda_stream)."""
        self._keep = []
        N.check(self._lib.nvproPyramidBeginCmd(self._h, stream), "begin")
        return self

    def bind_image(self, image: N.NvproPyramidImage) -> None:
        self._keep.append(image)
        N.check(self._lib.nvproPyramidCmdBindImage(self._h, ctypes.byref(image)), "bind image")

    def bind_pipeline(self, pipeline: int) -> None:
        N.check(self._lib.nvproPyramidCmdBindPipeline(self._h, pipeline), "bind pipeline")

    def push_constant(self, value: int) -> None:
        v = ctypes.c_uint32(value)
        N.check(self._lib.nvproPyramidCmdPushConstants(self._h, None, 0, 4, ctypes.byref(v)), "push constant")

    def dispatch(self, gx: int, gy: int = 1, gz: int = 1) -> None:
        N.check(self._lib.nvproPyramidCmdDispatch(self._h, gx, gy, gz), "dispatch")

    def barrier(self) -> None:
        N.check(self._lib.nvproPyramidCmdPipelineBarrier(self._h), "barrier")

    def end(self) -> None:
        N.check(self._lib.nvproPyramidEndCmd(self._h), "end")

    def records(self) -> list[dict]:
        n = self._lib.nvproPyramidCmdRecordCount(self._h)
        arr = (N.NvproPyramidDispatchRecord * max(n, 1))()
        N.check(self._lib.nvproPyramidCmdGetRecords(self._h, arr, n), "records")
        return [{f: getattr(arr[i], f) for f, _ in N.NvproPyramidDispatchRecord._fields_} for i in range(n)]

    @property
    def launch_count(self) -> int:
        return self._lib.nvproPyramidCmdLaunchCount(self._h)

    def close(self) -> None:
        if self._h.value:
            self._lib.nvproPyramidDestroyCmd(self._h)
            self._h.value = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


Dispatcher = Callable[[int, Optional[int], int, Optional[int], N.NvproPyramidState], int]


def wrap_dispatcher(fn: Dispatcher):
    """Turn fn(cmd, layout, push_constant_offset, pipeline_if_needed, state) into a C callback."""

    def trampoline(cmd, layout, pco, pipeline, state_ptr):
        return int(fn(cmd, layout, pco, pipeline, state_ptr.contents))

    return N.DISPATCHER(trampoline)


def cmd_pyramid_dispatch(cmd: Cmd, pipelines: Pipelines, width: int, height: int, mip_levels: int = 0,
                         general=None, fast=None) -> None:
    """nvproCmdPyramidDispatch (nvpro_pyramid_dispatch.hpp:54-59, :109-188).

    general / fast: optional dispatcher callbacks, either Python callables
    (see wrap_dispatcher) or ctypes function pointers of the library's own
    dispatchers; None selects the defaults.
    """
    lib = N.load()
    if general is None and fast is None:
        N.check(lib.nvproCmdPyramidDispatch(cmd.handle, pipelines.struct, width, height, mip_levels),
                "nvproCmdPyramidDispatch")
        return
    g = general if general is not None else N.DISPATCHER(("nvproPyramidDefaultGeneralDispatcher", lib))
    f = fast if fast is not None else N.DISPATCHER(("nvproPyramidDefaultFastDispatcher", lib))
    g = wrap_dispatcher(g) if callable(g) and not isinstance(g, ctypes._CFuncPtr) else g
    f = wrap_dispatcher(f) if callable(f) and not isinstance(f, ctypes._CFuncPtr) else f
    cmd._keep += [g, f]
    N.check(lib.nvproCmdPyramidDispatchEx(cmd.handle, pipelines.struct, width, height, mip_levels, g, f),
            "nvproCmdPyramidDispatchEx")


def blit_general_dispatcher():
    """The library's nvproPyramidBlitGeneralDispatcher as a dispatcher
    callback: with it as the general dispatcher, cmd_pyramid_dispatch is the
    demo's "generalblit" mode (fast pipeline where possible, else a linear
    blit of one level)."""
    return N.DISPATCHER(("nvproPyramidBlitGeneralDispatcher", N.load()))


# ---------------------------------------------------------------------------
# torch convenience: packed mip chains on the GPU.

_DTYPES = {N.PRESET_SRGBA8: "uint8", N.PRESET_RGBA32F: "float32", N.PRESET_RGBA16F: "float16"}


class MipChain:
    """A packed mip chain in device memory: `storage` is a flat uint8 tensor."""

    def __init__(self, width: int, height: int, preset: int = N.PRESET_SRGBA8, levels: int = 0,
                 device="cuda", storage=None):
        import torch
        self.width, self.height, self.preset = width, height, preset
        self.levels = levels or full_level_count(width, height)
        self.bpp = PRESET_BYTES[preset]
        self.offsets = packed_offsets(width, height, self.levels, self.bpp)
        if storage is None:
            storage = torch.empty(self.offsets[-1], dtype=torch.uint8, device=device)
        assert storage.dtype == torch.uint8 and storage.numel() >= self.offsets[-1]
        self.storage = storage

    def level(self, k: int):
        """Level k as a [h, w, 4] tensor view of the preset's dtype."""
        import torch
        w, h = level_sizes(self.width, self.height, self.levels)[k]
        raw = self.storage[self.offsets[k]:self.offsets[k + 1]]
        return raw.view(getattr(torch, _DTYPES[self.preset])).view(h, w, 4)

    def image(self) -> N.NvproPyramidImage:
        base = self.storage.data_ptr()
        return make_image([base + o for o in self.offsets[:-1]], self.width, self.height)


_tls = threading.local()


def _defaults(preset: int, flags: int):
    key = (preset, flags)
    cache = getattr(_tls, "cache", None)
    if cache is None:
        cache = _tls.cache = {}
    if key not in cache:
        cache[key] = (Pipelines(preset), Cmd(flags))
    return cache[key]


def generate(chain: MipChain, stream: Optional[int] = None, mip_levels: int = 0, flags: int = 0,
             pipelines: Optional[Pipelines] = None, cmd: Optional[Cmd] = None) -> int:
    """Fill levels 1.. of `chain` from level 0 on `stream` (default: torch's
    current stream).  Returns the number of kernels launched."""
    import torch
    if stream is None:
        stream = torch.cuda.current_stream(chain.storage.device).cuda_stream
    p, c = _defaults(chain.preset, flags)
    pipelines = pipelines or p
    cmd = cmd or c
    img = chain.image()
    lib = N.load()
    N.check(lib.nvproPyramidGenerate(cmd.handle, stream, pipelines.struct, ctypes.byref(img),
                                     mip_levels or chain.levels), "nvproPyramidGenerate")
    return cmd.launch_count


def write_levels_tga(chain: "MipChain", base_filename: str, levels: int = 0) -> None:
    """Write the levels of an sRGBA8 chain to TGA files (level 0 to
    base_filename, level k to base_filename with ".k" before the extension),
    as the reference's writeMipmapsTga does.  Copies the chain to the host."""
    import numpy as np
    if chain.preset != N.PRESET_SRGBA8:
        raise ValueError("TGA output exists for the sRGBA8 preset only")
    host = np.ascontiguousarray(chain.storage.cpu().numpy())
    N.check(N.load().nvproPyramidWriteLevelsTga(str(base_filename).encode(), host.ctypes.data, chain.width,
                                                 chain.height, levels or chain.levels), "write levels")


def read_tga(path: str):
    """A 24/32-bit TGA file as a [h, w, 4] uint8 numpy array (RGBA, top row first)."""
    import numpy as np
    lib = N.load()
    w, h = ctypes.c_uint32(), ctypes.c_uint32()
    N.check(lib.nvproPyramidReadTga(str(path).encode(), None, 0, ctypes.byref(w), ctypes.byref(h)), "read TGA")
    out = np.empty((h.value, w.value, 4), np.uint8)
    N.check(lib.nvproPyramidReadTga(str(path).encode(), out.ctypes.data, out.nbytes, ctypes.byref(w),
                                    ctypes.byref(h)), "read TGA")
    return out


def write_tga(path: str, rgba) -> None:
    """Write a [h, w, 4] uint8 array (numpy or a CPU/CUDA tensor) as a TGA file."""
    import numpy as np
    a = rgba.cpu().numpy() if hasattr(rgba, "cpu") else rgba
    a = np.ascontiguousarray(a, dtype=np.uint8)
    if a.ndim != 3 or a.shape[2] != 4:
        raise ValueError("expected [h, w, 4] uint8")
    N.check(N.load().nvproPyramidWriteTga(str(path).encode(), a.ctypes.data, a.shape[1], a.shape[0], 0),
            "write TGA")


_copy_streams_cache: dict = {}


def _copy_streams(dev):
    """Two side streams per device for host copies (created once)."""
    import torch
    key = (threading.get_ident(), str(dev))
    if key not in _copy_streams_cache:
        _copy_streams_cache[key] = (torch.cuda.Stream(dev), torch.cuda.Stream(dev))
    return _copy_streams_cache[key]


def _first_fast_levels(w: int, h: int, levels: int) -> int:
    """Levels of the first dispatch if the default schedule starts with a fast
    dispatch (nvproPyramidDefaultFastDispatcher<4, 6>: both sizes divisible by
    4, as many halvings as both stay even, at most 6), else 0."""
    if w % 4 or h % 4:
        return 0
    n = 0
    while w % 2 == 0 and h % 2 == 0 and n < levels - 1 and n < 6:
        w, h, n = w // 2, h // 2, n + 1
    return n


def _sub_image(chain: "MipChain", first: int, count: int, row0: int, rows: int) -> N.NvproPyramidImage:
    """Levels first..first+count-1 of `chain` restricted to level-`first` rows
    [row0, row0 + rows) (row ranges of the deeper levels scale by 2^k)."""
    sizes = level_sizes(chain.width, chain.height, chain.levels)
    base = chain.storage.data_ptr()
    ptrs, pitches = [], []
    for k in range(first, first + count):
        w = sizes[k][0]
        pitch = w * chain.bpp
        ptrs.append(base + chain.offsets[k] + (row0 >> (k - first)) * pitch)
        pitches.append(pitch)
    return make_image(ptrs, sizes[first][0], rows, pitches)


def premultiply_alpha(src, dst=None, stream: Optional[int] = None):
    """Premultiplied-alpha staging of an sRGBA8 image on the GPU
    (nvproPyramidPremultiplyAlpha): `src` is a CUDA uint8 tensor [h, w, 4]
    (rows may be strided); the result goes to `dst` (same shape; default:
    in place) and is returned."""
    import torch
    if src.dtype != torch.uint8 or src.dim() != 3 or src.shape[2] != 4 or not src.is_cuda:
        raise ValueError("expected a CUDA uint8 tensor [h, w, 4]")
    dst = src if dst is None else dst
    if dst.shape != src.shape or dst.dtype != torch.uint8 or not dst.is_cuda:
        raise ValueError("dst must match src")
    for t in (src, dst):
        if t.stride(2) != 1 or t.stride(1) != 4:
            raise ValueError("texels of a row must be contiguous")
    if stream is None:
        stream = torch.cuda.current_stream(src.device).cuda_stream
    h, w = src.shape[:2]
    N.check(N.load().nvproPyramidPremultiplyAlpha(stream, src.data_ptr(), src.stride(0), dst.data_ptr(),
                                                   dst.stride(0), w, h), "premultiply alpha")
    return dst


def generate_from_host(chain: "MipChain", host_base, host_levels, stream: Optional[int] = None,
                       bands: Optional[int] = None, flags: int = 0, premultiply: bool = False) -> None:
    """Level 0 from pinned host memory (`host_base`, chain.offsets[1] bytes),
    levels 1.. back to pinned host memory (`host_levels`, the rest of the
    packed chain), with the copies overlapped with the generation.

    When the chain starts with a fast dispatch of n levels, that dispatch is
    local to 2^n-row tiles, so level 0 goes in as row bands (multiples of 2^n
    rows): the band's dispatch runs while the next band is copied in and the
    previous band's levels 1..n are copied out; the remaining dispatches run
    on level n after the last band.  The dispatches, and so the bytes, are
    those of `generate` on the whole chain.  Otherwise: copy in, generate,
    copy out.  `bands` defaults to one per 32 MiB of level 0, at most 32
    (16384^2: 32 bands, 5.58 ms against 5.72 with 8 and 5.93 with 4; the host
    link's 210 GB/s make the upload alone 5.1 ms).  With `premultiply` (sRGBA8), each band of level 0 is
    premultiplied in place on the device right after its copy, as the
    reference's -do-premultiply-alpha staging does before the pyramid (the
    host copy of level 0 is left as it was).  Returns when the work is
    queued; `stream` (default: torch's current stream) waits for all of it."""
    import torch
    dev = chain.storage.device
    cur = torch.cuda.current_stream(dev) if stream is None else torch.cuda.ExternalStream(stream, device=dev)
    off = chain.offsets
    if bands is None:
        bands = max(1, min(32, off[1] >> 25))
    n = _first_fast_levels(chain.width, chain.height, chain.levels)
    rows_unit = 1 << n
    band_rows = -(-chain.height // max(bands, 1) // rows_unit) * rows_unit if n else chain.height
    if premultiply and chain.preset != N.PRESET_SRGBA8:
        raise ValueError("premultiplied alpha is an sRGBA8 staging step")
    lib = N.load()
    pitch0 = chain.width * chain.bpp

    def premultiply_rows(r0, rows):
        ptr = chain.storage.data_ptr() + r0 * pitch0
        N.check(lib.nvproPyramidPremultiplyAlpha(cur.cuda_stream, ptr, pitch0, ptr, pitch0, chain.width, rows),
                "premultiply alpha")

    if not n or bands <= 1 or band_rows >= chain.height:
        with torch.cuda.stream(cur):
            chain.storage[:off[1]].copy_(host_base, non_blocking=True)
        if premultiply:
            premultiply_rows(0, chain.height)
        generate(chain, stream=cur.cuda_stream, flags=flags)
        with torch.cuda.stream(cur):
            host_levels.copy_(chain.storage[off[1]:off[-1]], non_blocking=True)
        return
    p, c = _defaults(chain.preset, flags)
    copy_in, copy_out = _copy_streams(dev)
    copy_in.wait_stream(cur)
    copy_out.wait_stream(cur)
    sizes = level_sizes(chain.width, chain.height, chain.levels)
    r0 = 0
    while r0 < chain.height:
        rows = min(band_rows, chain.height - r0)
        a, b = r0 * pitch0, (r0 + rows) * pitch0
        with torch.cuda.stream(copy_in):
            chain.storage[a:b].copy_(host_base[a:b], non_blocking=True)
        cur.wait_stream(copy_in)
        if premultiply:
            premultiply_rows(r0, rows)
        img = _sub_image(chain, 0, n + 1, r0, rows)
        N.check(lib.nvproPyramidGenerate(c.handle, cur.cuda_stream, p.struct, ctypes.byref(img), n + 1),
                "nvproPyramidGenerate")
        copy_out.wait_stream(cur)
        with torch.cuda.stream(copy_out):
            for k in range(1, n + 1):
                pk = sizes[k][0] * chain.bpp
                lo, hi = off[k] + (r0 >> k) * pk, off[k] + ((r0 + rows) >> k) * pk
                host_levels[lo - off[1]:hi - off[1]].copy_(chain.storage[lo:hi], non_blocking=True)
        r0 += rows
    if n + 1 < chain.levels:  # the rest of the schedule, from level n
        img = _sub_image(chain, n, chain.levels - n, 0, sizes[n][1])
        N.check(lib.nvproPyramidGenerate(c.handle, cur.cuda_stream, p.struct, ctypes.byref(img), chain.levels - n),
                "nvproPyramidGenerate")
        copy_out.wait_stream(cur)
        with torch.cuda.stream(copy_out):
            host_levels[off[n + 1] - off[1]:].copy_(chain.storage[off[n + 1]:off[-1]], non_blocking=True)
    cur.wait_stream(copy_out)


class Batch:
    """Many sRGBA8 chains generated by one persistent launch
    (nvproPyramidCreateBatch / BatchBuild / BatchLaunch)."""

    def __init__(self, flags: int = 0, preset: int = N.PRESET_SRGBA8):
        self._lib = N.load()
        self._h = ctypes.c_void_p()
        N.check(self._lib.nvproPyramidCreateBatch(preset, flags, ctypes.byref(self._h)), "create batch")
        self._images = None

    def build(self, chains: Sequence["MipChain"], stream: Optional[int] = None, mip_levels: int = 0) -> None:
        import torch
        if stream is None:
            dev = chains[0].storage.device if chains else torch.device("cuda")
            stream = torch.cuda.current_stream(dev).cuda_stream
        arr = (N.NvproPyramidImage * max(len(chains), 1))()
        for i, c in enumerate(chains):
            arr[i] = c.image()
        self._images = arr  # the library copies them; kept for inspection
        N.check(self._lib.nvproPyramidBatchBuild(self._h, stream, arr, len(chains), mip_levels), "batch build")

    def set_strip_band(self, band: int) -> None:
        """Fix the general-pipeline unit size for the next build (0: default / autotuned)."""
        N.check(self._lib.nvproPyramidBatchSetStripBand(self._h, band), "batch strip band")

    def set_tuning(self, strip_band: int = 0, fast_region_rows: int = 0, threads_per_cta: int = 0) -> None:
        """Fix shape parameters of the next build (0 = default / autotuned)."""
        N.check(self._lib.nvproPyramidBatchSetTuning(self._h, strip_band, fast_region_rows, threads_per_cta),
                "batch tuning")

    def launch(self, stream: Optional[int] = None) -> None:
        import torch
        if stream is None:
            stream = torch.cuda.current_stream().cuda_stream
        N.check(self._lib.nvproPyramidBatchLaunch(self._h, stream), "batch launch")

    def info(self) -> dict:
        inf = N.NvproPyramidBatchInfo()
        N.check(self._lib.nvproPyramidBatchGetInfo(self._h, ctypes.byref(inf)), "batch info")
        return {name: getattr(inf, name) for name, _ in N.NvproPyramidBatchInfo._fields_}

    def device_status(self) -> None:
        N.check(self._lib.nvproPyramidBatchDeviceStatus(self._h), "batch device status")

    @property
    def handle(self):
        return self._h

    def close(self) -> None:
        if self._h.value:
            self._lib.nvproPyramidDestroyBatch(self._h)
            self._h.value = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pack_chains(sizes: Sequence[tuple], device="cuda", align: int = 256):
    """MipChains (sRGBA8) of the given (w, h) sizes in one device buffer, each
    starting on an `align`-byte boundary.  Returns (storage, chains)."""
    import torch
    offs, total = [], 0
    for w, h in sizes:
        offs.append(total)
        total += (packed_offsets(w, h, full_level_count(w, h), 4)[-1] + align - 1) // align * align
    storage = torch.empty(max(total, 1), dtype=torch.uint8, device=device)
    chains = []
    for (w, h), o in zip(sizes, offs):
        n = packed_offsets(w, h, full_level_count(w, h), 4)[-1]
        chains.append(MipChain(w, h, N.PRESET_SRGBA8, device=device, storage=storage[o:o + n]))
    return storage, chains
