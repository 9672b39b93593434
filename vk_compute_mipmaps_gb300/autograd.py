"""Differentiable linear image pyramid for PyTorch, over the same C ABI.

`pyramid(base)` returns levels 1..n-1 of the RGBA32F (float32) or RGBA16F
(float16 storage, FP32 arithmetic) pyramid of `base` ([B, H, W, 4] or
[H, W, 4], contiguous, on a CUDA device).  The forward pass is one
nvproPyramidGenerateStrided call and the backward pass one
nvproPyramidAdjointStrided call for all B images: the operator is linear, so
nothing of the forward pass is saved, and the base gradient is written once
per texel.
"""
from __future__ import annotations

import ctypes
import threading

import numpy as np
import torch

from . import _native as N
from .pyramid import Cmd, Pipelines, level_sizes

_PRESETS = {torch.float32: N.PRESET_RGBA32F, torch.float16: N.PRESET_RGBA16F}
_ELEMENT_BYTES = {torch.float32: 4, torch.float16: 2}
_tls = threading.local()
# The current stream's handle by device index without building a Stream
# object (a few microseconds per call otherwise).
_raw_stream = getattr(torch._C, "_cuda_getCurrentRawStream", None)


def _stream(device) -> int:
    if _raw_stream is not None:
        return _raw_stream(device.index if device.index is not None else torch.cuda.current_device())
    return torch.cuda.current_stream(device).cuda_stream


def _objects(preset: int):
    cache = getattr(_tls, "objs", None)
    if cache is None:
        cache = _tls.objs = {}
    if preset not in cache:
        cache[preset] = (Pipelines(preset), Cmd())
    return cache[preset]


def _check_base(base: torch.Tensor):
    if base.dtype not in _PRESETS:
        raise TypeError(f"pyramid needs float32 or float16 texels, got {base.dtype}")
    if not base.is_cuda or base.shape[-1] != 4 or base.dim() not in (3, 4):
        raise ValueError("base must be a CUDA tensor of shape [B, H, W, 4] or [H, W, 4]")


def _strides(sizes, esz: int, present=None) -> np.ndarray:
    """Bytes between images of each level of [B, h, w, 4] tensors (0 where
    present[k] is False), from the level sizes alone."""
    arr = np.zeros(N.MAX_LEVELS, np.uint64)
    for k, (w, h) in enumerate(sizes):
        if present is None or present[k]:
            arr[k] = w * h * 4 * esz
    return arr


def _image(ptrs, w: int, h: int) -> np.ndarray:
    """An NvproPyramidImage (packed rows) as raw words, filled without
    per-field ctypes assignments: {w, h, levelCount, 0}, levels[32], pitches[32]."""
    img = np.zeros(2 + 2 * N.MAX_LEVELS, np.uint64)
    img[0] = w | (h << 32)
    img[1] = len(ptrs)
    img[2:2 + len(ptrs)] = ptrs
    return img


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class _Plan:
    """Everything a call for one geometry (device, dtype, B, H, W, levels)
    needs besides the tensors' addresses, made once per thread: level sizes
    and shapes, per-image strides, the image structs to fill with addresses,
    the adjoint's workspace (one per stream: launches on one stream are
    ordered, so the calls on it may share it)."""

    def __init__(self, device, dtype, B: int, H: int, W: int, levels: int):
        self.lib = N.load()
        self.preset = _PRESETS[dtype]
        self.pipes, self.cmd = _objects(self.preset)
        self.pipes_struct = self.pipes.struct  # by value in every call
        self.esz = _ELEMENT_BYTES[dtype]
        self.sizes = level_sizes(W, H, levels)
        self.n = len(self.sizes)
        self.shapes = [(B, h, w, 4) for (w, h) in self.sizes]
        self.strides = _strides(self.sizes, self.esz)
        self.strides_ptr = _ptr(self.strides)
        self.img = _image([0] * self.n, W, H)
        self.img_ptr = _ptr(self.img)
        self.adj_img = _image([0] * self.n, W, H)
        self.adj_img_ptr = _ptr(self.adj_img)
        self.adj_strides = {}  # present-pattern -> (array, pointer)
        self.ws_bytes = max(int(self.lib.nvproPyramidAdjointWorkspaceBytes(W, H, self.n)) * B, 16)
        self.ws = {}  # stream -> workspace tensor
        self.base_stride = H * W * 4 * self.esz

    def workspace(self, stream: int, device):
        ws = self.ws.get(stream)
        if ws is None:
            ws = self.ws[stream] = torch.empty(self.ws_bytes, dtype=torch.uint8, device=device)
        return ws

    def adjoint_strides(self, present: tuple):
        e = self.adj_strides.get(present)
        if e is None:
            arr = _strides(self.sizes, self.esz, present)
            e = self.adj_strides[present] = (arr, _ptr(arr))
        return e[1]


def _plan(device, dtype, B: int, H: int, W: int, levels: int) -> _Plan:
    """The calling thread's plan for a geometry (a plan holds the thread's
    command object and image arrays it rewrites per call)."""
    plans = getattr(_tls, "plans", None)
    if plans is None:
        plans = _tls.plans = {}
    key = (device, dtype, B, H, W, levels)
    p = plans.get(key)
    if p is None:
        p = plans[key] = _Plan(device, dtype, B, H, W, levels)
    return p


def forward_levels(base: torch.Tensor, levels: int = 0) -> list[torch.Tensor]:
    """Levels 1..n-1 of the pyramid of base ([B, H, W, 4]); no autograd.  One
    strided call: every dispatch is one launch over the B images."""
    b4 = base if base.dim() == 4 else base.unsqueeze(0)
    b4 = b4.contiguous()
    B, H, W, _ = b4.shape
    device, dtype = b4.device, b4.dtype
    p = _plan(device, dtype, B, H, W, levels)
    # one tensor per level (views of one buffer would turn in-place changes of
    # a level into autograd errors)
    outs = [torch.empty(s, dtype=dtype, device=device) for s in p.shapes[1:]]
    p.img[2:2 + p.n] = [b4.data_ptr()] + [o.data_ptr() for o in outs]
    stream = _stream(device)
    rc = p.lib.nvproPyramidGenerateStrided(p.cmd.handle, stream, p.pipes_struct, p.img_ptr, p.strides_ptr, B, p.n)
    if rc:
        N.check(rc, "nvproPyramidGenerateStrided")
    return outs


def adjoint(grads: list, shape, dtype, device, levels: int = 0) -> torch.Tensor:
    """Base gradient for upstream gradients of levels 0..n-1 (entries may be
    None), one strided nvproPyramidAdjoint call for the B images."""
    B, H, W, _ = shape
    p = _plan(device, dtype, B, H, W, levels)
    stream = _stream(device)
    # [B, h, w, 4] contiguous as they come from autograd; reshape only what is not
    grads = [g if g is None or (g.dim() == 4 and g.is_contiguous()) else g.reshape(B, *g.shape[-3:]).contiguous()
             for g in grads]
    out = torch.empty(p.shapes[0], dtype=dtype, device=device)
    p.adj_img[2:2 + p.n] = [0 if g is None else g.data_ptr() for g in grads]
    strides_ptr = p.adjoint_strides(tuple(g is not None for g in grads))
    ws = p.workspace(stream, device)
    rc = p.lib.nvproPyramidAdjointStrided(stream, p.preset, p.adj_img_ptr, strides_ptr, out.data_ptr(), 0,
                                          p.base_stride, B, p.n, ws.data_ptr(), p.ws_bytes)
    if rc:
        N.check(rc, "nvproPyramidAdjointStrided")
    return out


class PyramidFunction(torch.autograd.Function):
    """levels 1..n-1 (or 0..n-1) = pyramid(base); backward = nvproPyramidAdjoint."""

    @staticmethod
    def forward(ctx, base: torch.Tensor, levels: int, with_base: bool):
        _check_base(base)
        ctx.squeeze = base.dim() == 3
        ctx.with_base = with_base
        b4 = base if base.dim() == 4 else base.unsqueeze(0)
        ctx.shape, ctx.dtype, ctx.device, ctx.levels = tuple(b4.shape), b4.dtype, b4.device, levels
        outs = forward_levels(b4, levels)
        if ctx.squeeze:
            outs = [o[0] for o in outs]
        # level 0 is the input itself (autograd makes it an alias whose
        # gradient comes to backward, so the adjoint adds it in-kernel)
        return tuple([base] + outs) if with_base else tuple(outs)

    @staticmethod
    @torch.autograd.function.once_differentiable
    def backward(ctx, *grads):
        g = list(grads) if ctx.with_base else [None] + list(grads)
        out = adjoint(g, ctx.shape, ctx.dtype, ctx.device, ctx.levels)
        return (out[0] if ctx.squeeze else out), None, None


def pyramid(base: torch.Tensor, levels: int = 0, with_base: bool = False) -> list[torch.Tensor]:
    """Differentiable levels 1..n-1 of the linear pyramid of `base`; with
    `with_base`, levels 0..n-1 (level 0 an alias of `base`), so that a loss on
    every level costs one adjoint pass (the level-0 gradient is added in the
    kernel instead of by a separate accumulation)."""
    return list(PyramidFunction.apply(base, levels, with_base))
