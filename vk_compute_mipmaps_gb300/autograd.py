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


_geometry_cache: dict = {}


def _geometry(W: int, H: int, levels: int, esz: int):
    """Per (W, H, levels, element size): the level sizes and the per-image
    byte stride of every level (cached: the same for every call of a
    training loop)."""
    key = (W, H, levels, esz)
    g = _geometry_cache.get(key)
    if g is None:
        sizes = level_sizes(W, H, levels)
        g = _geometry_cache[key] = (sizes, _strides(sizes, esz))
    return g


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


def forward_levels(base: torch.Tensor, levels: int = 0) -> list[torch.Tensor]:
    """Levels 1..n-1 of the pyramid of base ([B, H, W, 4]); no autograd.  One
    strided call: every dispatch is one launch over the B images."""
    b4 = base if base.dim() == 4 else base.unsqueeze(0)
    b4 = b4.contiguous()
    B, H, W, _ = b4.shape
    preset = _PRESETS[b4.dtype]
    sizes, strides = _geometry(W, H, levels, b4.element_size())
    # one tensor per level (views of one buffer would turn in-place changes of
    # a level into autograd errors)
    outs = [torch.empty((B, h, w, 4), dtype=b4.dtype, device=b4.device) for (w, h) in sizes[1:]]
    pipes, cmd = _objects(preset)
    lib = N.load()
    stream = torch.cuda.current_stream(b4.device).cuda_stream
    img = _image([b4.data_ptr()] + [o.data_ptr() for o in outs], W, H)
    N.check(lib.nvproPyramidGenerateStrided(cmd.handle, stream, pipes.struct, _ptr(img), _ptr(strides), B,
                                            len(sizes)),
            "nvproPyramidGenerateStrided")
    return outs


def adjoint(grads: list, shape, dtype, device, levels: int = 0) -> torch.Tensor:
    """Base gradient for upstream gradients of levels 0..n-1 (entries may be
    None), one strided nvproPyramidAdjoint call for the B images."""
    B, H, W, _ = shape
    preset = _PRESETS[dtype]
    sizes = _geometry(W, H, levels, _ELEMENT_BYTES[dtype])[0]
    lib = N.load()
    stream = torch.cuda.current_stream(device).cuda_stream
    ws_bytes = lib.nvproPyramidAdjointWorkspaceBytes(W, H, len(sizes)) * B
    ws = torch.empty(max(ws_bytes, 16), dtype=torch.uint8, device=device)
    # [B, h, w, 4] contiguous as they come from autograd; reshape only what is not
    grads = [g if g is None or (g.dim() == 4 and g.is_contiguous()) else g.reshape(B, *g.shape[-3:]).contiguous()
             for g in grads]
    out = torch.empty((B, H, W, 4), dtype=dtype, device=device)
    esz = out.element_size()
    img = _image([0 if g is None else g.data_ptr() for g in grads], W, H)
    strides = _strides(sizes, esz, [g is not None for g in grads])
    N.check(lib.nvproPyramidAdjointStrided(stream, preset, _ptr(img), _ptr(strides), out.data_ptr(), 0,
                                           H * W * 4 * esz, B, len(sizes), ws.data_ptr(), ws.numel()),
            "nvproPyramidAdjointStrided")
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
