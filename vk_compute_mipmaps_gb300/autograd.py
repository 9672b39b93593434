"""Differentiable linear image pyramid for PyTorch, over the same C ABI.

`pyramid(base)` returns levels 1..n-1 of the RGBA32F (float32) or RGBA16F
(float16 storage, FP32 arithmetic) pyramid of `base` ([B, H, W, 4] or
[H, W, 4], contiguous, on a CUDA device).  The backward pass calls
nvproPyramidAdjoint: the operator is linear, so nothing of the forward pass is
saved, and the base gradient is written once per texel.
"""
from __future__ import annotations

import ctypes
import threading

import torch

from . import _native as N
from .pyramid import Cmd, Pipelines, level_sizes, make_image

_PRESETS = {torch.float32: N.PRESET_RGBA32F, torch.float16: N.PRESET_RGBA16F}
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


def forward_levels(base: torch.Tensor, levels: int = 0) -> list[torch.Tensor]:
    """Levels 1..n-1 of the pyramid of base ([B, H, W, 4]); no autograd."""
    b4 = base if base.dim() == 4 else base.unsqueeze(0)
    b4 = b4.contiguous()
    B, H, W, _ = b4.shape
    preset = _PRESETS[b4.dtype]
    sizes = level_sizes(W, H, levels)
    outs = [torch.empty((B, h, w, 4), dtype=b4.dtype, device=b4.device) for (w, h) in sizes[1:]]
    pipes, cmd = _objects(preset)
    lib = N.load()
    stream = torch.cuda.current_stream(b4.device).cuda_stream
    for i in range(B):
        img = make_image([b4[i].data_ptr()] + [o[i].data_ptr() for o in outs], W, H)
        N.check(lib.nvproPyramidGenerate(cmd.handle, stream, pipes.struct, ctypes.byref(img), len(sizes)),
                "nvproPyramidGenerate")
    return outs


def adjoint(grads: list, shape, dtype, device, levels: int = 0) -> torch.Tensor:
    """Base gradient for upstream gradients of levels 0..n-1 (entries may be None)."""
    B, H, W, _ = shape
    preset = _PRESETS[dtype]
    sizes = level_sizes(W, H, levels)
    lib = N.load()
    stream = torch.cuda.current_stream(device).cuda_stream
    ws_bytes = lib.nvproPyramidAdjointWorkspaceBytes(W, H, len(sizes))
    ws = torch.empty(max(ws_bytes, 16), dtype=torch.uint8, device=device)
    grads = [None if g is None else g.reshape(B, *g.shape[-3:]).contiguous() for g in grads]
    out = torch.empty((B, H, W, 4), dtype=dtype, device=device)
    for i in range(B):
        ptrs = [0 if g is None else g[i].data_ptr() for g in grads]
        img = make_image(ptrs, W, H)
        N.check(lib.nvproPyramidAdjoint(stream, preset, ctypes.byref(img), out[i].data_ptr(), 0, len(sizes),
                                        ws.data_ptr(), ws.numel()), "nvproPyramidAdjoint")
    return out


class PyramidFunction(torch.autograd.Function):
    """levels 1..n-1 = pyramid(base); backward = nvproPyramidAdjoint."""

    @staticmethod
    def forward(ctx, base: torch.Tensor, levels: int):
        _check_base(base)
        ctx.squeeze = base.dim() == 3
        b4 = base if base.dim() == 4 else base.unsqueeze(0)
        ctx.shape, ctx.dtype, ctx.device, ctx.levels = tuple(b4.shape), b4.dtype, b4.device, levels
        outs = forward_levels(b4, levels)
        if ctx.squeeze:
            outs = [o[0] for o in outs]
        return tuple(outs)

    @staticmethod
    def backward(ctx, *grads):
        # the base level is the input itself: its own upstream gradient is
        # added by autograd, so level 0 enters the adjoint as zero
        g = [None] + list(grads)
        out = adjoint(g, ctx.shape, ctx.dtype, ctx.device, ctx.levels)
        return (out[0] if ctx.squeeze else out), None


def pyramid(base: torch.Tensor, levels: int = 0) -> list[torch.Tensor]:
    """Differentiable levels 1..n-1 of the linear pyramid of `base`."""
    return list(PyramidFunction.apply(base, levels))
