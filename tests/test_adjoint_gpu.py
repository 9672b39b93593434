"""Adjoint of the linear float pyramids (nvproPyramidAdjoint and the
torch.autograd.Function over it) against FP64 references computed by the
CPU oracle: a dense FP64 adjoint (explicit impulse responses) on small sizes,
and FP64 central finite differences (eps 1e-3) on 64 random pixels."""
import ctypes

import numpy as np
import pytest

import _oracle as O
from vk_compute_mipmaps_gb300 import _native as N
from vk_compute_mipmaps_gb300 import pyramid as P

pytestmark = pytest.mark.gpu

RTOL = 1e-6  # max |error| / max |reference| for FP32 storage


def gpu_adjoint(torch, cuda, grads_np, w, h, dtype=np.float32):
    """nvproPyramidAdjoint for per-level upstream gradients (numpy, [h_k, w_k, 4])."""
    lib = N.load()
    preset = N.PRESET_RGBA32F if dtype == np.float32 else N.PRESET_RGBA16F
    tdt = torch.float32 if dtype == np.float32 else torch.float16
    gt = [torch.from_numpy(g.astype(dtype)).to(cuda) for g in grads_np]
    img = P.make_image([g.data_ptr() for g in gt], w, h)
    out = torch.empty((h, w, 4), dtype=tdt, device=cuda)
    n = len(grads_np)
    ws = torch.empty(max(lib.nvproPyramidAdjointWorkspaceBytes(w, h, n), 16), dtype=torch.uint8, device=cuda)
    N.check(lib.nvproPyramidAdjoint(torch.cuda.current_stream(cuda).cuda_stream, preset, ctypes.byref(img),
                                    out.data_ptr(), 0, n, ws.data_ptr(), ws.numel()), "adjoint")
    torch.cuda.synchronize()
    return out.float().cpu().numpy().astype(np.float64)


def impulse_response(w, h, x, y):
    """FP64 pyramid (one channel) of a unit impulse at (x, y): list of [h_k, w_k]."""
    base = np.zeros((h, w, 4))
    base[y, x, 0] = 1.0
    return [lvl[..., 0] for lvl in O.f64_pyramid(base)]


def dense_adjoint(grads, w, h):
    """sum_k M_k^T g_k in FP64 from the impulse responses of every texel."""
    out = np.zeros((h, w, 4))
    for y in range(h):
        for x in range(w):
            resp = impulse_response(w, h, x, y)
            for k, r in enumerate(resp):
                out[y, x] += np.tensordot(r, grads[k], axes=([0, 1], [0, 1]))
    return out


def rel_err(got, ref):
    return np.max(np.abs(got - ref)) / max(np.max(np.abs(ref)), 1e-30)


@pytest.mark.parametrize("w,h", [(1, 1), (2, 1), (1, 5), (5, 3), (7, 7), (16, 16), (17, 9), (33, 20), (50, 37),
                                 (64, 64)])
def test_adjoint_matches_dense_fp64(cuda, w, h):
    import torch
    rng = np.random.default_rng(w * 100 + h)
    sizes = P.level_sizes(w, h)
    grads = [rng.standard_normal((lh, lw, 4)) for lw, lh in sizes]
    ref = dense_adjoint(grads, w, h)
    got = gpu_adjoint(torch, cuda, grads, w, h)
    assert rel_err(got, ref) <= RTOL, (w, h, rel_err(got, ref))


def test_adjoint_fd_1023x777(cuda):
    """FP64 central differences (eps 1e-3) of L(x) = sum_k <g_k, level_k(x)>
    on 64 random pixels of a 1023x777 image (the 3x3 kernel on every level).
    L(p) - L(m) is summed as sum_k <g_k, level_k(p) - level_k(m)>: the same
    number, without cancelling two sums of ~4M terms, so the difference
    quotient carries ~1e-12 relative noise and the bar is 1e-6."""
    import torch
    w, h = 1023, 777
    rng = np.random.default_rng(7)
    base = rng.random((h, w, 4))
    sizes = P.level_sizes(w, h)
    grads = [rng.standard_normal((lh, lw, 4)) for lw, lh in sizes]
    got = gpu_adjoint(torch, cuda, grads, w, h)

    def loss_difference(a, b):
        return sum(float(np.sum(g * (la - lb))) for g, la, lb in zip(grads, O.f64_pyramid(a), O.f64_pyramid(b)))

    eps = 1e-3
    pix = rng.integers(0, [w, h, 4], size=(64, 3))
    fd = []
    for x, y, c in pix:
        p, m = base.copy(), base.copy()
        p[y, x, c] += eps
        m[y, x, c] -= eps
        fd.append(loss_difference(p, m) / (2 * eps))
    fd = np.array(fd)
    g = np.array([got[y, x, c] for x, y, c in pix])
    assert np.max(np.abs(g - fd)) / np.max(np.abs(fd)) <= 1e-6


def test_autograd_function_fp32(cuda):
    import torch

    from vk_compute_mipmaps_gb300.autograd import adjoint, pyramid
    B, H, W = 3, 64, 48
    g = torch.Generator(device=cuda).manual_seed(3)
    base = torch.rand((B, H, W, 4), generator=g, device=cuda, requires_grad=True)
    levels = pyramid(base)
    # forward values: bit-exact against the oracle's FP32 mode
    for b in range(B):
        want = O.split_levels(O.pyramid(2, base[b].detach().cpu().numpy()), W, H, len(levels) + 1, 16, np.float32)
        for k, lvl in enumerate(levels, start=1):
            assert np.array_equal(lvl[b].detach().cpu().numpy(), want[k]), (b, k)
    ups = [torch.randn(l.shape, generator=g, device=cuda) for l in levels]
    torch.autograd.backward(levels, ups)
    direct = adjoint([None] + ups, tuple(base.shape), torch.float32, cuda)
    assert torch.equal(base.grad, direct)
    # and against the dense FP64 adjoint for image 1
    ref = dense_adjoint([np.zeros((H, W, 4))] + [u[1].double().cpu().numpy() for u in ups], W, H)
    assert rel_err(base.grad[1].double().cpu().numpy(), ref) <= RTOL


def test_autograd_function_fp16_storage(cuda):
    import torch

    from vk_compute_mipmaps_gb300.autograd import pyramid
    H, W = 37, 50
    g = torch.Generator(device=cuda).manual_seed(4)
    base = torch.rand((H, W, 4), generator=g, device=cuda).half().requires_grad_(True)
    levels = pyramid(base)
    want = O.split_levels(O.pyramid(3, base.detach().cpu().numpy()), W, H, len(levels) + 1, 8, np.float16)
    for k, lvl in enumerate(levels, start=1):
        assert np.array_equal(lvl.detach().cpu().numpy(), want[k]), k
    ups = [torch.randn(l.shape, generator=g, device=cuda).half() for l in levels]
    torch.autograd.backward(levels, ups)
    ref = dense_adjoint([np.zeros((H, W, 4))] + [u.double().cpu().numpy() for u in ups], W, H)
    # FP16 storage of the result: half an ulp of FP16 relative
    assert rel_err(base.grad.double().cpu().numpy(), ref) <= 2e-3


def test_adjoint_2048_batch_closed_form(cuda):
    """8 x 2048^2 FP32 (the benchmark shape): even sizes only, so the adjoint
    of texel p is g_0[p] + sum_k 4^-k g_k[p >> k]; checked in FP64 on 64 pixels."""
    import torch

    from vk_compute_mipmaps_gb300.autograd import adjoint
    B, S = 8, 2048
    g = torch.Generator(device=cuda).manual_seed(5)
    n = P.full_level_count(S, S)
    ups = [torch.randn((B, max(S >> k, 1), max(S >> k, 1), 4), generator=g, device=cuda) for k in range(n)]
    grad = adjoint(ups, (B, S, S, 4), torch.float32, cuda)
    rng = np.random.default_rng(9)
    errs, mags = [], []
    for _ in range(64):
        b, x, y, c = int(rng.integers(B)), int(rng.integers(S)), int(rng.integers(S)), int(rng.integers(4))
        ref = sum(float(ups[k][b, y >> k, x >> k, c]) * 0.25 ** k for k in range(n))
        errs.append(abs(float(grad[b, y, x, c]) - ref))
        mags.append(abs(ref))
    assert max(errs) / max(mags) <= RTOL


@pytest.mark.parametrize("dtype_name", ["float32", "float16"])
@pytest.mark.parametrize("w,h", [(64, 48), (33, 20), (1, 5), (255, 256)])
def test_strided_calls_equal_per_image_calls(cuda, dtype_name, w, h):
    """nvproPyramidGenerateStrided / AdjointStrided over B images (one launch
    per dispatch) write the bytes of B single-image calls."""
    import torch

    from vk_compute_mipmaps_gb300.autograd import adjoint, forward_levels
    dt = getattr(torch, dtype_name)
    B = 3
    g = torch.Generator(device=cuda).manual_seed(w * h)
    base = torch.rand((B, h, w, 4), generator=g, device=cuda).to(dt)
    levels = forward_levels(base)
    ups = [torch.randn((B, lh, lw, 4), generator=g, device=cuda).to(dt) for lw, lh in P.level_sizes(w, h)]
    grad = adjoint(ups, (B, h, w, 4), dt, cuda)
    for i in range(B):
        one = forward_levels(base[i:i + 1].clone())
        for a, b in zip(levels, one):
            assert torch.equal(a[i], b[0])
        gi = adjoint([u[i:i + 1].clone() for u in ups], (1, h, w, 4), dt, cuda)
        assert torch.equal(grad[i], gi[0])


def test_autograd_with_base_takes_level0_gradient(cuda):
    """pyramid(base, with_base=True): the level-0 gradient enters the adjoint
    (h_0 = g_0 + A^T h_1), the same as the direct call with g_0."""
    import torch

    from vk_compute_mipmaps_gb300.autograd import adjoint, pyramid
    B, H, W = 2, 40, 24
    g = torch.Generator(device=cuda).manual_seed(8)
    base = torch.rand((B, H, W, 4), generator=g, device=cuda, requires_grad=True)
    levels = pyramid(base, with_base=True)
    assert len(levels) == P.full_level_count(W, H) and torch.equal(levels[0], base)
    ups = [torch.randn(l.shape, generator=g, device=cuda) for l in levels]
    torch.autograd.backward(levels, ups)
    assert torch.equal(base.grad, adjoint(ups, tuple(base.shape), torch.float32, cuda))
    ref = dense_adjoint([u[0].double().cpu().numpy() for u in ups], W, H)
    assert rel_err(base.grad[0].double().cpu().numpy(), ref) <= RTOL


@pytest.mark.parametrize("shape", [(8, 256, 256), (1, 777, 1023), (2, 64, 48)])
def test_autograd_step_captures_in_cuda_graph(cuda, shape):
    """Forward + backward through the autograd Function captured in a CUDA
    graph (no host synchronisation, allocations from torch's allocator):
    replays give the eager gradient, also after the input changes in place."""
    import torch

    from vk_compute_mipmaps_gb300 import autograd as A
    B, H, W = shape
    g = torch.Generator(device=cuda).manual_seed(B * H + W)
    base = torch.rand((B, H, W, 4), generator=g, device=cuda).requires_grad_(True)
    ups = [torch.randn((B, h, w, 4), generator=g, device=cuda) for w, h in P.level_sizes(W, H)[1:]]

    def step():
        base.grad = None
        torch.autograd.backward(A.pyramid(base), ups)

    side = torch.cuda.Stream(cuda)
    side.wait_stream(torch.cuda.current_stream(cuda))
    with torch.cuda.stream(side):
        for _ in range(3):
            step()
    torch.cuda.current_stream(cuda).wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    base.grad = None
    with torch.cuda.graph(graph):
        levels = A.pyramid(base)
        torch.autograd.backward(levels, ups)
    static_grad = base.grad
    for _ in range(2):
        with torch.no_grad():
            base.mul_(0.5).add_(0.25)
            for u in ups:
                u.mul_(-1.0)
        graph.replay()
        torch.cuda.synchronize()
        want = A.adjoint([None] + ups, (B, H, W, 4), torch.float32, cuda)
        assert torch.equal(static_grad, want)
        eager = A.forward_levels(base.detach())
        assert all(torch.equal(a, b) for a, b in zip(levels, eager))
