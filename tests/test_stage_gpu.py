"""GPU parity of the premultiplied-alpha staging pass
(nvproPyramidPremultiplyAlpha; the reference's -do-premultiply-alpha staging,
include/scoped_image.hpp:233-255): every (colour code, alpha) pair against
the oracle and the hash of the reference's own output, random images in every
layout (in place, out of place, pitched, unaligned), and the staging fused
into the host-memory entry point.
"""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import _oracle as O
import vk_compute_mipmaps_gb300 as V

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden" / "premultiply_all_pairs.json"


def test_premultiply_all_pairs_bit_exact(cuda):
    import torch
    img = O.all_code_alpha_pairs()
    t = torch.from_numpy(img).to(cuda)
    out = V.premultiply_alpha(t, torch.empty_like(t))
    got = out.cpu().numpy()
    assert np.array_equal(got, O.premultiply(img))
    assert hashlib.sha256(got.tobytes()).hexdigest() == json.loads(GOLDEN.read_text())["sha256"]
    assert np.array_equal(t.cpu().numpy(), img)  # the source is untouched


@pytest.mark.parametrize("w,h", [(1, 1), (3, 5), (4, 4), (7, 3), (1023, 777), (4096, 17), (17, 4096), (1920, 1080)])
@pytest.mark.parametrize("layout", ["inplace", "copy", "pitched", "unaligned"])
def test_premultiply_layouts(cuda, w, h, layout):
    import torch
    base = np.random.default_rng(w * 3 + h).integers(0, 256, (h, w, 4), dtype=np.uint8)
    want = O.premultiply(base)
    if layout == "inplace":
        t = torch.from_numpy(base.copy()).to(cuda)
        got = V.premultiply_alpha(t)
    elif layout == "copy":
        t = torch.from_numpy(base).to(cuda)
        got = V.premultiply_alpha(t, torch.full_like(t, 0xA7))
    elif layout == "pitched":  # rows 16 texels apart beyond the width, in and out
        big = torch.full((h, w + 16, 4), 0xA7, dtype=torch.uint8, device=cuda)
        big[:, :w] = torch.from_numpy(base).to(cuda)
        dst = torch.full((h, w + 16, 4), 0x5C, dtype=torch.uint8, device=cuda)
        got = V.premultiply_alpha(big[:, :w], dst[:, :w])
        assert (dst[:, w:] == 0x5C).all() and (big[:, w:] == 0xA7).all()  # padding untouched
    else:  # 4-byte offsets and odd pitches: the scalar path
        big = torch.full((h, w + 1, 4), 0xA7, dtype=torch.uint8, device=cuda)
        big[:, 1:] = torch.from_numpy(base).to(cuda)
        got = V.premultiply_alpha(big[:, 1:])
        assert (big[:, 0] == 0xA7).all()
    assert np.array_equal(got.cpu().numpy(), want), layout


@pytest.mark.parametrize("w,h,bands", [(2048, 2048, 8), (2048, 2048, None), (1920, 1080, 4), (4096, 64, None),
                                       (8192, 8192, None)])
def test_generate_from_host_premultiply(cuda, w, h, bands):
    import torch
    base = np.random.default_rng(w + h).integers(0, 256, (h, w, 4), dtype=np.uint8)
    ref = V.MipChain(w, h, V.PRESET_SRGBA8, device=cuda)
    ref.level(0).copy_(torch.from_numpy(O.premultiply(base)))
    V.generate(ref)
    chain = V.MipChain(w, h, V.PRESET_SRGBA8, device=cuda)
    host_base = torch.from_numpy(base.reshape(-1).copy()).pin_memory()
    host_levels = torch.empty(chain.offsets[-1] - chain.offsets[1], dtype=torch.uint8).pin_memory()
    V.generate_from_host(chain, host_base, host_levels, bands=bands, premultiply=True)
    torch.cuda.synchronize()
    assert torch.equal(chain.storage, ref.storage)  # level 0 premultiplied on the device
    assert torch.equal(host_levels, ref.storage[chain.offsets[1]:].cpu())
    assert np.array_equal(host_base.numpy(), base.reshape(-1))  # the host copy of level 0 as it was


def vavg(a, b):
    return ((a.astype(np.uint16) + b + 1) >> 1).astype(np.uint8)


@pytest.mark.parametrize("w,h", [(2, 2), (5, 3), (64, 64), (1023, 777), (4096, 18), (2048, 2048)])
def test_speed_of_light_probe_traffic_pattern(cuda, w, h):
    """The probe writes every texel of levels 1.. exactly once (level 1: the
    rounded-up byte average of its 2x2 block, pairs first; level k texel
    (x, y): level 1's texel (x, y)) and nothing else."""
    import ctypes

    import torch

    from vk_compute_mipmaps_gb300 import _native as N
    chain = V.MipChain(w, h, V.PRESET_SRGBA8, device=cuda)
    chain.storage.fill_(0xA7)
    base = np.random.default_rng(w * h).integers(0, 256, (h, w, 4), dtype=np.uint8)
    chain.level(0).copy_(torch.from_numpy(base))
    img = chain.image()
    N.check(N.load().nvproPyramidSpeedOfLightProbe(torch.cuda.current_stream(cuda).cuda_stream, ctypes.byref(img), 0))
    torch.cuda.synchronize()
    h1, w1 = max(h >> 1, 1), max(w >> 1, 1)
    b = base[:2 * h1, :2 * w1]
    l1 = vavg(vavg(b[0::2, 0::2], b[0::2, 1::2]), vavg(b[1::2, 0::2], b[1::2, 1::2]))
    assert np.array_equal(chain.level(0).cpu().numpy(), base)
    assert np.array_equal(chain.level(1).cpu().numpy(), l1)
    for k in range(2, chain.levels):
        lw, lh = max(w >> k, 1), max(h >> k, 1)
        assert np.array_equal(chain.level(k).cpu().numpy(), l1[:lh, :lw]), k
