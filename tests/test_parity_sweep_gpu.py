"""GPU parity over a seeded sweep of image sizes: every level byte for byte
against the CPU oracle, through the C ABI, with the default pipelines and
launch planning (TMA launches with small-dispatch tails, general strip runs
with grid barriers, single-CTA launches, portable kernels where the layout
needs them), and with fusion off (one launch per dispatch).

The fixed size list of test_parity_gpu.py covers each schedule branch once;
the sweep adds many mixed cases: sides log-uniform in [2, 1536] (so both the
fast and the general pipeline start chains, and chains switch between them
at odd levels), sides at powers of two and one to three texels off them,
and very thin images.  A third of the sizes also run with shared-format
pipelines (SRGB_SHARED / F16_SHARED on one or both pipelines) against the
oracle's shared-format mode.  Outputs are pre-filled with a sentinel.
"""
import numpy as np
import pytest

import _oracle as O
from test_parity_gpu import assert_same, gpu_run, oracle_bytes, random_base
from test_shared_formats_gpu import check, gpu_run as gpu_run_formats, oracle as oracle_formats
from vk_compute_mipmaps_gb300 import _native as N
from vk_compute_mipmaps_gb300 import pyramid as P

pytestmark = pytest.mark.gpu


def sweep_sizes():
    rng = np.random.default_rng(20261204)
    sizes = set()
    while len(sizes) < 90:  # log-uniform sides
        w, h = np.exp(rng.uniform(0.0, np.log(1536.0), 2)).astype(int) + 1
        sizes.add((int(w), int(h)))
    for _ in range(40):  # a power of two, or up to three texels off it, on one or both sides
        k = int(rng.integers(2, 11))
        w = (1 << k) + int(rng.integers(-3, 4))
        h = (1 << int(rng.integers(2, 11))) + int(rng.integers(-3, 4)) if rng.random() < 0.5 else w
        sizes.add((max(w, 1), max(h, 1)))
    for _ in range(10):  # thin images
        long_side = int(rng.integers(2, 3000))
        short_side = int(rng.integers(1, 4))
        sizes.add((long_side, short_side) if rng.random() < 0.5 else (short_side, long_side))
    return sorted(sizes)


SWEEP = sweep_sizes()


@pytest.mark.parametrize("flags", [0, N.CMD_NO_FUSION])
@pytest.mark.parametrize("w,h", SWEEP)
def test_sweep_bit_exact(cuda, w, h, flags):
    base = random_base(N.PRESET_SRGBA8, w, h, w * 7919 + h * 104729)
    got, sched, _ = gpu_run(cuda, N.PRESET_SRGBA8, base, flags)
    mips = P.full_level_count(w, h)
    assert sched == [tuple(s) for s in O.default_schedule(w, h)]
    assert_same(got, oracle_bytes(N.PRESET_SRGBA8, base, sched, mips), w, h, 4, mips, f"{w}x{h} flags={flags}")


FORMATS = [(O.SHARED_SRGB, O.SHARED_SRGB), (O.SHARED_F16, O.SHARED_F16), (O.SHARED_FP32, O.SHARED_SRGB),
           (O.SHARED_SRGB, O.SHARED_F16)]


@pytest.mark.parametrize("w,h", SWEEP[::3])
def test_sweep_shared_formats_bit_exact(cuda, w, h):
    base = random_base(N.PRESET_SRGBA8, w, h, w * 31 + h * 17)
    fast_fmt, general_fmt = FORMATS[(w + h) % len(FORMATS)]
    got, _ = gpu_run_formats(cuda, base, fast_fmt, general_fmt)
    check(got, oracle_formats(base, fast_fmt, general_fmt), w, h, f"{w}x{h} fast {fast_fmt} general {general_fmt}")
