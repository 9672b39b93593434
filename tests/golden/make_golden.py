#!/usr/bin/env python3
"""Generate the golden fixtures in tests/golden/ by running the reference's own
code, compiled from its sources by `make -C oracle ref`:

* refcpu_vectors.npz -- cpuGenerateMipmaps_sRGBA (include/mipmap_storage.hpp)
  outputs for seeded uniform-random sRGBA8 images of many sizes.  Key
  "WxH" holds the packed pyramid; its level 0 is the input.
* dispatch_schedules.json.gz -- the commands that nvproCmdPyramidDispatch
  (nvpro_pyramid/nvpro_pyramid_dispatch.hpp) records for many image sizes,
  mip counts and dispatcher variants, captured through a recording stub of
  the Vulkan declarations it uses.
* premultiply_all_pairs.json -- the SHA-256 of the premultiplied-alpha
  staging (include/scoped_image.hpp:233-255: linearFromSrgb(c) *
  (A * (1.F / 255.F)) -> srgbFromLinear, shaders/srgb.h from the reference
  build) of the image holding every (colour code, alpha) pair in each
  channel (_oracle.all_code_alpha_pairs).

Run from the repository root: python tests/golden/make_golden.py [premultiply]
"""
from __future__ import annotations

import gzip
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
import _oracle as O  # noqa: E402

REFCPU_SIZES = [(1, 1), (2, 1), (1, 2), (1, 7), (7, 1), (2, 2), (3, 3), (4, 4), (5, 4), (4, 5), (6, 6), (7, 7),
                (8, 3), (9, 9), (17, 17), (31, 33), (33, 17), (64, 64), (65, 33), (127, 2), (100, 37), (257, 5)]
SCHED_W = list(range(2, 34)) + [63, 64, 65, 96, 127, 128, 129, 255, 256, 257, 513, 1080, 1920, 2047, 2048, 2052,
                                4094, 4095, 4096, 16384]
SCHED_H = [1, 2, 3, 4, 6, 8, 12, 17, 64, 1080, 4095, 4096]
# (has_fast, variant): variant 0 default <4,6>, 1 <2,5>, 2 <2,6>, 3 null fast, 4 null general
CONFIGS = [(1, 0), (1, 1), (1, 2), (1, 3), (1, 4), (0, 0)]


def seed_of(w: int, h: int) -> int:
    return 1000003 * w + h


def premultiply_golden(ref) -> None:
    import hashlib
    img = O.all_code_alpha_pairs()
    alpha = img[..., 3].astype(np.float32) * np.float32(1.0 / 255.0)
    out = img.copy()
    lin = np.array([ref.ref_linear_from_srgb(c) for c in range(256)], np.float32)
    for ch in range(3):
        prod = (lin[img[..., ch]] * alpha).astype(np.float32)
        out[..., ch] = np.array([ref.ref_srgb_from_linear(float(v)) for v in prod.reshape(-1)]).reshape(256, 256)
    digest = hashlib.sha256(out.tobytes()).hexdigest()
    (HERE / "premultiply_all_pairs.json").write_text(json.dumps({"sha256": digest, "shape": list(out.shape)}) + "\n")
    print("premultiply golden", digest)


def main() -> None:
    ref = O.ref_cpu()
    rd = O.ref_dispatch()
    if ref is None or rd is None:
        sys.exit("oracle/_ref is not built (make -C oracle ref needs the reference sources)")
    premultiply_golden(ref)
    if sys.argv[1:] == ["premultiply"]:
        return
    vec = {}
    for w, h in REFCPU_SIZES:
        base = np.random.default_rng(seed_of(w, h)).integers(0, 256, (h, w, 4), dtype=np.uint8)
        buf = O.packed_from_base(1, base)
        ref.ref_cpu_generate_srgba8(w, h, buf.ctypes.data_as(O.POINTER(O.c_uint8)))
        vec[f"{w}x{h}"] = buf
    np.savez_compressed(HERE / "refcpu_vectors.npz", **vec)

    sched = {}
    for w in SCHED_W:
        for h in SCHED_H:
            full = O.full_levels(w, h)
            if full < 2:
                continue  # the reference asserts on single-level images
            for mips in sorted({0, 3}):
                if mips > full:
                    continue
                for has_fast, var in CONFIGS:
                    ev = O.ref_events(rd, w, h, mips, has_fast, var)
                    sched[f"{w},{h},{mips},{has_fast},{var}"] = [list(e) for e in ev]
    with gzip.open(HERE / "dispatch_schedules.json.gz", "wt") as f:
        json.dump(sched, f, separators=(",", ":"))
    print(f"{len(vec)} CPU-generator vectors, {len(sched)} dispatch schedules")


if __name__ == "__main__":
    main()
