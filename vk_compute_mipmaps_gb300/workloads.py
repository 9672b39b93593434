"""Seeded synthetic workloads (the reference's image corpus cannot be decoded
here; these stand in for it with the same kinds of sizes)."""
from __future__ import annotations

import numpy as np


def batch_sizes(count: int = 256, seed: int = 2024, lo: int = 17, hi: int = 4096) -> list[tuple[int, int]]:
    """`count` image sizes: side log-uniform in [lo, hi], aspect ratio
    log-uniform in [1/4, 4] (about half the widths and heights odd)."""
    rng = np.random.default_rng(seed)
    side = np.exp(rng.uniform(np.log(lo), np.log(hi), count))
    aspect = np.exp(rng.uniform(np.log(0.25), np.log(4.0), count))
    w = np.clip(np.round(side * np.sqrt(aspect)), 1, hi).astype(int)
    h = np.clip(np.round(side / np.sqrt(aspect)), 1, hi).astype(int)
    return [(int(a), int(b)) for a, b in zip(w, h)]


def chain_bytes(w: int, h: int, bpp: int = 4) -> int:
    """Algorithmic bytes of one full chain: read the base once, write every
    other level once."""
    total, x, y = w * h, w, h
    while x > 1 or y > 1:
        x, y = max(x >> 1, 1), max(y >> 1, 1)
        total += x * y
    return total * bpp


def smooth_field(w: int, h: int, seed: int, opaque: bool = False) -> np.ndarray:
    """[h, w, 4] uint8: per colour channel a sum of 8 random-phase sinusoids
    (wavelengths log-uniform in 8..512 px) plus uniform +-16 noise around 128;
    alpha a radial gradient (255 at the centre), or 255 if opaque."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    img = np.zeros((h, w, 4))
    for c in range(3):
        acc = np.zeros((h, w))
        for _ in range(8):
            lam = np.exp(rng.uniform(np.log(8), np.log(512)))
            th = rng.uniform(0, 2 * np.pi)
            acc += np.sin(2 * np.pi * (x * np.cos(th) + y * np.sin(th)) / lam + rng.uniform(0, 2 * np.pi))
        img[..., c] = 128 + 14 * acc + rng.uniform(-16, 16, (h, w))
    r = np.hypot(x - w / 2, y - h / 2) / max(np.hypot(w / 2, h / 2), 1)
    img[..., 3] = 255 if opaque else 255 * (1 - r)
    return np.clip(np.rint(img), 0, 255).astype(np.uint8)


def shard_by_image(sizes, rank: int, world: int) -> list[int]:
    """Indices of the images rank `rank` of `world` generates when a batch is
    split by image (no exchange between ranks: every image is independent).
    Largest chains first, each to the rank with the fewest bytes so far (ties
    to the lowest rank), so every rank gets about the same traffic; the same
    on every rank, so the shares are disjoint and cover the batch."""
    load = [0] * world
    owner = [0] * len(sizes)
    order = sorted(range(len(sizes)), key=lambda i: (-chain_bytes(*sizes[i]), i))
    for i in order:
        r = min(range(world), key=lambda q: (load[q], q))
        owner[i] = r
        load[r] += chain_bytes(*sizes[i])
    return [i for i in range(len(sizes)) if owner[i] == rank]
