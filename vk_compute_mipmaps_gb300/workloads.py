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
