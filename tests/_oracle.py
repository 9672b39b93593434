"""ctypes access to the CPU oracle (oracle/liborc.so) and, where present, the
reference builds in oracle/_ref.  Test infrastructure only."""
from __future__ import annotations

import ctypes
import subprocess
from ctypes import POINTER, c_double, c_float, c_int, c_uint8, c_uint16, c_uint32, c_uint64
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
ORACLE_DIR = ROOT / "oracle"
ORC_PATH = ORACLE_DIR / "liborc.so"
REF_CPU_PATH = ORACLE_DIR / "_ref" / "libref_cpu.so"
REF_DISPATCH_PATH = ORACLE_DIR / "_ref" / "libref_dispatch.so"

BPP = {1: 4, 2: 16, 3: 8, 4: 8}
DTYPE = {1: np.uint8, 2: np.float32, 3: np.float16, 4: np.uint16}

_orc = None


def orc() -> ctypes.CDLL:
    global _orc
    if _orc is None:
        if not ORC_PATH.exists():
            subprocess.run(["make", "-s", "-C", str(ORACLE_DIR), "all"], check=True)
        lib = ctypes.CDLL(str(ORC_PATH))
        u32p = POINTER(c_uint32)
        lib.orc_full_level_count.restype = c_uint32
        lib.orc_full_level_count.argtypes = [c_uint32, c_uint32]
        lib.orc_default_schedule.argtypes = [c_uint32, c_uint32, c_uint32, c_int, c_uint32, c_uint32, u32p, u32p,
                                             u32p, c_int]
        lib.orc_run.argtypes = [c_int, c_uint32, c_uint32, c_uint32, u32p, u32p, u32p, c_int, POINTER(c_uint8)]
        lib.orc_run_ex.argtypes = [c_int, c_int, c_int, c_uint32, c_uint32, c_uint32, u32p, u32p, u32p, c_int,
                                   POINTER(c_uint8)]
        lib.orc_refcpu_srgba8.argtypes = [c_uint32, c_uint32, POINTER(c_uint8)]
        lib.orc_f64_pyramid.argtypes = [c_uint32, c_uint32, c_uint32, POINTER(c_double)]
        lib.orc_srgb_tables.argtypes = [POINTER(c_float)] * 3
        lib.orc_srgb_encode.argtypes = [c_float]
        lib.orc_srgb_encode.restype = c_uint32
        lib.orc_alpha_encode.argtypes = [c_float]
        lib.orc_alpha_encode.restype = c_uint32
        lib.orc_srgb_encode_array.argtypes = [POINTER(c_float), POINTER(c_uint8), c_uint64]
        lib.orc_premultiply_srgba8.argtypes = [POINTER(c_uint8), POINTER(c_uint8), c_uint64, c_int]
        lib.orc_premultiply_srgba8.restype = None
        lib.orc_half_to_float.argtypes = [c_uint16]
        lib.orc_half_to_float.restype = c_float
        lib.orc_float_to_half.argtypes = [c_float]
        lib.orc_float_to_half.restype = c_uint16
        _orc = lib
    return _orc


def full_levels(w: int, h: int) -> int:
    return orc().orc_full_level_count(w, h)


def offsets(w: int, h: int, levels: int, bpp: int) -> list[int]:
    out, o = [], 0
    for k in range(levels):
        out.append(o)
        o += max(w >> k, 1) * max(h >> k, 1) * bpp
    return out + [o]


def default_schedule(w, h, mips=0, has_fast=True, div=4, max_levels=6):
    n = 64
    a, b, c = (c_uint32 * n)(), (c_uint32 * n)(), (c_uint32 * n)()
    cnt = orc().orc_default_schedule(w, h, mips, int(has_fast), div, max_levels, a, b, c, n)
    assert cnt >= 0
    return [(a[i], b[i], c[i]) for i in range(cnt)]


# shared-memory formats of the sRGBA8 pipelines (SRGB_SHARED / F16_SHARED)
SHARED_FP32, SHARED_SRGB, SHARED_F16 = 0, 1, 2


def fast_or_blit_schedule(w, h, mips=0):
    """The demo's "generalblit" sequence (demo_app/mipmap_pipelines.cpp:
    350-452): the default fast dispatcher <4, 6> where it accepts the level,
    else a linear blit of one level (isFast = 2)."""
    mips = mips or full_levels(w, h)
    out, level, remaining, x, y = [], 0, mips - 1, w, h
    while remaining:
        if x % 4 == 0 and y % 4 == 0:
            tx, ty, done = x, y, 0
            while tx % 2 == 0 and ty % 2 == 0 and done < remaining and done < 6:
                tx, ty, done = tx // 2, ty // 2, done + 1
            shift, mask = (12, 4095) if done > 5 else (10, 1023)
            out.append((1, level << 5 | done, ((x * y + mask) & 0xFFFFFFFF) >> shift))
        else:
            done = 1
            out.append((2, level << 5 | 1, 1))
        level, remaining = level + done, remaining - done
        x, y = max(x >> done, 1), max(y >> done, 1)
    return out


def run(preset: int, w: int, h: int, packed: np.ndarray, schedule=None, mips: int = 0, fast_shared: int = 0,
        general_shared: int = 0) -> np.ndarray:
    """Apply a dispatch schedule (default: the reference's) to a packed image in
    place; fast_shared / general_shared: the pipelines' shared-memory formats."""
    mips = mips or full_levels(w, h)
    if schedule is None:
        schedule = default_schedule(w, h, mips)
    n = max(len(schedule), 1)
    a, b, c = (c_uint32 * n)(), (c_uint32 * n)(), (c_uint32 * n)()
    for i, (f, pc, g) in enumerate(schedule):
        a[i], b[i], c[i] = f, pc, g
    assert packed.flags.c_contiguous
    rc = orc().orc_run_ex(preset, fast_shared, general_shared, w, h, mips, a, b, c, len(schedule),
                          packed.ctypes.data_as(POINTER(c_uint8)))
    assert rc == 0, rc
    return packed


def packed_from_base(preset: int, base: np.ndarray, mips: int = 0) -> np.ndarray:
    """A zeroed packed byte buffer with level 0 = base ([h, w, 4])."""
    h, w = base.shape[:2]
    mips = mips or full_levels(w, h)
    off = offsets(w, h, mips, BPP[preset])
    buf = np.zeros(off[-1], np.uint8)
    buf[:off[1]] = np.ascontiguousarray(base).view(np.uint8).reshape(-1)
    return buf


def pyramid(preset: int, base: np.ndarray, schedule=None, mips: int = 0, fast_shared: int = 0,
            general_shared: int = 0) -> np.ndarray:
    h, w = base.shape[:2]
    buf = packed_from_base(preset, base, mips)
    return run(preset, w, h, buf, schedule, mips, fast_shared, general_shared)


def refcpu(base: np.ndarray) -> np.ndarray:
    """The restated reference CPU generator (cpuGenerateMipmaps_sRGBA)."""
    h, w = base.shape[:2]
    buf = packed_from_base(1, base)
    assert orc().orc_refcpu_srgba8(w, h, buf.ctypes.data_as(POINTER(c_uint8))) == 0
    return buf


def f64_pyramid(base: np.ndarray, mips: int = 0) -> list[np.ndarray]:
    """Exact-weight FP64 pyramid of a [h, w, 4] float image; returns levels."""
    h, w = base.shape[:2]
    mips = mips or full_levels(w, h)
    off = offsets(w, h, mips, 1)
    buf = np.zeros(off[-1] * 4, np.float64)
    buf[:off[1] * 4] = base.astype(np.float64).reshape(-1)
    orc().orc_f64_pyramid(w, h, mips, buf.ctypes.data_as(POINTER(c_double)))
    return split_levels(buf.view(np.uint8), w, h, mips, 32, np.float64)


def split_levels(packed: np.ndarray, w: int, h: int, levels: int, bpp: int, dtype) -> list[np.ndarray]:
    off = offsets(w, h, levels, bpp)
    out = []
    for k in range(levels):
        lw, lh = max(w >> k, 1), max(h >> k, 1)
        out.append(packed[off[k]:off[k + 1]].view(dtype).reshape(lh, lw, 4))
    return out


def tables():
    d, a, t = (c_float * 256)(), (c_float * 256)(), (c_float * 256)()
    orc().orc_srgb_tables(d, a, t)
    return (np.frombuffer(bytes(d), np.float32), np.frombuffer(bytes(a), np.float32),
            np.frombuffer(bytes(t), np.float32))


def srgb_encode_array(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, np.float32)
    out = np.empty(x.shape, np.uint8)
    orc().orc_srgb_encode_array(x.ctypes.data_as(POINTER(c_float)), out.ctypes.data_as(POINTER(c_uint8)), x.size)
    return out


def worst_delta(a: np.ndarray, b: np.ndarray, w: int, h: int) -> int:
    """Max per-channel delta over levels >= 1 (MipmapStorage::compare)."""
    off = offsets(w, h, full_levels(w, h), 4)
    d = np.abs(a[off[1]:].astype(np.int16) - b[off[1]:].astype(np.int16))
    return int(d.max()) if d.size else 0


# --- reference builds (present only where the reference sources were) -----

def ref_cpu():
    if not REF_CPU_PATH.exists():
        return None
    lib = ctypes.CDLL(str(REF_CPU_PATH))
    lib.ref_cpu_generate_srgba8.argtypes = [c_uint32, c_uint32, POINTER(c_uint8)]
    lib.ref_linear_from_srgb.argtypes = [c_uint32]
    lib.ref_linear_from_srgb.restype = c_float
    lib.ref_srgb_from_linear.argtypes = [c_float]
    lib.ref_srgb_from_linear.restype = c_uint32
    return lib


def ref_dispatch():
    if not REF_DISPATCH_PATH.exists():
        return None
    lib = ctypes.CDLL(str(REF_DISPATCH_PATH))
    lib.ref_dispatch_events.argtypes = [c_uint32, c_uint32, c_uint32, c_int, c_int, POINTER(c_uint32), c_int]
    return lib


def ref_events(lib, w, h, mips, has_fast, variant):
    buf = (c_uint32 * 4096)()
    n = lib.ref_dispatch_events(w, h, mips, int(has_fast), variant, buf, 1024)
    assert n >= 0
    return [tuple(buf[4 * i:4 * i + 4]) for i in range(n)]


def premultiply(rgba: np.ndarray, reference_math: bool = False) -> np.ndarray:
    """Premultiplied-alpha staging of uint8 RGBA texels (any shape [..., 4])."""
    src = np.ascontiguousarray(rgba, np.uint8)
    out = np.empty_like(src)
    orc().orc_premultiply_srgba8(src.ctypes.data_as(POINTER(c_uint8)), out.ctypes.data_as(POINTER(c_uint8)),
                                 src.size // 4, int(reference_math))
    return out


def all_code_alpha_pairs() -> np.ndarray:
    """[256, 256, 4] uint8: texel (x=c, y=A) = (c, 255 - c, c ^ 0x5A, A): every
    colour code with every alpha in each colour channel."""
    c = np.arange(256, dtype=np.uint8)
    img = np.empty((256, 256, 4), np.uint8)
    img[..., 0] = c[None, :]
    img[..., 1] = (255 - c)[None, :]
    img[..., 2] = (c ^ 0x5A)[None, :]
    img[..., 3] = c[:, None]
    return img
