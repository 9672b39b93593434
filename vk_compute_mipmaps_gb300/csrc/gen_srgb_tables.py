#!/usr/bin/env python3
"""Generate srgb_tables.h: the exact sRGB <-> linear tables shared by every
sRGBA8 kernel of this library.

The reference defines the sRGB transfer functions in shaders/srgb.h:18-41 and
nvpro_pyramid/srgba8_mipmap_preamble.glsl:110-128, evaluated with FP32 `pow`
(whose precision is implementation-defined on GPUs).  This library pins both
directions to the exact mathematical functions so that the CUDA kernels and
the CPU oracle agree bit for bit:

* decode  : kSrgbDecode[c]  = FP32 nearest to EOTF(c / 255), where
            EOTF(u) = u / 12.92                       for u <= 0.04045
                    = ((u + 0.055) / 1.055) ** 2.4    otherwise
            (srgb.h:18-28 writes the same function as u * (25/323) and
            ((200u + 11) / 211) ** 2.4).
* alpha   : kAlphaDecode[c] = FP32 nearest to c / 255 (UNORM decode).
* encode  : code(x) = floor(clamp(255 * OETF(x) + 0.5, 0, 255)) with
            OETF(x) = 12.92 x                          for x <= 0.0031308
                    = 1.055 x ** (1/2.4) - 0.055       otherwise
            evaluated exactly on the FP32 value x (srgb.h:30-41).
            kSrgbEncodeThreshold[a] is the smallest non-negative FP32 x with
            code(x) >= a + 1 (a = 0..254); entry 255 is +inf.  Hence
            code(x) = number of entries <= x, and for any candidate
            a in {code(x) - 1, code(x)}: code(x) = a + (x >= kSrgbEncodeThreshold[a]).

All arithmetic uses the decimal module at 60 significant digits; the result is
rounded to FP32 by comparing the two neighbouring FP32 values exactly.

Usage: python gen_srgb_tables.py > srgb_tables.h
"""
import decimal
import struct
import sys

D = decimal.Decimal
CTX = decimal.Context(prec=60)
decimal.setcontext(CTX)


def f32_bits(x: float) -> int:
    return struct.unpack("<I", struct.pack("<f", x))[0]


def bits_f32(b: int) -> float:
    return struct.unpack("<f", struct.pack("<I", b))[0]


def exact(b: int) -> D:
    """Exact decimal value of the FP32 with bit pattern b (b >= 0)."""
    return D(bits_f32(b))  # float -> Decimal conversion is exact


def nearest_f32(v: D) -> int:
    """Bit pattern of the FP32 nearest to the non-negative decimal v (ties to even)."""
    approx = struct.unpack("<f", struct.pack("<f", float(v)))[0]
    b = f32_bits(approx)
    cands = [c for c in (b - 1, b, b + 1) if c >= 0]
    best = min(cands, key=lambda c: (abs(exact(c) - v), c & 1))
    return best


def eotf(u: D) -> D:
    if u <= D("0.04045"):
        return u / D("12.92")
    return ((u + D("0.055")) / D("1.055")) ** D("2.4")


FIVE_TWELFTHS = D(5) / D(12)


def oetf(x: D) -> D:
    if x <= D("0.0031308"):
        return D("12.92") * x
    return D("1.055") * (x ** FIVE_TWELFTHS) - D("0.055")


def threshold_bits(a: int) -> int:
    """Smallest FP32 bit pattern b in [0, 1.0] with 255*oetf(x)+0.5 >= a+1."""
    target = (D(a) + D("0.5")) / D(255)
    lo, hi = 0, f32_bits(1.0)  # predicate false at lo (x=0), true at hi (x=1)
    assert not oetf(exact(lo)) >= target and oetf(exact(hi)) >= target
    while hi - lo > 1:
        mid = (lo + hi) // 2
        if oetf(exact(mid)) >= target:
            hi = mid
        else:
            lo = mid
    return hi


def main() -> None:
    # The OETF is not exactly continuous at 0.0031308; make sure no code
    # boundary (a + 0.5) / 255 falls inside that tiny gap, so that counting
    # thresholds equals the piecewise definition everywhere.
    t = D("0.0031308")
    lin = D("12.92") * t
    pw = D("1.055") * (t ** FIVE_TWELFTHS) - D("0.055")
    gap_lo, gap_hi = min(lin, pw), max(lin, pw)
    for a in range(255):
        edge = (D(a) + D("0.5")) / D(255)
        assert not (gap_lo <= edge <= gap_hi), a

    decode = [nearest_f32(eotf(D(c) / D(255))) for c in range(256)]
    alpha = [nearest_f32(D(c) / D(255)) for c in range(256)]
    thresholds = [threshold_bits(a) for a in range(255)] + [0x7F800000]
    for a in range(254):
        assert thresholds[a] < thresholds[a + 1]

    out = sys.stdout
    out.write("// Generated by gen_srgb_tables.py -- do not edit.\n")
    out.write("// Exact sRGB decode/encode tables; see the generator for the definitions.\n")
    out.write("#pragma once\n\n")

    def emit(macro, vals, comment):
        # An initializer-list macro, so that host arrays and __constant__
        # device arrays can both be defined from it.
        out.write(f"// {comment}\n")
        out.write(f"#define {macro} \\\n")
        for i in range(0, 256, 4):
            chunk = vals[i:i + 4]
            vals_txt = ", ".join(f"0x{v:08X}u" for v in chunk)
            cmt = " ".join(f"{bits_f32(v):.9g}" for v in chunk)
            sep = "" if i + 4 >= 256 else ","
            cont = "" if i + 4 >= 256 else " \\"
            out.write(f"  {vals_txt}{sep} /* {cmt} */{cont}\n")
        out.write("\n")

    emit("NVPYR_SRGB_DECODE_BITS", decode, "FP32 nearest to the sRGB EOTF of c/255, c = 0..255")
    emit("NVPYR_ALPHA_DECODE_BITS", alpha, "FP32 nearest to c/255, c = 0..255")
    emit("NVPYR_SRGB_ENCODE_THRESHOLD_BITS", thresholds,
         "smallest FP32 x with sRGB code(x) >= a+1, a = 0..254; [255] = +inf")


if __name__ == "__main__":
    main()
