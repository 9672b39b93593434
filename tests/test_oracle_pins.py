"""Pin the CPU oracle to the reference before trusting it (CPU only).

* The restated reference CPU generator must equal, bit for bit, the golden
  vectors made by the reference's own cpuGenerateMipmaps_sRGBA (and the live
  reference build where its sources are present).
* The restated dispatcher must equal the golden dispatch sequences recorded
  from the reference's nvpro_pyramid_dispatch.hpp.
* The sRGB tables of the library (decimal arithmetic) and of the oracle (long
  double arithmetic) must agree; the reference's FP32 formulas stay within one
  code of them.
* Shader semantics (the oracle's main mode) must stay within the reference's
  own delta bar against its CPU generator (demo_app/rtx3090.json: 2 on opaque
  images, 4-5 with alpha).
"""
import gzip
import json
import re
from pathlib import Path

import numpy as np
import pytest

import _oracle as O
from vk_compute_mipmaps_gb300.workloads import smooth_field

GOLDEN = Path(__file__).resolve().parent / "golden"


def golden_vectors():
    with np.load(GOLDEN / "refcpu_vectors.npz") as z:
        return {k: z[k] for k in z.files}


def golden_schedules():
    with gzip.open(GOLDEN / "dispatch_schedules.json.gz", "rt") as f:
        return json.load(f)


def test_refcpu_restatement_matches_golden_vectors():
    vecs = golden_vectors()
    assert len(vecs) >= 20
    for key, expected in vecs.items():
        w, h = map(int, key.split("x"))
        base = expected[:w * h * 4].reshape(h, w, 4)
        got = O.refcpu(base)
        assert np.array_equal(got, expected), key


@pytest.mark.skipif(O.ref_cpu() is None, reason="reference build oracle/_ref absent")
@pytest.mark.parametrize("w,h", [(1920, 1080), (4095, 17), (3, 257), (513, 129), (1023, 777)])
def test_refcpu_restatement_matches_live_reference(w, h):
    ref = O.ref_cpu()
    base = np.random.default_rng(w * 7 + h).integers(0, 256, (h, w, 4), dtype=np.uint8)
    expected = O.packed_from_base(1, base)
    ref.ref_cpu_generate_srgba8(w, h, expected.ctypes.data_as(O.POINTER(O.c_uint8)))
    assert np.array_equal(O.refcpu(base), expected)


def events_to_schedule(events):
    """(isFast, pushConstant, groups) per dispatch from recorded commands."""
    out, bound, pc = [], None, None
    for kind, a, b, c in events:
        if kind == 1:
            bound = a
        elif kind == 2:
            pc = a
        elif kind == 3:
            out.append((bound, pc, a))
    return out


def test_default_schedule_matches_reference_dispatcher():
    sched = golden_schedules()
    variants = {0: (4, 6), 1: (2, 5), 2: (2, 6)}
    checked = 0
    for key, events in sched.items():
        w, h, mips, has_fast, var = map(int, key.split(","))
        if var not in variants:
            continue
        div, mx = variants[var]
        expected = events_to_schedule(events)
        got = O.default_schedule(w, h, mips, bool(has_fast), div, mx)
        assert [tuple(x) for x in got] == expected, key
        checked += 1
    assert checked > 4000


def test_schedule_examples():
    # The schedules quoted for the benchmark sizes (F = fast, G = general).
    def kinds(w, h):
        return [("F" if f else "G") + str(pc & 31) for f, pc, _ in O.default_schedule(w, h)]
    assert kinds(2048, 2048) == ["F6", "F5"]
    assert kinds(4096, 4096) == ["F6", "F6"]
    assert kinds(16384, 16384) == ["F6", "F6", "F2"]
    assert kinds(4095, 4095) == ["G2"] * 5 + ["G1"]
    assert kinds(1920, 1080) == ["F3", "G2", "G2", "G2", "G1"]
    assert kinds(2052, 2052) == ["F2", "G2", "F6", "G1"]


def header_table(name):
    src = (Path(O.ROOT) / "vk_compute_mipmaps_gb300" / "csrc" / "srgb_tables.h").read_text()
    body = src.split(f"#define {name}")[1].split("\n\n")[0]
    vals = [int(x, 16) for x in re.findall(r"0x([0-9A-F]{8})u", body)]
    assert len(vals) == 256
    return np.array(vals, np.uint32)


def test_srgb_tables_two_independent_computations_agree():
    dec, alpha, thr = O.tables()
    assert np.array_equal(dec.view(np.uint32), header_table("NVPYR_SRGB_DECODE_BITS"))
    assert np.array_equal(alpha.view(np.uint32), header_table("NVPYR_ALPHA_DECODE_BITS"))
    assert np.array_equal(thr.view(np.uint32), header_table("NVPYR_SRGB_ENCODE_THRESHOLD_BITS"))
    assert dec[0] == 0.0 and dec[255] == 1.0 and alpha[255] == 1.0
    assert np.all(np.diff(dec) > 0) and np.all(np.diff(thr[:255]) > 0) and np.isinf(thr[255])


def test_encode_thresholds_are_exact_boundaries():
    _, _, thr = O.tables()
    t = thr[:255]
    below = np.nextafter(t, np.float32(-1))
    assert np.array_equal(O.srgb_encode_array(t), np.arange(1, 256))
    assert np.array_equal(O.srgb_encode_array(below), np.arange(0, 255))
    # decode -> encode is the identity on all 256 codes
    dec, _, _ = O.tables()
    assert np.array_equal(O.srgb_encode_array(dec), np.arange(256))


def test_reference_fp32_formulas_within_one_code():
    lib = O.orc()
    lib.orc_ref_srgb_from_linear.argtypes = [O.c_float]
    lib.orc_ref_srgb_from_linear.restype = O.c_uint32
    lib.orc_ref_linear_from_srgb.argtypes = [O.c_uint32]
    lib.orc_ref_linear_from_srgb.restype = O.c_float
    dec, _, thr = O.tables()
    ref_dec = np.array([lib.orc_ref_linear_from_srgb(c) for c in range(256)], np.float32)
    ulps = np.abs(ref_dec.view(np.int32).astype(np.int64) - dec.view(np.int32))
    assert ulps.max() <= 8
    xs = np.concatenate([np.random.default_rng(3).random(20000, dtype=np.float32), thr[:255],
                         np.nextafter(thr[:255], np.float32(-1))])
    mine = O.srgb_encode_array(xs).astype(int)
    ref = np.array([lib.orc_ref_srgb_from_linear(float(x)) for x in xs])
    assert np.abs(mine - ref).max() <= 1


@pytest.mark.parametrize("w,h", [(256, 256), (255, 255), (254, 254), (192, 108), (257, 129)])
def test_shader_semantics_within_reference_delta_bar(w, h):
    for opaque, bar in ((True, 2), (False, 5)):
        base = smooth_field(w, h, w + h, opaque)
        delta = O.worst_delta(O.pyramid(1, base), O.refcpu(base), w, h)
        assert delta <= bar, (w, h, opaque, delta)


def test_schedule_changes_output_negative_control():
    # Quantisation happens at every dispatch boundary, so a different (still
    # valid) schedule must give different bytes: the comparison has teeth.
    base = np.random.default_rng(7).integers(0, 256, (64, 64, 4), dtype=np.uint8)
    a = O.pyramid(1, base)  # F6
    b = O.pyramid(1, base, schedule=O.default_schedule(64, 64, 0, True, 2, 3))  # F3 F3
    c = O.pyramid(1, base, schedule=O.default_schedule(64, 64, 0, False))  # G2 G2 G2
    assert not np.array_equal(a, b) and not np.array_equal(a, c)
    assert O.worst_delta(a, b, 64, 64) <= 2 and O.worst_delta(a, c, 64, 64) <= 2


def test_float_oracle_close_to_fp64():
    base = np.random.default_rng(11).random((37, 50, 4), dtype=np.float32)
    f32 = O.split_levels(O.pyramid(2, base), 50, 37, O.full_levels(50, 37), 16, np.float32)
    f64 = O.f64_pyramid(base)
    for a, b in zip(f32, f64):
        assert np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-3)) < 1e-5
