"""The C ABI without a GPU: the library loads, exports every symbol the header
declares, records exactly the reference dispatcher's command sequence, and
turns the reference's asserts into error codes.  Commands here are created
with NVPRO_PYRAMID_CMD_RECORD_ONLY, which makes no CUDA call."""
import ctypes
import gzip
import json
import re
from pathlib import Path

import pytest

import _oracle as O
from vk_compute_mipmaps_gb300 import _native as N
from vk_compute_mipmaps_gb300 import pyramid as P

ROOT = Path(__file__).resolve().parents[1]


def header_functions():
    names = set()
    for hdr in (ROOT / "include").glob("*.h"):
        src = hdr.read_text()
        names |= set(re.findall(r"NVPRO_PYRAMID_API\s+[\w\s\*]+?\b(\w+)\s*\(", src))
    return names


def test_library_exports_every_declared_function(native):
    names = header_functions()
    assert len(names) >= 25
    for name in names:
        assert hasattr(native, name), name
    assert names <= set(N.SIGNATURES), names - set(N.SIGNATURES)


def fake_image(w, h, levels=0, bpp=4):
    """An image whose level pointers are aligned but never dereferenced."""
    levels = levels or P.full_level_count(w, h)
    return P.make_image([0x7F0000000000 + 0x100000 * k for k in range(levels)], w, h)


def record(w, h, mips=0, has_fast=True, general=None, fast=None, preset=N.PRESET_SRGBA8):
    cmd = P.Cmd(N.CMD_RECORD_ONLY)
    pipes = P.Pipelines(preset, fast=has_fast)
    cmd.begin(None)
    cmd.bind_image(fake_image(w, h))
    P.cmd_pyramid_dispatch(cmd, pipes, w, h, mips, general=general, fast=fast)
    cmd.end()
    return cmd.records()


def records_to_events(recs):
    ev = []
    for r in recs:
        if r["barrierBefore"]:
            ev.append([4, 0, 0, 0])
        if r["pipelineBound"]:
            ev.append([1, r["isFastPipeline"], 0, 0])
        ev.append([2, r["pushConstant"], 0, 4])
        ev.append([3, r["groupCountX"], r["groupCountY"], r["groupCountZ"]])
    return ev


def test_records_match_reference_dispatcher_golden(native):
    with gzip.open(ROOT / "tests" / "golden" / "dispatch_schedules.json.gz", "rt") as f:
        golden = json.load(f)

    def fast_variant(div, mx):
        return P.wrap_dispatcher(lambda c, lay, pco, pipe, st: native.nvproPyramidFastDispatch(
            c, lay, pco, pipe, ctypes.byref(st), div, mx))

    null = P.wrap_dispatcher(lambda c, lay, pco, pipe, st: st.remainingLevels)
    fasts = {1: fast_variant(2, 5), 2: fast_variant(2, 6), 3: null}
    checked = 0
    for key, events in golden.items():
        w, h, mips, has_fast, var = map(int, key.split(","))
        if checked > 2500 and w < 2047 and (w + h) % 3:
            continue  # keep the CPU suite quick: a large deterministic subset
        general = null if var == 4 else None
        fast = fasts.get(var)
        recs = record(w, h, mips, bool(has_fast), general=general, fast=fast)
        # A barrier after the last dispatch (possible when a null dispatcher
        # records nothing) orders nothing; records keep barriers as a flag of
        # the following dispatch, so such a barrier has no record.
        while events and events[-1][0] == 4:
            events = events[:-1]
        assert records_to_events(recs) == events, key
        checked += 1
    assert checked > 2500


def expect_error(code, fn):
    with pytest.raises(N.NativeLibraryError) as e:
        fn()
    assert e.value.code == code, str(e.value)


def test_error_codes_replace_asserts(native):
    pipes = P.Pipelines()
    cmd = P.Cmd(N.CMD_RECORD_ONLY)
    # more levels than the image size allows
    cmd.begin(None)
    cmd.bind_image(fake_image(16, 16))
    expect_error(N.ERROR_INVALID_ARGUMENT, lambda: P.cmd_pyramid_dispatch(cmd, pipes, 16, 16, 6))
    # general dispatcher returning 0 (the reference asserts levelsDone != 0)
    cmd.begin(None)
    cmd.bind_image(fake_image(15, 15))
    zero = P.wrap_dispatcher(lambda *a: 0)
    expect_error(N.ERROR_DISPATCHER, lambda: P.cmd_pyramid_dispatch(cmd, pipes, 15, 15, general=zero))
    # ... and more than remainingLevels (levelsDone <= state.remainingLevels)
    cmd.begin(None)
    cmd.bind_image(fake_image(15, 15))
    many = P.wrap_dispatcher(lambda c, l, o, p, st: st.remainingLevels + 1)
    expect_error(N.ERROR_DISPATCHER, lambda: P.cmd_pyramid_dispatch(cmd, pipes, 15, 15, general=many))
    expect_error(N.ERROR_DISPATCHER, cmd.end)  # the error is sticky until End
    # dispatch without a bound image
    cmd.begin(None)
    expect_error(N.ERROR_INVALID_STATE, lambda: P.cmd_pyramid_dispatch(cmd, pipes, 8, 8))
    # the image has fewer levels than the dispatch writes
    cmd.begin(None)
    cmd.bind_image(fake_image(64, 64, levels=3))
    expect_error(N.ERROR_INVALID_ARGUMENT, lambda: P.cmd_pyramid_dispatch(cmd, pipes, 64, 64))
    # push constant must be 4 bytes at offset 0
    cmd.begin(None)
    v = ctypes.c_uint32(1)
    expect_error(N.ERROR_INVALID_ARGUMENT,
                 lambda: N.check(native.nvproPyramidCmdPushConstants(cmd.handle, None, 4, 4, ctypes.byref(v))))
    # misaligned level pointer
    cmd.begin(None)
    img = fake_image(8, 8)
    img.levels[1] = img.levels[1] + 2
    cmd.bind_image(img)
    expect_error(N.ERROR_UNSUPPORTED, lambda: P.cmd_pyramid_dispatch(cmd, pipes, 8, 8))
    # unknown preset, missing general pipeline
    h = ctypes.c_void_p()
    expect_error(N.ERROR_UNSUPPORTED, lambda: N.check(native.nvproPyramidCreatePipeline(9, 0, ctypes.byref(h))))
    cmd.begin(None)
    cmd.bind_image(fake_image(8, 8))
    bad = N.NvproPyramidPipelines(None, pipes.fast, None, 0)
    expect_error(N.ERROR_INVALID_ARGUMENT,
                 lambda: N.check(native.nvproCmdPyramidDispatch(cmd.handle, bad, 8, 8, 0)))
    expect_error(N.ERROR_INVALID_ARGUMENT, cmd.end)  # reports the recorded error
    # End without Begin
    expect_error(N.ERROR_INVALID_STATE, cmd.end)
    # null handles are rejected, not dereferenced
    expect_error(N.ERROR_INVALID_ARGUMENT, lambda: N.check(native.nvproPyramidBeginCmd(None, None)))


def test_single_level_image_records_nothing(native):
    assert record(1, 1) == []


def test_packed_layout_matches_mipmap_storage(native):
    for w, h in [(1, 1), (3, 5), (64, 64), (4095, 17), (16384, 16384)]:
        levels = P.full_level_count(w, h)
        offs = (ctypes.c_uint64 * (levels + 1))()
        N.check(native.nvproPyramidPackedLayout(w, h, levels, 4, offs))
        assert list(offs) == O.offsets(w, h, levels, 4) == P.packed_offsets(w, h, levels, 4)
        assert native.nvproPyramidFullLevelCount(w, h) == O.full_levels(w, h) == levels


def test_partial_mip_count_and_general_only(native):
    recs = record(64, 64, mips=3)
    assert [(r["isFastPipeline"], r["pushConstant"] & 31) for r in recs] == [(1, 2)]
    recs = record(64, 64, has_fast=False)
    assert all(r["isFastPipeline"] == 0 for r in recs)
    assert sum(r["pushConstant"] & 31 for r in recs) == 6


def test_pipeline_config_bits(native):
    """nvproPyramidCreatePipelineEx: the demo's per-pipeline config bits
    (demo_app/pipeline_alternative.hpp:40-42) and their validation."""
    h = ctypes.c_void_p()

    def create(preset, fast, bits):
        return native.nvproPyramidCreatePipelineEx(preset, fast, bits, ctypes.byref(h))

    assert (N.CONFIG_SRGB_SHARED, N.CONFIG_F16_SHARED, N.CONFIG_NO_BILINEAR) == (1, 2, 4)
    for bits in (0, 1, 2, 4, 5, 6):
        assert create(N.PRESET_SRGBA8, 1, bits) == N.SUCCESS, bits
        native.nvproPyramidDestroyPipeline(h)
    assert create(N.PRESET_SRGBA8, 0, 3) == N.ERROR_INVALID_ARGUMENT  # both shared formats
    assert create(N.PRESET_SRGBA8, 0, 8) == N.ERROR_INVALID_ARGUMENT  # unknown bit
    assert create(N.PRESET_RGBA32F, 0, N.CONFIG_F16_SHARED) == N.ERROR_UNSUPPORTED  # sRGBA8 only
    assert create(N.PRESET_RGBA32F, 1, N.CONFIG_NO_BILINEAR) == N.SUCCESS
    native.nvproPyramidDestroyPipeline(h)
    # each record carries the bits of the pipeline bound for it
    cmd = P.Cmd(N.CMD_RECORD_ONLY)
    pipes = P.Pipelines(general_config=N.CONFIG_SRGB_SHARED, fast_config=N.CONFIG_F16_SHARED)
    cmd.begin(None)
    cmd.bind_image(fake_image(2052, 2052))
    P.cmd_pyramid_dispatch(cmd, pipes, 2052, 2052)
    cmd.end()
    recs = cmd.records()
    assert [(r["isFastPipeline"], r["configBits"]) for r in recs] == [(1, 2), (0, 1), (1, 2), (0, 1)]


def test_premultiply_argument_checks(native):
    # rejected before any CUDA call (the pointers are never dereferenced)
    base = 0x7F0000000000
    f = native.nvproPyramidPremultiplyAlpha
    assert f(None, None, 0, base, 0, 8, 8) == N.ERROR_INVALID_ARGUMENT  # null source
    assert f(None, base, 0, base, 0, 0, 8) == N.ERROR_INVALID_ARGUMENT  # empty
    assert f(None, base, 16, base, 0, 8, 8) == N.ERROR_INVALID_ARGUMENT  # pitch below 4 * width
    assert f(None, base + 2, 0, base + 2, 0, 8, 8) == N.ERROR_UNSUPPORTED  # texels not 4-byte aligned
    assert f(None, base, 0, base + 64, 0, 8, 8) == N.ERROR_INVALID_ARGUMENT  # overlapping, not equal
    assert f(None, base, 32, base, 64, 8, 8) == N.ERROR_INVALID_ARGUMENT  # same start, different pitches


def test_general_blit_mode_records(native):
    """nvproCmdPyramidDispatchEx with nvproPyramidBlitGeneralDispatcher: the
    demo's generalblit loop -- the fast dispatcher where it accepts a level,
    else one blit record per level."""
    blit = P.blit_general_dispatcher()
    for w, h in [(1920, 1080), (4095, 4095), (2052, 2052), (2048, 2048), (5, 3), (1, 9), (64, 1)]:
        recs = record(w, h, general=blit)
        got = [(2 if r["isBlit"] else r["isFastPipeline"], r["pushConstant"],
                r["groupCountX"] if r["isFastPipeline"] else 1) for r in recs]
        assert got == O.fast_or_blit_schedule(w, h), (w, h)
    cmd = P.Cmd(N.CMD_RECORD_ONLY)
    cmd.begin(None)
    expect_error(N.ERROR_INVALID_STATE, lambda: N.check(native.nvproPyramidCmdBlitLevel(cmd.handle, 0)))


def test_plain_c_caller(native, repo_tmp):
    """The header and library from a strict C99 program (gcc -pedantic
    -Werror): the recorded schedules equal the oracle's, with config bits and
    the blit dispatcher."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc") or shutil.which("cc")
    if gcc is None:
        pytest.skip("no C compiler")
    exe = repo_tmp / "c_caller"
    lib_dir = N.LIB_PATH.parent
    subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "c_caller.c"), "-o", str(exe), "-L", str(lib_dir), "-lnvpro_pyramid_cuda",
                    f"-Wl,-rpath,{lib_dir}"], check=True)
    for w, h, args in [(1920, 1080, []), (4095, 4095, []), (2052, 2052, ["2", "1", "0"]), (1920, 1080, ["0", "0", "1"])]:
        out = subprocess.run([str(exe), str(w), str(h), *args], check=True, capture_output=True, text=True).stdout
        lines = out.strip().splitlines()
        levels = O.full_levels(w, h)
        assert lines[0] == f"levels {levels} bytes {O.offsets(w, h, levels, 4)[-1]}"
        recs = [tuple(map(int, ln.split())) for ln in lines[1:]]
        fast_bits, general_bits, blit = map(int, args) if args else (0, 0, 0)
        want = O.fast_or_blit_schedule(w, h) if blit else O.default_schedule(w, h)
        got = [(2 if b else f, pc, g if (f or not b) else 1) for f, pc, g, b, _ in recs]
        assert got == [tuple(x) for x in want], (w, h, args)
        assert all(c == (fast_bits if f else general_bits) for f, _, _, b, c in recs if not b)


def header_prototypes():
    """name -> number of parameters, from every NVPRO_PYRAMID_API declaration."""
    protos = {}
    for hdr in (ROOT / "include").glob("*.h"):
        src = re.sub(r"/\*.*?\*/", "", hdr.read_text(), flags=re.S)
        for m in re.finditer(r"NVPRO_PYRAMID_API\s+[\w\s\*]+?\b(\w+)\s*\(([^;]*?)\)\s*;", src, flags=re.S):
            params = m.group(2).strip()
            protos[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    return protos


def test_python_signatures_match_header_arity(native):
    protos = header_prototypes()
    assert len(protos) >= 40
    for name, n in protos.items():
        assert len(N.SIGNATURES[name][1]) == n, (name, n, len(N.SIGNATURES[name][1]))
