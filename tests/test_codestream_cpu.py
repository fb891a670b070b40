"""Host codestream reader (jpxlg_codestream_*): headers, TOC, modular
sub-bitstreams and the VarDCT sections of cjxl-encoded fixtures, decoded to
the frame's integer content (jpxl-decode decode.rs:2513 decode_vardct_frame,
vardct/hf_coeff.rs:689).

The fixtures (tests/golden/codestream/, copied by make_codestream_golden.py
from the reference's tests/fixtures/handmade) are real encoder output, so a
wrong context model or a misread field shows up as an ANS stream that does
not end in its final state (an error) or a section whose reader stops short
of, or past, the size its TOC entry gives.  Host code only.
"""
from pathlib import Path

import numpy as np
import pytest

import jpxl_gb300 as jg

GOLDEN = Path(__file__).resolve().parent / "golden" / "codestream"
VARDCT = sorted(p.stem for p in GOLDEN.glob("*_vardct_*.jxl"))
PROGRESSIVE = sorted(p.stem for p in GOLDEN.glob("*progressive*.jxl"))
ERR_STREAM = -8


def load(name):
    return jg.Codestream((GOLDEN / (name + ".jxl")).read_bytes())


def test_fixtures_present():
    assert len(VARDCT) == 10, VARDCT
    assert len(PROGRESSIVE) == 3, PROGRESSIVE


@pytest.mark.parametrize("name", PROGRESSIVE)
def test_progressive_fixture_decodes_every_pass(name):
    """Several HF passes (each its own coefficient orders, histograms and
    group sections, coefficients shifted per pass) in a multi-section TOC."""
    cs = load(name)
    i = cs.info
    if name.startswith("73_"):
        return  # an LF frame first; see test_lf_frame_streams
    assert i["num_passes"] == (3 if name.startswith("70_") else 2)
    assert i["sections"] == 3 + i["num_passes"]  # LfGlobal, LF group, HfGlobal, a group per pass
    assert i["sections_exact"] == i["sections"]
    assert np.count_nonzero(cs.coefficients()) > 0


def test_two_lf_groups():
    """128 x 2176: two LF groups (2048 rows each) and nine groups, thirteen
    sections; varblocks of both LF groups land in one frame-wide map."""
    cs = load("64_vardct_lfgroupseam_rgb_128x2176_nofilters_d6")
    i = cs.info
    assert (i["width"], i["height"]) == (128, 2176)
    assert i["sections"] == 13 and i["sections_exact"] == 13
    b = cs.blocks()
    assert np.count_nonzero(b["block_map"] & 0x80) == i["num_varblocks"] == 16 * 272


@pytest.mark.parametrize("name", VARDCT)
def test_vardct_fixture_decodes_with_every_section_exact(name):
    cs = load(name)
    i = cs.info
    assert i["encoding"] == 0
    assert i["sections"] >= 1
    assert i["sections_exact"] == i["sections"], "a section ended away from its TOC size"
    side = 64 if name.startswith(("63_", "82_", "109_")) else 128
    if name.startswith("64_"):
        assert (i["width"], i["height"]) == (128, 2176)
        return
    if name.startswith("83_"):
        assert (i["width"], i["height"]) == (384, 320)
        return
    assert (i["width"], i["height"]) == (side, side)
    assert i["colour_space"] == (0 if ("_rgb_" in name or "_rgba_" in name) else 1)
    assert i["xyb_encoded"] == 1
    if "nofilters" in name:
        assert i["gaborish"] == 0 and i["epf_iters"] == 0
    else:
        assert i["gaborish"] == 1 and i["epf_iters"] >= 1
    assert i["blocks_w"] == side // 8 and i["blocks_h"] == side // 8
    assert i["num_varblocks"] == sum(i["transform_counts"])


# Block rows x columns of each DctSelect (Table I.1).
SHAPES = {0: (1, 1), 1: (1, 1), 2: (1, 1), 3: (1, 1), 4: (2, 2), 5: (4, 4), 6: (2, 1),
          7: (1, 2), 8: (4, 1), 9: (1, 4), 10: (4, 2), 11: (2, 4), 12: (1, 1), 13: (1, 1),
          14: (1, 1), 15: (1, 1), 16: (1, 1), 17: (1, 1), 18: (8, 8), 19: (8, 4), 20: (4, 8)}


@pytest.mark.parametrize("name", VARDCT)
def test_block_map_tiles_the_frame(name):
    cs = load(name)
    b = cs.blocks()
    bmap = b["block_map"]
    bh, bw = bmap.shape
    cover = np.zeros((bh, bw), np.int32)
    counts = np.zeros(27, np.int64)
    for by in range(bh):
        for bx in range(bw):
            if bmap[by, bx] & 0x80:
                sel = int(bmap[by, bx] & 0x7F)
                counts[sel] += 1
                r, c = SHAPES[sel]
                cover[by:by + r, bx:bx + c] += 1
                assert (bmap[by:by + r, bx:bx + c] & 0x7F == sel).all()
                assert (b["hf_mul"][by:by + r, bx:bx + c] == b["hf_mul"][by, bx]).all()
    assert (cover == 1).all()
    assert counts.tolist() == cs.info["transform_counts"]
    assert (b["hf_mul"] >= 1).all()
    assert b["sharpness"].max() <= 7


@pytest.mark.parametrize("name", VARDCT)
def test_coefficients_sit_outside_the_lf_corners(name):
    """The HF coefficients never fill a varblock's LLF corner (those cells
    come from the LF image), and the content is non-trivial."""
    cs = load(name)
    coeff = cs.coefficients()
    b = cs.blocks()
    bmap = b["block_map"]
    assert np.count_nonzero(coeff) > 0
    for by, bx in zip(*np.nonzero(bmap & 0x80)):
        r, c = SHAPES[int(bmap[by, bx] & 0x7F)]
        cr, cc = min(r, c), max(r, c)
        for ch in range(3):
            if r > c:  # portrait: stored transposed
                corner = coeff[ch, 8 * by:8 * by + cc, 8 * bx:8 * bx + cr][:c, :r]
            else:
                corner = coeff[ch, 8 * by:8 * by + cr, 8 * bx:8 * bx + cc][:r, :c]
            assert not corner.any(), (by, bx, ch)


@pytest.mark.parametrize("name", VARDCT)
def test_truncated_codestream_is_a_stream_error(name):
    data = (GOLDEN / (name + ".jxl")).read_bytes()
    for cut in (len(data) // 3, len(data) - 1):
        with pytest.raises(jg.JpxlError) as e:
            jg.Codestream(data[:cut])
        assert e.value.code == ERR_STREAM


def test_lf_planes_are_plausible():
    """Grey fixtures: the X and B LF planes of a grey image are close to
    constant while Y carries the picture."""
    cs = load("51_vardct_mixed_gray_128x128_nofilters_d4")
    lf = cs.blocks()["lf"]
    assert np.ptp(lf[1]) > 10 * max(1, np.ptp(lf[0]))


def test_not_a_codestream():
    with pytest.raises(jg.JpxlError) as e:
        jg.Codestream(b"\x00\x00\x00\x0cJXL \r\n\x87\x0b")
    assert e.value.code == ERR_STREAM


def test_unsupported_feature_is_reported_not_misdecoded():
    """110_noise_rgb_32x32 asks for photon noise, a feature the reader does
    not carry: it is reported with its name instead of decoded wrongly."""
    with pytest.raises(jg.JpxlError) as e:
        load("110_noise_rgb_32x32")
    assert e.value.code == ERR_STREAM
    assert "noise" in str(e.value)


@pytest.mark.parametrize("name,w,h,gen", [
    ("60_sawtooth_32x32_lossless", 32, 32, lambda x, y: [(x * 7 + y * 3) % 256]),
    ("40_checker_64x64_lossless", 64, 64,
     lambda x, y: [np.where((x // 8 + y // 8) % 2 == 0, 255, 0)] * 3),
    ("11_modular_gradient_256x256_lossless", 256, 256, lambda x, y: [x, y, (x + y) % 256]),
    ("07_modular_gray_8x8_lossless", 8, 8, lambda x, y: [(x + y) * 255 // 14]),
    ("03_gradient_8x8_lossless", 8, 8, lambda x, y: [x * 255 // 7, y * 255 // 7, (x + y) % 256]),
    ("09_modular_rgb_64x64_lossless", 64, 64,
     lambda x, y: [x * 255 // 63, y * 255 // 63, (x + y) % 256]),
    ("05_gradient_300x200_lossless", 300, 200,
     lambda x, y: [x * 255 // 299, y * 255 // 199, (x + y) % 256]),
    ("12_modular_gray_300x200_lossless", 300, 200, lambda x, y: [(x + y) * 255 // 498]),
    ("21_gradient_260x10_lossless", 260, 10,
     lambda x, y: [x * 255 // 259, y * 255 // 9, (x + y) % 256]),
    # several groups: G.2.3 / G.4.2 channel pieces in their own sections
    ("14_modular_gray_600x520_multisection_lossless", 600, 520,
     lambda x, y: [(x + y) * 255 // 1118]),
    ("15_modular_rgb_600x520_multisection_lossless", 600, 520,
     lambda x, y: [x * 255 // 599, y * 255 // 519, (x + y) % 256]),
    ("16_modular_gray_511x8_multisection_lossless", 511, 8, lambda x, y: [(x + y) * 255 // 517]),
])
def test_lossless_modular_frames_match_their_generators(name, w, h, gen):
    """Lossless modular frames (MA trees, the H.5 predictor, RCT, squeeze and
    palettes, cjxl -d 0): every channel equals the generator each sidecar
    states."""
    cs = load(name)
    assert cs.info["encoding"] == 1 and (cs.info["width"], cs.info["height"]) == (w, h)
    assert cs.info["sections_exact"] == cs.info["sections"]
    y, x = np.mgrid[0:h, 0:w]
    want = gen(x, y)
    assert cs.info["num_channels"] == len(want)
    for c, plane in enumerate(want):
        assert np.array_equal(cs.channel(c), plane), c


@pytest.mark.parametrize("name", ["72_lfframe_gray_128x128_nofilters",
                                  "73_progressive_all_gray_128x128_nofilters"])
def test_lf_frame_streams(name):
    """cjxl --progressive_dc: a modular LF frame (squeezed, 16x16) ahead of
    the VarDCT frame, which takes its LF from it (kUseLfFrame)."""
    cs = load(name)
    i = cs.info
    assert i["encoding"] == 0 and i["sections_exact"] == i["sections"]
    assert i["num_passes"] == (1 if name.startswith("72_") else 2)


def test_mutated_codestreams_fail_cleanly():
    """Seeded bit flips, byte overwrites, truncations and appended garbage over
    every fixture: each decodes or reports a stream error; nothing crashes or
    runs away (a few seconds in all)."""
    rng = np.random.default_rng(20261204)
    files = sorted(GOLDEN.glob("*.jxl"))
    decoded = 0
    for trial in range(2000):
        data = bytearray(files[trial % len(files)].read_bytes())
        kind = trial % 4
        if kind == 0:
            for _ in range(int(rng.integers(1, 4))):
                i = int(rng.integers(len(data)))
                data[i] ^= 1 << int(rng.integers(8))
        elif kind == 1:
            for _ in range(int(rng.integers(1, 6))):
                data[int(rng.integers(min(40, len(data))))] = int(rng.integers(256))
        elif kind == 2:
            data = data[:int(rng.integers(2, len(data)))]
        else:
            data += bytes(rng.integers(0, 256, int(rng.integers(1, 64))).tolist())
        try:
            jg.Codestream(bytes(data))
            decoded += 1
        except jg.JpxlError as e:
            assert e.code == ERR_STREAM
    assert 0 < decoded < 2000


def _box(kind: bytes, body: bytes) -> bytes:
    return (8 + len(body)).to_bytes(4, "big") + kind + body


SIGNATURE = bytes([0, 0, 0, 0x0C]) + b"JXL " + bytes([0x0D, 0x0A, 0x87, 0x0A])


def test_container_jxlc_and_jxlp():
    """The same stream bare, in one jxlc box, and split over jxlp fragments
    (18181-2; jpxl-decode container.rs) decodes to the same content; other
    boxes are skipped."""
    name = "52_vardct_mixed_gray_128x128_filters_d1"
    data = (GOLDEN / (name + ".jxl")).read_bytes()
    ftyp = _box(b"ftyp", b"jxl " + bytes(4) + b"jxl ")
    boxed = SIGNATURE + ftyp + _box(b"jxlc", data) + _box(b"Exif", bytes(8))
    cut = len(data) // 3
    parts = SIGNATURE + ftyp + _box(b"jxlp", (0).to_bytes(4, "big") + data[:cut]) + \
        _box(b"xml ", b"<x/>") + _box(b"jxlp", (1 | 1 << 31).to_bytes(4, "big") + data[cut:])
    ref = load(name).coefficients()
    for blob in (boxed, parts):
        cs = jg.Codestream(blob)
        assert cs.info["sections_exact"] == cs.info["sections"]
        assert np.array_equal(cs.coefficients(), ref)


def test_container_errors():
    data = (GOLDEN / "51_vardct_mixed_gray_128x128_nofilters_d4.jxl").read_bytes()
    bad = [SIGNATURE + _box(b"jxlp", (1).to_bytes(4, "big") + data),      # wrong first index
           SIGNATURE + _box(b"jxlp", (0).to_bytes(4, "big") + data),      # no final fragment
           SIGNATURE + _box(b"jxlc", data)[:-5] + b"\x00" * 2,            # box past the end
           SIGNATURE]                                                      # no codestream
    for blob in bad:
        with pytest.raises(jg.JpxlError) as e:
            jg.Codestream(blob)
        assert e.value.code == ERR_STREAM


def test_alpha_of_a_vardct_frame():
    """82_alpha_vardct_rgba_64x64_nofilters: the alpha channel, palette-coded
    in the frame's global modular section, equals djxl's to float rounding."""
    name = "82_alpha_vardct_rgba_64x64_nofilters"
    cs = load(name)
    ref = np.load(GOLDEN / (name + ".npy"))[0, :, :, 3]
    assert np.abs(cs.extra(0) - ref).max() < 1e-6


# Exif orientations 1-8 as the display transform of an [H, W, C] image
# (Table A.6 of 18181-1; djxl applies it, the reader reports it).
ORIENT = {1: lambda a: a, 2: lambda a: a[:, ::-1], 3: lambda a: a[::-1, ::-1],
          4: lambda a: a[::-1], 5: lambda a: a.transpose(1, 0, 2),
          6: lambda a: np.rot90(a, -1), 7: lambda a: a[::-1, ::-1].transpose(1, 0, 2),
          8: lambda a: np.rot90(a, 1)}
MODULAR_RGBA = ["80_alpha_rgba_8x8_lossless"] + sorted(
    p.stem for p in GOLDEN.glob("10[0-7]_orientation_*.jxl"))


@pytest.mark.parametrize("name", MODULAR_RGBA)
def test_modular_rgba_matches_djxl(name):
    """Lossless modular RGBA frames: the alpha channel follows the colour
    channels in the frame's channel list; after the stream's orientation the
    integers equal djxl's decode (f32 round trip only)."""
    cs = load(name)
    i = cs.info
    assert i["num_extra"] == 1 and i["num_channels"] == 4
    rgba = np.stack([cs.channel(k) for k in range(4)], -1).astype(np.float32) / 255.0
    assert np.array_equal(cs.extra(0), rgba[:, :, 3])
    assert rgba[:, :, 3].min() < rgba[:, :, 3].max()
    ref = np.load(GOLDEN / (name + ".npy"))[0]
    got = ORIENT[i["orientation"]](rgba)
    assert got.shape == ref.shape
    assert np.abs(got - ref).max() < 1e-6


def test_orientation_fixtures_cover_all_eight():
    assert sorted(load(n).info["orientation"] for n in MODULAR_RGBA[1:]) == list(range(1, 9))


def test_multigroup_rgba_decodes_every_section_exactly():
    """81_alpha_rgba_600x520_lossless: 3x3 groups of 256 with an alpha channel
    among the group pieces; twelve sections, each read to its TOC size, and
    an alpha plane that is not constant."""
    cs = load("81_alpha_rgba_600x520_lossless")
    i = cs.info
    assert (i["sections"], i["sections_exact"], i["num_channels"]) == (12, 12, 4)
    a = cs.channel(3)
    assert a.shape == (520, 600) and a.min() < a.max()
    assert np.array_equal(cs.extra(0), a.astype(np.float32) / 255.0)


def test_vardct_alpha_over_several_groups():
    """83_alpha_vardct_rgba_384x320_nofilters: an alpha channel larger than a
    group, decoded in the pass groups after each group's HF coefficients
    (G.4.2), so a wrong split desynchronises the colour, not just the alpha:
    all seven sections end at their TOC sizes, and the alpha (a radial ramp
    with a transparent notch) is continuous across the group seams."""
    cs = load("83_alpha_vardct_rgba_384x320_nofilters")
    i = cs.info
    assert (i["sections"], i["sections_exact"], i["num_extra"]) == (7, 7, 1)
    a = np.round(cs.extra(0) * 255).astype(np.int32)
    assert a.min() == 0 and a.max() > 250
    dx, dy = np.abs(np.diff(a, axis=1)), np.abs(np.diff(a, axis=0))
    assert dx[:, 255].max() <= 4 and dy[255].max() <= 4


def test_allocation_and_pixel_limits_reject_before_allocating():
    """jpxl-core limits.rs: every plane the reader allocates for a stream is
    charged to a cumulative meter before it is made; a stream past the limit
    (or an image past the pixel limit) is a stream error, not an allocation.
    Fixture 53 (128x128 VarDCT) needs a few hundred kB of planes: it opens
    under the defaults and under a 16 MB meter, and fails cleanly under a
    64 kB one or a 100-pixel limit."""
    data = (GOLDEN / "53_vardct_mixed_gray_128x128_filters_d4.jxl").read_bytes()
    jg.Codestream(data).close()
    jg.Codestream(data, max_alloc_bytes=16 << 20).close()
    with pytest.raises(jg.JpxlError) as e:
        jg.Codestream(data, max_alloc_bytes=64 << 10)
    assert e.value.code == -8 and "allocation limit" in str(e.value)
    with pytest.raises(jg.JpxlError) as e:
        jg.Codestream(data, max_pixels=100)
    assert e.value.code == -8 and "pixel limit" in str(e.value)
    # the limits are per stream: the next default open succeeds again
    jg.Codestream(data).close()


def test_parallel_open_matches_serial():
    """open_codestreams parses on host threads; every stream's headers,
    block data and coefficients equal a serial open's, in order."""
    datas = [(GOLDEN / (n + ".jxl")).read_bytes() for n in VARDCT] * 3
    par = jg.open_codestreams(datas, workers=8)
    try:
        assert len(par) == len(datas)
        for d, p in zip(datas, par):
            s = jg.Codestream(d)
            try:
                assert p.info == s.info
                pb, sb = p.blocks(), s.blocks()
                for k in sb:
                    assert np.array_equal(pb[k], sb[k]), k
                assert np.array_equal(p.coefficients(), s.coefficients())
            finally:
                s.close()
    finally:
        for p in par:
            p.close()


def test_parallel_open_reports_a_bad_stream():
    """A rejected stream among good ones raises its stream error; the
    others are closed."""
    good = (GOLDEN / (VARDCT[0] + ".jxl")).read_bytes()
    with pytest.raises(jg.JpxlError) as e:
        jg.open_codestreams([good, good[: len(good) // 3], good], workers=3)
    assert e.value.code == ERR_STREAM
