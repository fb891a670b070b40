"""Batched decode: the committed cjxl VarDCT streams, repeated to 256, rendered
to 8-bit sRGB by one graph launch (jpxlg_decode_batch_*).

Each stream's pixels must equal its own single-stream render bit for bit,
and against djxl's decode (the float .npy beside each fixture, quantized as
jpxl-decode decode.rs:3498 quantize_sample does: round half away from zero,
clamp to [0, 255]) every sample must lie within 1 DN; the samples that are
1 DN off are counted and reported."""
from pathlib import Path

import numpy as np
import pytest

import jpxl_gb300 as jg

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden" / "codestream"
WITH_DJXL = ["50_vardct_mixed_gray_128x128_nofilters_d1", "51_vardct_mixed_gray_128x128_nofilters_d4",
             "52_vardct_mixed_gray_128x128_filters_d1", "53_vardct_mixed_gray_128x128_filters_d4",
             "63_vardct_outofgamut_rgb_64x64_nofilters_d4", "70_progressive_ac_gray_128x128_nofilters",
             "71_qprogressive_ac_gray_128x128_nofilters", "72_lfframe_gray_128x128_nofilters",
             "73_progressive_all_gray_128x128_nofilters", "82_alpha_vardct_rgba_64x64_nofilters",
             "109_orientation_transpose_vardct_rgba_64x64"]
# streams without a djxl decode beside them: bit-exactness against the
# single-stream render only
RENDER_ONLY = ["06_gradient_300x200_lossy", "64_vardct_lfgroupseam_rgb_128x2176_nofilters_d6"]
ORIENT = {1: lambda a: a, 5: lambda a: a.transpose(1, 0, 2)}
N_STREAMS = 256


def quantize_8(v):
    """decode.rs:3498 quantize_sample at max 255 (f32 arithmetic)."""
    s = v.astype(np.float32) * np.float32(255.0)
    r = np.where(s >= 0, np.floor(s + np.float32(0.5)), np.ceil(s - np.float32(0.5)))
    r = np.where(np.isfinite(r), np.clip(r, 0, 255), 0)
    return r.astype(np.int32)


@pytest.mark.parametrize("precision", ["fp32", "bf16x6", "bf16x3"])
def test_256_streams_in_one_graph_match_single_renders_and_djxl(ctx, precision):
    names = WITH_DJXL + RENDER_ONLY
    order = [names[i % len(names)] for i in range(N_STREAMS)]
    data = {n: (GOLDEN / (n + ".jxl")).read_bytes() for n in names}
    streams = [jg.Codestream(data[n]) for n in order]
    single = {n: jg.Codestream(data[n]).render(ctx, "srgb8") for n in names}
    batch = jg.DecodeBatch(ctx, streams, "srgb8", precision=precision)
    try:
        outs = [b.copy() for b in batch.run()]
        again = batch.run()
        for a, b in zip(outs, again):
            assert np.array_equal(a, b)
    finally:
        batch.close()
    total = off = 0
    worst = 0
    differ = 0
    for n, out in zip(order, outs):
        if precision == "fp32":
            assert np.array_equal(out, single[n]), n
        else:
            differ += int((out != single[n]).sum())
        if n in RENDER_ONLY:
            continue
        ref = np.load(GOLDEN / (n + ".npy"))[0][:, :, :3]
        cs_orient = streams[order.index(n)].info["orientation"]
        got = ORIENT[cs_orient](out).astype(np.int32)[:, :, :ref.shape[2]]  # grey: plane 0
        want = quantize_8(ref)
        assert got.shape == want.shape, n
        d = np.abs(got - want)
        worst = max(worst, int(d.max()))
        off += int((d > 0).sum())
        total += d.size
    print(f"{precision}: {N_STREAMS} streams: {off} of {total} samples 1 DN off djxl, worst "
          f"{worst} DN; {differ} samples differ from the FP32 render")
    assert worst <= 1
    for s in streams:
        s.close()


def test_a_stream_the_renderer_does_not_carry_fails_creation(ctx):
    lossless = jg.Codestream((GOLDEN / "05_gradient_300x200_lossless.jxl").read_bytes())
    ok = jg.Codestream((GOLDEN / "52_vardct_mixed_gray_128x128_filters_d1.jxl").read_bytes())
    with pytest.raises(jg.JpxlError) as e:
        jg.DecodeBatch(ctx, [ok, lossless], "srgb8")
    assert e.value.code == -8 and "stream 1" in str(e.value)
