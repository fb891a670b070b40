"""Parity of the CUDA path (through the C ABI) with the CPU restatement.

Bar: quantized coefficients, LF samples, CfL factors and 8-bit pixels
bit-identical; float planes bit-identical where the reference arithmetic is
restated exactly (every stage before SSIMULACRA2's blur); SSIMULACRA2 within
0.01 points (the blur is the reference's f64 recursion restated as its f32
9-tap FIR).  Sizes are small enough for the CPU restatement to finish in
seconds; full-size configurations are covered by size-independent
properties in test_gpu_properties.py.
"""
import numpy as np
import pytest

import jpxl_gb300 as jg
from jpxl_gb300 import synth

pytestmark = pytest.mark.gpu

SCORE_TOL = 0.01  # SSIMULACRA2 points


def _run(ctx, oracle, rgb, bmap, req, sharp=7, hf=1):
    h, w = rgb.shape[:2]
    hf_mul = np.full(bmap.shape, hf, np.uint32)
    sh = np.full(bmap.shape, sharp, np.uint8)
    layout = jg.Layout(ctx, w, h, bmap, hf_mul, sh)
    plan = ctx.encode_transform(layout, rgb, req)
    rc, ref = oracle.encode(rgb, bmap, hf_mul, global_scale=req.global_scale,
                            quant_lf=req.quant_lf, x_qm_scale=req.x_qm_scale,
                            b_qm_scale=req.b_qm_scale, gaborish=req.gaborish, cfl=req.cfl)
    assert rc == 0
    return layout, plan, ref, hf_mul, sh


def _assert_plan_equal(plan, ref):
    assert tuple(plan.lf_factors) == tuple(ref["lf_factors"])
    assert np.array_equal(plan.cfl_x, ref["cfl_x"]), (plan.cfl_x, ref["cfl_x"])
    assert np.array_equal(plan.cfl_b, ref["cfl_b"])
    assert np.array_equal(plan.lf, ref["lf"]), np.argwhere(plan.lf != ref["lf"])[:5]
    diff = np.argwhere(plan.qcoeff != ref["qcoeff"])
    assert diff.size == 0, (len(diff), diff[:5])


def test_stages_are_bit_identical(ctx, oracle):
    w, h = 160, 96
    rgb = synth.synthetic_rgb(w, h, seed=4)
    bmap = synth.activity_cover(rgb)
    req = jg.EncodeRequest(global_scale=30000, gaborish=True)
    layout = jg.Layout(ctx, w, h, bmap)
    st = ctx.encode_stages(layout, rgb, req)
    rc, ref = oracle.encode(rgb, bmap, np.ones(bmap.shape, np.uint32), global_scale=30000,
                            gaborish=True, stages=True)
    assert rc == 0
    assert np.array_equal(st["xyb"].view(np.uint32), ref["xyb"].view(np.uint32))
    assert np.array_equal(st["pre"].view(np.uint32), ref["pre"].view(np.uint32))
    assert np.array_equal(st["coeff"].view(np.uint32), ref["coeff"].view(np.uint32))


@pytest.mark.parametrize("w,h", [(520, 330), (517, 331), (1001, 421), (250, 213), (130, 7),
                                 (7, 130), (9, 4), (5, 2), (3, 3), (2, 5), (1, 1)])
def test_precondition_interior_and_edge_tiles(ctx, oracle, w, h):
    """Frames with interior 104x104 tiles (the register-resident paired
    update) inside a ring of edge tiles (border taps, the columns past the
    groups of four, the n % 4 division tail: 517 x 331 and 1001 x 421), and
    frames smaller than one tile, down to a single sample."""
    rgb = synth.synthetic_rgb(w, h, seed=w + h, bits=16)
    bmap = synth.fixed_dct8_map(w, h)
    req = jg.EncodeRequest(global_scale=30000, gaborish=True)
    layout = jg.Layout(ctx, w, h, bmap)
    st = ctx.encode_stages(layout, rgb, req, bits=16)
    rc, ref = oracle.encode(rgb, bmap, np.ones(bmap.shape, np.uint32), bits=16,
                            global_scale=30000, gaborish=True, stages=True)
    assert rc == 0
    assert np.array_equal(st["xyb"].view(np.uint32), ref["xyb"].view(np.uint32))
    diff = np.argwhere(st["pre"].view(np.uint32) != ref["pre"].view(np.uint32))
    assert diff.size == 0, (len(diff), diff[:5])


def test_xyb_of_every_16bit_code_point(ctx, oracle):
    """All 65536 code points per channel pass the exact-parity cube root."""
    w, h = 256, 256
    v = np.arange(65536, dtype=np.uint16).reshape(h, w)
    rgb = np.stack([v, np.roll(v, 7919), np.roll(v, 31337)], axis=-1)
    bmap = synth.fixed_dct8_map(w, h)
    layout = jg.Layout(ctx, w, h, bmap)
    st = ctx.encode_stages(layout, rgb, jg.EncodeRequest(), bits=16)
    rc, ref = oracle.encode(rgb, bmap, np.ones(bmap.shape, np.uint32), global_scale=32768,
                            bits=16, stages=True)
    assert rc == 0
    assert np.array_equal(st["xyb"].view(np.uint32), ref["xyb"].view(np.uint32))


def test_c1_dct8_plan_and_pixels(ctx, oracle):
    """512x512 RGB8, DCT8 only, global_scale 40000, CfL, Gaborish + 3-step EPF
    with uniform sharpness 7."""
    w = h = 512
    rgb = synth.synthetic_rgb(w, h, seed=1)
    bmap = synth.fixed_dct8_map(w, h)
    req = jg.EncodeRequest.with_global_scale(40000, gaborish=True, epf_iters=3)
    layout, plan, ref, hf, sh = _run(ctx, oracle, rgb, bmap, req)
    _assert_plan_equal(plan, ref)
    r = jg.PlanRenderer(ctx)
    for kind, code in (("xyb", 0), ("linear", 1), ("srgb8", 2)):
        got = r.render(layout, plan, req, out=kind)
        rc, want = oracle.reconstruct(w, h, bmap, hf, sh, ref, global_scale=40000, gaborish=True,
                                      epf_iters=3, out_kind=code)
        assert rc == 0
        if kind == "srgb8":
            assert np.array_equal(got, want)
        else:
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), kind


@pytest.mark.parametrize("bits", [8, 16])
def test_square_cover_plan_and_pixels(ctx, oracle, bits):
    """Mixed DCT8/16/32 (activity cover), RGB8 and RGB16."""
    w, h = 384, 256
    rgb = synth.synthetic_rgb(w, h, seed=9, bits=bits)
    bmap = synth.activity_cover(rgb)
    assert len(np.unique(bmap & 0x1F)) == 3
    req = jg.EncodeRequest.with_global_scale(25000, gaborish=True, epf_iters=3)
    layout, plan, ref, hf, sh = _run(ctx, oracle, rgb, bmap, req)
    _assert_plan_equal(plan, ref)
    got = jg.PlanRenderer(ctx).render(layout, plan, req, out="linear_at_depth", bits=bits)
    rc, want = oracle.reconstruct(w, h, bmap, hf, sh, ref, global_scale=25000, gaborish=True,
                                  epf_iters=3, out_kind=3, bits=bits)
    assert rc == 0 and np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("w,h", [(7, 9), (33, 17), (257, 263)])
def test_ragged_frames(ctx, oracle, w, h):
    rgb = synth.synthetic_rgb(w, h, seed=w * h)
    bmap = synth.activity_cover(rgb, 12.0, 8.0)
    req = jg.EncodeRequest.with_global_scale(20000, gaborish=True, epf_iters=3)
    layout, plan, ref, hf, sh = _run(ctx, oracle, rgb, bmap, req)
    _assert_plan_equal(plan, ref)
    got = jg.PlanRenderer(ctx).render(layout, plan, req, out="srgb8")
    rc, want = oracle.reconstruct(w, h, bmap, hf, sh, ref, global_scale=20000, gaborish=True,
                                  epf_iters=3, out_kind=2)
    assert rc == 0 and np.array_equal(got, want)


@pytest.mark.parametrize("epf", [0, 1, 2])
def test_qm_scales_and_epf_steps(ctx, oracle, epf):
    w, h = 128, 120
    rgb = synth.synthetic_rgb(w, h, seed=21)
    bmap = synth.activity_cover(rgb)
    req = jg.EncodeRequest(global_scale=50000, quant_lf=4, x_qm_scale=3, b_qm_scale=4,
                           gaborish=False, epf_iters=epf)
    layout, plan, ref, hf, sh = _run(ctx, oracle, rgb, bmap, req, sharp=5, hf=2)
    _assert_plan_equal(plan, ref)
    got = jg.PlanRenderer(ctx).render(layout, plan, req, out="srgb8")
    rc, want = oracle.reconstruct(w, h, bmap, hf, sh, ref, global_scale=50000, quant_lf=4,
                                  x_qm_scale=3, b_qm_scale=4, epf_iters=epf, out_kind=2)
    assert rc == 0 and np.array_equal(got, want)


def test_grayscale_disables_cfl(ctx, oracle):
    w, h = 96, 64
    g = synth.synthetic_rgb(w, h, seed=2)[..., :1]
    rgb = np.ascontiguousarray(np.repeat(g, 3, axis=2))
    bmap = synth.fixed_dct8_map(w, h)
    req = jg.EncodeRequest.with_global_scale(30000)
    layout, plan, ref, hf, sh = _run(ctx, oracle, rgb, bmap, req)
    _assert_plan_equal(plan, ref)
    assert tuple(plan.lf_factors) == (128, 128) and not plan.cfl_x.any() and not plan.cfl_b.any()


def test_render_all_nine_shapes_from_random_coefficients(ctx, oracle):
    """The renderer over rectangles too (decoder streams carry them)."""
    w, h = 200, 136
    bmap = synth.mixed_cover(w, h, seed=0)
    assert len(np.unique(bmap & 0x1F)) == 9
    rng = np.random.default_rng(8)
    bw, bh = (w + 7) // 8, (h + 7) // 8
    plan = {"qcoeff": rng.integers(-6, 7, (3, bh * 8, bw * 8)).astype(np.int32)
            * (rng.random((3, bh * 8, bw * 8)) < 0.2),
            "lf": rng.integers(-40, 400, (3, bh, bw)).astype(np.int32),
            "cfl_x": rng.integers(-20, 20, ((bh + 7) // 8, (bw + 7) // 8)).astype(np.int8),
            "cfl_b": rng.integers(-20, 20, ((bh + 7) // 8, (bw + 7) // 8)).astype(np.int8),
            "lf_factors": (131, 120)}
    plan["qcoeff"] = plan["qcoeff"].astype(np.int32)
    hf = rng.integers(1, 4, bmap.shape).astype(np.uint32)
    sh = rng.integers(0, 8, bmap.shape).astype(np.uint8)
    layout = jg.Layout(ctx, w, h, bmap, hf, sh)
    p = jg.Plan(plan["qcoeff"], plan["lf"], plan["cfl_x"], plan["cfl_b"], plan["lf_factors"])
    req = jg.EncodeRequest(global_scale=12000, quant_lf=8, gaborish=True, epf_iters=3)
    for kind, code in (("xyb", 0), ("srgb8", 2)):
        got = jg.PlanRenderer(ctx).render(layout, p, req, out=kind)
        rc, want = oracle.reconstruct(w, h, bmap, hf, sh, plan, global_scale=12000, quant_lf=8,
                                      gaborish=True, epf_iters=3, out_kind=code)
        assert rc == 0
        if kind == "srgb8":
            assert np.array_equal(got, want)
        else:
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_score_identical_is_exactly_one_hundred(ctx, oracle):
    a, _ = oracle.perceptual_pair(256, 192, 1, 0.0, 1)
    assert jg.score_pair(ctx, a, a) == 100.0


# The blur reproduces the reference's f32 outputs (up to its f64 rounding
# ties), so scores agree far inside the 0.01-point contract; MEASURED_TOL
# holds that.  Sizes cover the minimum frame, widths and heights that are not
# multiples of the 32-column strips or 32-row tiles, a single strip, tall and
# wide frames (many segments along one axis) and the widest row the row pass
# stages.
MEASURED_TOL = 1e-4


@pytest.mark.parametrize("w,h,amp", [(320, 240, 0.002), (320, 240, 0.03), (67, 45, 0.01),
                                     (8, 8, 0.02), (33, 1000, 0.005), (1000, 33, 0.005),
                                     (8192, 24, 0.003), (517, 331, 0.0005)])
def test_score_matches_the_restatement(ctx, oracle, w, h, amp):
    a, b = oracle.perceptual_pair(w, h, 2, amp, 7)
    want, _, want_terms = oracle.ssim2(a, b)
    got = jg.score_pair(ctx, a, b)
    assert abs(got - want) < SCORE_TOL, (got, want)
    assert abs(got - want) < MEASURED_TOL, (got, want)
    ref = jg.PrecomputedReference(ctx, a)
    try:
        terms = np.asarray(jg.Ssimulacra2(ctx).score(ref, b).terms)[: len(want_terms)]
    finally:
        ref.close()
    # every pooled norm, not only their weighted sum (norms of near-zero maps
    # move by ~1e-8 where a blurred value sits on one of the reference's f64
    # rounding ties)
    assert np.allclose(terms, want_terms, rtol=1e-3, atol=1e-7), np.max(np.abs(terms - want_terms))


def test_score_of_the_recorded_4mp_pair(ctx, oracle):
    a, b = oracle.perceptual_pair(2400, 1800, 9, 0.01, 3)
    got = jg.score_pair(ctx, a, b)
    assert abs(got - 77.38494501660614) < SCORE_TOL
    assert abs(got - 77.38494501660614) < MEASURED_TOL


def test_wider_than_the_row_pass_is_an_error(ctx):
    a = np.zeros((3, 8, 8193), np.float32)
    with pytest.raises(jg.JpxlError):
        jg.PrecomputedReference(ctx, a)


def test_probe_equals_encode_render_score(ctx, oracle):
    w, h = 256, 192
    rgb = synth.synthetic_rgb(w, h, seed=12)
    bmap = synth.activity_cover(rgb)
    req = jg.EncodeRequest.with_global_scale(35000, gaborish=True, epf_iters=3)
    layout, plan, ref, hf, sh = _run(ctx, oracle, rgb, bmap, req)
    src = jg.srgb_to_linear_planes(rgb)
    pref = jg.PrecomputedReference(ctx, src)
    got = ctx.probe(layout, pref, rgb, req)
    rc, lin = oracle.reconstruct(w, h, bmap, hf, sh, ref, global_scale=35000, gaborish=True,
                                 epf_iters=3, out_kind=3, bits=8)
    want, _, _ = oracle.ssim2(src, lin)
    assert abs(got - want) < SCORE_TOL, (got, want)


def test_errors_are_statuses_not_crashes(ctx):
    w, h = 64, 64
    bad = synth.fixed_dct8_map(w, h)
    bad[0, 0] = 4 | 0x80
    with pytest.raises(jg.JpxlError) as e:
        jg.Layout(ctx, w, h, bad)
    assert e.value.code == -2
    layout = jg.Layout(ctx, w, h, synth.fixed_dct8_map(w, h))
    rgb = synth.synthetic_rgb(w, h, seed=1)
    with pytest.raises(jg.JpxlError) as e:
        ctx.encode_transform(layout, rgb, jg.EncodeRequest(global_scale=0))
    assert e.value.code == -1
    with pytest.raises(jg.JpxlError) as e:
        ctx.encode_transform(layout, rgb, jg.EncodeRequest(global_scale=1, quant_lf=1 << 30))
    assert e.value.code == -3  # an LF step so small the integer leaves 2^20
    tiny = np.zeros((3, 7, 7), np.float32)
    with pytest.raises(jg.JpxlError) as e:
        jg.score_pair(ctx, tiny, tiny)
    assert e.value.code == -6
    # the context stays usable
    plan = ctx.encode_transform(layout, rgb, jg.EncodeRequest())
    assert plan.qcoeff.any()
