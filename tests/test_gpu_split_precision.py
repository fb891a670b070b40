"""The split-precision form of the DCTs (tcgen05 tensor cores, f32 operands
as bf16 terms, FP32 accumulation) against the FP64 truth and the FP32 form.

The bounds for the split form: decoded pixels within 1e-5 max-abs
(linear, [0, 1]) of the FP64 truth, SSIMULACRA2 within 0.01 points.  BF16x6
(three bf16 terms) meets them (measured 3.3e-6 at 2048x2048, the FP32
kernels' own error is 2.9e-6); BF16x3 (two terms) does not (1.1e-4).  The
quantized coefficients are compared with the FP32 form's (which equals the
reference's) and their mismatches counted.  A mismatch between adjacent
integers is a coefficient at a decision boundary that the two arithmetics
resolve differently; any other mismatch would be an error of the split form.
"""
import ctypes as C

import numpy as np
import pytest

import jpxl_gb300 as jg
from jpxl_gb300 import synth

pytestmark = pytest.mark.gpu

PIXEL_TOL = 1e-5
SCORE_TOL = 0.01
# Two bf16 terms (three products) carry about 16 bits per operand: measured
# 1.1e-4 max-abs at 2048x2048 (RMSE 3.2e-6), outside the 1e-5 bound, which
# three terms (six products) meet.  The two-term form is held to its own
# measured envelope.
PIXEL_TOL_X3 = 3e-4


def _req(gs, precision="fp32"):
    return jg.EncodeRequest.with_global_scale(gs, gaborish=True, epf_iters=3,
                                              precision=precision)


def _frame(ctx, w, h, seed, bits=16, gs=40000):
    rgb = synth.synthetic_rgb(w, h, seed=seed, bits=bits)
    cover = jg.select_blocks(ctx, rgb, _req(gs), bits)
    layout = jg.Layout(ctx, w, h, cover, 1, 7)
    return rgb, cover, layout


def _render_error(ctx, oracle, layout, cover, plan, precision, gs=40000):
    h, w = layout.height, layout.width
    lin = jg.PlanRenderer(ctx).render(layout, plan, _req(gs, precision), out="linear")
    hf = np.ones(cover.shape, np.uint32)
    sh = np.full(cover.shape, 7, np.uint8)
    p = dict(qcoeff=plan.qcoeff, lf=plan.lf, cfl_x=plan.cfl_x, cfl_b=plan.cfl_b,
             lf_factors=plan.lf_factors)
    rc, truth = oracle.fp64_reconstruct(w, h, cover, hf, sh, p, global_scale=gs, gaborish=True,
                                        epf_iters=3, out_kind=1)
    assert rc == 0
    return np.abs(lin.astype(np.float64) - truth)


@pytest.mark.parametrize("w,h", [(512, 384), (333, 217)])
def test_split_render_is_within_the_fp64_bound(ctx, oracle, w, h):
    rgb, cover, layout = _frame(ctx, w, h, seed=w + h)
    plan = ctx.encode_transform(layout, rgb, _req(40000))
    assert set(np.unique(cover & 0x7F)) <= {0, 4, 5}
    e32 = _render_error(ctx, oracle, layout, cover, plan, "fp32")
    e6 = _render_error(ctx, oracle, layout, cover, plan, "bf16x6")
    e3 = _render_error(ctx, oracle, layout, cover, plan, "bf16x3")
    print(f"{w}x{h} render max|err| vs fp64: fp32 {e32.max():.3e} bf16x6 {e6.max():.3e} "
          f"bf16x3 {e3.max():.3e}")
    assert float(e32.max()) < PIXEL_TOL
    assert float(e6.max()) < PIXEL_TOL
    assert float(e3.max()) < PIXEL_TOL_X3
    layout.close()


def _mismatches(a, b):
    d = a.astype(np.int64) - b.astype(np.int64)
    return int(np.count_nonzero(np.abs(d) == 1)), int(np.count_nonzero(np.abs(d) > 1))


@pytest.mark.parametrize("precision", ["bf16x3", "bf16x6"])
def test_split_encode_differs_only_at_decision_boundaries(ctx, precision):
    rgb, cover, layout = _frame(ctx, 512, 512, seed=77)
    ref = ctx.encode_transform(layout, rgb, _req(40000))
    got = ctx.encode_transform(layout, rgb, _req(40000, precision))
    adjacent, other = _mismatches(got.qcoeff, ref.qcoeff)
    lf_adj, lf_other = _mismatches(got.lf, ref.lf)
    n = ref.qcoeff.size
    cfl = int(np.count_nonzero(got.cfl_x != ref.cfl_x) + np.count_nonzero(got.cfl_b != ref.cfl_b))
    print(f"{precision}: qcoeff mismatches {adjacent} adjacent + {other} other of {n}; "
          f"LF {lf_adj} + {lf_other}; CfL tile factors differing {cfl}")
    assert other == 0 and lf_other == 0
    assert adjacent <= 1e-3 * n
    layout.close()


@pytest.mark.parametrize("precision", ["bf16x3", "bf16x6"])
def test_split_probe_score_is_within_contract(ctx, precision):
    w = h = 2048
    rgb, cover, layout = _frame(ctx, w, h, seed=1003)
    ref = jg.PrecomputedReference(ctx, jg.srgb_to_linear_planes(rgb, 16))
    try:
        s32 = ctx.probe(layout, ref, rgb, _req(40000))
        ss = ctx.probe(layout, ref, rgb, _req(40000, precision))
        again = ctx.probe(layout, ref, rgb, _req(40000, precision))
    finally:
        ref.close()
        layout.close()
    print(f"2048x2048 probe: fp32 {s32:.6f} {precision} {ss:.6f} |d| {abs(ss - s32):.2e}")
    assert ss == again  # deterministic
    assert abs(ss - s32) < SCORE_TOL


def test_split_full_size_render_within_fp64_bound(ctx, oracle):
    w = h = 2048
    rgb, cover, layout = _frame(ctx, w, h, seed=1003)
    plan = ctx.encode_transform(layout, rgb, _req(40000))
    e6 = _render_error(ctx, oracle, layout, cover, plan, "bf16x6")
    e3 = _render_error(ctx, oracle, layout, cover, plan, "bf16x3")
    print(f"2048x2048 render max|err| vs fp64: bf16x6 {e6.max():.3e} (rmse "
          f"{np.sqrt(np.mean(e6 ** 2)):.2e}) bf16x3 {e3.max():.3e} (rmse "
          f"{np.sqrt(np.mean(e3 ** 2)):.2e})")
    assert float(e6.max()) < PIXEL_TOL
    assert float(e3.max()) < PIXEL_TOL_X3
    layout.close()


def test_unknown_precision_is_rejected(ctx):
    rgb, cover, layout = _frame(ctx, 64, 64, seed=5)
    plan = ctx.encode_transform(layout, rgb, _req(40000))
    bad = _req(40000)._struct()
    bad.precision = 7
    out = np.zeros((3, 64, 64), np.float32)
    s = plan._struct()
    rc = ctx.lib.jpxlg_reconstruct(ctx.handle, layout.handle, C.byref(s), C.byref(bad),
                                   jg.OUT_LINEAR, 8, out.ctypes.data, jg.MEM_HOST)
    assert rc == -1
    layout.close()
