"""The FP64 truth oracle (oracle/oracle_fp64.cpp) pinned on the CPU.

It is the yardstick every result's error is stated against, so it is held to
the reference's own known answers where the reference states them in exact
terms (dct.rs:1572 DCT-8 of a constant and of an impulse, metric.rs:20
identical images score 100), to exact invertibility of its transforms, and
to the f32 restatement within f32 rounding: a difference larger than f32
rounding can explain would mean one of the two departs from the algorithm.
"""
import math

import numpy as np
import pytest

from jpxl_gb300 import synth
import jpxl_gb300 as jg

SHAPES = [(8, 8), (16, 16), (32, 32), (8, 16), (16, 8), (8, 32), (32, 8), (16, 32), (32, 16)]


def test_fp64_dct_known_answers(oracle):
    """dct.rs:1572: DCT-8 (1-D, normative) of a constant is the constant at
    DC; of an impulse at 0, X0 = 1/8 and X1 = sqrt(2) cos(pi/16) / 8."""
    const = np.ones((1, 8))
    out = oracle.dct_2d(const, f64=True)
    assert abs(out[0, 0] - 1.0) < 1e-14 and np.abs(out[0, 1:]).max() < 1e-14
    imp = np.zeros((1, 8))
    imp[0, 0] = 1.0
    out = oracle.dct_2d(imp, f64=True)
    assert abs(out[0, 0] - 0.125) < 1e-15
    assert abs(out[0, 1] - math.sqrt(2) * math.cos(math.pi / 16) / 8) < 1e-15
    # the f32 butterflies give the same numbers to f32 rounding
    f32 = oracle.dct_2d(imp.astype(np.float32))
    assert np.abs(f32 - out).max() < 1e-7


@pytest.mark.parametrize("rows,cols", SHAPES)
def test_fp64_transforms_invert_and_match_the_f32_butterflies(oracle, rows, cols):
    rng = np.random.default_rng(rows * 100 + cols)
    blk = rng.standard_normal((rows, cols))
    c64 = oracle.dct_2d(blk, f64=True)
    back = oracle.idct_2d(c64, rows, cols, f64=True)
    assert np.abs(back - blk).max() < 1e-13
    c32 = oracle.dct_2d(blk.astype(np.float32))
    assert c32.shape == c64.shape
    assert np.abs(c32 - c64).max() < 2e-7 * max(1.0, np.abs(c64).max())
    s32 = oracle.idct_2d(c64.astype(np.float32), rows, cols)
    s64 = oracle.idct_2d(c64, rows, cols, f64=True)
    assert np.abs(s32 - s64).max() < 2e-6 * max(1.0, np.abs(s64).max())


def _plan(oracle, w, h, seed, gs=40000):
    rgb = synth.synthetic_rgb(w, h, seed=seed)
    bmap = synth.activity_cover(rgb)
    hf = np.ones(bmap.shape, np.uint32)
    sh = np.full(bmap.shape, 7, np.uint8)
    rc, plan = oracle.encode(rgb, bmap, hf, global_scale=gs, gaborish=True, stages=True)
    assert rc == 0
    return rgb, bmap, hf, sh, plan


def test_fp64_encode_transform_is_within_f32_rounding(oracle):
    rgb, bmap, _, _, plan = _plan(oracle, 136, 104, seed=11)
    rc, xyb, pre, coeff = oracle.fp64_encode_transform(rgb, bmap, gaborish=True)
    assert rc == 0
    assert np.abs(plan["xyb"] - xyb).max() < 1e-6
    assert np.abs(plan["pre"] - pre).max() < 2e-6
    assert np.abs(plan["coeff"] - coeff).max() < 4e-6


def test_fp64_render_is_within_f32_rounding(oracle):
    w, h = 136, 104
    _, bmap, hf, sh, plan = _plan(oracle, w, h, seed=12)
    kw = dict(global_scale=40000, gaborish=True, epf_iters=3)
    for kind in (4, 0, 1):
        rc, a = oracle.reconstruct(w, h, bmap, hf, sh, plan, out_kind=kind, **kw)
        assert rc == 0
        rc, b = oracle.fp64_reconstruct(w, h, bmap, hf, sh, plan, out_kind=kind, **kw)
        assert rc == 0
        # the f32 path's arithmetic error, measured at about 2e-6 (linear)
        assert np.abs(a - b).max() < 1e-5, kind


def test_fp64_score_known_answer_and_f32_distance(oracle):
    w, h = 136, 104
    rgb, bmap, hf, sh, plan = _plan(oracle, w, h, seed=13)
    src = jg.srgb_to_linear_planes(rgb)
    assert oracle.fp64_ssim2(src, src)[0] == 100.0
    rc, lin = oracle.reconstruct(w, h, bmap, hf, sh, plan, global_scale=40000, gaborish=True,
                                 epf_iters=3, out_kind=1)
    s32 = oracle.ssim2(src, lin)[0]
    s64, terms = oracle.fp64_ssim2(src, lin)
    assert len(terms) == 18 * 5
    assert abs(s32 - s64) < 0.01
    # f64 inputs give the same score as their f32 copies when exactly equal
    s64b = oracle.fp64_ssim2(src.astype(np.float64), lin.astype(np.float64))[0]
    assert s64b == s64
