"""Size-independent properties of the CUDA path at the bench's full size
(2048 x 2048 RGB16, DCT8/16/32 cover from select_blocks at global scale
40000), where a complete CPU
probe would take too long: determinism, the probe being exactly encode ->
render -> score, scores rising with the quantizer, a fine-quantizer round
trip, and one full-size plan checked bit for bit against the restatement."""
import numpy as np
import pytest

import jpxl_gb300 as jg
from jpxl_gb300 import synth

pytestmark = pytest.mark.gpu

W = H = 2048


@pytest.fixture(scope="module")
def frame(ctx):
    rgb = synth.synthetic_rgb(W, H, seed=1003, bits=16)
    cover = jg.select_blocks(ctx, rgb, _req(40000))
    assert len(np.unique(cover & 0x7F)) == 3  # DCT8, DCT16 and DCT32 all chosen
    layout = jg.Layout(ctx, W, H, cover, 1, 7)
    ref = jg.PrecomputedReference(ctx, jg.srgb_to_linear_planes(rgb, 16))
    yield rgb, cover, layout, ref
    ref.close()
    layout.close()


def _req(gs):
    return jg.EncodeRequest.with_global_scale(gs, gaborish=True, epf_iters=3)


def test_probe_is_deterministic_and_equals_its_stages(ctx, frame):
    rgb, _, layout, ref = frame
    a = ctx.probe(layout, ref, rgb, _req(40000))
    b = ctx.probe(layout, ref, rgb, _req(40000))
    assert a == b
    plan = ctx.encode_transform(layout, rgb, _req(40000))
    again = ctx.encode_transform(layout, rgb, _req(40000))
    assert np.array_equal(plan.qcoeff, again.qcoeff) and np.array_equal(plan.lf, again.lf)
    lin = jg.PlanRenderer(ctx).render(layout, plan, _req(40000), out="linear_at_depth", bits=16)
    assert jg.Ssimulacra2(ctx).score(ref, lin).score == a


def test_score_rises_with_the_quantizer(ctx, frame):
    rgb, _, layout, ref = frame
    s = [ctx.probe(layout, ref, rgb, _req(gs)) for gs in (8000, 20000, 40000, 90000, 200000)]
    assert all(x < y for x, y in zip(s, s[1:])), s
    assert 0.0 < s[0] and s[-1] < 100.0


def test_fine_quantizer_round_trip(ctx, frame):
    """A quantizer 100x finer than the bench's renders the source back closely
    (measured: mean |error| about 5e-4 linear, worst pixel 0.015 at a hard
    rectangle edge) and scores near 100."""
    rgb, _, layout, ref = frame
    req = _req(4000000)
    plan = ctx.encode_transform(layout, rgb, req)
    lin = jg.PlanRenderer(ctx).render(layout, plan, req, out="linear_at_depth", bits=16)
    err = np.abs(lin.astype(np.float64) - jg.srgb_to_linear_planes(rgb, 16))
    assert float(err.max()) < 0.03 and float(err.mean()) < 2e-3, (err.max(), err.mean())
    assert ctx.probe(layout, ref, rgb, req) > 95.0


def test_full_size_plan_matches_the_restatement(ctx, oracle, frame):
    rgb, cover, layout, _ = frame
    plan = ctx.encode_transform(layout, rgb, _req(40000))
    rc, want = oracle.encode(rgb, cover, np.ones(cover.shape, np.uint32), global_scale=40000,
                             gaborish=True)
    assert rc == 0
    assert tuple(plan.lf_factors) == tuple(want["lf_factors"])
    assert np.array_equal(plan.cfl_x, want["cfl_x"]) and np.array_equal(plan.cfl_b, want["cfl_b"])
    assert np.array_equal(plan.lf, want["lf"])
    diff = np.count_nonzero(plan.qcoeff != want["qcoeff"])
    assert diff == 0, diff
