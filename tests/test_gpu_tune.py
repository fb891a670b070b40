"""The batch autotuner on the GPU: it times every lanes x CTAs-per-SM shape
of a small split-precision batch, caches the fastest, leaves the tunable as
it found it, and the scores do not depend on the shape."""
import numpy as np
import pytest

import jpxl_gb300 as jg
from jpxl_gb300 import synth, tune

pytestmark = pytest.mark.gpu


def _items(ctx, torch):
    keep, items = [], []
    for i, (w, h) in enumerate([(256, 256), (320, 200), (192, 288)]):
        rgb = synth.synthetic_rgb(w, h, seed=8800 + i, bits=8)
        ref = jg.PrecomputedReference(ctx, jg.srgb_to_linear_planes(rgb, 8))
        dev = torch.from_numpy(rgb).cuda()
        for gs in (24000, 52000):
            req = jg.EncodeRequest.with_global_scale(gs, gaborish=True, epf_iters=3,
                                                     precision="bf16x6")
            layout = jg.Layout(ctx, w, h, jg.select_blocks(ctx, rgb, req), 1, 7)
            keep.append(layout)
            items.append(jg.BatchItem(layout, ref, dev.data_ptr(), 8, req))
        keep += [ref, dev]
    torch.cuda.synchronize()
    return items, keep


def test_tuner_picks_a_timed_shape_and_restores_the_knob(ctx, tmp_path):
    torch = pytest.importorskip("torch")
    items, keep = _items(ctx, torch)
    before = ctx.lib.jpxlg_tune_get(tune.TUNE_TC_CTAS_PER_SM)
    path = tmp_path / "tune.json"
    out = tune.tune_batch(ctx, items, precision="bf16x6", lanes=(1, 2), tc_ctas=(2, 4),
                          reps=1, warmup=1, path=path)
    assert ctx.lib.jpxlg_tune_get(tune.TUNE_TC_CTAS_PER_SM) == before
    shapes = {(t["lanes"], t["tc_ctas_per_sm"]) for t in out["trials"]}
    assert shapes == {(1, 2), (2, 2), (1, 4), (2, 4)}
    assert (out["lanes"], out["tc_ctas_per_sm"]) in shapes
    assert out["ms"] == min(t["ms"] for t in out["trials"])
    assert tune.tuned_shape(out["key"], path)["lanes"] == out["lanes"]


def test_scores_do_not_depend_on_the_shape(ctx):
    torch = pytest.importorskip("torch")
    items, keep = _items(ctx, torch)
    got = []
    before = ctx.lib.jpxlg_tune_get(tune.TUNE_TC_CTAS_PER_SM)
    try:
        for lanes, ctas in ((1, 1), (3, 4)):
            tune.set_tc_ctas_per_sm(ctx.lib, ctas)
            batch = jg.BatchProbe(ctx, items, lanes=lanes)
            try:
                got.append(batch.run())
            finally:
                batch.close()
    finally:
        tune.set_tc_ctas_per_sm(ctx.lib, before)
    assert np.array_equal(got[0], got[1])


def test_out_of_range_values_are_refused(ctx):
    assert ctx.lib.jpxlg_tune_set(tune.TUNE_TC_CTAS_PER_SM, 5) == -1
    assert ctx.lib.jpxlg_tune_set(7, 2) == -1
    with pytest.raises(ValueError):
        tune.set_tc_ctas_per_sm(ctx.lib, 0)
