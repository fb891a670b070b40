"""Batched probes (jpxlg_batch_*): one CUDA graph over many (frame, quantizer)
items must give exactly the scores of the same probes made one at a time —
the same kernels in the same order per item, on other streams."""
import numpy as np
import pytest

import jpxl_gb300 as jg
from jpxl_gb300 import synth

pytestmark = pytest.mark.gpu


def _frame(ctx, torch, w, h, seed, bits):
    rgb = synth.synthetic_rgb(w, h, seed=seed, bits=bits)
    cover = synth.activity_cover(rgb)
    layout = jg.Layout(ctx, w, h, cover, 1, 7)
    ref = jg.PrecomputedReference(ctx, jg.srgb_to_linear_planes(rgb, bits))
    view = rgb.view(np.int16) if bits == 16 else rgb
    dev = torch.from_numpy(np.ascontiguousarray(view)).cuda()
    return rgb, layout, ref, dev


def _req(gs):
    return jg.EncodeRequest.with_global_scale(gs, gaborish=True, epf_iters=3)


def test_batch_matches_single_probes_and_replays(ctx):
    torch = pytest.importorskip("torch")
    frames = [_frame(ctx, torch, 320, 240, 31, 16), _frame(ctx, torch, 257, 263, 32, 8)]
    plan = [(0, 20000), (0, 40000), (0, 60000), (1, 30000), (1, 50000)]
    torch.cuda.synchronize()
    items = [jg.BatchItem(frames[f][1], frames[f][2], frames[f][3].data_ptr(),
                          16 if f == 0 else 8, _req(gs)) for f, gs in plan]
    want = np.array([ctx.probe(frames[f][1], frames[f][2], frames[f][0], _req(gs))
                     for f, gs in plan])
    batch = jg.BatchProbe(ctx, items, lanes=2)
    first = batch.run()
    second = batch.run()  # graph replay
    np.testing.assert_array_equal(first, want)
    np.testing.assert_array_equal(second, want)
    assert np.all((want > 0) & (want < 100))
    # Scores follow the quantizer: a finer step scores higher on the same frame.
    assert want[0] < want[1] < want[2] and want[3] < want[4]
    # The graph reads the RGB buffers at run time: new contents, new scores.
    other = synth.synthetic_rgb(320, 240, seed=77, bits=16)
    frames[0][3].copy_(torch.from_numpy(other.view(np.int16)))
    torch.cuda.synchronize()
    changed = batch.run()
    for i, (f, gs) in enumerate(plan):
        if f == 0:
            assert changed[i] == ctx.probe(frames[0][1], frames[0][2], other, _req(gs))
        else:
            assert changed[i] == want[i]
    batch.close()
    for _, layout, ref, _ in frames:
        ref.close()
        layout.close()


def test_batch_probe_one_shot_and_errors(ctx):
    torch = pytest.importorskip("torch")
    rgb, layout, ref, dev = _frame(ctx, torch, 192, 128, 5, 16)
    torch.cuda.synchronize()
    items = (jg._lib.BatchItemStruct * 2)()
    for k, gs in enumerate((25000, 45000)):
        items[k].layout = layout.handle
        items[k].ref = ref.handle
        items[k].rgb = dev.data_ptr()
        items[k].bits = 16
        items[k].params = _req(gs)._struct()
    out = np.zeros(2, np.float64)
    ctx.check(ctx.lib.jpxlg_batch_probe(ctx.handle, 2, items, out.ctypes.data))
    for k, gs in enumerate((25000, 45000)):
        assert out[k] == ctx.probe(layout, ref, rgb, _req(gs))
    bad = jg.BatchItem(layout, ref, dev.data_ptr(), 16, jg.EncodeRequest(global_scale=0))
    with pytest.raises(jg.JpxlError) as e:
        jg.BatchProbe(ctx, [bad])
    assert e.value.code == -1
    ref.close()
    layout.close()
