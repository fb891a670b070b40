"""The GPU cover selection (jpxlg_select_blocks) against the CPU restatement
of select_blocks: block maps must be identical — same shapes at the same
origins — for every size, depth, quantizer and restoration setting here."""
import numpy as np
import pytest

import jpxl_gb300 as jg
from jpxl_gb300 import synth

pytestmark = pytest.mark.gpu


def _cover_mix(m):
    sel, org = m & 0x1F, (m & 0x80) != 0
    return {s: int(((sel == s) & org).sum()) for s in (jg.DCT8, jg.DCT16, jg.DCT32)}


@pytest.mark.parametrize("w,h,bits,gs,gab", [
    (256, 192, 8, 40000, True),
    (257, 263, 16, 20000, True),
    (512, 512, 16, 5000, True),
    (512, 512, 16, 10000, False),
    (333, 217, 8, 80000, True),
    (64, 40, 8, 3000, True),
])
def test_cover_matches_the_restatement(ctx, oracle, w, h, bits, gs, gab):
    rgb = synth.synthetic_rgb(w, h, seed=w * 7 + h, bits=bits)
    req = jg.EncodeRequest(global_scale=gs, gaborish=gab)
    got = jg.select_blocks(ctx, rgb, req)
    rc, want, _ = oracle.select_blocks(rgb, global_scale=gs, gaborish=gab)
    assert rc == 0
    diff = np.argwhere(got != want)
    assert diff.size == 0, (len(diff), diff[:5], _cover_mix(got), _cover_mix(want))
    jg.Layout(ctx, w, h, got).close()  # a valid cover


def test_cover_with_qm_scales(ctx, oracle):
    rgb = synth.synthetic_rgb(320, 240, seed=17, bits=16)
    req = jg.EncodeRequest(global_scale=15000, x_qm_scale=4, b_qm_scale=1, gaborish=True)
    got = jg.select_blocks(ctx, rgb, req)
    rc, want, _ = oracle.select_blocks(rgb, global_scale=15000, x_qm_scale=4, b_qm_scale=1,
                                       gaborish=True)
    assert rc == 0 and np.array_equal(got, want)


def test_full_size_cover_and_probe(ctx, oracle):
    """The bench's frame size: the selected cover equals the restatement's,
    mixes shapes, and drives a probe."""
    rgb = synth.synthetic_rgb(2048, 2048, seed=1000, bits=16)
    req = jg.EncodeRequest.with_global_scale(40000, gaborish=True, epf_iters=3)
    got = jg.select_blocks(ctx, rgb, req)
    rc, want, _ = oracle.select_blocks(rgb, global_scale=40000, gaborish=True)
    assert rc == 0 and np.array_equal(got, want)
    mix = _cover_mix(got)
    assert mix[jg.DCT8] > 0 and mix[jg.DCT16] > 0
    layout = jg.Layout(ctx, 2048, 2048, got, 1, 7)
    ref = jg.PrecomputedReference(ctx, jg.srgb_to_linear_planes(rgb, 16))
    assert 0.0 < ctx.probe(layout, ref, rgb, req) < 100.0
    ref.close()
    layout.close()
