"""Failure paths, injected on the host: non-finite samples, sizes past the
limits, a device allocation that cannot succeed, covers that no stream can
carry.  Every one must come back as a status (or, for non-finite samples,
as the reference's own arithmetic does), with the context still usable.
Nothing here faults or hangs the GPU: inputs are rejected before any kernel
reads them, or are finite-sized and in bounds."""
import numpy as np
import pytest

import jpxl_gb300 as jg
from jpxl_gb300 import synth

pytestmark = pytest.mark.gpu


def _usable(ctx):
    w, h = 64, 64
    layout = jg.Layout(ctx, w, h, synth.fixed_dct8_map(w, h))
    plan = ctx.encode_transform(layout, synth.synthetic_rgb(w, h, seed=1), jg.EncodeRequest())
    layout.close()
    assert plan.qcoeff.any()


def test_non_finite_samples_score_as_the_restatement(ctx, oracle):
    """perceptual color.rs:56 returns non-finite inputs of the cube root
    unchanged, the recursive blur carries them along its line, and pool.rs:208
    clamps with f64::max, which returns the other operand of a NaN: the score
    stays finite.  The GPU must give the restatement's score."""
    a, b = oracle.perceptual_pair(96, 80, 5, 0.01, 3)
    b[1, 10, 10] = np.nan
    b[0, 40, 60] = np.inf
    b[2, 70, 5] = -np.inf
    got = jg.score_pair(ctx, a, b)
    want = oracle.ssim2(a, b)[0]
    print(f"non-finite candidate: gpu {got} restatement {want}")
    assert np.isnan(got) == np.isnan(want)
    if not np.isnan(want):
        assert abs(got - want) < 1e-3, (got, want)
    _usable(ctx)


def test_oversized_dimensions_are_argument_errors(ctx):
    with pytest.raises(jg.JpxlError) as e:
        jg.Layout(ctx, 65536 * 8, 8, np.zeros((1, 65536), np.uint8))
    assert e.value.code == -1
    # the metric's row pass holds a line of at most 8192 samples: the width
    # is refused before any sample is read
    torch = pytest.importorskip("torch")
    import ctypes as C
    small = torch.zeros(16, dtype=torch.float32, device="cuda")
    h = C.c_void_p()
    rc = ctx.lib.jpxlg_ssim2_ref_create(ctx.handle, C.c_void_p(small.data_ptr()), 8200, 16,
                                        jg.MEM_DEVICE, C.byref(h))
    assert rc == -1 and "columns" in ctx.lib.jpxlg_last_error(ctx.handle).decode()
    _usable(ctx)


def test_device_allocation_failure_is_a_status(ctx):
    """A reference of 8192 x 2^21 samples needs about 600 GB of pyramid and
    moment planes, more than the device holds: the allocation fails before
    any kernel runs, and the call returns JPXLG_ERR_CUDA."""
    torch = pytest.importorskip("torch")
    import ctypes as C
    small = torch.zeros(16, dtype=torch.float32, device="cuda")
    h = C.c_void_p()
    rc = ctx.lib.jpxlg_ssim2_ref_create(ctx.handle, C.c_void_p(small.data_ptr()), 8192, 1 << 21,
                                        jg.MEM_DEVICE, C.byref(h))
    assert rc == -4, rc
    assert not h.value
    _usable(ctx)


def test_varblock_across_an_lf_group_is_rejected(ctx):
    """jpxl-decode hf_meta.rs:222: no stream carries a varblock that crosses
    the 32-block LF-group boundary, so the layout refuses one."""
    w, h = 320, 64
    bmap = synth.fixed_dct8_map(w, h)
    bmap[0:2, 31:33] = 4
    bmap[0, 31] = 4 | 0x80
    with pytest.raises(jg.JpxlError) as e:
        jg.Layout(ctx, w, h, bmap)
    assert e.value.code == -2 and "LF-group" in str(e.value)
    bmap = synth.fixed_dct8_map(w, h)
    bmap[0:2, 30:32] = 4
    bmap[0, 30] = 4 | 0x80
    jg.Layout(ctx, w, h, bmap).close()
    _usable(ctx)
