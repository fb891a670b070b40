"""The allocation-free scoring entry point (jpxlg_ssim2_score_static) against
the allocating one (jpxlg_ssim2_score) on the same reference and candidates.

Both run the same kernels in the same order, so the results agree to the
last bit; the tolerance below only guards the comparison itself.  The file
name sorts last so the test also runs after every other GPU test has used
the library.
"""
import numpy as np
import pytest

import jpxl_gb300 as jg
from jpxl_gb300 import synth

pytestmark = pytest.mark.gpu

TOL = 1e-9  # SSIMULACRA2 points, and relative on the raw error and terms


def _planes(w, h, seed, noise):
    rgb = synth.synthetic_rgb(w, h, seed=seed)
    lin = jg.srgb_to_linear_planes(rgb)
    if noise:
        rng = np.random.default_rng(seed + 100)
        lin = np.clip(lin + rng.normal(0.0, noise, lin.shape), 0.0, 1.0)
    return np.ascontiguousarray(lin, dtype=np.float32)


def test_static_scratch_score_matches_allocating_score(ctx):
    torch = pytest.importorskip("torch")
    w, h = 333, 217  # ragged: partial tiles at every scale
    ref_planes = _planes(w, h, 11, 0.0)
    ref = jg.PrecomputedReference(ctx, ref_planes)
    metric = jg.Ssimulacra2(ctx)
    out = torch.empty(110, dtype=torch.float64, device="cuda")
    for call, noise in enumerate((0.02, 0.05)):  # two consecutive calls
        cand = _planes(w, h, 11, noise)
        want = metric.score(ref, cand)
        cand_dev = torch.from_numpy(cand).cuda()
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        metric.score_static_device(ref, cand_dev.data_ptr(), out.data_ptr())
        ctx.synchronize()
        got = out.cpu().numpy()
        nterms = 18 * 6  # 333 x 217 keeps all six scales (the last is 11 x 7)
        assert abs(got[0] - want.score) <= TOL, (call, got[0], want.score)
        assert abs(got[1] - want.raw_error) <= TOL * max(1.0, abs(want.raw_error))
        np.testing.assert_allclose(got[2:2 + nterms], want.terms[:nterms], rtol=TOL, atol=1e-15)
        assert 0.0 < got[0] < 100.0
    ref.close()


@pytest.mark.parametrize("w,h", [(2048, 2048), (2048, 9), (9, 2048)])
def test_static_scratch_at_its_capacity_edge(ctx, w, h):
    """Frames at the side limit fill the scratch regions to their sizes:
    the result must still equal the allocating entry point's."""
    torch = pytest.importorskip("torch")
    ref_planes = _planes(w, h, 21, 0.0)
    cand = _planes(w, h, 21, 0.03)
    ref = jg.PrecomputedReference(ctx, ref_planes)
    metric = jg.Ssimulacra2(ctx)
    want = metric.score(ref, cand)
    out = torch.full((110,), float("nan"), dtype=torch.float64, device="cuda")
    cand_dev = torch.from_numpy(cand).cuda()
    torch.cuda.synchronize()
    metric.score_static_device(ref, cand_dev.data_ptr(), out.data_ptr())
    ctx.synchronize()
    got = out.cpu().numpy()
    assert abs(got[0] - want.score) <= TOL, (got[0], want.score)
    ref.close()


def test_static_scratch_rejects_frames_beyond_its_limit(ctx):
    torch = pytest.importorskip("torch")
    w, h = 2056, 8
    ref = jg.PrecomputedReference(ctx, np.full((3, h, w), 0.25, np.float32))
    cand = torch.full((3, h, w), 0.25, dtype=torch.float32, device="cuda")
    out = torch.zeros(110, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    with pytest.raises(jg.JpxlError) as e:
        jg.Ssimulacra2(ctx).score_static_device(ref, cand.data_ptr(), out.data_ptr())
    assert e.value.code == -1 and "2048" in str(e.value)
    ref.close()
