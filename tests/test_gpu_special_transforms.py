"""The decoder's 8x8 special transforms on the GPU (the kernels
jpxlg_codestream_render runs for DCT2x2, Hornuss, DCT4x4, DCT8x4, DCT4x8 and
AFV0-3; no committed stream exercises most of them) against the oracle's
restatement of jpxl-core varblock.rs:898-1230, bit for bit on random
dequantized blocks, and the reference's DC-only known answer."""
import json
from pathlib import Path

import numpy as np
import pytest

import jpxl_gb300 as jg

pytestmark = pytest.mark.gpu

AFV = np.array(json.loads((Path(__file__).resolve().parent / "golden" /
                           "reference_constants.json").read_text())["AFV_BASIS"], np.float64)


@pytest.mark.parametrize("name", list(jg.SPECIAL_KINDS))
def test_special_transform_matches_the_oracle(ctx, oracle, name):
    kind = jg.SPECIAL_KINDS[name]
    rng = np.random.default_rng(4000 + kind)
    n = 512
    # coefficients over several magnitudes, as dequantization produces them
    coef = (rng.standard_normal((n, 8, 8)) *
            (10.0 ** rng.integers(-3, 2, (n, 1, 1)))).astype(np.float32)
    got = jg.special_blocks(ctx, kind, coef)
    want = np.stack([oracle.special_block(kind, c, AFV) for c in coef])
    mism = int((got != want).sum())
    assert mism == 0, (name, mism, float(np.abs(got - want).max()))


@pytest.mark.parametrize("name", list(jg.SPECIAL_KINDS))
def test_dc_only_block_is_constant_on_the_gpu(ctx, name):
    c = np.zeros((1, 8, 8), np.float32)
    c[0, 0, 0] = 1.75
    out = jg.special_blocks(ctx, jg.SPECIAL_KINDS[name], c)
    assert np.abs(out - 1.75).max() < 2e-3


def test_a_bad_kind_is_an_argument_error(ctx):
    with pytest.raises(jg.JpxlError) as e:
        jg.special_blocks(ctx, 12, np.zeros((1, 8, 8), np.float32))
    assert e.value.code == -1
