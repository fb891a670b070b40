"""The oracle's restatement of the decoder's 8x8 special transforms
(oracle/oracle_special.cpp, jpxl-core varblock.rs:898-1230) against the
reference's own known answers (varblock.rs tests): the AFV basis is
orthonormal, a DC-only block reconstructs a constant for every kind, DCT8x4 is
the transpose of DCT4x8, the DCT8x4 halves land by row parity, and Hornuss's
centre and special cell are as hand-computed."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import loader as oracle

AFV = np.array(json.loads((Path(__file__).resolve().parent / "golden" /
                           "reference_constants.json").read_text())["AFV_BASIS"], np.float64)
KINDS = oracle.SPECIAL_KINDS


def test_afv_basis_is_orthonormal():
    assert AFV.shape == (16, 16)
    assert np.abs(AFV @ AFV.T - np.eye(16)).max() < 1e-12


@pytest.mark.parametrize("name", list(KINDS))
def test_dc_only_reconstructs_a_constant_block(name):
    c = np.zeros((8, 8), np.float32)
    c[0, 0] = 1.75
    out = oracle.special_block(KINDS[name], c, AFV)
    assert np.abs(out - 1.75).max() < 2e-3, name


def test_dct8x4_is_the_transpose_of_dct4x8():
    rng = np.random.default_rng(0x8A48)
    c = rng.uniform(-1, 1, (8, 8)).astype(np.float32)
    v = oracle.special_block(KINDS["dct8x4"], c)
    h = oracle.special_block(KINDS["dct4x8"], c)
    assert np.abs(v - h.T).max() < 1e-5


def test_dct8x4_halves_land_by_row_parity():
    c = np.zeros((8, 8), np.float32)
    c[2, 3] = 1.0  # column 3, row 2: an even row, half 0
    v = oracle.special_block(KINDS["dct8x4"], c)
    assert np.abs(v[:, 4:]).max() < 1e-6 and np.abs(v[:, :4]).max() > 1e-3
    h = oracle.special_block(KINDS["dct4x8"], c)
    assert np.abs(h[4:, :]).max() < 1e-6


def test_hornuss_residual_and_centre_are_hand_computable():
    c = np.zeros((8, 8), np.float32)
    c[0, 2] = 4.0  # (ix, iy) = (1, 0) of sub-block (0, 0)
    s = oracle.special_block(KINDS["hornuss"], c)
    centre = np.float32(-4.0) / np.float32(16.0)
    assert abs(s[1, 1] - centre) < 1e-6
    assert abs(s[0, 1] - (4.0 + centre)) < 1e-6
    assert abs(s[0, 0] - centre) < 1e-6  # reads coefficient (2, 2) == 0
    assert abs(s[3, 3] - centre) < 1e-6


def test_afv_flips_move_the_quadrants():
    """I.9.8: n's bits flip the AFV quadrant's samples and swap which side the
    DCT4x4 quadrant and the DCT4x8 half take; those two are not flipped."""
    rng = np.random.default_rng(77)
    c = rng.uniform(-1, 1, (8, 8)).astype(np.float32)
    a = [oracle.special_block(KINDS[f"afv{n}"], c, AFV) for n in range(4)]
    # AFV quadrant (rows y, columns x)
    assert np.array_equal(a[1][0:4, 4:8], a[0][0:4, 0:4][:, ::-1])
    assert np.array_equal(a[2][4:8, 0:4], a[0][0:4, 0:4][::-1, :])
    assert np.array_equal(a[3][4:8, 4:8], a[0][0:4, 0:4][::-1, ::-1])
    # DCT4x4 quadrant beside it, and the DCT4x8 half, moved but not flipped
    assert np.array_equal(a[1][0:4, 0:4], a[0][0:4, 4:8])
    assert np.array_equal(a[2][4:8, 4:8], a[0][0:4, 4:8])
    assert np.array_equal(a[1][4:8, :], a[0][4:8, :])
    assert np.array_equal(a[2][0:4, :], a[0][4:8, :])


def test_a_bad_kind_is_refused():
    with pytest.raises(ValueError):
        oracle.special_block(10, np.zeros((8, 8), np.float32))
    with pytest.raises(ValueError):
        oracle.special_block(KINDS["afv0"], np.zeros((8, 8), np.float32))
