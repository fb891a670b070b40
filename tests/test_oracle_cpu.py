"""The CPU restatement pinned against the reference: its constant tables (read
from the reference source into tests/golden/reference_constants.json) and
the known answers printed in the reference's own tests."""
import ctypes as C
import json
import math
import struct
from pathlib import Path

import numpy as np
import pytest

GOLDEN = json.loads((Path(__file__).parent / "golden" / "reference_constants.json").read_text())


def f32(x):
    return float(np.float32(x))


def test_dct_iv_leaves_match_the_reference_tables(oracle):
    lib = oracle.load()
    lib.orc_dct_iv_entry.restype = C.c_float
    lib.orc_dct_iv_entry.argtypes = [C.c_int, C.c_int, C.c_int]
    for name, m in (("DCT4_4", 4), ("DCT4_8", 8), ("DCT4_16", 16)):
        ref = GOLDEN[name]
        got = [lib.orc_dct_iv_entry(m, u, n) for u in range(m) for n in range(m)]
        assert got == [f32(v) for v in ref], name


def test_ssim_weights_and_blur_constants_match(oracle):
    lib = oracle.load()
    lib.orc_ssim2_weight.restype = C.c_double
    lib.orc_ssim2_weight.argtypes = [C.c_int]
    assert [lib.orc_ssim2_weight(i) for i in range(108)] == GOLDEN["SSIM_WEIGHTS"]


def test_blur_is_the_nine_tap_fir(oracle):
    """blur.rs: the f64 resonators reduce to taps at |k| <= 4 (impulse)."""
    lib = oracle.load()
    lib.orc_blur_plane.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    w = h = 33
    a = np.zeros((h, w), np.float32)
    a[16, 16] = 1.0
    out = np.zeros_like(a)
    lib.orc_blur_plane(a.ctypes.data, w, h, out.ctypes.data)
    mul_in, omega = GOLDEN["MUL_IN"], [math.pi / 10, 3 * math.pi / 10, math.pi / 2]
    taps = [sum(mi * math.sin((5 - k) * om) / math.sin(om) for mi, om in zip(mul_in, omega))
            for k in range(5)]
    row = out[16]
    for k in range(-6, 7):
        want = taps[abs(k)] * taps[0] if abs(k) <= 4 else 0.0
        assert abs(row[16 + k] - want) < 2e-8, (k, row[16 + k], want)
    assert abs(taps[0] + 2 * sum(taps[1:]) - 1.0) < 1e-6


def _weights(params, rows, cols):
    bands = [params[0]]
    for v in params[1:]:
        bands.append(bands[-1] * (1.0 + v if v > 0 else 1.0 / (1.0 - v)))
    out = np.zeros((rows, cols), np.float32)
    rng_ = math.sqrt(2.0) + 1e-6
    last = len(bands) - 1
    for y in range(rows):
        for x in range(cols):
            dx, dy = x / (cols - 1), y / (rows - 1)
            pos = math.sqrt(dx * dx + dy * dy) * last / rng_
            i = math.floor(pos)
            a, b = bands[i], bands[i + 1]
            out[y, x] = np.float32(1.0 / (a * (b / a) ** (pos - i)))
    return out


@pytest.mark.parametrize("sel,name,rows,cols", [
    (0, "DCT8X8_PARAMS", 8, 8), (4, "DCT16X16_PARAMS", 16, 16), (5, "DCT32X32_PARAMS", 32, 32),
    (6, "DCT16X8_PARAMS", 8, 16), (8, "DCT32X8_PARAMS", 8, 32), (10, "DCT16X32_PARAMS", 16, 32)])
def test_dequant_matrices_follow_table_i6(oracle, sel, name, rows, cols):
    lib = oracle.load()
    for c in range(3):
        out = np.zeros(rows * cols, np.float32)
        r, k = C.c_int(), C.c_int()
        assert lib.orc_dequant_matrix(sel, c, out.ctypes.data, C.byref(r), C.byref(k)) == 0
        assert (r.value, k.value) == (rows, cols)
        want = _weights(GOLDEN[name][c], rows, cols).ravel()
        np.testing.assert_allclose(out, want, rtol=2e-7)
        assert out[0] == np.float32(1.0 / GOLDEN[name][c][0])  # dequant.rs:1600


def test_reference_known_answers(oracle):
    lib = oracle.load()
    kat = GOLDEN["KAT"]
    p = lambda a: a.ctypes.data
    lib.orc_dct_ii_ortho.argtypes = [C.c_void_p, C.c_int]
    v = np.ones(8, np.float32)
    lib.orc_dct_ii_ortho(p(v), 8)
    assert abs(v[0] - kat["dct_ii_8_constant_dc"]) < 1e-5 and np.abs(v[1:]).max() < 1e-6
    v = np.zeros(8, np.float32)
    v[0] = 1
    lib.orc_dct_ii_ortho(p(v), 8)
    assert abs(v[0] - kat["dct_ii_8_impulse"][0]) < 1e-6
    assert abs(v[1] - kat["dct_ii_8_impulse"][1]) < 1e-6
    imp = np.zeros(9, np.float32)
    imp[4] = 1
    out = np.zeros(9, np.float32)
    lib.orc_gaborish_w(p(imp), 3, 3, 0.25, 0.125, p(out))
    np.testing.assert_allclose(out.reshape(3, 3), kat["gaborish_impulse_w1_0.25_w2_0.125"],
                               atol=1e-6)
    z = np.zeros(3, np.float32)
    y = np.array([0, 1, 0], np.float32)
    s = np.array([100], np.float32)
    o = [np.zeros(3, np.float32) for _ in range(3)]
    lib.orc_epf_step.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    lib.orc_epf_step(2, (C.c_void_p * 3)(p(z), p(y), p(z)), 3, 1, p(s),
                     (C.c_void_p * 3)(*[p(a) for a in o]))
    assert abs(o[1][1] - kat["epf_step2_three_pixel_row"]) < 1e-6
    assert o[0].tolist() == [0, 0, 0] and o[2].tolist() == [0, 0, 0]
    assert lib.orc_hf_multiplier(32768, 2) == kat["hf_multiplier_32768_2"]
    assert abs(lib.orc_bias_adjust(10, 0.9, 0.145) - kat["bias_adjust_10_0.9_0.145"]) < 1e-6
    # color.rs tests: black -> 0, grey -> X == 0
    lib.orc_linear_to_xyb.argtypes = [C.c_void_p, C.c_void_p]
    xyb = np.zeros(3, np.float32)
    lib.orc_linear_to_xyb(p(np.zeros(3, np.float32)), p(xyb))
    assert np.abs(xyb).max() < 1e-6
    lib.orc_linear_to_xyb(p(np.full(3, 0.5, np.float32)), p(xyb))
    assert abs(xyb[0]) < 1e-6


def test_identical_images_score_exactly_one_hundred(oracle):
    a, _ = oracle.perceptual_pair(256, 192, 1, 0.0, 1)
    score, raw, terms = oracle.ssim2(a, a)
    assert score == 100.0 and raw == 0.0 and terms.size == 6 * 18


def test_recorded_score_of_the_4mp_timing_pair(oracle):
    """evidence.akr:6424 records score bits 0x405358a2f06c4538 (77.38494501660614)
    for synthetic(2400,1800,9) vs add_noise(0.01,3) (perceptual tests/common).
    The restatement lands within 1e-12 (6 f64 ulps; the generator's powf is the
    host libm's)."""
    a, b = oracle.perceptual_pair(2400, 1800, 9, 0.01, 3)
    score, _, _ = oracle.ssim2(a, b)
    want = struct.unpack("<d", bytes.fromhex(GOLDEN["SCORE_BITS_4MP_PAIR"])[::-1])[0]
    assert abs(want - 77.38494501660614) < 1e-15
    assert abs(score - want) < 1e-12, (score, want)


def test_reproducible_cbrt_is_the_correctly_rounded_root(oracle):
    """Both reference cube roots (simd.rs:36, perceptual color.rs:46) return
    the correctly rounded f32 cube root on a dense sample of the XYB input
    range: the GPU fast path relies on that (with its f64 fallback near ties)."""
    lib = oracle.load()
    rng = np.random.default_rng(5)
    xs = np.concatenate([rng.uniform(0.0037, 1.2, 200000), 10.0 ** rng.uniform(-6, 6, 50000)])
    xs = xs.astype(np.float32)
    for fn in (lib.orc_cbrt_core, lib.orc_cbrt_perceptual):
        bad = 0
        for x in xs[:20000]:
            got = np.float32(fn(float(x)))
            exact = np.cbrt(np.float64(x))
            lo = np.nextafter(got, np.float32(-np.inf))
            hi = np.nextafter(got, np.float32(np.inf))
            # correctly rounded: exact lies within half an ulp of got
            if not (abs(exact - np.float64(got)) <= abs(exact - np.float64(lo)) and
                    abs(exact - np.float64(got)) <= abs(exact - np.float64(hi))):
                bad += 1
        assert bad == 0


def test_oracle_encode_then_render_round_trips(oracle):
    from jpxl_gb300 import synth

    w, h = 64, 48
    rgb = synth.synthetic_rgb(w, h, seed=3)
    bm = synth.fixed_dct8_map(w, h)
    hf = np.ones(bm.shape, np.uint32)
    rc, plan = oracle.encode(rgb, bm, hf, global_scale=20000, gaborish=True)
    assert rc == 0
    rc, px = oracle.reconstruct(w, h, bm, hf, np.full(bm.shape, 7, np.uint8), plan,
                                global_scale=20000, gaborish=True, epf_iters=3)
    assert rc == 0
    mse = ((px.astype(float) - rgb.astype(float)) ** 2).mean()
    assert 10 * math.log10(255 ** 2 / mse) > 25  # global_scale 20000 is a coarse quantizer


def test_oracle_rejects_bad_block_maps(oracle):
    from jpxl_gb300 import synth

    w, h = 32, 32
    rgb = synth.synthetic_rgb(w, h, seed=1)
    bm = synth.fixed_dct8_map(w, h)
    hf = np.ones(bm.shape, np.uint32)
    bad = bm.copy()
    bad[0, 0] = 4 | 0x80  # DCT16 overlapping DCT8 origins
    assert oracle.encode(rgb, bad, hf, global_scale=20000)[0] == -4
    bad = bm.copy()
    bad[1, 1] = 0  # uncovered block
    assert oracle.encode(rgb, bad, hf, global_scale=20000)[0] == -4


def test_cover_restatement_properties(oracle):
    """select_blocks (policy lib.rs:5260) restated: a flat frame stays DCT8 (a
    merge pays 34 fixed bits that zero residuals never earn back), covers tile
    the grid, and coarse quantizers merge more than fine ones."""
    from jpxl_gb300 import synth

    flat = np.full((96, 128, 3), 77, np.uint8)
    rc, m, n = oracle.select_blocks(flat, global_scale=20000, gaborish=True)
    assert rc == 0 and np.all(m == 0x80) and n > 0
    rgb = synth.synthetic_rgb(320, 256, seed=5, bits=16)
    merged = []
    for gs in (4000, 60000):
        rc, m, _ = oracle.select_blocks(rgb, global_scale=gs, gaborish=True)
        assert rc == 0
        covered = np.zeros(m.shape, np.int32)
        side = {0: 1, 4: 2, 5: 4}
        for by, bx in np.argwhere(m & 0x80):
            s = side[int(m[by, bx] & 0x1F)]
            assert np.all((m[by:by + s, bx:bx + s] & 0x1F) == (m[by, bx] & 0x1F))
            covered[by:by + s, bx:bx + s] += 1
        assert np.all(covered == 1)
        merged.append(int(np.count_nonzero((m & 0x1F) != 0)))
    assert merged[0] > merged[1]
