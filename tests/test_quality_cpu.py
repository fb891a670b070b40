"""The quality controller's navigation (jpxl_gb300.quality) on the CPU: the
ladder and local-model known answers of the reference's own unit tests
(quantizer_ladder.rs, navigation.rs, quality.rs tests), and the search over
the reference tests' curve evaluator (quality.rs:2752 CurveEvaluator: loss =
60 * (effective_scale / 1000)^-0.8)."""
import math

import pytest

from jpxl_gb300 import quality as q


def curve(r, fresh=True):
    return 100.0 - 60.0 * (q.effective_scale(r) / 1000.0) ** -0.8


START = q.rung_for_scale(8000.0)


# ---- quantizer_ladder.rs tests ----------------------------------------------


def test_every_rung_is_representable_and_the_ladder_is_ordered():
    previous = 0
    for index in [0, 1, q.MAX_GLOBAL_SCALE - 2, q.MAX_GLOBAL_SCALE - 1, q.MAX_GLOBAL_SCALE,
                  q.MAX_GLOBAL_SCALE + 1, q.LADDER_LEN - 1]:
        quant = q.quantizer_at(q.rung(index), 16)
        assert 1 <= quant.global_scale <= q.MAX_GLOBAL_SCALE and quant.hf_mul >= 1
        product = quant.global_scale * quant.hf_mul
        assert product > previous, index
        previous = product


def test_lf_coupling_follows_the_segment_up_to_the_bound():
    assert [q.coupled_quant_lf(4, k) for k in (1, 2, 4, 5, 65)] == [4, 8, 16, 16, 16]
    assert q.coupled_quant_lf(16, 3) == 16
    assert q.coupled_quant_lf(3, 6) == 15
    assert q.coupled_quant_lf(64, 4) == 64


def test_the_upper_ladder_is_dense_invertible_and_lf_coupled():
    previous = q.effective_scale(q.rung(q.MAX_GLOBAL_SCALE - 1))
    assert previous == q.MAX_GLOBAL_SCALE
    for index in range(q.MAX_GLOBAL_SCALE, q.LADDER_LEN):
        scale = q.effective_scale(index)
        assert scale > previous, index
        gs, mul = q.rung_fields(index)
        assert 1 <= gs <= q.MAX_GLOBAL_SCALE
        if gs == q.segment_first_scale(mul):
            assert scale - previous <= mul, index
        else:
            assert scale - previous == mul, index
        assert q.rung_for_effective_scale(scale) == index
        if scale - previous > 1:
            assert q.rung_for_effective_scale(scale - 1) == index - 1
        previous = scale
    assert q.effective_scale(q.TOP) == q.MAX_GLOBAL_SCALE * q.MAX_LADDER_MUL
    assert q.rung_fields(q.TOP) == (q.MAX_GLOBAL_SCALE, q.MAX_LADDER_MUL)
    for index in [0, 4096, q.MAX_GLOBAL_SCALE - 1]:
        quant = q.quantizer_at(index, 16)
        assert (quant.global_scale, quant.hf_mul, quant.quant_lf) == (index + 1, 1, 16)
    ceiling = q.quantizer_at(q.MAX_GLOBAL_SCALE - 1, 4)
    above = q.quantizer_at(q.MAX_GLOBAL_SCALE, 4)
    assert above.global_scale * above.quant_lf >= ceiling.global_scale * ceiling.quant_lf
    assert above.quant_lf == 8
    assert q.quantizer_at(q.MAX_GLOBAL_SCALE, 16).quant_lf == 16


def test_a_rung_out_of_range_saturates():
    assert q.rung(2**32 - 1) == q.TOP
    assert q.rung_for_global_scale(0) == q.FLOOR
    assert q.rung_for_global_scale(1) == q.FLOOR
    assert q.rung_for_global_scale(32768) == 32767


# ---- navigation.rs tests --------------------------------------------------------


def test_a_crossing_at_an_observed_point_returns_that_point():
    lo = (q.ln_scale(1000), 10.0)
    hi = (q.ln_scale(4000), 12.0)
    assert q.local_slope(lo, hi) > 0.0
    assert abs(q.local_crossing(lo, hi, lo[1]) - lo[0]) < 1e-12
    assert abs(q.local_crossing(lo, hi, hi[1]) - hi[0]) < 1e-9


def test_negating_the_y_axis_does_not_move_the_crossing():
    for lo_y, hi_y, target in [(2.0, 5.5, 4.25), (-1.5, 3.25, 0.0), (0.125, 0.126, 0.1255),
                               (11.7, 19.3, 30.0)]:
        lo_x, hi_x = q.ln_scale(700), q.ln_scale(9000)
        rising = q.local_crossing((lo_x, lo_y), (hi_x, hi_y), target)
        falling = q.local_crossing((lo_x, -lo_y), (hi_x, -hi_y), -target)
        assert rising == falling


def test_the_progress_rules_differ_only_on_an_aim_that_did_not_advance():
    frm, forward, backwards = 1000, 1400, 900
    for rule in (True, False):
        assert q.force_progress(forward, frm, True, rule) == forward
    assert q.force_progress(frm, frm, True, True) == 1001
    assert q.force_progress(frm, frm, True, False) == 1001
    assert q.force_progress(backwards, frm, True, True) == 1001
    assert q.force_progress(backwards, frm, True, False) == backwards


def test_a_scale_that_is_not_a_number_lands_on_the_floor():
    for v in (math.nan, math.inf, -1.0, 0.0, 1.0):
        assert q.rung_for_scale(v) == q.FLOOR
    assert q.rung_for_scale(2.4) == 1
    # f64::round takes halves away from zero (Python's round() would not)
    assert q.rung_for_scale(2.5) == 2 and q.rung_for_scale(4.5) == 4


# ---- quality.rs tests ---------------------------------------------------------------


def test_the_crossing_stays_strictly_inside_the_bracket():
    lo, hi = (999, 60.0), (7999, 91.0)
    r = q.log_loss_crossing(lo, hi, 85.0)
    assert r is not None and lo[0] < r < hi[0]
    assert q.log_loss_crossing((999, 70.0), (7999, 65.0), 68.0) is None
    assert q.log_loss_crossing((10, 50.0), (11, 60.0), 55.0) is None


def test_geometric_steps_move_and_stop_at_the_ladder_ends():
    r = 999
    assert q.geometric_step(r, True) > r > q.geometric_step(r, False)
    assert q.geometric_step(q.FLOOR, False) == q.FLOOR
    assert q.geometric_step(q.TOP, True) == q.TOP


def test_met_band_couples_to_the_reserve():
    # at 85 and above under Balanced the reserve margin is below one point
    assert q.met_band(85.0, 0.03) == 1.0
    # below that the band is twice the reserve's score margin
    assert q.met_band(30.0, 0.03) == pytest.approx(2 * 0.03 * 70.0)
    assert q.aim_score_for(85.0, 0.03) == pytest.approx(85.45)
    assert q.aim_score_for(99.0, 0.03) == 99.25


@pytest.mark.parametrize("preset", ["fast", "balanced"])
@pytest.mark.parametrize("target", [50.0, 70.0, 85.0])
def test_every_effort_meets_its_target_inside_its_budget(preset, target):
    calls = []
    out = q.solve(lambda r, f: calls.append(r) or curve(r), START, target, preset)
    budget = q.PRESETS[preset]
    assert out.score >= target
    nav_probes = len(out.probes)
    # finalist rebuilds run inside the pixel cap; only the rescue goes past it
    assert nav_probes <= budget.pixel_probes
    assert len(calls) == nav_probes
    assert out.status in ("met", "met_adjacent_rungs", "met_work_cap",
                          "rescued_fresh_structure")
    # the choice is the coarsest feasible probe
    feas = [r for r, s, _ in out.probes if s >= target]
    assert out.rung == min(feas)


def test_running_out_of_probes_reports_under_target_work_cap():
    budget = q.Budget(pixel_probes=1, exact_prices=1, structural_builds=1, reserve=0.03)
    out = q.solve(curve, START, 99.9, budget)
    assert out.status == "under_target_work_cap"
    assert out.score < 99.9
    assert len(out.probes) == 2  # the cap of one, plus the rescue probe


def test_an_unreachable_target_saturates_explicitly():
    out = q.solve(curve, START, 99.99, "fast")
    assert out.status == "saturated_top"
    assert out.rung == q.TOP and out.score < 99.99


def test_a_higher_target_never_lands_coarser_or_lower():
    low = q.solve(curve, START, 60.0, "balanced")
    high = q.solve(curve, START, 90.0, "balanced")
    assert high.score >= low.score and high.rung >= low.rung


def test_a_first_probe_in_band_ends_the_search():
    # a start whose score lands within one point above the target
    target = 85.0
    start = next(r for r in range(5000, 8000) if 85.0 <= curve(r) <= 85.5)
    out = q.solve(curve, start, target, "balanced")
    assert [p[0] for p in out.probes] == [start]
    assert out.status == "met"


def test_lockstep_search_equals_one_frame_at_a_time():
    curves = [lambda r, a=a: 100.0 - a * (q.effective_scale(r) / 1000.0) ** -0.8
              for a in (30.0, 60.0, 120.0, 240.0)]
    starts = [START, 3000, 20000, 60000]
    rounds = []

    def batch(reqs):
        rounds.append(len(reqs))
        return [curves[i](r) for i, r, _ in reqs]

    together = q.search(batch, starts, 80.0, "balanced")
    alone = [q.solve(lambda r, f, c=c: c(r), s, 80.0, "balanced") for c, s in zip(curves, starts)]
    for a, b in zip(together, alone):
        assert (a.rung, a.status, a.probes) == (b.rung, b.status, b.probes)
    assert sum(rounds) == sum(len(o.probes) for o in together)
    assert max(rounds) == len(curves)
