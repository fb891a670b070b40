"""The perceptual quality controller's navigation over the batched probe path.

A restatement, on the host, of how jpxl-encode-policy searches the quantizer
ladder for the coarsest quantizer whose SSIMULACRA2 score meets a target
(quality.rs:2405 search_frame_perceptual, its baseline solve quality.rs:1775
solve_baseline and the Navigator of quality.rs:1104-1620), with the ladder of
quantizer_ladder.rs and the local model of navigation.rs.  The policy decides
WHICH probes run; every probe is a full encode -> render -> SSIMULACRA2 pass
of the CUDA path (jpxlg_batch_* / jpxlg_probe).  Several frames navigate in
lockstep: each round gathers the next probe of every unfinished frame and
runs them as one batch (one graph launch), which is what the batched scorer
is for.

The navigator is written as a generator: it yields the probe it wants, a
(rung, fresh) pair, and receives the score.  `search` drives many of them
over one probe function; `solve` runs one.

Restated with the crate's default features (Cargo.toml: corrected-stop, which
implies trusted-first-probe; reserve-coupled-band; no surrogate-navigation):
  1. probe the start rung with a fresh structure (cover and CfL planned for
     that quantizer; it becomes the structure anchor);
  2. stop if it is feasible inside the accept band (trusted-first-probe,
     quality.rs:1828 in_band);
  3. otherwise one direct correction under the prior exponent and one
     slope-corrected retry (quality.rs:1566 corrected_stop);
  4. otherwise expand until a bracket exists (quality.rs:1381), tighten on
     the log-loss crossing (quality.rs:1603), one rescue probe past the
     budget when nothing met the target (quality.rs:1404);
  5. finalists: the coarsest feasible probes (at most min(exact_prices, 2));
     a reused-structure finalist far from the anchor is re-probed with a
     fresh structure (quality.rs:1932);
  6. status as quality.rs:2698.

What is outside the path and how it is stood in for:
  * the start rung and slope prior come from the reference's crossing model
    and source features (quality.rs:1030 predicted_effective_scale,
    quality_prediction.rs): here the caller passes them;
  * exact pricing (entropy coding the finalists) picks the smallest stream:
    here the coarsest feasible finalist is picked, which is the smallest
    stream whenever bytes fall with the rung;
  * policy-bank trials and the reducer (policy_trials = 0 and no reducer in
    the Fast and Balanced presets) are not run;
  * a reused-structure probe in the reference keeps the anchor's cover AND
    CfL factors; the probe function decides what it reuses (the CUDA probe
    reuses the cover and estimates CfL for each probe).
"""
from __future__ import annotations

import bisect
import math
from dataclasses import dataclass, field

# ---- the ladder (quantizer_ladder.rs) --------------------------------------

MAX_GLOBAL_SCALE = 8193 + 65535  # jpxl-encode vardct/ids.rs:20
MAX_QUANT_LF = 65536             # ids.rs MAX_QUANT_LF
HF_MUL_RUNGS = 64                # quantizer_ladder.rs:57
MAX_LADDER_MUL = HF_MUL_RUNGS + 1
LF_COUPLING_MAX_QUANT_LF = 16    # quantizer_ladder.rs:104


def segment_first_scale(k: int) -> int:
    """quantizer_ladder.rs:65: the smallest global_scale of segment k whose
    product with k exceeds (k - 1) * MAX."""
    floor = ((k - 1) * MAX_GLOBAL_SCALE) // k
    return MAX_GLOBAL_SCALE if floor >= MAX_GLOBAL_SCALE else floor + 1


def segment_len(k: int) -> int:
    return MAX_GLOBAL_SCALE - segment_first_scale(k) + 1


# First rung index of segment k (k = 2 .. MAX_LADDER_MUL), and one past the
# ladder's end.
_SEG_START = {}
_i = MAX_GLOBAL_SCALE
for _k in range(2, MAX_LADDER_MUL + 1):
    _SEG_START[_k] = _i
    _i += segment_len(_k)
LADDER_LEN = _i
FLOOR = 0
TOP = LADDER_LEN - 1
_SEG_KEYS = [_SEG_START[k] for k in range(2, MAX_LADDER_MUL + 1)]


def rung(index: int) -> int:
    """Rung::new: an index clamped into the ladder."""
    return TOP if index >= LADDER_LEN else max(int(index), 0)


def rung_for_global_scale(scale: int) -> int:
    return FLOOR if scale == 0 else rung(scale - 1)


def rung_fields(r: int) -> tuple[int, int]:
    """quantizer_ladder.rs:134: (global_scale, HfMul) of a rung."""
    if r < MAX_GLOBAL_SCALE:
        return r + 1, 1
    # the segment holding r (the walk of quantizer_ladder.rs:138, by bisection
    # over the segments' first indices); past the last segment's end the
    # offset runs on inside the last segment, as the walk leaves it
    k = min(bisect.bisect_right(_SEG_KEYS, r) + 1, MAX_LADDER_MUL)
    offset = r - _SEG_START[k]
    return min(segment_first_scale(k) + offset, MAX_GLOBAL_SCALE), k


def coupled_quant_lf(base: int, k: int) -> int:
    """quantizer_ladder.rs:117: the largest base * j, j <= k, within the
    coupling bound (or base itself)."""
    best = base
    for j in range(2, k + 1):
        cand = base * j
        if 1 <= cand <= MAX_QUANT_LF and cand <= LF_COUPLING_MAX_QUANT_LF:
            best = cand
        else:
            break
    return best


@dataclass(frozen=True)
class Quantizer:
    """QuantizerChoice (quantizer_ladder.rs:186): the three wire fields."""

    rung: int
    global_scale: int
    hf_mul: int
    quant_lf: int


def quantizer_at(r: int, quant_lf: int) -> Quantizer:
    """QuantizerChoice::at (quantizer_ladder.rs:204)."""
    gs, mul = rung_fields(r)
    return Quantizer(r, gs, mul, coupled_quant_lf(quant_lf, mul))


def effective_scale(r: int) -> int:
    """quantizer_ladder.rs:226: global_scale * HfMul."""
    gs, mul = rung_fields(r)
    return gs * mul


def rung_for_effective_scale(scale: int) -> int:
    """quantizer_ladder.rs:236: the finest rung not above `scale`."""
    mx = MAX_GLOBAL_SCALE
    if scale <= mx:
        return rung(max(scale - 1, 0))
    if scale >= mx * MAX_LADDER_MUL:
        return TOP
    k = min(max(-(-scale // mx), 2), MAX_LADDER_MUL)
    gs = scale // k
    index = _SEG_START[k]
    if gs < segment_first_scale(k):
        return rung(max(index - 1, 0))
    return rung(index + (gs - segment_first_scale(k)))


# ---- the local model (navigation.rs) ---------------------------------------


def ln_scale(r: int) -> float:
    """navigation.rs ln_scale."""
    return math.log(float(effective_scale(r)))


def _round_half_away(x: float) -> float:
    """f64::round: halves away from zero (Python's round() is half-even)."""
    f = math.floor(x)
    return f + 1.0 if x - f >= 0.5 else f


def rung_for_scale(scale: float) -> int:
    """navigation.rs rung_for_scale: non-finite scales land on the floor."""
    if not math.isfinite(scale):
        return FLOOR
    v = min(max(_round_half_away(scale), 1.0), 18446744073709551615.0)
    return rung_for_effective_scale(int(v))


def force_progress(aim: int, frm: int, finer: bool, at_least_one: bool = False) -> int:
    """navigation.rs force_progress (AtLeastOneRung / NudgeWhenStuck)."""
    if at_least_one:
        return max(aim, rung(frm + 1)) if finer else min(aim, rung(max(frm - 1, 0)))
    if aim != frm:
        return aim
    return rung(frm + 1) if finer else rung(max(frm - 1, 0))


def local_crossing(lo: tuple[float, float], hi: tuple[float, float], target_y: float) -> float:
    """LocalModel::through(lo, hi).crossing(target_y) (navigation.rs)."""
    slope = (hi[1] - lo[1]) / (hi[0] - lo[0])
    return lo[0] + (target_y - lo[1]) / slope


def local_slope(lo: tuple[float, float], hi: tuple[float, float]) -> float:
    """navigation.rs fit_slope (a zero run gives an infinite or NaN slope,
    as f64 division does)."""
    dy, dx = hi[1] - lo[1], hi[0] - lo[0]
    if dx == 0.0:
        return math.nan if dy == 0.0 else math.copysign(math.inf, dy)
    return dy / dx


# ---- the controller's constants and pure steps (quality.rs) ----------------

BRACKET_RATIO = 1.8            # quality.rs:169
PRIOR_LOSS_EXPONENT = 0.9      # :173
EXPANSION_MARGIN = 1.25        # :178
MAX_EXPANSION_JUMP = 16.0      # :181
STRUCTURE_REBUILD_RATIO = 1.8  # :186
LOSS_EPSILON = 1e-3            # :190
MET_OVERSHOOT_BAND = 1.0       # :199
MET_BAND_RESERVE_MULTIPLE = 2.0  # :213 (reserve-coupled-band)
MIN_AIM_MARGIN = 0.25          # :233
CORRECTED_STOP_MOVE_GATE = 0.5  # :242 (corrected-stop)


def loss(score: float) -> float:
    """quality.rs:867: the metric loss, floored."""
    return max(100.0 - score, LOSS_EPSILON)


def neg_ln_loss(score: float) -> float:
    return -math.log(loss(score))


def met_band(threshold: float, reserve: float) -> float:
    """quality.rs:219 with reserve-coupled-band."""
    return max(MET_BAND_RESERVE_MULTIPLE * reserve * loss(threshold), MET_OVERSHOOT_BAND)


def log_loss_crossing(infeasible: tuple[int, float], feasible: tuple[int, float],
                      aim_score: float) -> int | None:
    """quality.rs:888: the rung where -ln(loss) against ln(scale) reaches the
    aim, strictly inside the bracket; None when the points do not order."""
    lo_rung, lo_score = infeasible
    hi_rung, hi_score = feasible
    if hi_rung <= lo_rung + 1:
        return None
    x_lo, x_hi = ln_scale(lo_rung), ln_scale(hi_rung)
    y_lo, y_hi = neg_ln_loss(lo_score), neg_ln_loss(hi_score)
    if y_hi <= y_lo or x_hi <= x_lo:
        return None
    x = local_crossing((x_lo, y_lo), (x_hi, y_hi), neg_ln_loss(aim_score))
    r = rung_for_scale(math.exp(x))
    return min(max(r, rung(lo_rung + 1)), rung(hi_rung - 1))


def geometric_step(frm: int, finer: bool) -> int:
    """quality.rs:914: one BRACKET_RATIO step from exp(ln_scale(from))."""
    scale = math.exp(ln_scale(frm))
    nxt = scale * BRACKET_RATIO if finer else scale / BRACKET_RATIO
    return force_progress(rung_for_scale(nxt), frm, finer)


def extrapolated_step_from(points: list[tuple[int, float]], threshold: float,
                           prior_beta: float | None, finer: bool, attempt: int) -> int | None:
    """quality.rs:933: aim past the extrapolated crossing by a margin that
    grows with each attempt, one bounded jump at most."""
    pts = sorted(points, key=lambda p: p[0])
    if not pts:
        return None
    if finer:
        frm = pts[-1]
        other = pts[-2] if len(pts) >= 2 else None
    else:
        frm = pts[0]
        other = pts[1] if len(pts) >= 2 else None
    if (finer and frm[0] == TOP) or (not finer and frm[0] == FLOOR):
        return None
    alpha = None
    if other is not None:
        a = (ln_scale(other[0]), neg_ln_loss(other[1]))
        b = (ln_scale(frm[0]), neg_ln_loss(frm[1]))
        slope = local_slope(a, b)
        if abs(ln_scale(frm[0]) - ln_scale(other[0])) > 2.220446049250313e-16 and slope > 0.0:
            alpha = min(max(slope, 0.2), 3.0)
    if alpha is None:
        alpha = prior_beta if prior_beta is not None else PRIOR_LOSS_EXPONENT
    margin = EXPANSION_MARGIN ** (attempt + 1)
    ratio = (loss(frm[1]) / loss(threshold)) ** (1.0 / alpha)
    ratio = ratio * margin if finer else ratio / margin
    ratio = min(max(ratio, 1.0 / MAX_EXPANSION_JUMP), MAX_EXPANSION_JUMP)
    if (finer and ratio <= 1.0) or (not finer and ratio >= 1.0):
        return geometric_step(frm[0], finer)
    r = rung_for_scale(math.exp(ln_scale(frm[0])) * ratio)
    return geometric_step(frm[0], finer) if r == frm[0] else r


def aim_score_for(threshold: float, reserve: float) -> float:
    """quality.rs:991: the threshold plus the effort's loss-relative reserve."""
    relative = 100.0 - loss(threshold) * (1.0 - reserve)
    return max(relative, threshold + MIN_AIM_MARGIN)


def crossing_aim_from(lo: tuple[int, float], hi: tuple[int, float], threshold: float,
                      reserve: float) -> int | None:
    """quality.rs:999."""
    aim = aim_score_for(threshold, reserve)
    if aim >= hi[1]:
        return None
    return log_loss_crossing(lo, hi, aim)


def structure_is_far(anchor: int, r: int) -> bool:
    """quality.rs:1016."""
    return abs(ln_scale(r) - ln_scale(anchor)) > math.log(STRUCTURE_REBUILD_RATIO)


# ---- budgets and results -----------------------------------------------------


@dataclass(frozen=True)
class Budget:
    """QualityBudget (quality.rs:300) fields the baseline solve reads."""

    pixel_probes: int
    exact_prices: int
    structural_builds: int
    reserve: float


PRESETS = {  # QualityBudget::for_preset (quality.rs:395)
    "fast": Budget(3, 2, 2, 0.06),
    "balanced": Budget(5, 3, 2, 0.03),
    "quality": Budget(10, 4, 3, 0.02),
}


@dataclass
class ProbeRecord:
    rung: int
    score: float
    feasible: bool
    fresh: bool


@dataclass
class Outcome:
    """The search's answer: the chosen rung and quantizer, its score, the
    status name of quality.rs:854 and every probe in order."""

    rung: int
    quantizer: Quantizer
    score: float
    status: str
    probes: list = field(default_factory=list)
    bracket: tuple | None = None


class _Navigator:
    """Navigator (quality.rs:1104) without surrogates, pricing or trials.
    The methods that probe are generators: `yield (rung, fresh)` receives
    the score."""

    def __init__(self, target: float, budget: Budget, quant_lf: int,
                 prior_beta: float | None, guard: float):
        self.target, self.budget, self.quant_lf = target, budget, quant_lf
        self.prior_beta, self.guard = prior_beta, guard
        self.probes: list[ProbeRecord] = []
        self.pixel_probes = 0
        self.structural_builds = 0
        self.anchor_rung: int | None = None

    def threshold(self) -> float:
        return self.target + self.guard

    def band(self) -> float:
        return met_band(self.threshold(), self.budget.reserve)

    def pixel_budget_left(self) -> bool:
        return self.pixel_probes < self.budget.pixel_probes

    def already_probed(self, r: int) -> bool:
        return any(p.rung == r for p in self.probes)

    def probe(self, r: int, fresh: bool):
        """quality.rs:1153: a fresh probe plans its own structure and becomes
        the anchor when none exists yet."""
        fresh = fresh or self.anchor_rung is None
        score = yield (r, fresh)
        if fresh:
            self.structural_builds += 1
            if self.anchor_rung is None:
                self.anchor_rung = r
        self.pixel_probes += 1
        self.probes.append(ProbeRecord(r, float(score), float(score) >= self.threshold(), fresh))
        return len(self.probes) - 1

    def bracket(self):
        """quality.rs:1343: the finest infeasible and coarsest feasible probes."""
        inf = [p for p in self.probes if not p.feasible]
        fea = [p for p in self.probes if p.feasible]
        if not inf or not fea:
            return None
        lo = _max_by_rung(inf)
        hi = _min_by_rung(fea)
        return ((lo.rung, lo.score), (hi.rung, hi.score)) if lo.rung < hi.rung else None

    def coarsest_feasible(self):
        fea = [p for p in self.probes if p.feasible]
        return _min_by_rung(fea) if fea else None

    def extrapolated_step(self, finer: bool, attempt: int):
        pts = [(p.rung, p.score) for p in self.probes]
        return extrapolated_step_from(pts, self.threshold(), self.prior_beta, finer, attempt)

    def in_band(self, index: int) -> bool:
        p = self.probes[index] if 0 <= index < len(self.probes) else None
        return p is not None and p.feasible and p.score - self.threshold() <= self.band()

    def expand_until_bracketed(self):
        """quality.rs:1381."""
        attempt = 0
        while self.bracket() is None and self.pixel_budget_left():
            if not self.probes:
                return
            finer = not self.probes[-1].feasible
            nxt = self.extrapolated_step(finer, attempt)
            if nxt is None or self.already_probed(nxt):
                return
            yield from self.probe(nxt, False)
            attempt += 1

    def rescue_probe(self):
        """quality.rs:1404: one probe past the budget when nothing met."""
        if self.coarsest_feasible() is not None:
            return
        nxt = self.extrapolated_step(True, 3)
        if nxt is None or self.already_probed(nxt):
            return
        yield from self.probe(nxt, False)

    def crossing_is_tight(self) -> bool:
        """quality.rs:1420."""
        b = self.bracket()
        if b is None:
            return True
        (lo, _), (hi, hi_score) = b
        return hi <= lo + 1 or hi_score - self.threshold() <= self.band()

    def tighten_aim(self):
        """quality.rs:1431."""
        b = self.bracket()
        if b is None:
            return None
        r = crossing_aim_from(b[0], b[1], self.threshold(), self.budget.reserve)
        return None if r is None or self.already_probed(r) else r

    def corrected_aim(self, frm: tuple[int, float], beta: float) -> int:
        """quality.rs:1537."""
        aim = aim_score_for(self.threshold(), self.budget.reserve)
        ratio = (loss(frm[1]) / loss(aim)) ** (1.0 / beta)
        ratio = min(max(ratio, 1.0 / MAX_EXPANSION_JUMP), MAX_EXPANSION_JUMP)
        r = rung_for_scale(math.exp(ln_scale(frm[0])) * ratio)
        return force_progress(r, frm[0], frm[1] < aim)

    def corrected_stop(self):
        """quality.rs:1566: one correction under the prior exponent, one
        through the measured slope; True when a probe lands in band."""
        if not self.probes:
            return False
        first = (self.probes[0].rung, self.probes[0].score)
        aim = aim_score_for(self.threshold(), self.budget.reserve)
        implied = abs(math.log(loss(first[1]) / loss(aim))) / PRIOR_LOSS_EXPONENT
        if implied > CORRECTED_STOP_MOVE_GATE or not self.pixel_budget_left():
            return False
        second_rung = self.corrected_aim(first, PRIOR_LOSS_EXPONENT)
        if self.already_probed(second_rung):
            return False
        i2 = yield from self.probe(second_rung, False)
        if self.in_band(i2):
            return True
        if not self.pixel_budget_left():
            return False
        second = (self.probes[i2].rung, self.probes[i2].score)
        x1, x2 = ln_scale(first[0]), ln_scale(second[0])
        if abs(x2 - x1) <= 2.220446049250313e-16:
            return False
        slope = local_slope((x1, neg_ln_loss(first[1])), (x2, neg_ln_loss(second[1])))
        if math.isnan(slope) or slope <= 0.0:
            return False
        near = second if abs(second[1] - aim) < abs(first[1] - aim) else first
        third_rung = self.corrected_aim(near, min(max(slope, 0.2), 3.0))
        if self.already_probed(third_rung):
            return False
        i3 = yield from self.probe(third_rung, False)
        return self.in_band(i3)

    def tighten(self):
        """quality.rs:1603."""
        while self.pixel_budget_left() and not self.crossing_is_tight():
            r = self.tighten_aim()
            if r is None:
                break
            yield from self.probe(r, False)


def _min_by_rung(ps):
    # Iterator::min_by_key keeps the first of equal keys.
    best = ps[0]
    for p in ps[1:]:
        if p.rung < best.rung:
            best = p
    return best


def _max_by_rung(ps):
    # Iterator::max_by_key keeps the last of equal keys.
    best = ps[0]
    for p in ps[1:]:
        if p.rung >= best.rung:
            best = p
    return best


def navigate(start: int, target: float, budget: Budget | str = "balanced", *,
             quant_lf: int = 16, prior_beta: float | None = None, guard: float = 0.0):
    """The baseline solve of quality.rs:1775 as a generator: yields
    (rung, fresh) for every probe it wants, receives the probe's score, and
    returns the Outcome."""
    if isinstance(budget, str):
        budget = PRESETS[budget]
    nav = _Navigator(target, budget, quant_lf, prior_beta, guard)
    start = rung(start)
    yield from nav.probe(start, True)
    one_shot_hit = nav.in_band(0)
    corrected_hit = False
    if not one_shot_hit:
        corrected_hit = yield from nav.corrected_stop()
    if not one_shot_hit and not corrected_hit:
        yield from nav.expand_until_bracketed()
    yield from nav.tighten()
    yield from nav.rescue_probe()
    bracket = nav.bracket()

    # Finalists: the coarsest feasible probes (quality.rs:1882).
    anchor_rung = nav.anchor_rung if nav.anchor_rung is not None else start
    max_finalists = min(max(budget.exact_prices, 1), 2)
    ordered = sorted((i for i, p in enumerate(nav.probes) if p.feasible),
                     key=lambda i: nav.probes[i].rung)[:max_finalists]
    under_target = saturated = rescued = False
    if not ordered:
        under_target = True
        finest = _max_by_rung(nav.probes)
        saturated = finest.rung == TOP
        ordered = [max(range(len(nav.probes)), key=lambda i: (nav.probes[i].rung, i))]
    finalists: list[ProbeRecord] = []
    exact_prices = 0
    for index in ordered:
        if exact_prices >= budget.exact_prices:
            break
        p = nav.probes[index]
        rebuild = (not p.fresh and structure_is_far(anchor_rung, p.rung)
                   and nav.structural_builds < budget.structural_builds
                   and nav.pixel_budget_left() and not under_target)
        if rebuild:
            fi = yield from nav.probe(p.rung, True)
            if nav.probes[fi].feasible:
                exact_prices += 1
                rescued = True
                finalists.append(nav.probes[fi])
                continue
        exact_prices += 1
        finalists.append(p)
    # Selection: pricing would take the smallest feasible stream; the
    # coarsest feasible finalist stands in for it, else the finest.
    feasible = [f for f in finalists if f.feasible]
    chosen = _min_by_rung(feasible) if feasible else _max_by_rung(finalists)
    coarsest = nav.coarsest_feasible()
    adjacent_infeasible = coarsest is not None and any(
        (not p.feasible) and p.rung + 1 == coarsest.rung for p in nav.probes)
    threshold = target + guard
    if saturated:
        status = "saturated_top"
    elif under_target:
        status = "under_target_work_cap"
    elif rescued and chosen.fresh:
        status = "rescued_fresh_structure"
    elif chosen.rung == FLOOR:
        status = "saturated_floor"
    elif chosen.score - threshold <= met_band(threshold, budget.reserve):
        status = "met"
    elif adjacent_infeasible:
        status = "met_adjacent_rungs"
    else:
        status = "met_work_cap"
    return Outcome(chosen.rung, quantizer_at(chosen.rung, quant_lf), chosen.score, status,
                   [(p.rung, p.score, p.fresh) for p in nav.probes], bracket)


def solve(probe_fn, start: int, target: float, budget: Budget | str = "balanced",
          **kw) -> Outcome:
    """One frame: probe_fn(rung, fresh) -> score."""
    return search(lambda reqs: [probe_fn(r, f) for _, r, f in reqs], [start], target, budget,
                  **kw)[0]


def search(batch_fn, starts: list[int], target: float, budget: Budget | str = "balanced",
           **kw) -> list[Outcome]:
    """Many frames in lockstep: every round collects the pending probe of
    each unfinished frame as (frame index, rung, fresh) and calls
    batch_fn(requests) once for their scores (in request order)."""
    gens = [navigate(s, target, budget, **kw) for s in starts]
    pending: dict[int, tuple[int, bool]] = {}
    out: list[Outcome | None] = [None] * len(gens)
    for i, g in enumerate(gens):
        try:
            pending[i] = next(g)
        except StopIteration as stop:
            out[i] = stop.value
    while pending:
        reqs = [(i, r, f) for i, (r, f) in sorted(pending.items())]
        scores = list(batch_fn(reqs))
        if len(scores) != len(reqs):
            raise ValueError("batch_fn returned the wrong number of scores")
        pending = {}
        for (i, _, _), s in zip(reqs, scores):
            try:
                pending[i] = gens[i].send(float(s))
            except StopIteration as stop:
                out[i] = stop.value
    return out


# ---- the CUDA probes -----------------------------------------------------------


@dataclass
class SearchFrame:
    """One frame of a search: its interleaved samples on the host (the cover
    is selected from them) and in device memory (the probes read them), and
    its SSIMULACRA2 reference built from the same source."""

    rgb: object          # numpy [h, w, 3] uint8 or uint16
    rgb_ptr: int         # device address of the same samples
    ref: object          # PrecomputedReference
    bits: int = 8


class BatchedProber:
    """The probe function of `search` over the CUDA path: every round's
    probes, one per unfinished frame, run as one jpxlg batch (one CUDA
    graph over several lanes).  A probe at rung r encodes with the rung's
    quantizer (quantizer_at), renders at the source depth and scores
    against the frame's reference.  Structure: a fresh probe selects the
    cover for its own quantizer (select_blocks); a reused probe takes the
    frame's anchor cover, the cover of its first fresh probe.  CfL is
    estimated by every probe."""

    def __init__(self, ctx, frames: list, request=None, *, sharpness: int = 7, lanes: int = 0):
        from . import EncodeRequest
        self.ctx, self.frames = ctx, list(frames)
        self.request = request or EncodeRequest(gaborish=True, epf_iters=3)
        self.sharpness, self.lanes = sharpness, lanes
        self.anchor: dict[int, object] = {}
        self.covers: dict[tuple[int, int], object] = {}
        self.batches = 0
        self.probes = 0

    def request_for(self, q: Quantizer):
        from dataclasses import replace
        return replace(self.request, global_scale=q.global_scale, quant_lf=q.quant_lf)

    def cover(self, i: int, r: int, fresh: bool):
        from . import select_blocks
        if not fresh and i in self.anchor:
            return self.anchor[i]
        key = (i, r)
        if key not in self.covers:
            q = quantizer_at(r, self.request.quant_lf)
            f = self.frames[i]
            self.covers[key] = select_blocks(self.ctx, f.rgb, self.request_for(q), f.bits)
        self.anchor.setdefault(i, self.covers[key])
        return self.covers[key]

    def __call__(self, reqs) -> list[float]:
        from . import BatchItem, BatchProbe, Layout
        items, layouts = [], []
        for i, r, fresh in reqs:
            f = self.frames[i]
            q = quantizer_at(r, self.request.quant_lf)
            h, w = f.rgb.shape[:2]
            layout = Layout(self.ctx, w, h, self.cover(i, r, fresh), q.hf_mul, self.sharpness)
            layouts.append(layout)
            items.append(BatchItem(layout, f.ref, f.rgb_ptr, f.bits, self.request_for(q)))
        batch = BatchProbe(self.ctx, items, lanes=self.lanes)
        try:
            scores = batch.run()
        finally:
            batch.close()
            for layout in layouts:
                layout.close()
        self.batches += 1
        self.probes += len(items)
        return [float(s) for s in scores]


def search_frames(ctx, frames: list, target: float, starts: list[int],
                  budget: Budget | str = "balanced", request=None, **kw) -> list[Outcome]:
    """search_frame_perceptual for many frames over the CUDA path, in
    lockstep: one batch per navigation round."""
    prober = BatchedProber(ctx, frames, request)
    quant_lf = prober.request.quant_lf
    return search(prober, starts, target, budget, quant_lf=quant_lf, **kw)
