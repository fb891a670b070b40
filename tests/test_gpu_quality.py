"""The quality controller's search over the batched CUDA probes, against the
same search over the oracle's probes.

Eight frames of uneven sizes navigate in lockstep (one jpxlg batch per
round) toward SSIMULACRA2 targets under the Balanced and Fast budgets
(quality.rs:2405 search_frame_perceptual's baseline solve, restated in
jpxl_gb300.quality).  The oracle side runs the same navigation with every
probe computed by the CPU restatement (select_blocks for a fresh structure,
encode, render at the source depth, SSIMULACRA2).  Every probe the GPU search
made must score within 1e-4 points of the oracle's probe of the same frame,
rung and structure, and both searches must probe the same rungs in the same
order and choose the same quantizer with the same status."""
import numpy as np
import pytest

import jpxl_gb300 as jg
from jpxl_gb300 import quality as q
from jpxl_gb300 import synth

pytestmark = pytest.mark.gpu

SCORE_TOL = 1e-4


def _frames():
    rng = np.random.default_rng(9191)
    out = []
    for i in range(8):
        w, h = int(rng.integers(160, 321)), int(rng.integers(144, 289))
        out.append(synth.synthetic_rgb(w, h, seed=7100 + i, bits=8))
    return out


class OracleProber:
    """The CPU restatement's probes with BatchedProber's structure rule."""

    def __init__(self, oracle, frames, request):
        self.oracle, self.frames, self.request = oracle, frames, request
        self.anchor, self.covers, self.scores = {}, {}, {}

    def cover(self, i, r, fresh):
        if not fresh and i in self.anchor:
            return self.anchor[i]
        if (i, r) not in self.covers:
            quant = q.quantizer_at(r, self.request.quant_lf)
            rc, cov, _ = self.oracle.select_blocks(self.frames[i], global_scale=quant.global_scale,
                                                   quant_lf=quant.quant_lf, gaborish=True)
            assert rc == 0
            self.covers[(i, r)] = cov
        self.anchor.setdefault(i, self.covers[(i, r)])
        return self.covers[(i, r)]

    def __call__(self, reqs):
        out = []
        for i, r, fresh in reqs:
            rgb = self.frames[i]
            h, w = rgb.shape[:2]
            quant = q.quantizer_at(r, self.request.quant_lf)
            cover = self.cover(i, r, fresh)
            hf = np.full(cover.shape, quant.hf_mul, np.uint32)
            sh = np.full(cover.shape, 7, np.uint8)
            rc, plan = self.oracle.encode(rgb, cover, hf, global_scale=quant.global_scale,
                                          quant_lf=quant.quant_lf, gaborish=True)
            assert rc == 0
            rc, lin = self.oracle.reconstruct(w, h, cover, hf, sh, plan,
                                              global_scale=quant.global_scale,
                                              quant_lf=quant.quant_lf, gaborish=True,
                                              epf_iters=3, out_kind=3, bits=8)
            assert rc == 0
            s = self.oracle.ssim2(jg.srgb_to_linear_planes(rgb, 8), lin)[0]
            self.scores[(i, r, fresh)] = s
            out.append(s)
        return out


@pytest.mark.parametrize("preset,target", [("balanced", 80.0), ("fast", 60.0)])
def test_search_over_batched_probes_matches_the_oracle(ctx, oracle, preset, target):
    torch = pytest.importorskip("torch")
    frames = _frames()
    refs, devs, sframes = [], [], []
    for rgb in frames:
        ref = jg.PrecomputedReference(ctx, jg.srgb_to_linear_planes(rgb, 8))
        dev = torch.from_numpy(np.ascontiguousarray(rgb)).cuda()
        refs.append(ref)
        devs.append(dev)
        sframes.append(q.SearchFrame(rgb, dev.data_ptr(), ref, 8))
    torch.cuda.synchronize()
    request = jg.EncodeRequest(gaborish=True, epf_iters=3)
    # starts spread around the crossings so that expansion, correction and
    # tightening all run
    starts = [q.rung_for_scale(s) for s in (4000, 12000, 30000, 70000, 9000, 150000, 2500,
                                            45000)]
    prober = q.BatchedProber(ctx, sframes, request)
    got = q.search(prober, starts, target, preset, quant_lf=request.quant_lf)
    oprober = OracleProber(oracle, frames, request)
    want = q.search(oprober, starts, target, preset, quant_lf=request.quant_lf)
    try:
        assert prober.batches == max(len(o.probes) for o in got)
        for i, (g, w) in enumerate(zip(got, want)):
            print(f"frame {i} {frames[i].shape[1]}x{frames[i].shape[0]}: gpu {g.status} rung "
                  f"{g.rung} score {g.score:.6f} probes {[p[0] for p in g.probes]} | oracle "
                  f"{w.status} rung {w.rung} score {w.score:.6f}")
            for (rg, sg, fg), (rw, sw, fw) in zip(g.probes, w.probes):
                if (rg, fg) == (rw, fw):
                    assert abs(sg - sw) < SCORE_TOL, (i, rg, sg, sw)
            assert [(p[0], p[2]) for p in g.probes] == [(p[0], p[2]) for p in w.probes], i
            assert (g.rung, g.status) == (w.rung, w.status), i
            assert g.quantizer == w.quantizer
        statuses = {o.status for o in got}
        assert statuses & {"met", "met_adjacent_rungs", "met_work_cap",
                           "rescued_fresh_structure"}
    finally:
        for ref in refs:
            ref.close()
