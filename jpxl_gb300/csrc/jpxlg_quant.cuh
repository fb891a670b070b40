// jpxlg_quant.cuh — the HF quantizer shared by the encoder's kernels
// (jpxl-encode-policy quantize.rs): clamp_round, the nearest-reconstruction
// choice and the residual bit proxy.
#pragma once
#include "jpxlg_common.cuh"

namespace jpxlg {

// 1 - the reference's per-channel quant bias (color.rs:591), defined in k_encode.cu.
extern __constant__ float c_quant_bias[3];

// quantize.rs:1720 clamp_round: v +- 0.5 then truncate; false = Err.
__device__ __forceinline__ bool clamp_round(float v, int32_t* out) {
  if (!isfinite(v)) return false;
  float adjusted = signbit(v) ? v - 0.5f : v + 0.5f;
  if (!(fabsf(adjusted) < 2147483648.0f)) return false;
  int32_t q = (int32_t)adjusted;
  if ((q < 0 ? -q : q) > (1 << 20)) return false;
  *out = q;
  return true;
}

__device__ __forceinline__ float bias_adjust(int32_t q, float bias) { return bias_adjust_q(q, bias); }

// quantize.rs:1400 HfQuantizer::choose (nearest reconstruction, ties to the
// smaller magnitude) with step = scale * matrix and the zero threshold
// 0.5 * bias * step, both formed as quantize.rs:334 forms them.
//
// The reference centres its candidates {0, e-1, e, e+1} on
// e = clamp_round(target / step).  The winner is always within one of
// target / step (a reconstruction bias_adjust(q) * step lies within 0.08
// steps of q * step), so a centre taken from target * (1 / step), which can
// differ from e by one only next to a half-integer, yields a candidate set
// holding the same winner, and the exact error comparison below picks it.
// `rstep` is 1.0f / step, formed once per cell by the caller.  Quotients
// near the 2^20 range limit, where the reference's error condition is
// decided, take the exact division.
__device__ __forceinline__ int32_t choose(float target, float step, float rstep, float bias,
                                          uint32_t* err, float* recon) {
  if (!(isfinite(step) && step > 0.0f)) {
    raise_error(err, kDevBadStep);
    *recon = 0.0f;
    return 0;
  }
  float thr = 0.5f * bias * step;
  if (fabsf(target) <= thr) {
    *recon = bias_adjust(0, bias) * step;
    return 0;
  }
  int32_t e;
  const float va = target * rstep;
  if (fabsf(va) < 1048000.0f) {
    e = (int32_t)(signbit(va) ? va - 0.5f : va + 0.5f);
  } else if (!clamp_round(target / step, &e)) {
    raise_error(err, kDevQuantRange);
    *recon = 0.0f;
    return 0;
  }
  // Reconstruction levels increase with q, so of {e-1, e, e+1} only e and
  // its neighbour on the target's side can be nearest; the third is strictly
  // farther.  Candidates in the reference's update rule: q = 0 first (its
  // level is 0, error |target|), then the pair in increasing q.
  const float re = bias_adjust(e, bias) * step;
  const int32_t nb = re < target ? e + 1 : e - 1;
  const float rn = bias_adjust(nb, bias) * step;
  int32_t best = 0;
  float best_err = fabsf(target);
  float best_recon = 0.0f;
  const int32_t q_lo = min(e, nb), q_hi = max(e, nb);
  const float r_lo = e < nb ? re : rn, r_hi = e < nb ? rn : re;
  // (|q| > 2^20 is outside the reference's candidate range; only the exact
  // path near the limit can reach it.)
  if (abs(q_lo) <= (1 << 20)) {
    const float er = fabsf(r_lo - target);
    if (er < best_err || (er == best_err && abs(q_lo) < abs(best))) {
      best = q_lo;
      best_err = er;
      best_recon = r_lo;
    }
  }
  if (abs(q_hi) <= (1 << 20)) {
    const float er = fabsf(r_hi - target);
    if (er < best_err || (er == best_err && abs(q_hi) < abs(best))) {
      best = q_hi;
      best_err = er;
      best_recon = r_hi;
    }
  }
  *recon = best_recon;
  return best;
}

__device__ __forceinline__ uint32_t residual_bits(int32_t q) {
  if (q == 0) return 0;
  uint32_t aq = (uint32_t)(q < 0 ? -q : q);
  return (32u - __clz(aq)) + 1u;
}

}  // namespace jpxlg
