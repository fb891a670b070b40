// oracle_abi.cpp — extern "C" entry points of the CPU restatement's scalar
// and plane stages (test infrastructure only; see oracle.h).
#include <algorithm>
#include <vector>

#include "oracle.h"
#include "oracle_internal.h"

using namespace orc;

extern "C" {

float orc_cbrt_core(float v) { return cbrt_core(v); }
float orc_cbrt_perceptual(float v) { return cbrt_perceptual(v); }
float orc_srgb_to_linear(float v) { return srgb_to_linear(v); }
float orc_linear_to_srgb(float v) { return linear_to_srgb(v); }
void orc_linear_to_xyb(const float* rgb3, float* xyb3) { linear_to_xyb(rgb3, xyb3); }
void orc_opsin_inverse(const float* xyb3, float* rgb3) { opsin_inverse(xyb3, rgb3); }
float orc_hf_multiplier(uint32_t gs, uint32_t hf_mul) { return hf_multiplier(gs, hf_mul); }
float orc_bias_adjust(int32_t q, float bias, float num) { return bias_adjust(q, bias, num); }
float orc_scale_f(int c, int lf_count) { return scale_f(c, lf_count); }

int orc_dequant_matrix(int dct_select, int channel, float* out, int* rows, int* cols) {
  TransformInfo t;
  if (!transform_info(dct_select, &t) || channel < 0 || channel > 2) return kErrParam;
  dequant_matrix(t.dq_index, channel, out, rows, cols);
  return kOk;
}

float orc_dct_iv_entry(int M, int u, int n) { return dct_iv_entry(M, u, n); }
void orc_dct_ii_ortho(float* v, int n) { dct_ii_ortho(v, n); }
void orc_dct_iii_ortho(float* v, int n) { dct_iii_ortho(v, n); }
void orc_dct_1d(float* v, int n) { dct_1d(v, n); }
void orc_idct_1d(float* v, int n) { idct_1d(v, n); }
void orc_dct_2d(float* work, int rows, int cols) { dct_2d(work, rows, cols); }
void orc_idct_2d(float* work, int rows, int cols) { idct_2d(work, rows, cols); }

// source.rs:226 — 256-entry LUT then planar XYB.
void orc_srgb8_to_xyb(const uint8_t* rgb, int w, int h, float* x, float* y, float* b) {
  float lut[256];
  for (int i = 0; i < 256; ++i) lut[i] = srgb_to_linear((float)i / 255.0f);
  size_t n = (size_t)w * h;
  for (size_t i = 0; i < n; ++i) {
    float lin[3] = {lut[rgb[3 * i]], lut[rgb[3 * i + 1]], lut[rgb[3 * i + 2]]}, o[3];
    linear_to_xyb(lin, o);
    x[i] = o[0]; y[i] = o[1]; b[i] = o[2];
  }
}

// source.rs:355 — per-code-point transfer curve over 2^bits - 1.
void orc_srgb16_to_xyb(const uint16_t* rgb, int w, int h, int bits, float* x, float* y,
                       float* b) {
  float max = std::min(65535.0f, (float)((1u << bits) - 1));
  float divisor = max > 0.0f ? max : 1.0f;
  std::vector<float> lut(65536);
  for (int i = 0; i < 65536; ++i) lut[i] = srgb_to_linear((float)i / divisor);
  size_t n = (size_t)w * h;
  for (size_t i = 0; i < n; ++i) {
    float lin[3] = {lut[rgb[3 * i]], lut[rgb[3 * i + 1]], lut[rgb[3 * i + 2]]}, o[3];
    linear_to_xyb(lin, o);
    x[i] = o[0]; y[i] = o[1]; b[i] = o[2];
  }
}

void orc_gab_precondition(const float* in, int w, int h, float* out) {
  gab_precondition(in, w, h, out);
}
void orc_gaborish(const float* in, int w, int h, float* out) { gaborish(in, w, h, out); }
void orc_gaborish_w(const float* in, int w, int h, float w1, float w2, float* out) {
  gaborish_w(in, w, h, w1, w2, out);
}
void orc_epf_step(int step, const float* const* in, int w, int h, const float* sigma,
                  float* const* out) {
  epf_step(step, in, w, h, sigma, out);
}
void orc_depth_thresholds(int bits, float* out) { depth_thresholds(bits, out); }

}  // extern "C"
