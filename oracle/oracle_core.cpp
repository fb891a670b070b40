// oracle_core.cpp — CPU restatement of the scalar kernels of JPXL's lossy
// VarDCT pixel path: colour, cube roots, DCT, dequantization tables,
// quantizers, Gaborish, EPF and the output depth quantizer.
//
// TEST INFRASTRUCTURE ONLY (the checker, never the product).  Built with
// -ffp-contract=off so that every a*b+c rounds twice exactly as the Rust
// reference does; std::fma appears only where the reference writes mul_add.
// Citations are file:line within the reference project's JPXL/crates tree.
#include "oracle_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace orc {

// ---------------------------------------------------------------------------
// Cube roots
// ---------------------------------------------------------------------------

// jpxl-core/src/simd.rs:36 reproducible_cbrt: 5-bit integer estimate, two
// f64 Halley steps, one rounding to f32.
float cbrt_core(float value) {
  const uint32_t B1 = 709958130u;
  const uint32_t B2 = 642849266u;
  uint32_t bits = fbits(value);
  uint32_t magnitude = bits & 0x7fffffffu;
  if (magnitude == 0 || magnitude >= 0x7f800000u) return value;
  uint32_t estimate;
  if (magnitude < 0x00800000u) {
    float scaled = value * 16777216.0f;
    estimate = (fbits(scaled) & 0x7fffffffu) / 3u + B2;
  } else {
    estimate = magnitude / 3u + B1;
  }
  uint32_t estimate_bits = (bits & 0x80000000u) | estimate;
  double x = (double)value;
  double t = (double)ffrom(estimate_bits);
  for (int i = 0; i < 2; ++i) {
    double r = (t * t) * t;
    t = (t * ((x + x) + r)) / ((x + r) + r);
  }
  return (float)t;
}

// jpxl-perceptual/src/color.rs:46 reproducible_cbrt: f64 bit estimate and
// four Newton steps on |x|, sign reapplied.
float cbrt_perceptual(float value) {
  double x = (double)value;
  double a = std::fabs(x);
  uint64_t abits;
  std::memcpy(&abits, &a, 8);
  uint64_t ybits = abits / 3u + (0x2A9F7893ull << 32);
  double y;
  std::memcpy(&y, &ybits, 8);
  for (int i = 0; i < 4; ++i) {
    y -= (((y * y) * y) - a) / ((3.0 * y) * y);
  }
  float root = (float)y;
  float signed_root = x < 0.0 ? -root : root;
  if (value == 0.0f || !std::isfinite(value)) return value;
  return signed_root;
}

// ---------------------------------------------------------------------------
// Colour (jpxl-core/src/color.rs)
// ---------------------------------------------------------------------------

static const float kOpsinMix[3][3] = {
    {0.3f, 0.622f, 0.078f},
    {0.23f, 0.692f, 0.078f},
    {0.2434227f, 0.2047674f, 0.5518099f},
};
static const float kOpsinBias = 0.0037930734f;      // color.rs:54
static const float kOpsinBiasCbrt = 0.1559542f;     // color.rs:81

// color.rs:84 linear_srgb_to_xyb (no FMA; left-to-right sums).
void linear_to_xyb(const float rgb[3], float out[3]) {
  float r = rgb[0], g = rgb[1], b = rgb[2];
  float lm = kOpsinMix[0][0] * r + kOpsinMix[0][1] * g + kOpsinMix[0][2] * b + kOpsinBias;
  float mm = kOpsinMix[1][0] * r + kOpsinMix[1][1] * g + kOpsinMix[1][2] * b + kOpsinBias;
  float sm = kOpsinMix[2][0] * r + kOpsinMix[2][1] * g + kOpsinMix[2][2] * b + kOpsinBias;
  float lg = cbrt_core(lm) - kOpsinBiasCbrt;
  float mg = cbrt_core(mm) - kOpsinBiasCbrt;
  float sg = cbrt_core(sm) - kOpsinBiasCbrt;
  out[0] = 0.5f * (lg - mg);
  out[1] = 0.5f * (lg + mg);
  out[2] = sg;
}

// jpxl-perceptual/src/color.rs:66 linear_srgb_to_positive_xyb.
void linear_to_positive_xyb(const float rgb[3], float out[3]) {
  float r = rgb[0], g = rgb[1], b = rgb[2];
  float lm = kOpsinMix[0][0] * r + kOpsinMix[0][1] * g + kOpsinMix[0][2] * b + kOpsinBias;
  float mm = kOpsinMix[1][0] * r + kOpsinMix[1][1] * g + kOpsinMix[1][2] * b + kOpsinBias;
  float sm = kOpsinMix[2][0] * r + kOpsinMix[2][1] * g + kOpsinMix[2][2] * b + kOpsinBias;
  float lg = cbrt_perceptual(lm) - kOpsinBiasCbrt;
  float mg = cbrt_perceptual(mm) - kOpsinBiasCbrt;
  float sg = cbrt_perceptual(sm) - kOpsinBiasCbrt;
  float x = 0.5f * (lg - mg);
  float y = 0.5f * (lg + mg);
  out[0] = x * 14.0f + 0.42f;
  out[1] = y + 0.01f;
  out[2] = (sg - y) + 0.55f;
}

// color.rs:517 srgb_to_linear (odd extension below zero).
float srgb_to_linear(float v) {
  float a = std::fabs(v);
  float d = (a <= 12.92f * 0.0031308f) ? a / 12.92f : powf((a + 0.055f) / 1.055f, 2.4f);
  return v < 0.0f ? -d : d;
}

// color.rs:490 linear_to_srgb.
float linear_to_srgb(float v) {
  float a = std::fabs(v);
  float e = (a <= 0.0031308f) ? 12.92f * a : 1.055f * powf(a, 1.0f / 2.4f) - 0.055f;
  return v < 0.0f ? -e : e;
}

// jpxl-plan-render/src/lib.rs:55-68: Table L.1 defaults as the decoder reads
// them, and color.rs:626 OpsinInverse::new/convert.
static const float kInvMatrix[9] = {11.031567f, -9.866944f,  -0.16462299f,
                                    -3.2541474f, 4.4187705f, -0.16462299f,
                                    -3.6588513f, 2.712923f,  1.9459282f};
static const float kSignalledBias = -0.0037930733f;

void opsin_inverse(const float xyb[3], float out[3]) {
  static const float root = cbrt_core(kSignalledBias);
  const float itscale = 255.0f / 255.0f;
  float x = xyb[0], y = xyb[1], b = xyb[2];
  float gamma[3] = {y + x, y - x, b};
  float mix[3];
  for (int c = 0; c < 3; ++c) {
    float v = gamma[c] - root;
    mix[c] = ((v * v) * v + kSignalledBias) * itscale;
  }
  for (int r = 0; r < 3; ++r) {
    float acc = 0.0f;
    for (int c = 0; c < 3; ++c) acc = std::fma(kInvMatrix[r * 3 + c], mix[c], acc);
    out[r] = acc;
  }
}

// ---------------------------------------------------------------------------
// DCT (jpxl-core/src/dct.rs)
// ---------------------------------------------------------------------------

static const float kSqrtHalf = 0.707106769f;   // core::f32::consts::FRAC_1_SQRT_2
static const float kCosPi8 = 0.9238795f;       // dct.rs:143
static const float kSinPi8 = 0.38268343f;      // dct.rs:145

// The DCT-IV leaves of dct.rs:148-211 are the orthonormal matrices
// sqrt(2/M) cos(pi (2n+1)(2u+1) / 4M).  Every entry is +-m_j for the first
// row's magnitudes m_j (j = index of the odd angle), so each table is stored
// as that row: for M = 4 and 8 those are the correctly rounded f32 values,
// for M = 16 four of them sit one ulp away from correct rounding exactly as
// the reference's printed table does, and they are kept as printed.
static const float kIv4[4] = {0.69351995f, 0.587937772f, 0.392847478f, 0.13794969f};
static const float kIv8[8] = {0.49759236f,  0.478470176f, 0.440960646f, 0.386505216f,
                              0.317196637f, 0.235698372f, 0.145142332f, 0.0490085706f};
static const float kIv16[16] = {0.353127509f, 0.349726707f, 0.342957854f, 0.3328861f,
                                0.31960848f,  0.303252846f, 0.283976763f, 0.261965781f,
                                0.237431943f, 0.210611507f, 0.18176277f,  0.151163548f,
                                0.11910855f,  0.0859064683f, 0.051877059f, 0.0173480399f};

float dct_iv_entry(int M, int u, int n) {
  const float* mags = M == 4 ? kIv4 : (M == 8 ? kIv8 : kIv16);
  int k = ((2 * n + 1) * (2 * u + 1)) % (8 * M);
  float sign = 1.0f;
  if (k > 4 * M) k = 8 * M - k;          // cos symmetric about 2pi
  if (k > 2 * M) { k = 4 * M - k; sign = -1.0f; }  // cos(pi - t) = -cos t
  return sign * mags[(k - 1) / 2];
}

// dct.rs:243-280: dense DCT-IV, acc starts at zero, acc + c*x in column order.
static void dct_iv(float* v, int M) {
  if (M == 2) {
    float x0 = v[0], x1 = v[1];
    v[0] = kCosPi8 * x0 + kSinPi8 * x1;
    v[1] = kSinPi8 * x0 - kCosPi8 * x1;
    return;
  }
  float x[16];
  for (int i = 0; i < M; ++i) x[i] = v[i];
  for (int u = 0; u < M; ++u) {
    float acc = 0.0f;
    for (int n = 0; n < M; ++n) acc = acc + dct_iv_entry(M, u, n) * x[n];
    v[u] = acc;
  }
}

static void dct_ii(float* v, int N);
static void dct_iii(float* v, int N);

// dct.rs:286 (2-point) and :294 (4-point).
static void dct_ii_2(float* v) {
  float x0 = v[0], x1 = v[1];
  v[0] = (x0 + x1) * kSqrtHalf;
  v[1] = (x0 - x1) * kSqrtHalf;
}

static void dct_ii(float* v, int N) {
  if (N <= 1) return;
  if (N == 2) { dct_ii_2(v); return; }
  int H = N / 2;
  float even[16], odd[16];
  for (int k = 0; k < H; ++k) {          // split_even_odd, dct.rs:327
    even[k] = v[k] + v[N - 1 - k];
    odd[k] = v[k] - v[N - 1 - k];
  }
  if (N == 4) {                          // dct_ii_4, dct.rs:294
    dct_ii_2(even);
    dct_iv(odd, 2);
  } else {
    dct_ii(even, H);
    dct_iv(odd, H);
  }
  for (int k = 0; k < H; ++k) {          // merge_scaled, dct.rs:340
    v[2 * k] = even[k] * kSqrtHalf;
    v[2 * k + 1] = odd[k] * kSqrtHalf;
  }
}

static void dct_iii(float* v, int N) {
  if (N <= 1) return;
  if (N == 2) { dct_ii_2(v); return; }
  int H = N / 2;
  float even[16], odd[16];
  for (int k = 0; k < H; ++k) {          // split_scaled, dct.rs:350
    even[k] = v[2 * k] * kSqrtHalf;
    odd[k] = v[2 * k + 1] * kSqrtHalf;
  }
  if (N == 4) {                          // dct_iii_4, dct.rs:307
    dct_ii_2(even);
    dct_iv(odd, 2);
  } else {
    dct_iii(even, H);
    dct_iv(odd, H);
  }
  for (int k = 0; k < H; ++k) {          // merge_even_odd, dct.rs:363
    v[k] = even[k] + odd[k];
    v[N - 1 - k] = even[k] - odd[k];
  }
}

void dct_ii_ortho(float* v, int n) { dct_ii(v, n); }
void dct_iii_ortho(float* v, int n) { dct_iii(v, n); }

// dct.rs:731 dct_1d / :749 idct_1d (butterfly lengths up to 32).
void dct_1d(float* v, int n) {
  dct_ii(v, n);
  float factor = 1.0f / sqrtf((float)n);
  for (int i = 0; i < n; ++i) v[i] *= factor;
}
void idct_1d(float* v, int n) {
  dct_iii(v, n);
  float factor = sqrtf((float)n);
  for (int i = 0; i < n; ++i) v[i] *= factor;
}

// dct.rs:805 column_pass: the 1-D transform down every column.
static void column_pass(float* m, int rows, int cols, bool forward) {
  float col[32];
  for (int c = 0; c < cols; ++c) {
    for (int r = 0; r < rows; ++r) col[r] = m[r * cols + c];
    if (forward) dct_1d(col, rows); else idct_1d(col, rows);
    for (int r = 0; r < rows; ++r) m[r * cols + c] = col[r];
  }
}

static void transpose_into(const float* src, float* dst, int rows, int cols) {
  for (int r = 0; r < rows; ++r)
    for (int c = 0; c < cols; ++c) dst[c * rows + r] = src[r * cols + c];
}

// dct.rs:956 dct_2d_in_place.
void dct_2d(float* work, int rows, int cols) {
  float scratch[1024];
  int n = rows * cols;
  column_pass(work, rows, cols, true);
  transpose_into(work, scratch, rows, cols);
  column_pass(scratch, cols, rows, true);
  if (cols <= rows) std::memcpy(work, scratch, sizeof(float) * n);
  else transpose_into(scratch, work, cols, rows);
}

// dct.rs:982 idct_2d_in_place.
void idct_2d(float* work, int rows, int cols) {
  float scratch[1024];
  int n = rows * cols;
  if (cols > rows) transpose_into(work, scratch, rows, cols);
  else std::memcpy(scratch, work, sizeof(float) * n);
  column_pass(scratch, cols, rows, false);
  transpose_into(scratch, work, cols, rows);
  column_pass(work, rows, cols, false);
}

// ---------------------------------------------------------------------------
// Transforms (jpxl-core/src/varblock.rs:205 TRANSFORM_INFO) — the nine plain
// DCTRxC types this path carries.
// ---------------------------------------------------------------------------

bool transform_info(int sel, TransformInfo* t) {
  // (DctSelect, block rows, block cols, dequant matrix index)
  static const int table[][4] = {{0, 1, 1, 0},  {4, 2, 2, 4},  {5, 4, 4, 5},
                                 {6, 2, 1, 6},  {7, 1, 2, 6},  {8, 4, 1, 7},
                                 {9, 1, 4, 7},  {10, 4, 2, 8}, {11, 2, 4, 8}};
  for (auto& e : table) {
    if (e[0] == sel) {
      t->sel = sel;
      t->brows = e[1];
      t->bcols = e[2];
      t->dq_index = e[3];
      t->crows = std::min(e[1], e[2]) * 8;
      t->ccols = std::max(e[1], e[2]) * 8;
      return true;
    }
  }
  return false;
}

// varblock.rs:789 scale_f_closed_form (the tabled and closed forms agree).
float scale_f(int c, int lf_count) {
  int b = lf_count * 8;
  if (b == 0) return 1.0f;
  double cf = (double)c, bf = (double)b;
  const double pi = M_PI;
  double inv = std::cos(cf * pi / (2.0 * bf)) * std::cos(cf * pi / bf) *
               std::cos(2.0 * cf * pi / bf);
  return (float)(1.0 / inv);
}

// ---------------------------------------------------------------------------
// Dequantization weights (jpxl-core/src/dequant.rs) — Table I.6 DCT rows.
// ---------------------------------------------------------------------------

static const double kDct8x8[3][6] = {{3150.0, 0.0, -0.4, -0.4, -0.4, -2.0},
                                      {560.0, 0.0, -0.3, -0.3, -0.3, -0.3},
                                      {512.0, -2.0, -1.0, 0.0, -1.0, -2.0}};
static const double kDct16x16[3][7] = {
    {8996.8725711814115328, -1.3000777393353804, -0.49424529824571225, -0.439093774457103443,
     -0.6350101832695744, -0.90177264050827612, -1.6162099239887414},
    {3191.48366296844234752, -0.67424582104194355, -0.80745813428471001,
     -0.44925837484843441, -0.35865440981033403, -0.31322389111877305, -0.37615025315725483},
    {1157.50408145487200256, -2.0531423165804414, -1.4, -0.50687130033378396,
     -0.42708730624733904, -1.4856834539296244, -4.9209142884401604}};
static const double kDct32x32[3][8] = {
    {15718.40830982518931456, -1.025, -0.98, -0.9012, -0.4, -0.48819395464, -0.421064, -0.27},
    {7305.7636810695983104, -0.8041958212306401, -0.7633036457487539, -0.55660379990111464,
     -0.49785304658857626, -0.43699592683512467, -0.40180866526242109, -0.27321683125358037},
    {3803.53173721215041536, -3.060733579805728, -2.0413270132490346, -2.0235650159727417,
     -0.5495389509954993, -0.4, -0.4, -0.3}};
static const double kDct16x8[3][7] = {{7240.7734393502, -0.7, -0.7, -0.2, -0.2, -0.2, -0.5},
                                       {1448.15468787004, -0.5, -0.5, -0.5, -0.2, -0.2, -0.2},
                                       {506.854140754517, -1.4, -0.2, -0.5, -0.5, -1.5, -3.6}};
static const double kDct32x8[3][8] = {
    {16283.2494710648897, -1.7812845336559429, -1.6309059012653515, -1.0382179034313539, -0.85,
     -0.7, -0.9, -1.2360638576849587},
    {5089.15750884921511936, -0.320049391452786891, -0.35362849922161446, -0.30340000000000003,
     -0.61, -0.5, -0.5, -0.6},
    {3397.77603275308720128, -0.321327362693153371, -0.34507619223117997, -0.70340000000000003,
     -0.9, -1.0, -1.0, -1.1754605576265209}};
static const double kDct16x32[3][8] = {
    {13844.97076442300573, -0.97113799999999995, -0.658, -0.42026, -0.22712, -0.2206, -0.226,
     -0.6},
    {4798.964084220744293, -0.61125308982767057, -0.83770786552491361, -0.79014862079498627,
     -0.2692727459704829, -0.38272769465388551, -0.22924222653091453, -0.20719098826199578},
    {1807.236946760964614, -1.2, -1.2, -0.7, -0.7, -0.7, -0.4, -0.5}};

// dequant.rs:400 Mult.
static double mult(double v) { return v > 0.0 ? 1.0 + v : 1.0 / (1.0 - v); }

// dequant.rs:416 Interpolate.
static double interpolate(double pos, double max, const double* bands, int n) {
  int last = n - 1;
  if (last == 0) return bands[0];
  double scaled_pos = pos * (double)last / max;
  double scaled_index = std::floor(scaled_pos);
  int idx = (int)scaled_index;
  double frac = scaled_pos - scaled_index;
  double a = bands[idx];
  double b = bands[idx + 1];
  return a * std::pow(b / a, frac);
}

// dequant.rs:485 dct_quant_weights and :321 reciprocal narrowed to f32.
static void dct_matrix(const double* params, int np, int rows, int cols, float* out) {
  double bands[8];
  bands[0] = params[0];
  for (int i = 1; i < np; ++i) bands[i] = bands[i - 1] * mult(params[i]);
  double max = M_SQRT2 + 1e-6;
  double x_span = (double)(cols - 1), y_span = (double)(rows - 1);
  for (int y = 0; y < rows; ++y) {
    for (int x = 0; x < cols; ++x) {
      double dx = (double)x / x_span;
      double dy = (double)y / y_span;
      double distance = std::sqrt(dx * dx + dy * dy);
      double w = interpolate(distance, max, bands, np);
      out[y * cols + x] = (float)(1.0 / w);
    }
  }
}

// The dequantization matrix of Table I.4 index `dq` (DCT modes only), of the
// transform's landscape coefficient shape.
void dequant_matrix(int dq, int channel, float* out, int* rows, int* cols) {
  switch (dq) {
    case 0: *rows = 8; *cols = 8; dct_matrix(kDct8x8[channel], 6, 8, 8, out); break;
    case 4: *rows = 16; *cols = 16; dct_matrix(kDct16x16[channel], 7, 16, 16, out); break;
    case 5: *rows = 32; *cols = 32; dct_matrix(kDct32x32[channel], 8, 32, 32, out); break;
    case 6: *rows = 8; *cols = 16; dct_matrix(kDct16x8[channel], 7, 8, 16, out); break;
    case 7: *rows = 8; *cols = 32; dct_matrix(kDct32x8[channel], 8, 8, 32, out); break;
    case 8: *rows = 16; *cols = 32; dct_matrix(kDct16x32[channel], 8, 16, 32, out); break;
    default: *rows = 0; *cols = 0; break;
  }
}

const float* dequant_matrix_cached(int dq, int channel) {
  static float store[9][3][1024];
  static bool ready[9][3];
  if (!ready[dq][channel]) {
    int r, c;
    dequant_matrix(dq, channel, store[dq][channel], &r, &c);
    ready[dq][channel] = true;
  }
  return store[dq][channel];
}

// ---------------------------------------------------------------------------
// Scalar quantization rules
// ---------------------------------------------------------------------------

const float kQuantBias[3] = {1.0f - 0.054650073f, 1.0f - 0.0700545f, 1.0f - 0.049935103f};
const float kQuantBiasNumerator = 0.145f;

// reconstruct.rs:27 hf_multiplier.
float hf_multiplier(uint32_t gs, uint32_t hf_mul) {
  double denom = (double)gs * (double)hf_mul;
  if (denom <= 0.0) return 0.0f;
  return (float)(65536.0 / denom);
}

// reconstruct.rs:37 qm_multiplier: 0.8f32.powi(qm_scale - 2), evaluated by
// repeated squaring as the powi builtin does.
float qm_multiplier(uint32_t qm_scale) {
  int b = (int)qm_scale - 2;
  bool recip = b < 0;
  float a = 0.8f, r = 1.0f;
  for (;;) {
    if (b & 1) r *= a;
    b /= 2;
    if (b == 0) break;
    a *= a;
  }
  return recip ? 1.0f / r : r;
}

// reconstruct.rs:50 bias_adjust.
float bias_adjust(int32_t q, float bias, float num) {
  float f = (float)q;
  if (std::abs(q) <= 1) return f * bias;
  return f - num / f;
}

// quantize.rs:1720 clamp_round; false where the reference returns Err.
bool clamp_round(float v, int32_t* out) {
  if (!std::isfinite(v)) return false;
  float adjusted = std::signbit(v) ? v - 0.5f : v + 0.5f;
  // Rust's float-to-int cast saturates; |adjusted| > 2^31 is out of range anyway.
  if (!(std::fabs(adjusted) < 2147483648.0f)) return false;
  int32_t value = (int32_t)adjusted;
  if ((uint32_t)std::abs((int64_t)value) > (1u << 20)) return false;
  *out = value;
  return true;
}

// quantize.rs:1599 cfl_multiplier / reconstruct.rs:96 cfl_factors.
float cfl_multiplier(float base, int32_t factor, uint32_t colour_factor) {
  float ratio = (float)factor / (float)(colour_factor < 1 ? 1 : colour_factor);
  return base + ratio;
}

// quantize.rs:150 LfQuantizer.
LfQuant::LfQuant(uint32_t gs, uint32_t quant_lf, int extra_precision) : ep(extra_precision) {
  static const double w[3] = {1.0 / 32.0, 1.0 / 4.0, 1.0 / 2.0};
  double denom = (double)gs * (double)quant_lf;
  for (int c = 0; c < 3; ++c) {
    double wc = w[c] / 128.0;
    m_dc[c] = denom > 0.0 ? (float)(65536.0 * wc / denom) : 0.0f;
  }
}
float LfQuant::reconstruct(int32_t q, int c) const {
  return m_dc[c] * (float)q / (float)(1u << ep);
}
bool LfQuant::quantize(float target, int c, int32_t* q) const {
  float m = m_dc[c];
  if (!(std::isfinite(m) && m > 0.0f)) return false;
  float scaled = target * (float)(1u << ep) / m;
  return clamp_round(scaled, q);
}

// quantize.rs:301 HfQuantizer::new_with_matrices: step = (Mul*qm) * matrix,
// zero threshold = 0.5 * bias * step.
HfQuant::HfQuant(const TransformInfo& t, uint32_t gs, uint32_t hf_mul, uint32_t x_qm,
                 uint32_t b_qm) {
  float mul = hf_multiplier(gs, hf_mul);
  float scale[3] = {mul * qm_multiplier(x_qm), mul, mul * qm_multiplier(b_qm)};
  cells = t.crows * t.ccols;
  for (int c = 0; c < 3; ++c) {
    const float* m = dequant_matrix_cached(t.dq_index, c);
    for (int i = 0; i < cells; ++i) {
      steps[c][i] = scale[c] * m[i];
      thr[c][i] = 0.5f * kQuantBias[c] * steps[c][i];
    }
  }
}

float HfQuant::reconstruct(int32_t q, int c, int cell) const {
  return bias_adjust(q, kQuantBias[c], kQuantBiasNumerator) * steps[c][cell];
}

// quantize.rs:1400 choose (nearest-reconstruction rule, ties to smaller |q|).
bool HfQuant::choose(float target, int c, int cell, int32_t* out) const {
  float step = steps[c][cell];
  if (!(std::isfinite(step) && step > 0.0f)) return false;
  if (std::fabs(target) <= thr[c][cell]) { *out = 0; return true; }
  int32_t estimate;
  if (!clamp_round(target / step, &estimate)) return false;
  int32_t cand[4] = {0, estimate - 1, estimate, estimate + 1};
  int32_t best = 0;
  float best_error = INFINITY;
  for (int i = 0; i < 4; ++i) {
    int32_t q = cand[i];
    if (std::abs(q) > (1 << 20)) continue;
    float err = std::fabs(bias_adjust(q, kQuantBias[c], kQuantBiasNumerator) * step - target);
    if (err < best_error || (err == best_error && std::abs(q) < std::abs(best))) {
      best = q;
      best_error = err;
    }
  }
  *out = best;
  return true;
}

// ---------------------------------------------------------------------------
// Mirroring (jpxl-core/src/restoration.rs:56 mirror1d)
// ---------------------------------------------------------------------------

int mirror1d(int64_t c, int size) {
  if (size == 0) return 0;
  for (;;) {
    if (c < 0) c = -c - 1;
    else if (c >= size) c = 2 * (int64_t)size - 1 - c;
    else return (int)c;
  }
}

// A plane extended by r samples on every side with mirror1d's values.
std::vector<float> pad_mirror(const float* in, int w, int h, int r) {
  const int pw = w + 2 * r, ph = h + 2 * r;
  std::vector<float> out((size_t)pw * ph);
  for (int y = 0; y < ph; ++y) {
    const float* row = in + (size_t)mirror1d(y - r, h) * w;
    for (int x = 0; x < pw; ++x) out[(size_t)y * pw + x] = row[mirror1d(x - r, w)];
  }
  return out;
}

// ---------------------------------------------------------------------------
// Encoder inverse Gaborish (jpxl-encode/src/vardct/gaborish.rs)
// ---------------------------------------------------------------------------

struct EncKernel { float centre, edge, corner; };

// gaborish.rs:31 GaborKernel::new — normalised without FMA.
static EncKernel enc_kernel() {
  const float w1 = 0.115169525f, w2 = 0.061248592f;
  float unnorm = 1.0f + 4.0f * w1 + 4.0f * w2;
  float scale = 1.0f / unnorm;
  return {scale, w1 * scale, w2 * scale};
}

static float enc_weight(const EncKernel& k, int dx, int dy) {
  if (dx == 0 && dy == 0) return k.centre;
  if (dx == 0 || dy == 0) return k.edge;
  return k.corner;
}

// gaborish.rs:66 gaborish_forward: scalar 9-tap `acc += w*s` (dy outer, dx
// inner) on the border and on interior tails; the interior from x = 1 in
// groups of four as mid*c + (N+S+W+E)*e + (NW+NE+SW+SE)*k (:146).
static void enc_gaborish_forward(const float* in, int w, int h, const EncKernel& k,
                                 float* out) {
  for (int y = 0; y < h; ++y) {
    for (int x = 0; x < w; ++x) {
      bool edge = x == 0 || y == 0 || x + 1 == w || y + 1 == h;
      if (!edge) continue;
      float acc = 0.0f;
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          int sx = mirror1d(x + dx, w), sy = mirror1d(y + dy, h);
          acc += enc_weight(k, dx, dy) * in[(size_t)sy * w + sx];
        }
      out[(size_t)y * w + x] = acc;
    }
  }
  if (h >= 3 && w >= 3) {
    for (int y = 1; y < h - 1; ++y) {
      int x = 1;
      int x_end = w - 1;
      const float* rn = in + (size_t)(y - 1) * w;
      const float* rm = in + (size_t)y * w;
      const float* rs = in + (size_t)(y + 1) * w;
      for (; x + 4 <= x_end; x += 4) {
        for (int i = 0; i < 4; ++i) {
          int xi = x + i;
          float mid = rm[xi], north = rn[xi], south = rs[xi], west = rm[xi - 1],
                east = rm[xi + 1];
          float nw = rn[xi - 1], ne = rn[xi + 1], sw = rs[xi - 1], se = rs[xi + 1];
          out[(size_t)y * w + xi] = mid * k.centre + (north + south + west + east) * k.edge +
                                    (nw + ne + sw + se) * k.corner;
        }
      }
      for (; x < x_end; ++x) {
        float acc = 0.0f;
        for (int dy = -1; dy <= 1; ++dy)
          for (int dx = -1; dx <= 1; ++dx)
            acc += enc_weight(k, dx, dy) * in[(size_t)(y + dy) * w + (x + dx)];
        out[(size_t)y * w + x] = acc;
      }
    }
  }
}

// gaborish.rs:218 precondition_xyb_planes / :238 gaborish_inverse, 12 Jacobi
// steps x <- x + (f - Kx) * (1/centre) for the first 4*floor(n/4) samples and
// x + (f - Kx) / centre for the tail.
void gab_precondition(const float* f, int w, int h, float* x) {
  EncKernel k = enc_kernel();
  size_t n = (size_t)w * h;
  std::vector<float> kx(n);
  std::memcpy(x, f, sizeof(float) * n);
  float inv_c = 1.0f / k.centre;
  size_t bulk = n - n % 4;
  for (int it = 0; it < 12; ++it) {
    enc_gaborish_forward(x, w, h, k, kx.data());
    for (size_t i = 0; i < bulk; ++i) x[i] = x[i] + (f[i] - kx[i]) * inv_c;
    for (size_t i = bulk; i < n; ++i) x[i] = x[i] + (f[i] - kx[i]) / k.centre;
  }
}

// ---------------------------------------------------------------------------
// Decoder J.3 (jpxl-core/src/restoration.rs:111 GaborKernel::new, :148)
// ---------------------------------------------------------------------------

void gaborish(const float* in, int w, int h, float* out) {
  gaborish_w(in, w, h, 0.115169525f, 0.061248592f, out);
}

void gaborish_w(const float* in, int w, int h, float w1, float w2, float* out) {
  float unnorm = std::fma(4.0f, w2, std::fma(4.0f, w1, 1.0f));
  float scale = 1.0f / unnorm;
  float centre = scale, edge = w1 * scale, corner = w2 * scale;
  const std::vector<float> pad = pad_mirror(in, w, h, 1);
  const int pw = w + 2;
  for (int y = 0; y < h; ++y) {
    for (int x = 0; x < w; ++x) {
      float acc = 0.0f;
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          float wt = (dx == 0 && dy == 0) ? centre : ((dx == 0 || dy == 0) ? edge : corner);
          float s = pad[(size_t)(y + 1 + dy) * pw + (x + 1 + dx)];
          acc = std::fma(wt, s, acc);
        }
      out[(size_t)y * w + x] = acc;
    }
  }
}

// ---------------------------------------------------------------------------
// J.4 EPF (jpxl-core/src/restoration.rs:201-731)
// ---------------------------------------------------------------------------

static const int kCross[5][2] = {{0, 0}, {-1, 0}, {1, 0}, {0, -1}, {0, 1}};
static const int kStep0[13][2] = {{0, 0}, {-1, 0}, {1, 0},  {0, -1}, {0, 1},  {1, -1}, {1, 1},
                                  {-1, 1}, {-1, -1}, {-2, 0}, {2, 0}, {0, 2}, {0, -2}};

float epf_inv_sigma(int step, float sigma) {
  float scale = step == 0 ? 0.9f : (step == 1 ? 1.0f : 6.5f);
  float sm = 1.65f * scale;
  return sm * 4.0f * (1.0f - sqrtf(0.5f)) / sigma;
}

float vardct_sigma(float mul, int sharpness) {
  static const float lut[8] = {0.0f,        1.0f / 7.0f, 2.0f / 7.0f, 3.0f / 7.0f,
                               4.0f / 7.0f, 5.0f / 7.0f, 6.0f / 7.0f, 1.0f};
  return mul * 0.46f * lut[sharpness > 7 ? 7 : sharpness];
}

// restoration.rs:619 epf_step_rows_impl over the whole plane.
void epf_step(int step, const float* const* in, int w, int h, const float* sigma,
              float* const* out) {
  const int(*taps)[2] = step == 0 ? kStep0 : kCross;
  int ntaps = step == 0 ? 13 : 5;
  int ncross = step == 2 ? 1 : 5;
  const float scale[3] = {40.0f, 5.0f, 3.5f};
  int bw = (w + 7) / 8;
  // The taps reach 3 samples out (offset 2 plus the cross's 1): each plane
  // mirrored by 3 once, so that a sample is one lookup.
  const std::vector<float> pad[3] = {pad_mirror(in[0], w, h, 3), pad_mirror(in[1], w, h, 3),
                                     pad_mirror(in[2], w, h, 3)};
  const int pw = w + 6;
  auto at = [&](int c, int x, int y) -> float { return pad[c][(size_t)(y + 3) * pw + (x + 3)]; };
  for (int y = 0; y < h; ++y) {
    int ry = y % 8;
    bool border_row = ry == 0 || ry == 7;
    for (int x = 0; x < w; ++x) {
      size_t idx = (size_t)y * w + x;
      float bs = sigma[(size_t)(y / 8) * bw + x / 8];
      if (bs < 0.3f) {
        for (int c = 0; c < 3; ++c) out[c][idx] = in[c][idx];
        continue;
      }
      float inv_sigma = epf_inv_sigma(step, bs);
      int rx = x % 8;
      bool at_border = border_row || rx == 0 || rx == 7;
      float sum_w = 0.0f;
      float acc[3] = {0.0f, 0.0f, 0.0f};
      for (int t = 0; t < ntaps; ++t) {
        int kx = taps[t][0], ky = taps[t][1];
        float d = 0.0f;
        for (int c = 0; c < 3; ++c) {
          for (int i = 0; i < ncross; ++i) {
            int ix = kCross[i][0], iy = kCross[i][1];
            float a = at(c, x + ix, y + iy);
            float b = at(c, x + kx + ix, y + ky + iy);
            d = std::fma(std::fabs(a - b), scale[c], d);
          }
        }
        float pos_mul = at_border ? 2.0f / 3.0f : 1.0f;
        float sd = pos_mul * d;
        float weight;
        if (sd == 0.0f) {
          weight = 1.0f;
        } else {
          float v = std::fma(sd, -inv_sigma, 1.0f);
          weight = v > 0.0f ? v : 0.0f;
        }
        sum_w += weight;
        for (int c = 0; c < 3; ++c) acc[c] = std::fma(at(c, x + kx, y + ky), weight, acc[c]);
      }
      for (int c = 0; c < 3; ++c) out[c][idx] = acc[c] / sum_w;
    }
  }
}

// ---------------------------------------------------------------------------
// Output depth (jpxl-plan-render/src/lib.rs:153-468)
// ---------------------------------------------------------------------------

float full_scale(int bits) { return bits >= 32 ? 65535.0f : (float)((1u << std::max(bits, 1)) - 1); }

// lib.rs:198 composed_level: round(linear_to_srgb(x) * max) clamped.
int composed_level(float x, float max) {
  float scaled = roundf(linear_to_srgb(x) * max);
  if (!std::isfinite(scaled)) return 0;
  return (int)std::min(std::max(scaled, 0.0f), max);
}

// lib.rs:333 quantize_thresholds by bisection over the f32 bit lattice.
void depth_thresholds(int bits, float* out) {
  float max = full_scale(bits);
  int levels = bits >= 32 ? 65536 : (1 << std::min(std::max(bits, 1), 16));
  for (int q = 1; q < levels; ++q) {
    uint32_t lo = 0, hi = fbits(2.0f);
    while (lo < hi) {
      uint32_t mid = lo + (hi - lo) / 2;
      if (composed_level(ffrom(mid), max) >= q) hi = mid;
      else lo = mid + 1;
    }
    out[q - 1] = ffrom(lo);
  }
}

}  // namespace orc
