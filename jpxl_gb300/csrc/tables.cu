// tables.cu — host-side constant tables of the lossy VarDCT pixel path,
// built once per context in the precision the reference builds them (f64
// where the reference uses f64, narrowed to f32 once) and uploaded to the
// device.  This file is compiled with -ffp-contract=off so that table
// arithmetic rounds exactly as the reference's.
//
// References are to files of the JPXL project (crates/...).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "jpxlg_common.cuh"
#include "jpxlg_internal.h"

namespace jpxlg {

// ---- I.2.5 / Table I.6 DCT parameter rows (jpxl-core dequant.rs:712-1020) ----
// The data table of the standard: kept digit-for-digit as the reference
// prints it, because every weight is a function of these literals.
namespace {
const double kP8x8[3][8] = {{3150.0, 0.0, -0.4, -0.4, -0.4, -2.0},
                            {560.0, 0.0, -0.3, -0.3, -0.3, -0.3},
                            {512.0, -2.0, -1.0, 0.0, -1.0, -2.0}};
const double kP16x16[3][8] = {
    {8996.8725711814115328, -1.3000777393353804, -0.49424529824571225, -0.439093774457103443,
     -0.6350101832695744, -0.90177264050827612, -1.6162099239887414},
    {3191.48366296844234752, -0.67424582104194355, -0.80745813428471001,
     -0.44925837484843441, -0.35865440981033403, -0.31322389111877305, -0.37615025315725483},
    {1157.50408145487200256, -2.0531423165804414, -1.4, -0.50687130033378396,
     -0.42708730624733904, -1.4856834539296244, -4.9209142884401604}};
const double kP32x32[3][8] = {
    {15718.40830982518931456, -1.025, -0.98, -0.9012, -0.4, -0.48819395464, -0.421064, -0.27},
    {7305.7636810695983104, -0.8041958212306401, -0.7633036457487539, -0.55660379990111464,
     -0.49785304658857626, -0.43699592683512467, -0.40180866526242109, -0.27321683125358037},
    {3803.53173721215041536, -3.060733579805728, -2.0413270132490346, -2.0235650159727417,
     -0.5495389509954993, -0.4, -0.4, -0.3}};
const double kP16x8[3][8] = {{7240.7734393502, -0.7, -0.7, -0.2, -0.2, -0.2, -0.5},
                             {1448.15468787004, -0.5, -0.5, -0.5, -0.2, -0.2, -0.2},
                             {506.854140754517, -1.4, -0.2, -0.5, -0.5, -1.5, -3.6}};
const double kP32x8[3][8] = {
    {16283.2494710648897, -1.7812845336559429, -1.6309059012653515, -1.0382179034313539, -0.85,
     -0.7, -0.9, -1.2360638576849587},
    {5089.15750884921511936, -0.320049391452786891, -0.35362849922161446,
     -0.30340000000000003, -0.61, -0.5, -0.5, -0.6},
    {3397.77603275308720128, -0.321327362693153371, -0.34507619223117997,
     -0.70340000000000003, -0.9, -1.0, -1.0, -1.1754605576265209}};
const double kP16x32[3][8] = {
    {13844.97076442300573, -0.97113799999999995, -0.658, -0.42026, -0.22712, -0.2206, -0.226,
     -0.6},
    {4798.964084220744293, -0.61125308982767057, -0.83770786552491361, -0.79014862079498627,
     -0.2692727459704829, -0.38272769465388551, -0.22924222653091453, -0.20719098826199578},
    {1807.236946760964614, -1.2, -1.2, -0.7, -0.7, -0.7, -0.4, -0.5}};

// Indices 11 (DCT64x64) and 12 (DCT64x32 / DCT32x64): {base, SeqA | SeqB |
// SeqC} per channel (jpxl-core dequant.rs:746-790).
const double kSeqA[7] = {-1.025, -0.78, -0.65012, -0.19041574084286472, -0.20819395464,
                         -0.421064, -0.32733845535848671};
const double kSeqB[7] = {-0.3041958212306401, -0.3633036457487539, -0.35660379990111464,
                         -0.3443074455424403, -0.33699592683512467, -0.30180866526242109,
                         -0.27321683125358037};
const double kSeqC[7] = {-1.2, -1.2, -0.8, -0.7, -0.7, -0.4, -0.5};
const double kLargeBase[2][3] = {{23966.1665298448605, 8380.19148390090414, 4493.02378009847706},
                                 {15358.89804933239925, 5597.360516150652990,
                                  2919.961618960011210}};
double kP64x64[3][8], kP64x32[3][8];
struct LargeInit {
  LargeInit() {
    const double* seq[3] = {kSeqA, kSeqB, kSeqC};
    for (int c = 0; c < 3; ++c) {
      kP64x64[c][0] = kLargeBase[0][c];
      kP64x32[c][0] = kLargeBase[1][c];
      for (int i = 0; i < 7; ++i) kP64x64[c][i + 1] = kP64x32[c][i + 1] = seq[c][i];
    }
  }
} g_large_init;

// Table I.6 DCT2 params (dequant.rs:986), used as weights directly.
const double kDct2[3][6] = {{3840.0, 2560.0, 1280.0, 640.0, 480.0, 300.0},
                            {960.0, 640.0, 320.0, 180.0, 140.0, 120.0},
                            {640.0, 320.0, 128.0, 64.0, 32.0, 16.0}};

struct Slot {
  const double (*params)[8];
  int np, rows, cols;
};
const Slot kSlots[9] = {{kP8x8, 6, 8, 8},    {kP16x16, 7, 16, 16}, {kP32x32, 8, 32, 32},
                        {kP16x8, 7, 8, 16},  {kP32x8, 8, 8, 32},   {kP16x32, 8, 16, 32},
                        {nullptr, 0, 8, 8},  {kP64x64, 8, 64, 64}, {kP64x32, 8, 32, 64}};

// I.2.4 mode DCT2 (dequant.rs:1328): six rectangles of the 8x8 weights
// matrix, (0, 0) set to one; the matrix is the f32 reciprocal.
void dct2_into(const double* p, float* out) {
  double w[64] = {};
  auto fill = [&](int x0, int y0, int x1, int y1, double v) {
    for (int y = y0; y < y1; ++y)
      for (int x = x0; x < x1; ++x) w[y * 8 + x] = v;
  };
  fill(4, 4, 8, 8, p[5]);
  fill(4, 0, 8, 4, p[4]);
  fill(0, 4, 4, 8, p[4]);
  fill(2, 2, 4, 4, p[3]);
  fill(2, 0, 4, 2, p[2]);
  fill(0, 2, 2, 4, p[2]);
  fill(1, 1, 2, 2, p[1]);
  fill(0, 1, 1, 2, p[0]);
  fill(1, 0, 2, 1, p[0]);
  w[0] = 1.0;
  for (int i = 0; i < 64; ++i) out[i] = (float)(1.0 / w[i]);
}

// I.2.4 GetDctQuantWeights: geometric interpolation of the band sequence
// over the radial distance, then the f32 reciprocal (dequant.rs:321).
void weights_into(const double* params, int np, int rows, int cols, float* out) {
  double bands[8];
  bands[0] = params[0];
  for (int i = 1; i < np; ++i) {
    double v = params[i];
    double m = v > 0.0 ? 1.0 + v : 1.0 / (1.0 - v);
    bands[i] = bands[i - 1] * m;
  }
  const double range = M_SQRT2 + 1e-6;
  const int last = np - 1;
  for (int y = 0; y < rows; ++y) {
    for (int x = 0; x < cols; ++x) {
      double dx = (double)x / (double)(cols - 1);
      double dy = (double)y / (double)(rows - 1);
      double dist = std::sqrt(dx * dx + dy * dy);
      double pos = dist * (double)last / range;
      double fl = std::floor(pos);
      int idx = (int)fl;
      double frac = pos - fl;
      double a = bands[idx], b = bands[idx + 1];
      double w = a * std::pow(b / a, frac);
      out[y * cols + x] = (float)(1.0 / w);
    }
  }
}
}  // namespace

void build_dequant_tables(float* out) {
  for (int c = 0; c < 3; ++c)
    for (int s = 0; s < 9; ++s) {
      float* dst = out + c * kDequantTableFloats + dq_offset(s);
      if (s == 6) dct2_into(kDct2[c], dst);
      else weights_into(kSlots[s].params[c], kSlots[s].np, kSlots[s].rows, kSlots[s].cols, dst);
    }
}

// dct.rs:631 build_dct_matrix(64): orthonormal DCT-II rows in f64, narrowed.
void build_dct64_matrix(float* out) {
  const int n = 64;
  for (int u = 0; u < n; ++u) {
    const double scale = std::sqrt(u == 0 ? 1.0 / n : 2.0 / n);
    for (int x = 0; x < n; ++x) {
      const double angle = M_PI * (double)(2 * x + 1) * (double)u / (2.0 * n);
      out[u * n + x] = (float)(scale * std::cos(angle));
    }
  }
}

// ---- DCT-IV leaves (dct.rs:148-211) ------------------------------------------
// Entry (u, n) of the orthonormal DCT-IV of size M is +-m_j, where m_j is the
// j-th entry of the matrix's first row and (2n+1)(2u+1) folds onto 2j+1.  The
// first rows are those the reference prints: correctly rounded for M = 4 and
// 8; four of the sixteen M = 16 magnitudes are one ulp off correct rounding
// in the reference's table and are kept that way.
void build_iv_tables(float* iv4, float* iv8, float* iv16) {
  static const float m4[4] = {0.69351995f, 0.587937772f, 0.392847478f, 0.13794969f};
  static const float m8[8] = {0.49759236f,  0.478470176f, 0.440960646f, 0.386505216f,
                              0.317196637f, 0.235698372f, 0.145142332f, 0.0490085706f};
  static const float m16[16] = {0.353127509f, 0.349726707f, 0.342957854f, 0.3328861f,
                                0.31960848f,  0.303252846f, 0.283976763f, 0.261965781f,
                                0.237431943f, 0.210611507f, 0.18176277f,  0.151163548f,
                                0.11910855f,  0.0859064683f, 0.051877059f, 0.0173480399f};
  auto fill = [](int M, const float* mags, float* out) {
    for (int u = 0; u < M; ++u)
      for (int n = 0; n < M; ++n) {
        int k = ((2 * n + 1) * (2 * u + 1)) % (8 * M);
        float sign = 1.0f;
        if (k > 4 * M) k = 8 * M - k;
        if (k > 2 * M) {
          k = 4 * M - k;
          sign = -1.0f;
        }
        out[u * M + n] = sign * mags[(k - 1) / 2];
      }
  };
  fill(4, m4, iv4);
  fill(8, m8, iv8);
  fill(16, m16, iv16);
}

// varblock.rs:789 ScaleF closed form, for LF counts 1, 2, 4, 8 (b = 8*count).
void build_scale_f(float* out) {
  const int counts[4] = {1, 2, 4, 8};
  for (int i = 0; i < 4; ++i)
    for (int c = 0; c < 8; ++c) {
      double cf = (double)c, bf = (double)(counts[i] * 8);
      double inv = std::cos(cf * M_PI / (2.0 * bf)) * std::cos(cf * M_PI / bf) *
                   std::cos(2.0 * cf * M_PI / bf);
      out[i * 8 + c] = (float)(1.0 / inv);
    }
}

// reconstruct.rs:27 / quantize.rs:301: Mul = 65536 / (gs * hf_mul) in f64.
float host_hf_multiplier(uint32_t gs, uint32_t hf_mul) {
  double denom = (double)gs * (double)hf_mul;
  return denom <= 0.0 ? 0.0f : (float)(65536.0 / denom);
}

// reconstruct.rs:37: 0.8f32.powi(qm_scale - 2) by repeated squaring.
float host_qm_multiplier(uint32_t qm_scale) {
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

// reconstruct.rs:67 lf_multipliers with the G.1.2 default weights over 128.
void host_lf_multipliers(uint32_t gs, uint32_t quant_lf, float out[3]) {
  static const float w[3] = {1.0f / 32.0f, 1.0f / 4.0f, 1.0f / 2.0f};
  double denom = (double)gs * (double)quant_lf;
  for (int c = 0; c < 3; ++c) {
    float wc = w[c] / 128.0f;
    out[c] = denom > 0.0 ? (float)(65536.0 * (double)wc / denom) : 0.0f;
  }
}

// color.rs:517 / :490 transfer pair (odd below zero), host libm powf.
float host_srgb_to_linear(float v) {
  float a = std::fabs(v);
  float d = (a <= 12.92f * 0.0031308f) ? a / 12.92f : powf((a + 0.055f) / 1.055f, 2.4f);
  return v < 0.0f ? -d : d;
}
float host_linear_to_srgb(float v) {
  float a = std::fabs(v);
  float e = (a <= 0.0031308f) ? 12.92f * a : 1.055f * powf(a, 1.0f / 2.4f) - 0.055f;
  return v < 0.0f ? -e : e;
}

// source.rs:210/:355 — the per-code-point sRGB->linear table.
void build_srgb_lut(int bits, float* out) {
  if (bits == 8) {
    for (int i = 0; i < 256; ++i) out[i] = host_srgb_to_linear((float)i / 255.0f);
    return;
  }
  float max = std::min(65535.0f, (float)((1u << bits) - 1));
  float divisor = max > 0.0f ? max : 1.0f;
  for (int i = 0; i < 65536; ++i) out[i] = host_srgb_to_linear((float)i / divisor);
}

// plan-render lib.rs:333 quantize_thresholds: the smallest f32 reaching each
// level of round(linear_to_srgb(x) * max), by bisection on the bit lattice;
// lib.rs:161 linear_lut: the linear value of every level.
int build_depth_thresholds(int bits, float* thresholds, float* levels_linear) {
  float max = bits >= 32 ? 65535.0f : (float)((1u << std::max(bits, 1)) - 1);
  int levels = bits >= 32 ? 65536 : (1 << std::min(std::max(bits, 1), 16));
  auto level = [&](float x) -> int {
    float scaled = roundf(host_linear_to_srgb(x) * max);
    if (!std::isfinite(scaled)) return 0;
    return (int)std::min(std::max(scaled, 0.0f), max);
  };
  for (int q = 1; q < levels; ++q) {
    uint32_t lo = 0, hi = 0x40000000u;
    while (lo < hi) {
      uint32_t mid = lo + (hi - lo) / 2;
      float m;
      std::memcpy(&m, &mid, 4);
      if (level(m) >= q) hi = mid;
      else lo = mid + 1;
    }
    std::memcpy(&thresholds[q - 1], &lo, 4);
  }
  for (int q = 0; q < levels; ++q) levels_linear[q] = host_srgb_to_linear((float)q / max);
  return levels;
}

// jpxl-core simd.rs:36 on the host (used for the opsin bias cube roots).
float host_cbrt_core(float value) {
  const uint32_t B1 = 709958130u, B2 = 642849266u;
  uint32_t bits;
  std::memcpy(&bits, &value, 4);
  uint32_t magnitude = bits & 0x7fffffffu;
  if (magnitude == 0 || magnitude >= 0x7f800000u) return value;
  uint32_t estimate;
  if (magnitude < 0x00800000u) {
    float scaled = value * 16777216.0f;
    uint32_t sb;
    std::memcpy(&sb, &scaled, 4);
    estimate = (sb & 0x7fffffffu) / 3u + B2;
  } else {
    estimate = magnitude / 3u + B1;
  }
  uint32_t eb = (bits & 0x80000000u) | estimate;
  float ef;
  std::memcpy(&ef, &eb, 4);
  double x = (double)value, t = (double)ef;
  for (int i = 0; i < 2; ++i) {
    double r = (t * t) * t;
    t = (t * ((x + x) + r)) / ((x + r) + r);
  }
  return (float)t;
}

// plan-render lib.rs:55-68: Table L.1 defaults as signalled; color.rs:626
// OpsinInverse::new hoists cbrt(bias).
void build_opsin_inverse(float* matrix9, float* bias3, float* bias_cbrt3) {
  static const float m[9] = {11.031567f, -9.866944f,  -0.16462299f, -3.2541474f, 4.4187705f,
                             -0.16462299f, -3.6588513f, 2.712923f,  1.9459282f};
  for (int i = 0; i < 9; ++i) matrix9[i] = m[i];
  for (int c = 0; c < 3; ++c) {
    bias3[c] = -0.0037930733f;
    bias_cbrt3[c] = host_cbrt_core(bias3[c]);
  }
}

}  // namespace jpxlg
