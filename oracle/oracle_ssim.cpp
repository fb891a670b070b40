// oracle_ssim.cpp — CPU restatement of jpxl-perceptual's SSIMULACRA2:
// 2x2 pyramid, positive XYB, the recursive Gaussian with f64 state, the SSIM
// and edge maps with f64 pooled sums in raster order, the 108 weights and the
// final remap.
//
// TEST INFRASTRUCTURE ONLY (the checker, never the product).
#include <algorithm>
#include <cmath>

#include "oracle.h"
#include "oracle_internal.h"

namespace orc {

// blur.rs:41 / :47 — Charalampidis truncated-cosine constants for sigma 1.5.
static const double kMulIn[3] = {0.05529523572608661, -0.05883668702694998,
                                 0.012955819110517063};
static const double kMulPrev[3] = {1.902113032590307, 1.1755705045849463,
                                   1.2246467991473532e-16};
static const int kRadius = 5;

// blur.rs:164 step.
struct Rec {
  double prev[3] = {0, 0, 0}, prev2[3] = {0, 0, 0};
  float step(float sum) {
    double s = (double)sum;
    double o[3];
    for (int k = 0; k < 3; ++k) o[k] = s * kMulIn[k] + kMulPrev[k] * prev[k] - prev2[k];
    for (int k = 0; k < 3; ++k) { prev2[k] = prev[k]; prev[k] = o[k]; }
    return (float)((o[0] + o[1]) + o[2]);
  }
};

// blur.rs:414 horizontal_padded over one row of `padded` (2N zeros, the row,
// N zeros) and blur.rs:574 vertical pass with zero rows outside the plane.
static void blur(const float* a, const float* b, int w, int h, float* out) {
  std::vector<float> temp((size_t)w * h), padded(w + 3 * kRadius);
  for (int y = 0; y < h; ++y) {
    std::fill(padded.begin(), padded.end(), 0.0f);
    for (int x = 0; x < w; ++x) {
      size_t i = (size_t)y * w + x;
      padded[2 * kRadius + x] = b ? a[i] * b[i] : a[i];
    }
    Rec r;
    const int warm = kRadius - 1;
    for (int i = 0; i < warm; ++i) r.step(padded[i] + padded[i + 2 * kRadius]);
    for (int x = 0; x < w; ++x) {
      int i = x + warm;
      temp[(size_t)y * w + x] = r.step(padded[i] + padded[i + 2 * kRadius]);
    }
  }
  for (int x = 0; x < w; ++x) {
    Rec r;
    auto row = [&](int i) -> float { return (i < 0 || i >= h) ? 0.0f : temp[(size_t)i * w + x]; };
    for (int n = 1 - kRadius; n < h; ++n) {
      float v = r.step(row(n - kRadius - 1) + row(n + kRadius - 1));
      if (n >= 0) out[(size_t)n * w + x] = v;
    }
  }
}

// pyramid.rs:19 downscale_by_2.
static void downscale(const float* in, int w, int h, float* out) {
  int ow = (w + 1) / 2, oh = (h + 1) / 2;
  for (int oy = 0; oy < oh; ++oy) {
    int y0 = std::min(2 * oy, h - 1), y1 = std::min(2 * oy + 1, h - 1);
    for (int ox = 0; ox < ow; ++ox) {
      int x0 = std::min(2 * ox, w - 1), x1 = std::min(2 * ox + 1, w - 1);
      float a = in[(size_t)y0 * w + x0], b = in[(size_t)y0 * w + x1];
      float c = in[(size_t)y1 * w + x0], d = in[(size_t)y1 * w + x1];
      out[(size_t)oy * ow + ox] = (a + b + c + d) * 0.25f;
    }
  }
}

// ssimulacra2.rs:391 WEIGHTS.
static const double kWeights[108] = {
    0.0, 0.0007376606707406586, 0.0, 0.0, 0.0007793481682867309, 0.0, 0.0,
    0.0004371155730107379, 0.0, 1.1041726426657346, 0.00066284834129271, 0.00015231632783718752,
    0.0, 0.0016406437456599754, 0.0, 1.8422455520539298, 11.441172603757666, 0.0,
    0.0007989109436015163, 0.000176816438078653, 0.0, 1.8787594979546387, 10.94906990605142, 0.0,
    0.0007289346991508072, 0.9677937080626833, 0.0, 0.00014003424285435884, 0.9981766977854967,
    0.00031949755934435053, 0.0004550992113792063, 0.0, 0.0, 0.0013648766163243398, 0.0, 0.0,
    0.0, 0.0, 0.0, 7.466890328078848, 0.0, 17.445833984131262, 0.0006235601634041466, 0.0, 0.0,
    6.683678146179332, 0.00037724407979611296, 1.027889937768264, 225.20515300849274, 0.0, 0.0,
    19.213238186143016, 0.0011401524586618361, 0.001237755635509985, 176.39317598450694, 0.0,
    0.0, 24.43300999870476, 0.28520802612117757, 0.0004485436923833408, 0.0, 0.0, 0.0,
    34.77906344483772, 44.835625328877896, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0,
    0.0008680556573291698, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0005313191874358747, 0.0,
    0.00016533814161379112, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0004179171803251336,
    0.0017290828234722833, 0.0, 0.0020827005846636437, 0.0, 0.0, 8.826982764996862,
    23.19243343998926, 0.0, 95.1080498811086, 0.9863978034400682, 0.9834382792465353,
    0.0012286405048278493, 171.2667255897307, 0.9807858872435379, 0.0, 0.0, 0.0,
    0.0005130064588990679, 0.0, 0.00010854057858411537};

// ssimulacra2.rs:531 remap.
static double remap(double error) {
  double s = error * 0.9562382616834844;
  s = 6.248496625763138e-5 * s * s * s + 2.326765642916932 * s - 0.020884521182843837 * s * s;
  if (s > 0.0) return 100.0 - 10.0 * std::pow(s, 0.6276336467831387);
  return 100.0;
}

}  // namespace orc

using namespace orc;

// perceptual lib.rs:195 score_pair = PrecomputedReference::new (Moments) +
// Ssimulacra2::score; pool.rs:248 accumulate_scalar per pixel in raster
// order; pool.rs:60 ChannelTerms::from_sums; ssimulacra2.rs:509 weighted_error.
extern "C" int orc_ssim2(const float* const* ref, const float* const* cand, int w, int h,
                         double* score, double* raw_error, double* terms_out) {
  if (w < 8 || h < 8) return kErrShape;
  std::vector<float> r[3], c[3];
  for (int k = 0; k < 3; ++k) {
    r[k].assign(ref[k], ref[k] + (size_t)w * h);
    c[k].assign(cand[k], cand[k] + (size_t)w * h);
  }
  double terms[6][3][6];
  int scales = 0;
  int cw = w, ch = h;
  for (int s = 0; s < 6; ++s) {
    if (s > 0) {
      if (cw < 8 || ch < 8) break;
      int nw = (cw + 1) / 2, nh = (ch + 1) / 2;
      for (int k = 0; k < 3; ++k) {
        std::vector<float> t((size_t)nw * nh), u((size_t)nw * nh);
        downscale(r[k].data(), cw, ch, t.data());
        downscale(c[k].data(), cw, ch, u.data());
        r[k].swap(t);
        c[k].swap(u);
      }
      cw = nw;
      ch = nh;
    }
    size_t n = (size_t)cw * ch;
    std::vector<float> rx[3], cx[3];
    for (int k = 0; k < 3; ++k) { rx[k].resize(n); cx[k].resize(n); }
    for (size_t i = 0; i < n; ++i) {
      float a[3] = {r[0][i], r[1][i], r[2][i]}, o[3];
      linear_to_positive_xyb(a, o);
      for (int k = 0; k < 3; ++k) rx[k][i] = o[k];
      float b[3] = {c[0][i], c[1][i], c[2][i]};
      linear_to_positive_xyb(b, o);
      for (int k = 0; k < 3; ++k) cx[k][i] = o[k];
    }
    for (int k = 0; k < 3; ++k) {
      std::vector<float> mu1(n), s11(n), mu2(n), s22(n), s12(n);
      blur(rx[k].data(), nullptr, cw, ch, mu1.data());
      blur(rx[k].data(), rx[k].data(), cw, ch, s11.data());
      blur(cx[k].data(), nullptr, cw, ch, mu2.data());
      blur(cx[k].data(), cx[k].data(), cw, ch, s22.data());
      blur(rx[k].data(), cx[k].data(), cw, ch, s12.data());
      double sums[6] = {0, 0, 0, 0, 0, 0};  // ssim0, ssim1, art0, art1, lost0, lost1
      const float C2 = 0.0009f;
      for (size_t i = 0; i < n; ++i) {
        float m1 = mu1[i], m2 = mu2[i];
        float mu11 = m1 * m1, mu22 = m2 * m2, mu12 = m1 * m2;
        float md = m1 - m2;
        float num_m = 1.0f - md * md;
        float num_s = 2.0f * (s12[i] - mu12) + C2;
        float den_s = (s11[i] - mu11) + (s22[i] - mu22) + C2;
        // Rust's f64::max returns the other operand of a NaN: fmax
        double d = std::fmax(1.0 - (double)((num_m * num_s) / den_s), 0.0);
        sums[0] += d;
        sums[1] += d * d * d * d;
        double d1 = (1.0 + (double)std::fabs(cx[k][i] - m2)) /
                        (1.0 + (double)std::fabs(rx[k][i] - m1)) - 1.0;
        double art = std::fmax(d1, 0.0);
        sums[2] += art;
        sums[3] += art * art * art * art;
        double lost = std::fmax(-d1, 0.0);
        sums[4] += lost;
        sums[5] += lost * lost * lost * lost;
      }
      double inv = 1.0 / (double)std::max<size_t>(n, 1);
      // norms: [inv*s0, sqrt(sqrt(inv*s1))] for ssim, artifact, detail-lost.
      terms[s][k][0] = inv * sums[0];
      terms[s][k][1] = inv * sums[2];
      terms[s][k][2] = inv * sums[4];
      terms[s][k][3] = std::sqrt(std::sqrt(inv * sums[1]));
      terms[s][k][4] = std::sqrt(std::sqrt(inv * sums[3]));
      terms[s][k][5] = std::sqrt(std::sqrt(inv * sums[5]));
    }
    ++scales;
  }
  // weighted_error: for c, for scale, for n in 0..2: ssim[n], artifact[n], lost[n].
  double err = 0.0;
  int wi = 0;
  for (int k = 0; k < 3; ++k)
    for (int s = 0; s < scales; ++s)
      for (int nn = 0; nn < 2; ++nn)
        for (int m = 0; m < 3; ++m) {
          double v = terms[s][k][nn * 3 + m];
          double weight = wi < 108 ? kWeights[wi] : 0.0;
          ++wi;
          err += weight * std::fabs(v);
        }
  if (raw_error) *raw_error = err;
  if (score) *score = remap(err);
  if (terms_out)
    for (int s = 0; s < scales; ++s)
      for (int k = 0; k < 3; ++k)
        for (int m = 0; m < 6; ++m) terms_out[(s * 3 + k) * 6 + m] = terms[s][k][m];
  return scales;
}

extern "C" double orc_ssim2_weight(int i) { return (i >= 0 && i < 108) ? kWeights[i] : 0.0; }
extern "C" void orc_blur_plane(const float* in, int w, int h, float* out) {
  blur(in, nullptr, w, h, out);
}

// tests/common/mod.rs:15 Lcg (xorshift32) and :66 synthetic, :112 add_noise
// of the reference's perceptual tests.
namespace {
struct Xs {
  uint32_t s;
  explicit Xs(uint32_t seed) : s(seed < 1 ? 1 : seed) {}
  float next() {
    uint32_t x = s;
    x ^= x << 13;
    x ^= x >> 17;
    x ^= x << 5;
    s = x;
    return (float)(x >> 8) / (float)(1u << 24);
  }
};
float test_srgb_to_linear(float v) {
  if (v <= 12.92f * 0.0031308f) return v / 12.92f;
  return powf((v + 0.055f) / 1.055f, 2.4f);
}
float clamp01(float v) { return std::min(std::max(v, 0.0f), 1.0f); }
}  // namespace

extern "C" void orc_perceptual_synthetic(int w, int h, uint32_t seed, float* r, float* g,
                                         float* b) {
  Xs rng(seed);
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      float fx = (float)x / (float)w, fy = (float)y / (float)h;
      float pr = 0.2f + 0.6f * fx;
      float pg = 0.25f + 0.5f * fy;
      float pb = 0.3f + 0.4f * (1.0f - fx) * fy;
      if (fy >= 0.3f && fy < 0.6f) {
        float t = (float)((x * 7 + y * 3) % 11) / 11.0f - 0.5f;
        pr += 0.15f * t;
        pg += 0.1f * t;
        pb -= 0.1f * t;
      }
      if (fx > 0.7f) { pr *= 0.5f; pg *= 0.5f; pb *= 0.5f; }
      if (fx >= 0.1f && fx < 0.2f && fy >= 0.7f && fy < 0.8f) { pr = 0.95f; pg = 0.95f; pb = 0.9f; }
      float nz = (rng.next() - 0.5f) * 0.02f;
      size_t i = (size_t)y * w + x;
      r[i] = clamp01(test_srgb_to_linear(pr + nz));
      g[i] = clamp01(test_srgb_to_linear(pg + nz));
      b[i] = clamp01(test_srgb_to_linear(pb + nz));
    }
}

extern "C" void orc_perceptual_add_noise(float* r, float* g, float* b, int n, float amp,
                                         uint32_t seed) {
  Xs rng(seed);
  float* planes[3] = {r, g, b};
  for (float* p : planes)
    for (int i = 0; i < n; ++i) p[i] = clamp01(p[i] + (rng.next() - 0.5f) * 2.0f * amp);
}
