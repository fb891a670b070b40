// oracle_fp64.cpp — the FP64 truth of the lossy VarDCT pixel path and of
// SSIMULACRA2: the same algorithm as the f32 restatement (oracle_core.cpp,
// oracle_pipeline.cpp, oracle_ssim.cpp), stage for stage, with every
// arithmetic operation in f64 and every transform as an exact cosine sum.
//
// TEST INFRASTRUCTURE ONLY (the yardstick results are measured against; the
// product never loads it).
//
// Definition of "truth" used throughout: every table and constant takes the
// value the f32 path holds (an f32 literal or an f32 table entry, promoted
// exactly to f64: the dequantization matrices of dequant.rs:321, the opsin
// matrices of color.rs:54-81 and plan-render lib.rs:55-68, the quant biases of
// color.rs:591, the Gabor weights, the EPF constants of restoration.rs:201-256,
// SSIMULACRA2's C2 and weights), while the arithmetic is carried out in f64:
// the DCTs are dense sums with cosines evaluated in f64 (not the butterflies
// of dct.rs:235-465 with their f32 leaves), the cube roots are std::cbrt, the
// transfer curves std::pow, the recursive Gaussian runs on f64 inputs with its
// pair sums unrounded and its output unrounded (blur.rs:164/:414/:574), the
// encoder's inverse Gaborish is the uniform Jacobi update (gaborish.rs:218
// without its position-dependent f32 forms).  The distance of an f32 result
// from this oracle is therefore that result's arithmetic rounding error.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "oracle.h"
#include "oracle_internal.h"

namespace orc {
namespace {

// ---------------------------------------------------------------------------
// Normative 1-D transforms of jpxl-core dct.rs:731 (DCT: orthonormal DCT-II
// times 1/sqrt(n)) and :749 (IDCT: orthonormal DCT-III times sqrt(n)) as
// dense f64 matrices:
//   forward  D_n[u][i] = (u == 0 ? 1 : sqrt 2) cos(pi (2i+1) u / 2n) / n
//   inverse  I_n[i][u] = (u == 0 ? 1 : sqrt 2) cos(pi (2i+1) u / 2n)
// ---------------------------------------------------------------------------

struct Basis {
  double fwd[64 * 64];  // fwd[u * n + i]
  double inv[64 * 64];  // inv[i * n + u]
};

const Basis& basis(int n) {
  static Basis tables[7];
  static std::once_flag once;
  std::call_once(once, [] {
    for (int k = 0; k <= 6; ++k) {
      const int m = 1 << k;
      for (int u = 0; u < m; ++u)
        for (int i = 0; i < m; ++i) {
          const double cu = u == 0 ? 1.0 : std::sqrt(2.0);
          const double c = cu * std::cos(M_PI * (2.0 * i + 1.0) * u / (2.0 * m));
          tables[k].fwd[u * m + i] = c / m;
          tables[k].inv[i * m + u] = c;
        }
    }
  });
  int k = 0;
  while ((1 << k) < n) ++k;
  return tables[k];
}

// DCT_2D (dct.rs:956) of a rows x cols sample matrix into the landscape
// layout of the f32 path: rows x cols when cols > rows, else cols x rows with
// the horizontal frequency first.
void dct2d(const double* in, int rows, int cols, double* out) {
  const Basis& br = basis(rows);
  const Basis& bc = basis(cols);
  std::vector<double> tmp((size_t)rows * cols);
  for (int u = 0; u < rows; ++u)
    for (int x = 0; x < cols; ++x) {
      double acc = 0.0;
      for (int y = 0; y < rows; ++y) acc += br.fwd[u * rows + y] * in[y * cols + x];
      tmp[u * cols + x] = acc;
    }
  for (int u = 0; u < rows; ++u)
    for (int v = 0; v < cols; ++v) {
      double acc = 0.0;
      for (int x = 0; x < cols; ++x) acc += bc.fwd[v * cols + x] * tmp[u * cols + x];
      if (cols > rows) out[u * cols + v] = acc;
      else out[v * rows + u] = acc;
    }
}

// IDCT_2D (dct.rs:982): landscape coefficients (layout as dct2d's output)
// into rows x cols samples.
void idct2d(const double* coef, int rows, int cols, double* out) {
  const Basis& br = basis(rows);
  const Basis& bc = basis(cols);
  std::vector<double> tmp((size_t)rows * cols);
  auto F = [&](int u, int v) { return cols > rows ? coef[u * cols + v] : coef[v * rows + u]; };
  for (int u = 0; u < rows; ++u)
    for (int x = 0; x < cols; ++x) {
      double acc = 0.0;
      for (int v = 0; v < cols; ++v) acc += bc.inv[x * cols + v] * F(u, v);
      tmp[u * cols + x] = acc;
    }
  for (int y = 0; y < rows; ++y)
    for (int x = 0; x < cols; ++x) {
      double acc = 0.0;
      for (int u = 0; u < rows; ++u) acc += br.inv[y * rows + u] * tmp[u * cols + x];
      out[y * cols + x] = acc;
    }
}

// varblock.rs:789 scale_f closed form, not narrowed to f32.
double scale_f64(int c, int lf_count) {
  const int b = lf_count * 8;
  if (b == 0) return 1.0;
  const double cf = c, bf = b;
  return 1.0 / (std::cos(cf * M_PI / (2.0 * bf)) * std::cos(cf * M_PI / bf) *
                std::cos(2.0 * cf * M_PI / bf));
}

// ---------------------------------------------------------------------------
// Colour (jpxl-core color.rs, jpxl-perceptual color.rs) with the f32 path's
// constants.
// ---------------------------------------------------------------------------

const double kMix[3][3] = {{(double)0.3f, (double)0.622f, (double)0.078f},
                           {(double)0.23f, (double)0.692f, (double)0.078f},
                           {(double)0.2434227f, (double)0.2047674f, (double)0.5518099f}};
const double kBias = (double)0.0037930734f;       // color.rs:54
const double kBiasCbrt = (double)0.1559542f;      // color.rs:81
const double kInvM[9] = {(double)11.031567f,  (double)-9.866944f, (double)-0.16462299f,
                         (double)-3.2541474f, (double)4.4187705f, (double)-0.16462299f,
                         (double)-3.6588513f, (double)2.712923f,  (double)1.9459282f};
const double kSignalledBias = (double)-0.0037930733f;  // plan-render lib.rs:55

double srgb_to_linear64(double v) {
  const double a = std::fabs(v);
  const double d = a <= (double)12.92f * (double)0.0031308f
                       ? a / (double)12.92f
                       : std::pow((a + (double)0.055f) / (double)1.055f, (double)2.4f);
  return v < 0.0 ? -d : d;
}

void linear_to_xyb64(const double rgb[3], double out[3], bool positive) {
  double g[3];
  for (int k = 0; k < 3; ++k) {
    const double m = kMix[k][0] * rgb[0] + kMix[k][1] * rgb[1] + kMix[k][2] * rgb[2] + kBias;
    g[k] = std::cbrt(m) - kBiasCbrt;
  }
  const double x = 0.5 * (g[0] - g[1]), y = 0.5 * (g[0] + g[1]);
  if (!positive) {
    out[0] = x;
    out[1] = y;
    out[2] = g[2];
  } else {  // perceptual color.rs:66
    out[0] = x * 14.0 + (double)0.42f;
    out[1] = y + (double)0.01f;
    out[2] = (g[2] - y) + (double)0.55f;
  }
}

// color.rs:673 OpsinInverse::convert.
void opsin_inverse64(const double xyb[3], double out[3]) {
  const double root = std::cbrt(kSignalledBias);
  const double gamma[3] = {xyb[1] + xyb[0], xyb[1] - xyb[0], xyb[2]};
  double mix[3];
  for (int c = 0; c < 3; ++c) {
    const double v = gamma[c] - root;
    mix[c] = v * v * v + kSignalledBias;
  }
  for (int r = 0; r < 3; ++r)
    out[r] = kInvM[r * 3] * mix[0] + kInvM[r * 3 + 1] * mix[1] + kInvM[r * 3 + 2] * mix[2];
}

// ---------------------------------------------------------------------------
// Filters
// ---------------------------------------------------------------------------

std::vector<double> pad_mirror64(const double* in, int w, int h, int r) {
  const int pw = w + 2 * r, ph = h + 2 * r;
  std::vector<double> out((size_t)pw * ph);
  for (int y = 0; y < ph; ++y) {
    const double* row = in + (size_t)mirror1d(y - r, h) * w;
    for (int x = 0; x < pw; ++x) out[(size_t)y * pw + x] = row[mirror1d(x - r, w)];
  }
  return out;
}

// restoration.rs:148 J.3 with the Table J.1 weights (the decoder's kernel;
// the encoder's gaborish.rs:31 kernel has the same exact value).
void gaborish64(const double* in, int w, int h, double* out) {
  const double w1 = (double)0.115169525f, w2 = (double)0.061248592f;
  const double un = 1.0 + 4.0 * w1 + 4.0 * w2;
  const double centre = 1.0 / un, edge = w1 / un, corner = w2 / un;
  const std::vector<double> pad = pad_mirror64(in, w, h, 1);
  const int pw = w + 2;
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const double* p = &pad[(size_t)(y + 1) * pw + x + 1];
      out[(size_t)y * w + x] = centre * p[0] + edge * (p[-1] + p[1] + p[-pw] + p[pw]) +
                               corner * (p[-pw - 1] + p[-pw + 1] + p[pw - 1] + p[pw + 1]);
    }
}

// encode gaborish.rs:218 precondition_xyb_planes: 12 Jacobi steps
// x <- x + (f - Kx) / centre.
void precondition64(const double* f, int w, int h, double* x) {
  const double w1 = (double)0.115169525f, w2 = (double)0.061248592f;
  const double centre = 1.0 / (1.0 + 4.0 * w1 + 4.0 * w2);
  const size_t n = (size_t)w * h;
  std::vector<double> kx(n);
  std::memcpy(x, f, sizeof(double) * n);
  for (int it = 0; it < 12; ++it) {
    gaborish64(x, w, h, kx.data());
    for (size_t i = 0; i < n; ++i) x[i] = x[i] + (f[i] - kx[i]) / centre;
  }
}

// restoration.rs:619 epf_step_rows_impl, one step over the three planes.
void epf_step64(int step, const double* const* in, int w, int h, const double* sigma,
                double* const* out) {
  static const int kCross[5][2] = {{0, 0}, {-1, 0}, {1, 0}, {0, -1}, {0, 1}};
  static const int kStep0[13][2] = {{0, 0},  {-1, 0}, {1, 0},  {0, -1}, {0, 1},
                                    {1, -1}, {1, 1},  {-1, 1}, {-1, -1}, {-2, 0},
                                    {2, 0},  {0, 2},  {0, -2}};
  const int(*taps)[2] = step == 0 ? kStep0 : kCross;
  const int ntaps = step == 0 ? 13 : 5, ncross = step == 2 ? 1 : 5;
  const double scale[3] = {(double)40.0f, (double)5.0f, (double)3.5f};
  const double step_scale = step == 0 ? (double)0.9f : (step == 1 ? 1.0 : (double)6.5f);
  const int bw = (w + 7) / 8;
  const std::vector<double> pad[3] = {pad_mirror64(in[0], w, h, 3), pad_mirror64(in[1], w, h, 3),
                                      pad_mirror64(in[2], w, h, 3)};
  const int pw = w + 6;
  auto at = [&](int c, int x, int y) { return pad[c][(size_t)(y + 3) * pw + (x + 3)]; };
  for (int y = 0; y < h; ++y) {
    const bool border_row = y % 8 == 0 || y % 8 == 7;
    for (int x = 0; x < w; ++x) {
      const size_t idx = (size_t)y * w + x;
      const double bs = sigma[(size_t)(y / 8) * bw + x / 8];
      if (bs < (double)0.3f) {
        for (int c = 0; c < 3; ++c) out[c][idx] = in[c][idx];
        continue;
      }
      const double inv_sigma =
          (double)1.65f * step_scale * 4.0 * (1.0 - std::sqrt(0.5)) / bs;
      const bool at_border = border_row || x % 8 == 0 || x % 8 == 7;
      double sum_w = 0.0, acc[3] = {0.0, 0.0, 0.0};
      for (int t = 0; t < ntaps; ++t) {
        const int kx = taps[t][0], ky = taps[t][1];
        double d = 0.0;
        for (int c = 0; c < 3; ++c)
          for (int i = 0; i < ncross; ++i) {
            const int ix = kCross[i][0], iy = kCross[i][1];
            d += std::fabs(at(c, x + ix, y + iy) - at(c, x + kx + ix, y + ky + iy)) * scale[c];
          }
        const double sd = (at_border ? (double)(2.0f / 3.0f) : 1.0) * d;
        const double weight = sd == 0.0 ? 1.0 : std::max(1.0 - sd * inv_sigma, 0.0);
        sum_w += weight;
        for (int c = 0; c < 3; ++c) acc[c] += at(c, x + kx, y + ky) * weight;
      }
      for (int c = 0; c < 3; ++c) out[c][idx] = acc[c] / sum_w;
    }
  }
}

// ---------------------------------------------------------------------------
// SSIMULACRA2 (jpxl-perceptual) in f64.
// ---------------------------------------------------------------------------

const double kMulIn[3] = {0.05529523572608661, -0.05883668702694998, 0.012955819110517063};
const double kMulPrev[3] = {1.902113032590307, 1.1755705045849463, 1.2246467991473532e-16};
constexpr int kRadius = 5;

// blur.rs:164/:414/:574 with f64 inputs, unrounded pair sums and outputs.
void blur64(const double* a, const double* b, int w, int h, double* out) {
  struct Rec {
    double prev[3] = {0, 0, 0}, prev2[3] = {0, 0, 0};
    double step(double s) {
      double o[3];
      for (int k = 0; k < 3; ++k) o[k] = s * kMulIn[k] + kMulPrev[k] * prev[k] - prev2[k];
      for (int k = 0; k < 3; ++k) {
        prev2[k] = prev[k];
        prev[k] = o[k];
      }
      return (o[0] + o[1]) + o[2];
    }
  };
  std::vector<double> temp((size_t)w * h), padded(w + 3 * kRadius);
  for (int y = 0; y < h; ++y) {
    std::fill(padded.begin(), padded.end(), 0.0);
    for (int x = 0; x < w; ++x) {
      const size_t i = (size_t)y * w + x;
      padded[2 * kRadius + x] = b ? a[i] * b[i] : a[i];
    }
    Rec r;
    const int warm = kRadius - 1;
    for (int i = 0; i < warm; ++i) r.step(padded[i] + padded[i + 2 * kRadius]);
    for (int x = 0; x < w; ++x) {
      const int i = x + warm;
      temp[(size_t)y * w + x] = r.step(padded[i] + padded[i + 2 * kRadius]);
    }
  }
  for (int x = 0; x < w; ++x) {
    Rec r;
    auto row = [&](int i) { return (i < 0 || i >= h) ? 0.0 : temp[(size_t)i * w + x]; };
    for (int n = 1 - kRadius; n < h; ++n) {
      const double v = r.step(row(n - kRadius - 1) + row(n + kRadius - 1));
      if (n >= 0) out[(size_t)n * w + x] = v;
    }
  }
}

void downscale64(const double* in, int w, int h, double* out) {
  const int ow = (w + 1) / 2, oh = (h + 1) / 2;
  for (int oy = 0; oy < oh; ++oy) {
    const int y0 = std::min(2 * oy, h - 1), y1 = std::min(2 * oy + 1, h - 1);
    for (int ox = 0; ox < ow; ++ox) {
      const int x0 = std::min(2 * ox, w - 1), x1 = std::min(2 * ox + 1, w - 1);
      out[(size_t)oy * ow + ox] = (in[(size_t)y0 * w + x0] + in[(size_t)y0 * w + x1] +
                                   in[(size_t)y1 * w + x0] + in[(size_t)y1 * w + x1]) * 0.25;
    }
  }
}

double remap64(double error) {
  double s = error * 0.9562382616834844;
  s = 6.248496625763138e-5 * s * s * s + 2.326765642916932 * s - 0.020884521182843837 * s * s;
  return s > 0.0 ? 100.0 - 10.0 * std::pow(s, 0.6276336467831387) : 100.0;
}

}  // namespace
}  // namespace orc

using namespace orc;

// ---------------------------------------------------------------------------
// C ABI (oracle.h)
// ---------------------------------------------------------------------------

extern "C" void orc64_dct_2d(const double* in, int rows, int cols, double* out) {
  dct2d(in, rows, cols, out);
}
extern "C" void orc64_idct_2d(const double* coef, int rows, int cols, double* out) {
  idct2d(coef, rows, cols, out);
}

// The encoder's transform in f64: source.rs:226/:355 (sRGB -> linear ->
// XYB), gaborish.rs:218 (12 Jacobi steps when `gaborish`), forward.rs:451
// per varblock with the edge replication of policy lib.rs:3008, into the
// coefficient image of the f32 path (oracle.h layout).
extern "C" int orc64_encode_transform(const void* rgb, int w, int h, int bits,
                                      const uint8_t* block_map, int gaborish, double* xyb_out,
                                      double* pre_out, double* coeff_out) {
  if (w <= 0 || h <= 0 || !(bits >= 1 && bits <= 16)) return kErrShape;
  const int bw = (w + 7) / 8, bh = (h + 7) / 8, W8 = bw * 8, H8 = bh * 8;
  std::vector<Varblock> vbs;
  int rc = parse_block_map(block_map, bw, bh, &vbs);
  if (rc) return rc;
  const size_t n = (size_t)w * h;
  std::vector<double> xyb(3 * n);
  const double max = bits == 8 ? 255.0 : std::min(65535.0, (double)((1u << bits) - 1));
  for (size_t i = 0; i < n; ++i) {
    double lin[3], o[3];
    for (int c = 0; c < 3; ++c) {
      const uint32_t v = bits == 8 ? ((const uint8_t*)rgb)[3 * i + c]
                                   : ((const uint16_t*)rgb)[3 * i + c];
      lin[c] = srgb_to_linear64((double)v / max);
    }
    linear_to_xyb64(lin, o, false);
    for (int c = 0; c < 3; ++c) xyb[c * n + i] = o[c];
  }
  if (xyb_out) std::memcpy(xyb_out, xyb.data(), sizeof(double) * 3 * n);
  std::vector<double> pre = xyb;
  if (gaborish)
    for (int c = 0; c < 3; ++c) precondition64(&xyb[c * n], w, h, &pre[c * n]);
  if (pre_out) std::memcpy(pre_out, pre.data(), sizeof(double) * 3 * n);
  if (coeff_out) {
    const size_t plane8 = (size_t)W8 * H8;
    std::fill(coeff_out, coeff_out + 3 * plane8, 0.0);
    std::vector<double> blk(4096), co(4096);
    for (const Varblock& vb : vbs) {
      const int rows = vb.t.brows * 8, cols = vb.t.bcols * 8;
      for (int c = 0; c < 3; ++c) {
        for (int dy = 0; dy < rows; ++dy)
          for (int dx = 0; dx < cols; ++dx) {
            const int xx = std::min(vb.bx * 8 + dx, w - 1), yy = std::min(vb.by * 8 + dy, h - 1);
            blk[dy * cols + dx] = pre[c * n + (size_t)yy * w + xx];
          }
        dct2d(blk.data(), rows, cols, co.data());
        for (int y = 0; y < vb.t.crows; ++y)
          for (int x = 0; x < vb.t.ccols; ++x)
            coeff_out[c * plane8 + coeff_index(vb, y, x, W8)] = co[y * vb.t.ccols + x];
      }
    }
  }
  return kOk;
}

// plan-render lib.rs:749 render_inner in f64.  out_kind: 0 = XYB after
// restoration, 1 = linear sRGB, 4 = XYB before restoration (3 planes each).
extern "C" int orc64_reconstruct(int w, int h, const uint8_t* block_map,
                                 const uint32_t* hf_mul_blocks, const uint8_t* sharpness,
                                 const int32_t* qcoeff, const int32_t* lf, const int8_t* cfl_x,
                                 const int8_t* cfl_b, const orc_render_params* p, int out_kind,
                                 double* out) {
  if (w <= 0 || h <= 0 || p->epf_iters > 3) return kErrShape;
  if (out_kind != 0 && out_kind != 1 && out_kind != 4) return kErrParam;
  const int bw = (w + 7) / 8, bh = (h + 7) / 8, W8 = bw * 8;
  const int tw = (bw + 7) / 8;
  std::vector<Varblock> vbs;
  int rc = parse_block_map(block_map, bw, bh, &vbs);
  if (rc) return rc;
  const size_t n = (size_t)w * h, nb = (size_t)bw * bh, plane8 = (size_t)W8 * bh * 8;
  auto powi = [](double a, int b) {  // reconstruct.rs:37, 0.8^(qm_scale - 2)
    double r = 1.0;
    for (int i = 0; i < std::abs(b); ++i) r *= a;
    return b < 0 ? 1.0 / r : r;
  };
  const double qm[3] = {powi((double)0.8f, (int)p->x_qm_scale - 2), 1.0,
                        powi((double)0.8f, (int)p->b_qm_scale - 2)};
  double lf_mul[3];
  const double wts[3] = {1.0 / 32.0, 1.0 / 4.0, 1.0 / 2.0};
  const double denom = (double)p->global_scale * (double)p->quant_lf;
  for (int c = 0; c < 3; ++c) lf_mul[c] = denom > 0.0 ? 65536.0 * (wts[c] / 128.0) / denom : 0.0;
  const double k_x_lf = (double)(p->x_factor_lf - 128) / 84.0;
  const double k_b_lf = 1.0 + (double)(p->b_factor_lf - 128) / 84.0;
  std::vector<double> lfd(3 * nb);
  for (size_t i = 0; i < nb; ++i) {
    double d[3];
    for (int c = 0; c < 3; ++c) d[c] = lf_mul[c] * (double)lf[c * nb + i];
    lfd[i] = d[0] + k_x_lf * d[1];
    lfd[nb + i] = d[1];
    lfd[2 * nb + i] = d[2] + k_b_lf * d[1];
  }
  std::vector<double> planes(3 * n, 0.0), sigma(nb, 0.0);
  std::vector<double> co[3], samp(4096), rect(64), rect_c(64);
  for (auto& v : co) v.resize(4096);
  for (const Varblock& vb : vbs) {
    const int rows = vb.t.crows, cols = vb.t.ccols;
    const uint32_t hf = hf_mul_blocks[(size_t)vb.by * bw + vb.bx];
    const double mul = (double)p->global_scale * hf > 0.0 ? 65536.0 / ((double)p->global_scale * hf)
                                                          : 0.0;
    for (int c = 0; c < 3; ++c) {
      const float* m = dequant_matrix_cached(vb.t.dq_index, c);
      const double bias = (double)kQuantBias[c], num = (double)kQuantBiasNumerator;
      for (int y = 0; y < rows; ++y)
        for (int x = 0; x < cols; ++x) {
          const int32_t q = qcoeff[c * plane8 + coeff_index(vb, y, x, W8)];
          const double adj = std::abs(q) <= 1 ? (double)q * bias : (double)q - num / (double)q;
          co[c][y * cols + x] = adj * mul * qm[c] * (double)m[y * cols + x];
        }
    }
    const size_t tile = (size_t)(vb.by / 8) * tw + (vb.bx / 8);
    const double k_x = (double)cfl_x[tile] / 84.0, k_b = 1.0 + (double)cfl_b[tile] / 84.0;
    for (int i = 0; i < rows * cols; ++i) {
      co[0][i] += k_x * co[1][i];
      co[2][i] += k_b * co[1][i];
    }
    const int br = vb.t.brows, bc = vb.t.bcols;
    const int cx = std::max(br, bc), cy = std::min(br, bc);
    for (int c = 0; c < 3; ++c) {
      for (int dy = 0; dy < br; ++dy)
        for (int dx = 0; dx < bc; ++dx) {
          const double v = lfd[c * nb + (size_t)(vb.by + dy) * bw + vb.bx + dx];
          if (br > bc) rect[dx * br + dy] = v;
          else rect[dy * bc + dx] = v;
        }
      dct2d(rect.data(), cy, cx, rect_c.data());
      for (int y = 0; y < cy; ++y)
        for (int x = 0; x < cx; ++x)
          co[c][y * cols + x] = rect_c[y * cx + x] * scale_f64(y, cy) * scale_f64(x, cx);
    }
    const int srows = br * 8, scols = bc * 8;
    for (int c = 0; c < 3; ++c) {
      idct2d(co[c].data(), srows, scols, samp.data());
      for (int y = 0; y < srows; ++y) {
        const int fy = vb.by * 8 + y;
        if (fy >= h) continue;
        for (int x = 0; x < scols; ++x) {
          const int fx = vb.bx * 8 + x;
          if (fx < w) planes[c * n + (size_t)fy * w + fx] = samp[y * scols + x];
        }
      }
    }
    for (int dy = 0; dy < br; ++dy)
      for (int dx = 0; dx < bc; ++dx) {
        const size_t bi = (size_t)(vb.by + dy) * bw + vb.bx + dx;
        const int s = std::min<int>(sharpness[bi], 7);
        sigma[bi] = mul * (double)0.46f * (s == 7 ? 1.0 : (double)((float)s / 7.0f));
      }
  }
  if (out_kind == 4) {
    std::memcpy(out, planes.data(), sizeof(double) * 3 * n);
    return kOk;
  }
  std::vector<double> aux(3 * n);
  if (p->gaborish) {
    for (int c = 0; c < 3; ++c) gaborish64(&planes[c * n], w, h, &aux[c * n]);
    planes.swap(aux);
  }
  static const int steps_for[4][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 2, -1}, {0, 1, 2}};
  for (int s = 0; s < 3; ++s) {
    const int step = steps_for[p->epf_iters][s];
    if (step < 0) break;
    const double* in[3] = {&planes[0], &planes[n], &planes[2 * n]};
    double* o[3] = {&aux[0], &aux[n], &aux[2 * n]};
    epf_step64(step, in, w, h, sigma.data(), o);
    planes.swap(aux);
  }
  if (out_kind == 0) {
    std::memcpy(out, planes.data(), sizeof(double) * 3 * n);
    return kOk;
  }
  for (size_t i = 0; i < n; ++i) {
    const double xyb[3] = {planes[i], planes[n + i], planes[2 * n + i]};
    double rgb[3];
    opsin_inverse64(xyb, rgb);
    for (int c = 0; c < 3; ++c) out[c * n + i] = rgb[c];
  }
  return kOk;
}

// SSIMULACRA2 (perceptual lib.rs:195 score_pair) in f64 on linear planes
// given as f32 (promoted) or f64 (`ref64`/`cand64`, either may be NULL).
extern "C" int orc64_ssim2(const float* const* ref, const float* const* cand,
                           const double* const* ref64, const double* const* cand64, int w, int h,
                           double* score, double* terms_out) {
  if (w < 8 || h < 8) return kErrShape;
  const size_t n0 = (size_t)w * h;
  std::vector<double> r[3], c[3];
  for (int k = 0; k < 3; ++k) {
    r[k].resize(n0);
    c[k].resize(n0);
    for (size_t i = 0; i < n0; ++i) {
      r[k][i] = ref64 ? ref64[k][i] : (double)ref[k][i];
      c[k][i] = cand64 ? cand64[k][i] : (double)cand[k][i];
    }
  }
  double terms[6][3][6];
  int scales = 0, cw = w, ch = h;
  for (int s = 0; s < 6; ++s) {
    if (s > 0) {
      if (cw < 8 || ch < 8) break;
      const int nw = (cw + 1) / 2, nh = (ch + 1) / 2;
      for (int k = 0; k < 3; ++k) {
        std::vector<double> t((size_t)nw * nh), u((size_t)nw * nh);
        downscale64(r[k].data(), cw, ch, t.data());
        downscale64(c[k].data(), cw, ch, u.data());
        r[k].swap(t);
        c[k].swap(u);
      }
      cw = nw;
      ch = nh;
    }
    const size_t n = (size_t)cw * ch;
    std::vector<double> rx[3], cx[3];
    for (int k = 0; k < 3; ++k) {
      rx[k].resize(n);
      cx[k].resize(n);
    }
    for (size_t i = 0; i < n; ++i) {
      double a[3] = {r[0][i], r[1][i], r[2][i]}, o[3];
      linear_to_xyb64(a, o, true);
      for (int k = 0; k < 3; ++k) rx[k][i] = o[k];
      double b[3] = {c[0][i], c[1][i], c[2][i]};
      linear_to_xyb64(b, o, true);
      for (int k = 0; k < 3; ++k) cx[k][i] = o[k];
    }
    for (int k = 0; k < 3; ++k) {
      std::vector<double> mu1(n), s11(n), mu2(n), s22(n), s12(n);
      blur64(rx[k].data(), nullptr, cw, ch, mu1.data());
      blur64(rx[k].data(), rx[k].data(), cw, ch, s11.data());
      blur64(cx[k].data(), nullptr, cw, ch, mu2.data());
      blur64(cx[k].data(), cx[k].data(), cw, ch, s22.data());
      blur64(rx[k].data(), cx[k].data(), cw, ch, s12.data());
      double sums[6] = {0, 0, 0, 0, 0, 0};
      const double C2 = (double)0.0009f;
      for (size_t i = 0; i < n; ++i) {
        const double m1 = mu1[i], m2 = mu2[i], md = m1 - m2;
        const double num_m = 1.0 - md * md;
        const double num_s = 2.0 * (s12[i] - m1 * m2) + C2;
        const double den_s = (s11[i] - m1 * m1) + (s22[i] - m2 * m2) + C2;
        const double d = std::fmax(1.0 - (num_m * num_s) / den_s, 0.0);
        sums[0] += d;
        sums[1] += d * d * d * d;
        const double d1 =
            (1.0 + std::fabs(cx[k][i] - m2)) / (1.0 + std::fabs(rx[k][i] - m1)) - 1.0;
        const double art = std::fmax(d1, 0.0), lost = std::fmax(-d1, 0.0);
        sums[2] += art;
        sums[3] += art * art * art * art;
        sums[4] += lost;
        sums[5] += lost * lost * lost * lost;
      }
      const double inv = 1.0 / (double)n;
      terms[s][k][0] = inv * sums[0];
      terms[s][k][1] = inv * sums[2];
      terms[s][k][2] = inv * sums[4];
      terms[s][k][3] = std::sqrt(std::sqrt(inv * sums[1]));
      terms[s][k][4] = std::sqrt(std::sqrt(inv * sums[3]));
      terms[s][k][5] = std::sqrt(std::sqrt(inv * sums[5]));
    }
    ++scales;
  }
  double err = 0.0;
  int wi = 0;
  for (int k = 0; k < 3; ++k)
    for (int s = 0; s < scales; ++s)
      for (int nn = 0; nn < 2; ++nn)
        for (int m = 0; m < 3; ++m) {
          err += orc_ssim2_weight(wi) * std::fabs(terms[s][k][nn * 3 + m]);
          ++wi;
        }
  if (score) *score = remap64(err);
  if (terms_out)
    for (int s = 0; s < scales; ++s)
      for (int k = 0; k < 3; ++k)
        for (int m = 0; m < 6; ++m) terms_out[(s * 3 + k) * 6 + m] = terms[s][k][m];
  return scales;
}
