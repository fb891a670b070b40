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

// Table I.6 params of the 8x8 special matrices (dequant.rs:714-1004).
const double kHornuss[3][3] = {{280.0, 3160.0, 3160.0}, {60.0, 864.0, 864.0},
                               {18.0, 200.0, 200.0}};
const double kDct4x4[3][4] = {{2200.0, 0.0, 0.0, 0.0}, {392.0, 0.0, 0.0, 0.0},
                              {112.0, -0.25, -0.25, -0.5}};
const double kDct4x8[3][4] = {
    {2198.050556016380522, -0.96269623020744692, -0.76194253026666783, -0.6551140670773547},
    {764.3655248643528689, -0.92630200888366945, -0.9675229603596517, -0.27845290869168118},
    {527.107573587542228, -1.4594385811273854, -1.450082094097871593, -1.5843722511996204}};
const double kAfv[3][9] = {{3072.0, 3072.0, 256.0, 256.0, 256.0, 414.0, 0.0, 0.0, 0.0},
                           {1024.0, 1024.0, 50.0, 50.0, 50.0, 58.0, 0.0, 0.0, 0.0},
                           {384.0, 384.0, 12.0, 12.0, 12.0, 22.0, -0.25, -0.25, -0.25}};
// AFV's band positions (dequant.rs:512-580): the frequency of each 4x4 cell.
const double kAfvFreqs[16] = {0.0,
                              0.0,
                              0.8517778890324296,
                              5.37778436506804,
                              0.0,
                              0.0,
                              4.734747904497923,
                              5.449245381693219,
                              1.6598270267479331,
                              4.0,
                              7.275749096817861,
                              10.423227632456525,
                              2.662932286148962,
                              7.630657783650829,
                              8.962388608184032,
                              12.97166202570235};

double band_mult(double v) { return v > 0.0 ? 1.0 + v : 1.0 / (1.0 - v); }

// dequant.rs:416 Interpolate.
double interpolate(double pos, double max, const double* bands, int n) {
  const int last = n - 1;
  if (last == 0) return bands[0];
  const double scaled = pos * (double)last / max;
  const double fl = std::floor(scaled);
  const int idx = (int)fl;
  const double frac = scaled - fl;
  const double a = bands[idx], b = bands[idx + 1];
  return a * std::pow(b / a, frac);
}

// dequant.rs:461 GetDctQuantWeights as weights (not reciprocals), cols x rows.
void dct_weights(int cols, int rows, const double* params, int np, double* w) {
  double bands[8];
  bands[0] = params[0];
  for (int i = 1; i < np; ++i) bands[i] = bands[i - 1] * band_mult(params[i]);
  const double max = M_SQRT2 + 1e-6;
  for (int y = 0; y < rows; ++y)
    for (int x = 0; x < cols; ++x) {
      const double dx = (double)x / (double)(cols - 1), dy = (double)y / (double)(rows - 1);
      w[y * cols + x] = interpolate(std::sqrt(dx * dx + dy * dy), max, bands, np);
    }
}

// I.2.4 modes Hornuss, DCT4, DCT4x8 and AFV (dequant.rs:1300-1450) for
// slots 9..12, as f32 reciprocals of the 8x8 weights.
void special_into(int slot, int c, float* out) {
  double w[64];
  auto set = [&](int x, int y, double v) { w[y * 8 + x] = v; };
  auto at = [&](int x, int y) { return w[y * 8 + x]; };
  if (slot == 9) {
    for (int i = 0; i < 64; ++i) w[i] = kHornuss[c][0];
    set(0, 1, kHornuss[c][1]);
    set(1, 0, kHornuss[c][1]);
    set(1, 1, kHornuss[c][2]);
    set(0, 0, 1.0);
  } else if (slot == 10) {
    double base[16];
    dct_weights(4, 4, kDct4x4[c], 4, base);
    for (int y = 0; y < 8; ++y)
      for (int x = 0; x < 8; ++x) set(x, y, base[(y / 2) * 4 + x / 2]);
    // params (1, 1): the divisions leave the matrix as it is
    set(0, 1, at(0, 1) / 1.0);
    set(1, 0, at(1, 0) / 1.0);
    set(1, 1, at(1, 1) / 1.0);
  } else if (slot == 11) {
    double base[32];
    dct_weights(8, 4, kDct4x8[c], 4, base);
    for (int y = 0; y < 8; ++y)
      for (int x = 0; x < 8; ++x) set(x, y, base[(y / 2) * 8 + x]);
    set(0, 1, at(0, 1) / 1.0);
  } else {
    double w4x8[32], w4x4[16], bands[4];
    dct_weights(8, 4, kDct4x8[c], 4, w4x8);
    dct_weights(4, 4, kDct4x4[c], 4, w4x4);
    const double* p = kAfv[c];
    bands[0] = p[5];
    for (int i = 1; i < 4; ++i) bands[i] = bands[i - 1] * band_mult(p[i + 5]);
    for (int i = 0; i < 64; ++i) w[i] = 0.0;
    set(0, 0, 1.0);
    set(0, 1, p[0]);
    set(1, 0, p[1]);
    set(0, 2, p[2]);
    set(2, 0, p[3]);
    set(2, 2, p[4]);
    const double lo = kAfvFreqs[2], hi = kAfvFreqs[15];
    const double range = hi - lo + 1e-6;
    for (int y = 0; y < 4; ++y)
      for (int x = 0; x < 4; ++x) {
        if (x < 2 && y < 2) continue;
        set(2 * x, 2 * y, interpolate(kAfvFreqs[y * 4 + x] - lo, range, bands, 4));
      }
    for (int y = 0; y < 4; ++y)
      for (int x = 0; x < 8; ++x)
        if (x || y) set(x, 2 * y + 1, w4x8[y * 8 + x]);
    for (int y = 0; y < 4; ++y)
      for (int x = 0; x < 4; ++x)
        if (x || y) set(2 * x + 1, 2 * y, w4x4[y * 4 + x]);
  }
  for (int i = 0; i < 64; ++i) out[i] = (float)(1.0 / w[i]);
}

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
    for (int s = 0; s < 13; ++s) {
      float* dst = out + c * kDequantTableFloats + dq_offset(s);
      if (s == 6) dct2_into(kDct2[c], dst);
      else if (s >= 9) special_into(s, c, dst);
      else weights_into(kSlots[s].params[c], kSlots[s].np, kSlots[s].rows, kSlots[s].cols, dst);
    }
}

// Table I.11, the AFV basis (standard data, as jpxl-core varblock.rs prints
// it): row j is basis function j over the 4x4 samples in raster order.
const double kAfvBasis[16][16] = {
    {0.25, 0.25, 0.25, 0.25, 0.25, 0.25, 0.25, 0.25, 0.25, 0.25, 0.25, 0.25, 0.25, 0.25, 0.25,
     0.25},
    {0.876902929799142, 0.2206518106944235, -0.10140050393753763, -0.1014005039375375,
     0.2206518106944236, -0.10140050393753777, -0.10140050393753772, -0.10140050393753763,
     -0.10140050393753758, -0.10140050393753769, -0.1014005039375375, -0.10140050393753768,
     -0.10140050393753768, -0.10140050393753759, -0.10140050393753763, -0.10140050393753741},
    {0.0, 0.0, 0.40670075830260755, 0.44444816619734445, 0.0, 0.0, 0.19574399372042936,
     0.2929100136981264, -0.40670075830260716, -0.19574399372042872, 0.0, 0.11379074460448091,
     -0.44444816619734384, -0.29291001369812636, -0.1137907446044814, 0.0},
    {0.0, 0.0, -0.21255748058288748, 0.3085497062849767, 0.0, 0.4706702258572536,
     -0.1621205195722993, 0.0, -0.21255748058287047, -0.16212051957228327,
     -0.47067022585725277, -0.1464291867126764, 0.3085497062849487, 0.0, -0.14642918671266536,
     0.4251149611657548},
    {0.0, -0.7071067811865474, 0.0, 0.0, 0.7071067811865476, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0,
     0.0, 0.0, 0.0, 0.0},
    {-0.4105377591765233, 0.6235485373547691, -0.06435071657946274, -0.06435071657946266,
     0.6235485373547694, -0.06435071657946284, -0.0643507165794628, -0.06435071657946274,
     -0.06435071657946272, -0.06435071657946279, -0.06435071657946266, -0.06435071657946277,
     -0.06435071657946277, -0.06435071657946273, -0.06435071657946274, -0.0643507165794626},
    {0.0, 0.0, -0.4517556589999482, 0.15854503551840063, 0.0, -0.04038515160822202,
     0.0074182263792423875, 0.39351034269210167, -0.45175565899994635, 0.007418226379244351,
     0.1107416575309343, 0.08298163094882051, 0.15854503551839705, 0.3935103426921022,
     0.0829816309488214, -0.45175565899994796},
    {0.0, 0.0, -0.304684750724869, 0.5112616136591823, 0.0, 0.0, -0.290480129728998,
     -0.06578701549142804, 0.304684750724884, 0.2904801297290076, 0.0, -0.23889773523344604,
     -0.5112616136592012, 0.06578701549142545, 0.23889773523345467, 0.0},
    {0.0, 0.0, 0.3017929516615495, 0.25792362796341184, 0.0, 0.16272340142866204,
     0.09520022653475037, 0.0, 0.3017929516615503, 0.09520022653475055, -0.16272340142866173,
     -0.35312385449816297, 0.25792362796341295, 0.0, -0.3531238544981624, -0.6035859033230976},
    {0.0, 0.0, 0.40824829046386274, 0.0, 0.0, 0.0, 0.0, -0.4082482904638628,
     -0.4082482904638635, 0.0, 0.0, -0.40824829046386296, 0.0, 0.4082482904638634,
     0.408248290463863, 0.0},
    {0.0, 0.0, 0.1747866975480809, 0.0812611176717539, 0.0, 0.0, -0.3675398009862027,
     -0.307882213957909, -0.17478669754808135, 0.3675398009862011, 0.0, 0.4826689115059883,
     -0.08126111767175039, 0.30788221395790305, -0.48266891150598584, 0.0},
    {0.0, 0.0, -0.21105601049335784, 0.18567180916109802, 0.0, 0.0, 0.49215859013738733,
     -0.38525013709251915, 0.21105601049335806, -0.49215859013738905, 0.0, 0.17419412659916217,
     -0.18567180916109904, 0.3852501370925211, -0.1741941265991621, 0.0},
    {0.0, 0.0, -0.14266084808807264, -0.3416446842253372, 0.0, 0.7367497537172237,
     0.24627107722075148, -0.08574019035519306, -0.14266084808807344, 0.24627107722075137,
     0.14883399227113567, -0.04768680350229251, -0.3416446842253373, -0.08574019035519267,
     -0.047686803502292804, -0.14266084808807242},
    {0.0, 0.0, -0.13813540350758585, 0.3302282550303788, 0.0, 0.08755115000587084,
     -0.07946706605909573, -0.4613374887461511, -0.13813540350758294, -0.07946706605910261,
     0.49724647109535086, 0.12538059448563663, 0.3302282550303805, -0.4613374887461554,
     0.12538059448564315, -0.13813540350758452},
    {0.0, 0.0, -0.17437602599651067, 0.0702790691196284, 0.0, -0.2921026642334881,
     0.3623817333531167, 0.0, -0.1743760259965108, 0.36238173335311646, 0.29210266423348785,
     -0.4326608024727445, 0.07027906911962818, 0.0, -0.4326608024727457, 0.34875205199302267},
    {0.0, 0.0, 0.11354987314994337, -0.07417504595810355, 0.0, 0.19402893032594343,
     -0.435190496523228, 0.21918684838857466, 0.11354987314994257, -0.4351904965232251,
     0.5550443808910661, -0.25468277124066463, -0.07417504595810233, 0.2191868483885728,
     -0.25468277124066413, 0.1135498731499429},
};


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
