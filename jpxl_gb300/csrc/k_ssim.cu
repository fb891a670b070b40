// k_ssim.cu — sm_103a kernels of SSIMULACRA2 (jpxl-perceptual):
//   S1 k_downscale3        pyramid.rs:19 2x2 mean, edge replicated
//   S2 k_positive_xyb      color.rs:66 positive XYB (reproducible cube root)
//   S3 k_blur_h / k_blur_v blur.rs recursive Gaussian as its 9-tap FIR
//   S4 k_score_tile        fused candidate side of one scale: XYB, the three
//                          candidate blurs (mu2, sigma22, sigma12) in shared
//                          memory, the SSIM and edge maps and their pooled
//                          1st/4th powers
//   S5 k_score_finish      norms, 108 weights, remap (ssimulacra2.rs:509/:531)
//
// The reference's blur is three f64 resonators fed by f32 pair sums; in exact
// arithmetic they form a 9-tap symmetric FIR with zero padding (the host
// derives the taps).  The kernels evaluate that FIR in f32, paired and from
// the smallest tap inward, and pool per-pixel terms in f32 per thread and in
// f64 across threads and CTAs (fixed order).  The score agrees with the
// reference's to far inside the 0.01-point contract; the tests state the
// measured difference.
#include <algorithm>
#include <cstdint>

#include "jpxlg_common.cuh"
#include "jpxlg_internal.h"
#include "jpxlg_kernels.h"

namespace jpxlg {

__constant__ float c_taps[5];

// The 9-tap FIR on nine values in registers, outer pairs first.
__device__ __forceinline__ float fir9v(float m4, float m3, float m2, float m1, float c0, float p1,
                                       float p2, float p3, float p4) {
  float acc = c_taps[4] * (m4 + p4);
  acc = __fmaf_rn(c_taps[3], m3 + p3, acc);
  acc = __fmaf_rn(c_taps[2], m2 + p2, acc);
  acc = __fmaf_rn(c_taps[1], m1 + p1, acc);
  acc = __fmaf_rn(c_taps[0], c0, acc);
  return acc;
}

__device__ __forceinline__ float fir9(const float* p, int stride) {
  // p points at the centre sample; taps symmetric.
  return fir9v(p[-4 * stride], p[-3 * stride], p[-2 * stride], p[-stride], p[0], p[stride],
               p[2 * stride], p[3 * stride], p[4 * stride]);
}

// S1 — one output pixel per thread, all three channels; with `xyb` set the
// pixel's positive XYB (S2) is written too, for the scale's candidate side.
__global__ void __launch_bounds__(256) k_downscale3(const float* __restrict__ in, int w, int h,
                                                    float* __restrict__ out,
                                                    float* __restrict__ xyb) {
  const int ow = (w + 1) / 2, oh = (h + 1) / 2;
  const size_t ip = (size_t)w * h, op = (size_t)ow * oh;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ow * oh; i += gridDim.x * blockDim.x) {
    int ox = i % ow, oy = i / ow;
    int x0 = min(2 * ox, w - 1), x1 = min(2 * ox + 1, w - 1);
    int y0 = min(2 * oy, h - 1), y1 = min(2 * oy + 1, h - 1);
    float v[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float* p = in + ip * c;
      float a = p[(size_t)y0 * w + x0], b = p[(size_t)y0 * w + x1];
      float cc = p[(size_t)y1 * w + x0], d = p[(size_t)y1 * w + x1];
      v[c] = (a + b + cc + d) * 0.25f;
      out[op * c + i] = v[c];
    }
    if (xyb) {
      float o[3];
      positive_xyb(v[0], v[1], v[2], o);
      xyb[i] = o[0];
      xyb[op + i] = o[1];
      xyb[2 * op + i] = o[2];
    }
  }
}

void launch_downscale3(const float* in, int w, int h, float* out, float* xyb, cudaStream_t s) {
  int n = ((w + 1) / 2) * ((h + 1) / 2);
  dim3 grid(std::max(1, std::min((n + 255) / 256, 4096)));
  k_downscale3<<<grid, 256, 0, s>>>(in, w, h, out, xyb);
}

__global__ void __launch_bounds__(256) k_positive_xyb(const float* __restrict__ rgb,
                                                      float* __restrict__ xyb, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    float o[3];
    positive_xyb(rgb[i], rgb[n + i], rgb[2 * n + i], o);
    xyb[i] = o[0];
    xyb[n + i] = o[1];
    xyb[2 * n + i] = o[2];
  }
}

void launch_positive_xyb(const float* rgb, float* xyb, size_t n, int num_sms, cudaStream_t s) {
  int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)num_sms * 8);
  k_positive_xyb<<<std::max(1, blocks), 256, 0, s>>>(rgb, xyb, n);
}

// S3 — separable FIR with zero padding; `b` (optional) forms a*b rounded to
// f32 before the horizontal pass, as blur.rs:395 does.
constexpr int kBT = 32;
__global__ void __launch_bounds__(256) k_blur_h(const float* __restrict__ a,
                                                const float* __restrict__ b, int w, int h,
                                                float* __restrict__ out) {
  __shared__ float row[8][kBT * 4 + 8];
  const int x0 = blockIdx.x * kBT * 4;
  const int y = blockIdx.y * 8 + threadIdx.x / 32;
  const int lane = threadIdx.x % 32;
  float* r = row[threadIdx.x / 32];
  for (int i = lane; i < kBT * 4 + 8; i += 32) {
    int gx = x0 + i - 4;
    float v = 0.0f;
    if (y < h && gx >= 0 && gx < w) {
      size_t p = (size_t)y * w + gx;
      v = b ? a[p] * b[p] : a[p];
    }
    r[i] = v;
  }
  __syncwarp();
  if (y >= h) return;
  for (int i = lane; i < kBT * 4; i += 32) {
    int gx = x0 + i;
    if (gx < w) out[(size_t)y * w + gx] = fir9(&r[i + 4], 1);
  }
}

__global__ void __launch_bounds__(256) k_blur_v(const float* __restrict__ in, int w, int h,
                                                float* __restrict__ out) {
  __shared__ float t[kBT + 8][kBT + 1];
  const int x0 = blockIdx.x * kBT, y0 = blockIdx.y * kBT;
  for (int i = threadIdx.x; i < (kBT + 8) * kBT; i += blockDim.x) {
    int lx = i % kBT, ly = i / kBT;
    int gx = x0 + lx, gy = y0 + ly - 4;
    t[ly][lx] = (gx < w && gy >= 0 && gy < h) ? in[(size_t)gy * w + gx] : 0.0f;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kBT * kBT; i += blockDim.x) {
    int lx = i % kBT, ly = i / kBT;
    int gx = x0 + lx, gy = y0 + ly;
    if (gx < w && gy < h) out[(size_t)gy * w + gx] = fir9(&t[ly + 4][lx], kBT + 1);
  }
}

static void blur(const float* a, const float* b, float* tmp, float* out, int w, int h,
                 cudaStream_t s) {
  dim3 gh((w + kBT * 4 - 1) / (kBT * 4), (h + 7) / 8);
  k_blur_h<<<gh, 256, 0, s>>>(a, b, w, h, tmp);
  dim3 gv((w + kBT - 1) / kBT, (h + kBT - 1) / kBT);
  k_blur_v<<<gv, 256, 0, s>>>(tmp, w, h, out);
}

// Reference side (reference.rs:90 PrecomputedReference, Moments retention):
// mu = blur(xyb), sigma11 = blur(xyb*xyb), per channel.
void launch_ref_moments(const float* xyb, float* mu, float* s11, float* tmp, int w, int h,
                        cudaStream_t s) {
  const size_t n = (size_t)w * h;
  for (int c = 0; c < 3; ++c) {
    blur(xyb + n * c, nullptr, tmp, mu + n * c, w, h, s);
    blur(xyb + n * c, xyb + n * c, tmp, s11 + n * c, w, h, s);
  }
}

// S4 — candidate side of one scale, fused.  One CTA per 32x32 output tile:
// the candidate's positive XYB over the tile plus a 4-sample halo (zero
// outside the frame: the blur's zero padding) — read from precomputed
// planes, or converted here from linear RGB when kFromLinear — then per
// channel the horizontal and vertical FIR of c, c*c and r*c in shared memory
// and pool.rs:248's per-pixel terms.  Both passes are register-blocked: a
// thread produces four adjacent outputs from twelve inputs read as float4s
// (horizontal) or down one column (vertical).  Per-thread sums are f32,
// folded per warp in f32 and across warps in double-float into one row of 18
// sums per tile.
constexpr int kST = 32;
constexpr int kSH = 4;
constexpr int kSS = kST + 2 * kSH;  // 40: haloed side, rows float4-aligned
constexpr int kScoreThreads = 256;
constexpr int kScoreLoads = (kSS * kSS + kScoreThreads - 1) / kScoreThreads;  // 7
constexpr int kHItems = kSS * (kST / 4);  // 320 horizontal items: row x 4-column group
constexpr size_t kScoreSmem = (6 * kSS * kSS + 3 * kSS * kST) * sizeof(float);

// Four symmetric 9-tap FIR outputs from twelve inputs v[0..11]: output k
// is centred on v[k + 4].
__device__ __forceinline__ void fir9x4(const float* v, float* o) {
#pragma unroll
  for (int k = 0; k < 4; ++k)
    o[k] = fir9v(v[k], v[k + 1], v[k + 2], v[k + 3], v[k + 4], v[k + 5], v[k + 6], v[k + 7],
                 v[k + 8]);
}

template <bool kFromLinear>
__global__ void __launch_bounds__(kScoreThreads, 3) k_score_tile(const float* __restrict__ cand,
                                                              const float* __restrict__ rxyb,
                                                              const float* __restrict__ rmu,
                                                              const float* __restrict__ rs11,
                                                              int w, int h,
                                                              DF* __restrict__ partial) {
  extern __shared__ __align__(16) float ssm[];
  float* cx = ssm;                      // [3][kSS][kSS] candidate positive XYB
  float* rx = ssm + 3 * kSS * kSS;      // [3][kSS][kSS] reference positive XYB
  float* hp = ssm + 6 * kSS * kSS;      // [3][kSS][kST] horizontal pass of c, c*c, r*c
  __shared__ float red[kScoreThreads / 32][18];
  const size_t n = (size_t)w * h;
  const int lane = threadIdx.x % 32, warp = threadIdx.x / 32;
  const int x0 = blockIdx.x * kST - kSH, y0 = blockIdx.y * kST - kSH;
  // Phase 1: all candidate and reference samples of the haloed tile.
  {
    float v[kScoreLoads][6];
#pragma unroll
    for (int k = 0; k < kScoreLoads; ++k) {
      const int i = threadIdx.x + k * kScoreThreads;
      const int lx = i % kSS, ly = i / kSS;
      const int gx = x0 + lx, gy = y0 + ly;
      const bool ok = i < kSS * kSS && gx >= 0 && gy >= 0 && gx < w && gy < h;
      const size_t p = ok ? (size_t)gy * w + gx : 0;
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        v[k][q] = ok ? cand[n * q + p] : 0.0f;
        v[k][3 + q] = ok ? rxyb[n * q + p] : 0.0f;
      }
    }
#pragma unroll
    for (int k = 0; k < kScoreLoads; ++k) {
      const int i = threadIdx.x + k * kScoreThreads;
      if (i >= kSS * kSS) continue;
      const int lx = i % kSS, ly = i / kSS;
      const int gx = x0 + lx, gy = y0 + ly;
      const bool ok = gx >= 0 && gy >= 0 && gx < w && gy < h;
      float o[3] = {v[k][0], v[k][1], v[k][2]};
      if (kFromLinear) {
        o[0] = o[1] = o[2] = 0.0f;
        if (ok) positive_xyb(v[k][0], v[k][1], v[k][2], o);
      }
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        cx[(q * kSS + ly) * kSS + lx] = o[q];
        rx[(q * kSS + ly) * kSS + lx] = v[k][3 + q];
      }
    }
  }
  const float C2 = 0.0009f;
  // Vertical pass: column j = lane, output rows 4 * warp .. 4 * warp + 3.
  const int oj = lane, oi0 = 4 * warp;
  const int gxo = x0 + kSH + oj;
#pragma unroll 1
  for (int c = 0; c < 3; ++c) {
    float m1[4], v11[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int gy = y0 + kSH + oi0 + k;
      const bool ok = gxo < w && gy < h;
      const size_t p = n * c + (ok ? (size_t)gy * w + gxo : 0);
      m1[k] = ok ? rmu[p] : 0.0f;
      v11[k] = ok ? rs11[p] : 0.0f;
    }
    __syncthreads();
    const float* cc = cx + c * kSS * kSS;
    const float* rr = rx + c * kSS * kSS;
    // Horizontal pass: item = (row y, columns 4g .. 4g+3), inputs 4g .. 4g+11.
    for (int it = threadIdx.x; it < kHItems; it += kScoreThreads) {
      const int y = it / (kST / 4), g = it % (kST / 4);
      const float4* pc = reinterpret_cast<const float4*>(cc + y * kSS + 4 * g);
      const float4* pr = reinterpret_cast<const float4*>(rr + y * kSS + 4 * g);
      float a[12], sq[12], cr[12];
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const float4 u = pc[q], r = pr[q];
        a[4 * q] = u.x; a[4 * q + 1] = u.y; a[4 * q + 2] = u.z; a[4 * q + 3] = u.w;
        cr[4 * q] = r.x * u.x; cr[4 * q + 1] = r.y * u.y;
        cr[4 * q + 2] = r.z * u.z; cr[4 * q + 3] = r.w * u.w;
      }
#pragma unroll
      for (int q = 0; q < 12; ++q) sq[q] = a[q] * a[q];
      float o[4];
      fir9x4(a, o);
      *reinterpret_cast<float4*>(hp + (0 * kSS + y) * kST + 4 * g) = make_float4(o[0], o[1], o[2], o[3]);
      fir9x4(sq, o);
      *reinterpret_cast<float4*>(hp + (1 * kSS + y) * kST + 4 * g) = make_float4(o[0], o[1], o[2], o[3]);
      fir9x4(cr, o);
      *reinterpret_cast<float4*>(hp + (2 * kSS + y) * kST + 4 * g) = make_float4(o[0], o[1], o[2], o[3]);
    }
    __syncthreads();
    float sums[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    float m2[4], s22[4], s12[4];
    {
      float col[12];
#pragma unroll
      for (int q = 0; q < 12; ++q) col[q] = hp[(0 * kSS + oi0 + q) * kST + oj];
      fir9x4(col, m2);
#pragma unroll
      for (int q = 0; q < 12; ++q) col[q] = hp[(1 * kSS + oi0 + q) * kST + oj];
      fir9x4(col, s22);
#pragma unroll
      for (int q = 0; q < 12; ++q) col[q] = hp[(2 * kSS + oi0 + q) * kST + oj];
      fir9x4(col, s12);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int gy = y0 + kSH + oi0 + k;
      if (gxo >= w || gy >= h) continue;
      const int ctr = (oi0 + k + kSH) * kSS + oj + kSH;
      const float i1 = rr[ctr], i2 = cc[ctr];
      const float mu11 = m1[k] * m1[k], mu22 = m2[k] * m2[k], mu12 = m1[k] * m2[k];
      const float md = m1[k] - m2[k];
      const float num_m = 1.0f - md * md;
      const float num_s = 2.0f * (s12[k] - mu12) + C2;
      const float den_s = (v11[k] - mu11) + (s22[k] - mu22) + C2;
      // IEEE division here: identical images give num_s == den_s, and x / x
      // must be exactly 1 for the reference's score of exactly 100.
      const float d = fmaxf(1.0f - (num_m * num_s) / den_s, 0.0f);
      const float d2 = d * d;
      // (1 + |i2-m2|) / (1 + |i1-m1|) - 1, written as a difference over the
      // denominator so that the result keeps its relative precision.
      const float a1 = fabsf(i1 - m1[k]), a2 = fabsf(i2 - m2[k]);
      // Within the 0.01-point contract the fast division (at most 2 ulp off)
      // serves; identical images give a zero numerator, exact either way.
      const float d1 = __fdividef(a2 - a1, 1.0f + a1);
      const float art = fmaxf(d1, 0.0f), lost = fmaxf(-d1, 0.0f);
      const float art2 = art * art, lost2 = lost * lost;
      sums[0] += d;
      sums[1] += d2 * d2;
      sums[2] += art;
      sums[3] += art2 * art2;
      sums[4] += lost;
      sums[5] += lost2 * lost2;
    }
    // This channel's sums: warp fold in f32 (the warps are combined below).
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      float v = sums[k];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) red[warp][c * 6 + k] = v;
    }
  }
  // the 8 warps in order in double-float
  __syncthreads();
  if (threadIdx.x < 18) {
    DF t{red[0][threadIdx.x], 0.0f};
    for (int i = 1; i < kScoreThreads / 32; ++i) t = df_add(t, DF{red[i][threadIdx.x], 0.0f});
    partial[(size_t)(blockIdx.y * gridDim.x + blockIdx.x) * 18 + threadIdx.x] = t;
  }
}

int launch_score_scale(const float* cand, bool cand_is_linear, const SsimScale& ref, DF* partial,
                       int num_sms, cudaStream_t s) {
  (void)num_sms;
  dim3 grid((ref.w + kST - 1) / kST, (ref.h + kST - 1) / kST);
  if (cand_is_linear) {
    k_score_tile<true><<<grid, kScoreThreads, kScoreSmem, s>>>(cand, ref.xyb, ref.mu, ref.s11,
                                                                ref.w, ref.h, partial);
  } else {
    k_score_tile<false><<<grid, kScoreThreads, kScoreSmem, s>>>(cand, ref.xyb, ref.mu, ref.s11,
                                                                 ref.w, ref.h, partial);
  }
  return (int)(grid.x * grid.y);
}

cudaError_t configure_ssim_kernels() {
  cudaError_t e = cudaFuncSetAttribute(k_score_tile<true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kScoreSmem);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_score_tile<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)kScoreSmem);
}

// S5 — ssimulacra2.rs:391 WEIGHTS (the metric's data table), :509
// weighted_error, :531 remap; pool.rs:60 norms.
__constant__ double c_weights[108] = {
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

struct FinishArgs {
  int nscales;
  int ctas[6];
  long long pixels[6];
};

constexpr int kFinishThreads = 1024;
constexpr int kFinishGroups = kFinishThreads / 18;  // 56 groups of 18 threads

__global__ void __launch_bounds__(kFinishThreads) k_score_finish(const DF* __restrict__ partials,
                                                                 FinishArgs fa,
                                                                 double* __restrict__ out) {
  // Per scale: thread (g, k) sums quantity k of tile rows g, g + 56, ... in
  // order in double-float; the 56 group sums of each quantity are added in
  // group order.  Deterministic for a given frame size, f32 issue rates.
  __shared__ DF gsum[kFinishGroups][18];
  __shared__ double scale_sums[6][18];
  __shared__ double terms[6][3][6];
  __shared__ double wterm[108];
  const int g = threadIdx.x / 18, k = threadIdx.x % 18;
  size_t base = 0;
  for (int s = 0; s < fa.nscales; ++s) {
    if (g < kFinishGroups) {
      DF acc{0.0f, 0.0f};
      for (int i = g; i < fa.ctas[s]; i += kFinishGroups)
        acc = df_add(acc, partials[(base + i) * 18 + k]);
      gsum[g][k] = acc;
    }
    __syncthreads();
    if (threadIdx.x < 18) {
      DF t = gsum[0][threadIdx.x];
      for (int i = 1; i < kFinishGroups; ++i) t = df_add(t, gsum[i][threadIdx.x]);
      scale_sums[s][threadIdx.x] = df_value(t);
    }
    __syncthreads();
    base += fa.ctas[s];
  }
  // pool.rs:60 norms, one (scale, channel) per thread.
  if (threadIdx.x < fa.nscales * 3) {
    const int s = threadIdx.x / 3, c = threadIdx.x % 3;
    const double inv = 1.0 / (double)(fa.pixels[s] > 0 ? fa.pixels[s] : 1);
    const double* q = &scale_sums[s][c * 6];
    terms[s][c][0] = inv * q[0];
    terms[s][c][1] = inv * q[2];
    terms[s][c][2] = inv * q[4];
    terms[s][c][3] = sqrt(sqrt(inv * q[1]));
    terms[s][c][4] = sqrt(sqrt(inv * q[3]));
    terms[s][c][5] = sqrt(sqrt(inv * q[5]));
  }
  __syncthreads();
  // ssimulacra2.rs:509 weighted error: weight i belongs to channel c, scale
  // s, norm nn, map m with i = ((c * scales + s) * 2 + nn) * 3 + m.
  if (threadIdx.x < 108) {
    const int i = threadIdx.x;
    const int m = i % 3, nn = (i / 3) % 2, cs = i / 6;
    const int c = cs / fa.nscales, s = cs % fa.nscales;
    wterm[i] = c < 3 ? c_weights[i] * fabs(terms[s][c][nn * 3 + m]) : 0.0;
  }
  __syncthreads();
  if (threadIdx.x >= 32) return;
  double part = 0.0;
  for (int i = threadIdx.x; i < 3 * fa.nscales * 6; i += 32) part += wterm[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if (threadIdx.x != 0) return;
  const double err = part;
  double sc = err * 0.9562382616834844;
  sc = 6.248496625763138e-5 * sc * sc * sc + 2.326765642916932 * sc -
       0.020884521182843837 * sc * sc;
  out[0] = sc > 0.0 ? 100.0 - 10.0 * pow(sc, 0.6276336467831387) : 100.0;
  out[1] = err;
  for (int s = 0; s < fa.nscales; ++s)
    for (int c = 0; c < 3; ++c)
      for (int m = 0; m < 6; ++m) out[2 + (s * 3 + c) * 6 + m] = terms[s][c][m];
}

void launch_score_finish(const DF* partials, const int* ctas_per_scale, int nscales,
                         const int* pixels_per_scale, double* out, cudaStream_t s) {
  FinishArgs fa;
  fa.nscales = nscales;
  for (int i = 0; i < 6; ++i) {
    fa.ctas[i] = i < nscales ? ctas_per_scale[i] : 0;
    fa.pixels[i] = i < nscales ? pixels_per_scale[i] : 0;
  }
  k_score_finish<<<1, kFinishThreads, 0, s>>>(partials, fa, out);
}

void upload_blur_taps(const float* taps, cudaStream_t s) {
  cudaMemcpyToSymbolAsync(c_taps, taps, sizeof(float) * 5, 0, cudaMemcpyHostToDevice, s);
}

}  // namespace jpxlg
