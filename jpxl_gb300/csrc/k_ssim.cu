// k_ssim.cu — sm_103a kernels of SSIMULACRA2 (jpxl-perceptual) besides the
// blur (k_blur.cu):
//   S1 k_downscale3        pyramid.rs:19 2x2 mean, edge replicated
//   S2 k_positive_xyb      color.rs:66 positive XYB (reproducible cube root)
//   S5 k_score_reduce      the partial rows' sums per scale and quantity
//      k_score_finish      norms, 108 weights, remap (ssimulacra2.rs:509/:531)
//
// The per-strip partial sums that S5 folds come from k_blur_cols (f32 per
// 32 rows of a column, double-float above that, fixed order).
#include <algorithm>
#include <cstdint>

#include "jpxlg_common.cuh"
#include "jpxlg_internal.h"
#include "jpxlg_kernels.h"

namespace jpxlg {

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

constexpr int kReduceThreads = 256;
constexpr int kFinishThreads = 128;

// S5a: one CTA per (quantity, scale): thread t sums the quantity's tile rows
// t, t + 256, ... of the scale in order in double-float, then the threads'
// sums meet in a fixed tree (warps, then warps in order).  The total goes to
// row 0 of the scale's partial rows, column k (only this CTA reads that
// column).  Deterministic for a given frame size; every load of a scale is
// in flight at once instead of behind one CTA's sequential chains.
__global__ void __launch_bounds__(kReduceThreads) k_score_reduce(DF* __restrict__ partials,
                                                                 FinishArgs fa) {
  __shared__ DF wsum[kReduceThreads / 32];
  const int k = blockIdx.x, s = blockIdx.y, t = threadIdx.x;
  size_t base = 0;
  for (int i = 0; i < s; ++i) base += fa.ctas[i];
  DF acc{0.0f, 0.0f};
#pragma unroll 4
  for (int i = t; i < fa.ctas[s]; i += kReduceThreads)
    acc = df_add(acc, partials[(base + i) * 18 + k]);
  const DF w = df_warp_sum(acc);
  if ((t & 31) == 0) wsum[t >> 5] = w;
  __syncthreads();
  if (t == 0) {
    DF tot = wsum[0];
    for (int i = 1; i < kReduceThreads / 32; ++i) tot = df_add(tot, wsum[i]);
    partials[base * 18 + k] = tot;
  }
}

// S5b: the norms, weights and remap from the 6 x 18 sums.
__global__ void __launch_bounds__(kFinishThreads) k_score_finish(const DF* __restrict__ partials,
                                                                 FinishArgs fa,
                                                                 double* __restrict__ out) {
  __shared__ double scale_sums[6][18];
  __shared__ double terms[6][3][6];
  __shared__ double wterm[108];
  if (threadIdx.x < 18) {
    size_t base = 0;
    for (int s = 0; s < fa.nscales; ++s) {
      scale_sums[s][threadIdx.x] = df_value(partials[base * 18 + threadIdx.x]);
      base += fa.ctas[s];
    }
  }
  __syncthreads();
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

int launch_score_finish(DF* partials, const int* ctas_per_scale, int nscales,
                        const int* pixels_per_scale, double* out, cudaStream_t s) {
  FinishArgs fa;
  fa.nscales = nscales;
  for (int i = 0; i < 6; ++i) {
    fa.ctas[i] = i < nscales ? ctas_per_scale[i] : 0;
    fa.pixels[i] = i < nscales ? pixels_per_scale[i] : 0;
  }
  k_score_reduce<<<dim3(18, nscales), kReduceThreads, 0, s>>>(partials, fa);
  k_score_finish<<<1, kFinishThreads, 0, s>>>(partials, fa, out);
  return 2;
}


}  // namespace jpxlg
