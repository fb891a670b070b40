// k_render.cu — sm_103a kernels of the plan renderer / decoder tail:
//   R1 k_render_vb<R,C>  dequantize, HF CfL, LLF from the LF planes, IDCT_2D,
//                        in-frame scatter and the per-block EPF sigma
//   R2 k_gaborish        J.3 3x3 with FMA, mirrored borders
//   R3 k_epf<step>       J.4 steps 0/1/2
//   R4 k_colour_out      L.2.2 opsin inverse and the output encoding
// Operation order follows jpxl-plan-render lib.rs:749 render_inner and the
// jpxl-core kernels it calls; -fmad=false keeps every unfused product.
#include <algorithm>
#include <cstdint>

#include "jpxlg_common.cuh"
#include "jpxlg_internal.h"
#include "jpxlg_kernels.h"

namespace jpxlg {

extern __constant__ float c_scale_f[32];
extern __constant__ float c_quant_bias[3];

__constant__ float c_opsin_m[9];
__constant__ float c_opsin_bias[3];
__constant__ float c_opsin_bias_cbrt[3];
// dct.rs:631 the 64-point DCT-II matrix (rows u, columns x), f32 entries.
__device__ float g_dct64[64 * 64];

// dct.rs:678 matrix_pass for N = 64 (the reference's transforms above 32
// points): each output an f64 dot product of f32 entries, rounded once, then
// the normative factor sqrt(64) = 8.  The dot product runs in double-float on
// the FP32 pipe (GB300's FP64 rate is a small fraction of its FP32 rate):
// each product is exact as p + e (e from one FMA), four independent
// compensated partial sums carry the rest, and one rounding to f32 ends it.
// Both that sum and the reference's sequential f64 sum lie within ~1e-15
// (relative) of the exact dot product, so they round to the same f32 unless
// the exact value lies that close to a rounding midpoint.
__device__ __forceinline__ void df_acc(float& hi, float& lo, float a, float b) {
  const float p = a * b;
  const float e = __fmaf_rn(a, b, -p);  // a*b = p + e exactly
  const float s = hi + p;
  const float bb = s - hi;
  const float err = (hi - (s - bb)) + (p - bb);  // hi + p = s + err exactly
  hi = s;
  lo = lo + (err + e);
}

__device__ __forceinline__ void idct_64(float* v) {
  float out[64];
#pragma unroll 1
  for (int k = 0; k < 64; ++k) {
    float h[4] = {0.0f, 0.0f, 0.0f, 0.0f}, l[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int j = 0; j < 64; j += 4)
#pragma unroll
      for (int i = 0; i < 4; ++i) df_acc(h[i], l[i], g_dct64[(j + i) * 64 + k], v[j + i]);
    // combine the four partial sums (double-float additions)
    float hi = h[0], lo = l[0];
#pragma unroll
    for (int i = 1; i < 4; ++i) {
      const float s = hi + h[i];
      const float bb = s - hi;
      const float err = (hi - (s - bb)) + (h[i] - bb);
      hi = s;
      lo = lo + (err + l[i]);
    }
    const float r = hi + lo;
    // one correct rounding of hi + lo: r is f32(hi + lo) (round to nearest)
    out[k] = r;
  }
#pragma unroll
  for (int k = 0; k < 64; ++k) v[k] = out[k] * 8.0f;
}

// jpxl-core dct.rs:982 idct_2d_in_place for the small shapes of the 8x8
// special transforms: coef is landscape (min x max), out ROWS x COLS samples.
template <int ROWS, int COLS>
__device__ __forceinline__ void idct2d_raw(const float* coef, float* out) {
  float s[ROWS * COLS];
#pragma unroll
  for (int r = 0; r < ROWS; ++r)
#pragma unroll
    for (int c = 0; c < COLS; ++c)
      s[c * ROWS + r] = COLS > ROWS ? coef[r * COLS + c] : coef[c * ROWS + r];
#pragma unroll
  for (int k = 0; k < ROWS; ++k) {
    float v[COLS];
#pragma unroll
    for (int i = 0; i < COLS; ++i) v[i] = s[i * ROWS + k];
    idct_1d<COLS>(v);
#pragma unroll
    for (int i = 0; i < COLS; ++i) s[i * ROWS + k] = v[i];
  }
#pragma unroll
  for (int r = 0; r < ROWS; ++r)
#pragma unroll
    for (int c = 0; c < COLS; ++c) out[r * COLS + c] = s[c * ROWS + r];
#pragma unroll
  for (int c = 0; c < COLS; ++c) {
    float v[ROWS];
#pragma unroll
    for (int i = 0; i < ROWS; ++i) v[i] = out[i * COLS + c];
    idct_1d<ROWS>(v);
#pragma unroll
    for (int i = 0; i < ROWS; ++i) out[i * COLS + c] = v[i];
  }
}

__device__ double g_afv[256];  // Table I.11, uploaded by the host

// varblock.rs:917 DCT2x2: aux_idct_2x2 (:898) with s = 2, 4, 8, each stage
// reading the previous one; b (row-major, LLF at 0) becomes the samples.
__device__ __forceinline__ void dct2x2_block(float* b) {
  float r[64];
#pragma unroll
  for (int st = 2; st <= 8; st *= 2) {
    const int h = st / 2;
#pragma unroll
    for (int i = 0; i < 64; ++i) r[i] = b[i];
#pragma unroll
    for (int y = 0; y < h; ++y)
#pragma unroll
      for (int x = 0; x < h; ++x) {
        const float c00 = b[y * 8 + x], c01 = b[y * 8 + h + x];
        const float c10 = b[(y + h) * 8 + x], c11 = b[(y + h) * 8 + h + x];
        r[(2 * y) * 8 + 2 * x] = ((c00 + c01) + c10) + c11;
        r[(2 * y) * 8 + 2 * x + 1] = ((c00 + c01) - c10) - c11;
        r[(2 * y + 1) * 8 + 2 * x] = ((c00 - c01) + c10) - c11;
        r[(2 * y + 1) * 8 + 2 * x + 1] = ((c00 - c01) - c10) + c11;
      }
#pragma unroll
    for (int i = 0; i < 64; ++i) b[i] = r[i];
  }
}


// The 8x8 special transforms of jpxl-core varblock.rs:926-1230 on a
// dequantized block b (row-major, LLF at 0): KIND 2 Hornuss, 3 DCT4x4,
// 4 DCT8x4, 5 DCT4x8, 6..9 AFV0..AFV3.  Evaluation order follows the
// reference expression by expression.
template <int KIND>
__device__ __forceinline__ void special_block(const float* b, float* o) {
  auto at = [&](int x, int y) { return b[y * 8 + x]; };
  auto set = [&](int x, int y, float v) { o[y * 8 + x] = v; };
  if constexpr (KIND == 2 || KIND == 3) {
    const float c00 = b[0], c01 = b[1], c10 = b[8], c11 = b[9];
    const float dcs[4] = {((c00 + c01) + c10) + c11, ((c00 + c01) - c10) - c11,
                          ((c00 - c01) + c10) - c11, ((c00 - c01) - c10) + c11};
#pragma unroll
    for (int y = 0; y < 2; ++y)
#pragma unroll
      for (int x = 0; x < 2; ++x) {
        if constexpr (KIND == 2) {
          float rs = 0.0f;
#pragma unroll
          for (int iy = 0; iy < 4; ++iy)
#pragma unroll
            for (int ix = (iy == 0 ? 1 : 0); ix < 4; ++ix) rs += at(x + ix * 2, y + iy * 2);
          const float centre = dcs[y * 2 + x] - rs / 16.0f;
          set(4 * x + 1, 4 * y + 1, centre);
#pragma unroll
          for (int iy = 0; iy < 4; ++iy)
#pragma unroll
            for (int ix = 0; ix < 4; ++ix)
              if (!(ix == 1 && iy == 1)) set(x * 4 + ix, y * 4 + iy, at(x + ix * 2, y + iy * 2) + centre);
          set(4 * x, 4 * y, at(x + 2, y + 2) + centre);
        } else {
          float blk[16], smp[16];
#pragma unroll
          for (int iy = 0; iy < 4; ++iy)
#pragma unroll
            for (int ix = 0; ix < 4; ++ix) blk[iy * 4 + ix] = at(x + ix * 2, y + iy * 2);
          blk[0] = dcs[y * 2 + x];
          idct2d_raw<4, 4>(blk, smp);
#pragma unroll
          for (int l = 0; l < 4; ++l)
#pragma unroll
            for (int k = 0; k < 4; ++k) set(4 * x + k, 4 * y + l, smp[l * 4 + k]);
        }
      }
  } else if constexpr (KIND == 4 || KIND == 5) {
    const float coef0 = at(0, 0), coef1 = at(0, 1);
    const float dcs[2] = {coef0 + coef1, coef0 - coef1};
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      float g[32], smp[32];
#pragma unroll
      for (int iy = 0; iy < 4; ++iy)
#pragma unroll
        for (int ix = 0; ix < 8; ++ix) g[iy * 8 + ix] = at(ix, half + iy * 2);
      g[0] = dcs[half];
      if constexpr (KIND == 4) {
        idct2d_raw<8, 4>(g, smp);
#pragma unroll
        for (int iy = 0; iy < 8; ++iy)
#pragma unroll
          for (int ix = 0; ix < 4; ++ix) set(4 * half + ix, iy, smp[iy * 4 + ix]);
      } else {
        idct2d_raw<4, 8>(g, smp);
#pragma unroll
        for (int iy = 0; iy < 4; ++iy)
#pragma unroll
          for (int ix = 0; ix < 8; ++ix) set(ix, 4 * half + iy, smp[iy * 8 + ix]);
      }
    }
  } else {
    constexpr int n = KIND - 6, fx = n & 1, fy = n / 2;
    float ca[16], sa[16];
    ca[0] = ((at(0, 0) + at(0, 1)) + at(1, 0)) * 4.0f;
#pragma unroll
    for (int iy = 0; iy < 4; ++iy)
#pragma unroll
      for (int ix = (iy == 0 ? 1 : 0); ix < 4; ++ix) ca[iy * 4 + ix] = at(ix * 2, iy * 2);
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      double acc = 0.0;
#pragma unroll
      for (int j = 0; j < 16; ++j) acc += (double)ca[j] * g_afv[j * 16 + q];
      sa[q] = (float)acc;
    }
#pragma unroll
    for (int iy = 0; iy < 4; ++iy)
#pragma unroll
      for (int ix = 0; ix < 4; ++ix) {
        const int sx = fx ? 3 - ix : ix, sy = fy ? 3 - iy : iy;
        set(fx * 4 + ix, fy * 4 + iy, sa[sy * 4 + sx]);
      }
    float c44[16], s44[16];
#pragma unroll
    for (int iy = 0; iy < 4; ++iy)
#pragma unroll
      for (int ix = 0; ix < 4; ++ix) c44[iy * 4 + ix] = at(ix * 2 + 1, iy * 2);
    c44[0] = (at(0, 0) - at(1, 0)) + at(0, 1);
    idct2d_raw<4, 4>(c44, s44);
#pragma unroll
    for (int iy = 0; iy < 4; ++iy)
#pragma unroll
      for (int ix = 0; ix < 4; ++ix) set((fx ? 0 : 4) + ix, fy * 4 + iy, s44[iy * 4 + ix]);
    float c48[32], s48[32];
#pragma unroll
    for (int iy = 0; iy < 4; ++iy)
#pragma unroll
      for (int ix = 0; ix < 8; ++ix) c48[iy * 8 + ix] = at(ix, 1 + iy * 2);
    c48[0] = at(0, 0) - at(0, 1);
    idct2d_raw<4, 8>(c48, s48);
#pragma unroll
    for (int iy = 0; iy < 4; ++iy)
#pragma unroll
      for (int ix = 0; ix < 8; ++ix) set(ix, (fy ? 0 : 4) + iy, s48[iy * 8 + ix]);
  }
}

template <int N>
__device__ __forceinline__ void idct_n(float* v) {
  if constexpr (N == 64) idct_64(v);
  else idct_1d<N>(v);
}

// ---------------------------------------------------------------------------
// R1 — one varblock of R x C samples per group of T = max(R, C) threads.
// Landscape coefficients are crows = min x ccols = max.  IDCT_2D
// (dct.rs:982): scratch S (C x R) is L transposed when C > R, else L; step A
// runs length-C IDCTs down S's R columns; step B runs length-R IDCTs along
// the C rows of the result, producing sample column i in thread i.
// ---------------------------------------------------------------------------

// KIND 1: DCT2x2 (R = C = 8): the dequantized block goes through the three
// aux_idct_2x2 stages of jpxl-core varblock.rs:917 instead of IDCT_2D.
template <int R, int C, int KIND = 0>
__global__ void __launch_bounds__(128) k_render_vb(RenderArgs a, const uint32_t* __restrict__ list,
                                                   int count) {
  constexpr int T = R > C ? R : C;
  constexpr int CR = R < C ? R : C;   // landscape rows
  constexpr int CC = T;               // landscape cols
  constexpr bool portrait = R > C;
  constexpr int BR = R / 8, BC = C / 8;
  constexpr int LY = CR / 8, LX = CC / 8;  // LLF corner
  constexpr int VPB = 128 / T;
  __shared__ float L[VPB][CR][CC + 1];
  __shared__ float LLF[VPB][3][64];
  const int g = threadIdx.x / T, j = threadIdx.x % T;
  const int vi = blockIdx.x * VPB + g;
  const bool active = vi < count;
  const uint32_t packed = active ? list[vi] : 0u;
  const int bx = packed & 0xffff, by = packed >> 16;
  const int x0 = bx * 8, y0 = by * 8;
  const Geo& geo = a.geo;
  const size_t cplane = (size_t)geo.W8 * geo.H8;
  const size_t bplane = (size_t)geo.bw * geo.bh;
  const size_t plane = (size_t)geo.w * geo.h;

  float mul = 0.0f, kx = 0.0f, kb = 0.0f;
  if (active) {
    mul = hf_multiplier(a.mul_table, a.qs.global_scale,
                        a.hf_mul[(size_t)by * geo.bw + bx]);  // reconstruct.rs:27
    const int tile = (by / 8) * geo.tw + bx / 8;
    kx = 0.0f + (float)a.cfl_x[tile] / 84.0f;  // reconstruct.rs:96 cfl_factors
    kb = 1.0f + (float)a.cfl_b[tile] / 84.0f;
    // LLF rectangles (varblock.rs:817 llf_from_lf) of the three channels:
    // LF dequantized (reconstruct.rs:84) with the LF CfL (plan-render
    // lib.rs:1314), laid out landscape, DCT_2D, times scale_f(y)*scale_f(x).
    if (j < 3) {
      const int c = j;
      float k_x_lf = a.k_x_lf, k_b_lf = a.k_b_lf;
      if (a.lf_factors_dev) {
        k_x_lf = 0.0f + (float)a.lf_factors_dev[0] / 84.0f;
        k_b_lf = 1.0f + (float)a.lf_factors_dev[1] / 84.0f;
      }
      float rect[64];
      for (int dy = 0; dy < BR; ++dy)
        for (int dx = 0; dx < BC; ++dx) {
          size_t bi = (size_t)(by + dy) * geo.bw + bx + dx;
          float v;
          if (a.lf_float) {
            v = a.lf_float[bplane * c + bi];  // dequantized, LF CfL and smoothing applied
          } else {
            float dY = a.qs.m_dc[1] * (float)a.lfq[bplane + bi] / 1.0f;
            if (c == 1) v = dY;
            else {
              float d = a.qs.m_dc[c] * (float)a.lfq[bplane * c + bi] / 1.0f;
              v = d + (c == 0 ? k_x_lf : k_b_lf) * dY;
            }
          }
          if (portrait) rect[dx * BR + dy] = v; else rect[dy * BC + dx] = v;
        }
      if (LY * LX > 1) dct2d_small(rect, LY, LX);
      constexpr int sfiy = LY == 1 ? 0 : (LY == 2 ? 1 : (LY == 4 ? 2 : 3));
      constexpr int sfix = LX == 1 ? 0 : (LX == 2 ? 1 : (LX == 4 ? 2 : 3));
      const float* sfy = &c_scale_f[sfiy * 8];
      const float* sfx = &c_scale_f[sfix * 8];
      for (int y = 0; y < LY; ++y)
        for (int x = 0; x < LX; ++x) LLF[g][c][y * LX + x] = rect[y * LX + x] * sfy[y] * sfx[x];
    }
  }
  __syncthreads();

  // Dequantize landscape column x = j of each channel (plan-render
  // lib.rs:913: adjusted * (mul*qm) * matrix, left to right).
  float dY[CR];
  // compact dequant slot of this shape (Table I.4 indices 0,4,5,6,7,8)
  constexpr int slot = KIND == 1 ? 6
                       : KIND == 2 ? 9
                       : KIND == 3 ? 10
                       : (KIND == 4 || KIND == 5) ? 11
                       : KIND >= 6 ? 12
                       : (R == 64 && C == 64) ? 7
                       : (T == 64) ? 8
                       : (R == C) ? (R == 8 ? 0 : (R == 16 ? 1 : 2))
                                  : (CC == 16 ? 3 : (CR == 8 ? 4 : 5));
  const int off = dq_offset(slot);
  // The channel loop stays rolled, and for square shapes both IDCT passes
  // run through one copy of the transform: a 32-point transform inlined six
  // times does not fit the instruction cache.
#pragma unroll 1
  for (int ci = 0; ci < 3; ++ci) {
    const int c = ci == 0 ? 1 : (ci == 1 ? 0 : 2);  // luma first: CfL needs it
    if (active) {
      const float scale = mul * a.qs.qm[c];
      const float bias = c_quant_bias[c];
      const float* m = a.dq + c * kDequantTableFloats + off;
      const float kc = c == 0 ? kx : kb;
#pragma unroll
      for (int y = 0; y < CR; ++y) {
        const int x = j;
        size_t pos = portrait ? (size_t)(y0 + x) * geo.W8 + x0 + y : (size_t)(y0 + y) * geo.W8 + x0 + x;
        int32_t q = a.qcoeff[cplane * c + pos];
        float d = bias_adjust_q(q, bias) * scale * __ldg(&m[y * CC + x]);
        if (c == 1) dY[y] = d;
        else d = d + kc * dY[y];  // lib.rs:1344 apply_hf_cfl
        if (y < LY && x < LX) d = LLF[g][c][y * LX + x];
        L[g][y][x] = d;
      }
    }
    __syncthreads();
    float v[T];
    if constexpr (KIND >= 2) {
      // thread 0 of the group reconstructs the block, then thread j writes
      // sample column j.
      if (active && j == 0) {
        float b[64], o[64];
#pragma unroll
        for (int i = 0; i < 64; ++i) b[i] = L[g][i / 8][i % 8];
        special_block<KIND>(b, o);
#pragma unroll
        for (int i = 0; i < 64; ++i) L[g][i / 8][i % 8] = o[i];
      }
      __syncthreads();
      if (active) {
        const int fx = x0 + j;
        if (fx < geo.w) {
#pragma unroll
          for (int rr = 0; rr < 8; ++rr) {
            const int fy = y0 + rr;
            if (fy < geo.h) a.planes[plane * c + (size_t)fy * geo.w + fx] = L[g][rr][j];
          }
        }
      }
      __syncthreads();
    } else if constexpr (KIND == 1) {
      // varblock.rs:895 aux_idct_2x2 with s = 2, 4, 8, each stage reading the
      // previous one; thread 0 of the group runs the cascade, then thread j
      // writes sample column j.
      if (active && j == 0) {
        float b[64];
#pragma unroll
        for (int i = 0; i < 64; ++i) b[i] = L[g][i / 8][i % 8];
        dct2x2_block(b);
#pragma unroll
        for (int i = 0; i < 64; ++i) L[g][i / 8][i % 8] = b[i];
      }
      __syncthreads();
      if (active) {
        const int fx = x0 + j;
        if (fx < geo.w) {
#pragma unroll
          for (int rr = 0; rr < 8; ++rr) {
            const int fy = y0 + rr;
            if (fy < geo.h) a.planes[plane * c + (size_t)fy * geo.w + fx] = L[g][rr][j];
          }
        }
      }
      __syncthreads();
    } else if constexpr (R == C) {
      // Step A (st = 0): thread j transforms column j of L in place.
      // Step B (st = 1): thread j transforms row j of the result into sample
      // column j and scatters it inside the frame.
#pragma unroll 1
      for (int st = 0; st < 2; ++st) {
        if (active) {
#pragma unroll
          for (int i = 0; i < T; ++i) v[i] = st == 0 ? L[g][i][j] : L[g][j][i];
          idct_n<T>(v);
        }
        if (st == 0) {
          __syncthreads();
          if (active) {
#pragma unroll
            for (int i = 0; i < T; ++i) L[g][i][j] = v[i];
          }
        } else if (active) {
          const int fx = x0 + j;
          if (fx < geo.w) {
#pragma unroll
            for (int r = 0; r < T; ++r) {
              const int fy = y0 + r;
              if (fy < geo.h) a.planes[plane * c + (size_t)fy * geo.w + fx] = v[r];
            }
          }
        }
        __syncthreads();
      }
    } else {
      // Step A: thread jj < R transforms column jj of S (length C).
      if (active && j < R) {
#pragma unroll
        for (int i = 0; i < C; ++i) v[i] = (C > R) ? L[g][j][i] : L[g][i][j];
        idct_n<C>(v);
      }
      __syncthreads();
      if (active && j < R) {
#pragma unroll
        for (int i = 0; i < C; ++i) {
          if (C > R) L[g][j][i] = v[i]; else L[g][i][j] = v[i];
        }
      }
      __syncthreads();
      // Step B: thread i < C transforms row i of the step-A result (length R)
      // into sample column i and scatters it inside the frame.
      if (active && j < C) {
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = (C > R) ? L[g][r][j] : L[g][j][r];
        idct_n<R>(v);
        const int fx = x0 + j;
        if (fx < geo.w) {
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const int fy = y0 + r;
            if (fy < geo.h) a.planes[plane * c + (size_t)fy * geo.w + fx] = v[r];
          }
        }
      }
      __syncthreads();
    }
  }
  // J.4.3 sigma per block (restoration.rs:338 vardct_sigma).
  if (active && j < BR * BC) {
    const int dy = j / BC, dx = j % BC;
    size_t bi = (size_t)(by + dy) * geo.bw + bx + dx;
    int s = a.sharpness[bi];
    s = s > 7 ? 7 : s;
    const float lut = s == 7 ? 1.0f : (float)s / 7.0f;
    a.sigma[bi] = mul * 0.46f * lut;
  }
}

// The LLF rectangles and EPF sigma of the square varblocks of size N that
// the split-precision render (k_tc.cu) transforms: varblock.rs:817
// llf_from_lf (LF dequantized by reconstruct.rs:84 with the LF CfL of
// plan-render lib.rs:1314, DCT_2D, times scale_f) and restoration.rs:338
// vardct_sigma, exactly as k_render_vb forms them.  One thread per
// (varblock, channel); llf receives 16 floats per channel per varblock.
template <int N>
__global__ void __launch_bounds__(128) k_llf_sigma(RenderArgs a, const uint32_t* __restrict__ list,
                                                   int count, float* __restrict__ llf) {
  constexpr int n = N / 8;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= count * 3) return;
  const int vi = idx / 3, c = idx % 3;
  const uint32_t packed = list[vi];
  const int bx = packed & 0xffff, by = packed >> 16;
  const Geo& geo = a.geo;
  const size_t bplane = (size_t)geo.bw * geo.bh;
  float k_x_lf = a.k_x_lf, k_b_lf = a.k_b_lf;
  if (a.lf_factors_dev) {
    k_x_lf = 0.0f + (float)a.lf_factors_dev[0] / 84.0f;
    k_b_lf = 1.0f + (float)a.lf_factors_dev[1] / 84.0f;
  }
  if (c == 0) {
    const float mul = hf_multiplier(a.mul_table, a.qs.global_scale,
                                    a.hf_mul[(size_t)by * geo.bw + bx]);
    for (int i = 0; i < n * n; ++i) {
      const size_t bi = (size_t)(by + i / n) * geo.bw + bx + i % n;
      int sh = a.sharpness[bi];
      sh = sh > 7 ? 7 : sh;
      const float lut = sh == 7 ? 1.0f : (float)sh / 7.0f;
      a.sigma[bi] = mul * 0.46f * lut;
    }
  }
  float rect[64];
  for (int dy = 0; dy < n; ++dy)
    for (int dx = 0; dx < n; ++dx) {
      const size_t bi = (size_t)(by + dy) * geo.bw + bx + dx;
      float v;
      if (a.lf_float) {
        v = a.lf_float[bplane * c + bi];
      } else {
        const float dY = a.qs.m_dc[1] * (float)a.lfq[bplane + bi] / 1.0f;
        if (c == 1) {
          v = dY;
        } else {
          const float d = a.qs.m_dc[c] * (float)a.lfq[bplane * c + bi] / 1.0f;
          v = d + (c == 0 ? k_x_lf : k_b_lf) * dY;
        }
      }
      rect[dy * n + dx] = v;
    }
  if (n > 1) dct2d_small(rect, n, n);
  constexpr int sfi = n == 1 ? 0 : (n == 2 ? 1 : (n == 4 ? 2 : 3));
  const float* sf = &c_scale_f[sfi * 8];
  float* o = llf + (size_t)vi * 48 + c * 16;
  for (int y = 0; y < n; ++y)
    for (int x = 0; x < n; ++x) o[y * n + x] = rect[y * n + x] * sf[y] * sf[x];
}

int launch_llf_sigma(const RenderArgs& a, const uint32_t* const* lists, const int* counts,
                     float* const* llf, const cudaStream_t* s) {
  int k = 0;
  if (counts[0]) { k_llf_sigma<8><<<(3 * counts[0] + 127) / 128, 128, 0, s[0]>>>(a, lists[0], counts[0], llf[0]); ++k; }
  if (counts[1]) { k_llf_sigma<16><<<(3 * counts[1] + 127) / 128, 128, 0, s[1]>>>(a, lists[1], counts[1], llf[1]); ++k; }
  if (counts[2]) { k_llf_sigma<32><<<(3 * counts[2] + 127) / 128, 128, 0, s[2]>>>(a, lists[2], counts[2], llf[2]); ++k; }
  return k;
}

void launch_render_varblocks(const RenderArgs& a, const uint32_t* const* lists, const int* counts,
                             const cudaStream_t* s) {
#define JPXLG_RV(IDX, R, C)                                                              \
  if (counts[IDX])                                                                       \
    k_render_vb<R, C><<<(counts[IDX] + (128 / ((R) > (C) ? (R) : (C))) - 1) /            \
                            (128 / ((R) > (C) ? (R) : (C))),                             \
                        128, 0, s[IDX]>>>(a, lists[IDX], counts[IDX]);
#define JPXLG_RVK(IDX, R, C, K)                                                          \
  if (counts[IDX])                                                                       \
    k_render_vb<R, C, K><<<(counts[IDX] + (128 / ((R) > (C) ? (R) : (C))) - 1) /         \
                               (128 / ((R) > (C) ? (R) : (C))),                          \
                           128, 0, s[IDX]>>>(a, lists[IDX], counts[IDX]);
  // shape classes in kShapeSel order: DCT8, 16x16, 32x32, 16x8, 8x16, 32x8,
  // 8x32, 32x16, 16x32, DCT2x2, 64x64, 64x32, 32x64 (rows x cols of samples)
  JPXLG_RV(0, 8, 8)
  JPXLG_RV(1, 16, 16)
  JPXLG_RV(2, 32, 32)
  JPXLG_RV(3, 16, 8)
  JPXLG_RV(4, 8, 16)
  JPXLG_RV(5, 32, 8)
  JPXLG_RV(6, 8, 32)
  JPXLG_RV(7, 32, 16)
  JPXLG_RV(8, 16, 32)
  JPXLG_RVK(9, 8, 8, 1)
  JPXLG_RV(10, 64, 64)
  JPXLG_RV(11, 64, 32)
  JPXLG_RV(12, 32, 64)
  JPXLG_RVK(13, 8, 8, 2)  // Hornuss
  JPXLG_RVK(14, 8, 8, 3)  // DCT4x4
  JPXLG_RVK(15, 8, 8, 4)  // DCT8x4
  JPXLG_RVK(16, 8, 8, 5)  // DCT4x8
  JPXLG_RVK(17, 8, 8, 6)  // AFV0..AFV3
  JPXLG_RVK(18, 8, 8, 7)
  JPXLG_RVK(19, 8, 8, 8)
  JPXLG_RVK(20, 8, 8, 9)
#undef JPXLG_RV
#undef JPXLG_RVK
}

// ---------------------------------------------------------------------------
// R2 — restoration.rs:148 gaborish_into: acc = fma(w, s, acc) over (dy, dx)
// in row-major order from 0, kernel from GaborKernel::new (:111, with FMA).
// ---------------------------------------------------------------------------

constexpr int kGT = 32;
__global__ void __launch_bounds__(256) k_gaborish(const float* __restrict__ in,
                                                  float* __restrict__ out, int w, int h,
                                                  float centre, float edge, float corner) {
  __shared__ float t[kGT + 2][kGT + 3];
  const size_t plane = (size_t)w * h;
  in += plane * blockIdx.z;
  out += plane * blockIdx.z;
  const int x0 = blockIdx.x * kGT, y0 = blockIdx.y * kGT;
  for (int i = threadIdx.x; i < (kGT + 2) * (kGT + 2); i += blockDim.x) {
    int lx = i % (kGT + 2), ly = i / (kGT + 2);
    int gx = mirror1d(x0 + lx - 1, w), gy = mirror1d(y0 + ly - 1, h);
    t[ly][lx] = in[(size_t)gy * w + gx];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kGT * kGT; i += blockDim.x) {
    int lx = i % kGT, ly = i / kGT;
    int gx = x0 + lx, gy = y0 + ly;
    if (gx >= w || gy >= h) continue;
    float acc = 0.0f;
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
      for (int dx = -1; dx <= 1; ++dx) {
        float wt = (dx == 0 && dy == 0) ? centre : ((dx == 0 || dy == 0) ? edge : corner);
        acc = __fmaf_rn(wt, t[ly + 1 + dy][lx + 1 + dx], acc);
      }
    out[(size_t)gy * w + gx] = acc;
  }
}

void launch_gaborish(const float* in, float* out, int w, int h, cudaStream_t s) {
  const float w1 = 0.115169525f, w2 = 0.061248592f;
  float unnorm = fmaf(4.0f, w2, fmaf(4.0f, w1, 1.0f));
  float scale = 1.0f / unnorm;
  dim3 grid((w + kGT - 1) / kGT, (h + kGT - 1) / kGT, 3);
  k_gaborish<<<grid, 256, 0, s>>>(in, out, w, h, scale, w1 * scale, w2 * scale);
}

// ---------------------------------------------------------------------------
// R3 — restoration.rs:619 epf_step_rows_impl.  Distances: per tap,
// d = fma(|a-b|, channel_scale[c], d) over channels then the cross (step 2:
// the pixel alone); weight max(0, fma(pos_mul*d, -inv_sigma, 1)) (exactly 1
// for zero distance); output sum_t fma(v, w, acc) / sum_t w.  Blocks with
// sigma < 0.3 are copied.  pos_mul = 2/3 on the 8x8 border of the reference
// pixel.  Mirrored padding of 3.
// ---------------------------------------------------------------------------

constexpr int kET = 32;
constexpr int kEP = 3;
constexpr int kES = kET + 2 * kEP;

template <int STEP>
__global__ void __launch_bounds__(256, 3) k_epf(const float* __restrict__ in, float* __restrict__ out,
                                             const float* __restrict__ sigma, int w, int h,
                                             float step_mul4) {
  __shared__ float t[3][kES][kES + 1];
  const size_t plane = (size_t)w * h;
  const int x0 = blockIdx.x * kET, y0 = blockIdx.y * kET;
  for (int i = threadIdx.x; i < kES * kES; i += blockDim.x) {
    int lx = i % kES, ly = i / kES;
    int gx = mirror1d(x0 + lx - kEP, w), gy = mirror1d(y0 + ly - kEP, h);
    size_t p = (size_t)gy * w + gx;
    t[0][ly][lx] = in[p];
    t[1][ly][lx] = in[plane + p];
    t[2][ly][lx] = in[2 * plane + p];
  }
  __syncthreads();
  const int bw = (w + 7) / 8;
  const float scale[3] = {40.0f, 5.0f, 3.5f};
  for (int i = threadIdx.x; i < kET * kET; i += blockDim.x) {
    int lx = i % kET, ly = i / kET;
    int gx = x0 + lx, gy = y0 + ly;
    if (gx >= w || gy >= h) continue;
    const int cx = lx + kEP, cy = ly + kEP;
    size_t p = (size_t)gy * w + gx;
    float bs = sigma[(size_t)(gy / 8) * bw + gx / 8];
    if (bs < 0.3f) {
      out[p] = t[0][cy][cx];
      out[plane + p] = t[1][cy][cx];
      out[2 * plane + p] = t[2][cy][cx];
      continue;
    }
    const float inv_sigma = step_mul4 / bs;
    const int rx = gx % 8, ry = gy % 8;
    const bool at_border = ry == 0 || ry == 7 || rx == 0 || rx == 7;
    const float pos_mul = at_border ? 2.0f / 3.0f : 1.0f;
    float sum_w = 0.0f, acc0 = 0.0f, acc1 = 0.0f, acc2 = 0.0f;
    constexpr int NT = STEP == 0 ? 13 : 5;
    // J.4.4 kernels: the 5-pixel cross, plus the diagonals and +-2 for step 0.
    constexpr int tkx[13] = {0, -1, 1, 0, 0, 1, 1, -1, -1, -2, 2, 0, 0};
    constexpr int tky[13] = {0, 0, 0, -1, 1, -1, 1, 1, -1, 0, 0, 2, -2};
    auto dist = [&](int kx, int ky) {
      float d = 0.0f;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if (STEP == 2) {
          d = __fmaf_rn(fabsf(t[c][cy][cx] - t[c][cy + ky][cx + kx]), scale[c], d);
        } else {
          const int ix[5] = {0, -1, 1, 0, 0}, iy[5] = {0, 0, 0, -1, 1};
#pragma unroll
          for (int q = 0; q < 5; ++q) {
            float av = t[c][cy + iy[q]][cx + ix[q]];
            float bv = t[c][cy + ky + iy[q]][cx + kx + ix[q]];
            d = __fmaf_rn(fabsf(av - bv), scale[c], d);
          }
        }
      }
      return d;
    };
    auto weight = [&](float d) {
      float sd = pos_mul * d;
      if (sd == 0.0f) return 1.0f;
      float v = __fmaf_rn(sd, -inv_sigma, 1.0f);
      return v > 0.0f ? v : 0.0f;
    };
    // The centre tap's distance sums |s - s| over the centre's own patch:
    // exactly 0 (weight 1) when every sample there is finite, not a number
    // otherwise.  The next tap's distance takes |s - s'| of the same samples
    // with positive scales, so it is finite only if they all are; then the
    // centre's terms are skipped, else evaluated as written.
    const float d1 = dist(tkx[1], tky[1]);
    float wts[NT];
    wts[0] = isfinite(d1) ? 1.0f : weight(dist(0, 0));
    wts[1] = weight(d1);
#pragma unroll
    for (int tp = 0; tp < NT; ++tp) {
      const int kx = tkx[tp], ky = tky[tp];
      const float wt = tp < 2 ? wts[tp] : weight(dist(kx, ky));
      sum_w += wt;
      acc0 = __fmaf_rn(t[0][cy + ky][cx + kx], wt, acc0);
      acc1 = __fmaf_rn(t[1][cy + ky][cx + kx], wt, acc1);
      acc2 = __fmaf_rn(t[2][cy + ky][cx + kx], wt, acc2);
    }
    out[p] = acc0 / sum_w;
    out[plane + p] = acc1 / sum_w;
    out[2 * plane + p] = acc2 / sum_w;
  }
}

void launch_epf_step(int step, const float* in, float* out, const float* sigma, int w, int h,
                     cudaStream_t s) {
  // restoration.rs:356 epf_inv_sigma: step_multiplier * 4 * (1 - sqrt(0.5)) / sigma,
  // evaluated left to right; the numerator is formed here once.
  float sc = step == 0 ? 0.9f : (step == 1 ? 1.0f : 6.5f);
  float sm = 1.65f * sc;
  float num = sm * 4.0f * (1.0f - sqrtf(0.5f));
  dim3 grid((w + kET - 1) / kET, (h + kET - 1) / kET);
  if (step == 0) k_epf<0><<<grid, 256, 0, s>>>(in, out, sigma, w, h, num);
  else if (step == 1) k_epf<1><<<grid, 256, 0, s>>>(in, out, sigma, w, h, num);
  else k_epf<2><<<grid, 256, 0, s>>>(in, out, sigma, w, h, num);
}

// ---------------------------------------------------------------------------
// R4 — color.rs:673 OpsinInverse::convert (cube without pow, FMA matrix),
// then the output: linear planes; 8-bit sRGB as the decoder writes it
// (decode.rs:3498 round(linear_to_srgb(v)*255) clamped) found by binary
// search in the host-bisected level thresholds (plan-render lib.rs:333,
// identical by construction); or the level's linear value (lib.rs:437).
// ---------------------------------------------------------------------------

__device__ __forceinline__ int level_of(float x, const float* thr, int n) {
  if (!isfinite(x)) return 0;
  int lo = 0, hi = n;  // count of thresholds <= x
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (thr[mid] <= x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// The linear value of x's level among n + 1 levels, for deep outputs
// (65536 levels): the level is first estimated from the transfer curve with
// the fast powf (its error, a few ulp, moves the estimate by well under one
// level), then confirmed against the exact thresholds around it, stepping by
// one where the estimate sits on the wrong side; one 16-byte load of the
// bracket table per try gives both thresholds and the level's value.  The
// binary search remains the fallback.  The thresholds decide, so the result
// is exactly the bisected level's.
__device__ __forceinline__ float level_value_bracketed(float x, const float4* __restrict__ br,
                                                       const float* __restrict__ thr,
                                                       const float* __restrict__ levels, int n,
                                                       float maxv) {
  if (!isfinite(x)) return __ldg(&levels[0]);
  float a = fabsf(x);
  float e = a <= 0.0031308f ? 12.92f * a : 1.055f * __powf(a, 1.0f / 2.4f) - 0.055f;
  float s = rintf((x < 0.0f ? -e : e) * maxv);
  int est = (int)fminf(fmaxf(s, 0.0f), maxv);
#pragma unroll 1
  for (int it = 0; it < 4; ++it) {
    const float4 v = __ldg(&br[est]);
    const bool lo_ok = v.x <= x, hi_ok = x < v.y;
    if (lo_ok && hi_ok) return v.z;
    est += lo_ok ? 1 : -1;
  }
  return __ldg(&levels[level_of(x, thr, n)]);
}

template <int KIND>
__global__ void __launch_bounds__(256) k_colour_out(const float* __restrict__ xyb, size_t n,
                                                    const float* __restrict__ thr,
                                                    const float* __restrict__ levels,
                                                    const float4* __restrict__ bracket, int nlev,
                                                    void* __restrict__ out,
                                                    float* __restrict__ pxyb) {
  __shared__ float s_thr[255];
  __shared__ float s_lev[256];
  if (KIND == 2 || (KIND == 3 && nlev <= 256)) {
    for (int i = threadIdx.x; i < nlev - 1; i += blockDim.x) s_thr[i] = thr[i];
    for (int i = threadIdx.x; i < nlev; i += blockDim.x) s_lev[i] = levels[i];
    __syncthreads();
  }
  const float* T = (nlev <= 256) ? s_thr : thr;
  const float* LV = (nlev <= 256) ? s_lev : levels;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    float x = xyb[i], y = xyb[n + i], b = xyb[2 * n + i];
    float gm[3] = {y + x, y - x, b};
    float mix[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      float v = gm[c] - c_opsin_bias_cbrt[c];
      mix[c] = ((v * v) * v + c_opsin_bias[c]) * 1.0f;
    }
    float rgb[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      float acc = 0.0f;
#pragma unroll
      for (int c = 0; c < 3; ++c) acc = __fmaf_rn(c_opsin_m[r * 3 + c], mix[c], acc);
      rgb[r] = acc;
    }
    if (KIND == 1) {
      float* o = (float*)out;
      o[i] = rgb[0];
      o[n + i] = rgb[1];
      o[2 * n + i] = rgb[2];
    } else if (KIND == 4) {
      // jpxl-core color.rs:490 linear_to_srgb, odd-symmetric, unclipped.
      float* o = (float*)out;
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const float v = rgb[q], av = fabsf(v);
        const float e = av <= 0.0031308f ? 12.92f * av : 1.055f * powf(av, 1.0f / 2.4f) - 0.055f;
        o[q * n + i] = v < 0.0f ? -e : e;
      }
    } else if (KIND == 2) {
      uint8_t* o = (uint8_t*)out;
      o[3 * i] = (uint8_t)level_of(rgb[0], T, nlev - 1);
      o[3 * i + 1] = (uint8_t)level_of(rgb[1], T, nlev - 1);
      o[3 * i + 2] = (uint8_t)level_of(rgb[2], T, nlev - 1);
    } else {
      float lin[3];
      if (nlev <= 256) {
#pragma unroll
        for (int q = 0; q < 3; ++q) lin[q] = LV[level_of(rgb[q], T, nlev - 1)];
      } else {
        const float maxv = (float)(nlev - 1);
#pragma unroll
        for (int q = 0; q < 3; ++q)
          lin[q] = level_value_bracketed(rgb[q], bracket, T, LV, nlev - 1, maxv);
      }
      float* o = (float*)out;
      o[i] = lin[0];
      o[n + i] = lin[1];
      o[2 * n + i] = lin[2];
      // The metric's positive XYB of the rendered pixel (candidate side of
      // SSIMULACRA2's first scale), when the caller scores it next.
      if (pxyb) {
        float px[3];
        positive_xyb(lin[0], lin[1], lin[2], px);
        pxyb[i] = px[0];
        pxyb[n + i] = px[1];
        pxyb[2 * n + i] = px[2];
      }
    }
  }
}

void launch_colour_out(const float* xyb, int w, int h, int out_kind, const float* thresholds,
                       const float* levels, const float4* bracket, int nlevels, void* out,
                       float* pxyb, int num_sms, cudaStream_t s) {
  size_t n = (size_t)w * h;
  int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)num_sms * 8);
  if (blocks < 1) blocks = 1;
  if (out_kind == 1)
    k_colour_out<1><<<blocks, 256, 0, s>>>(xyb, n, thresholds, levels, bracket, nlevels, out,
                                           nullptr);
  else if (out_kind == 2)
    k_colour_out<2><<<blocks, 256, 0, s>>>(xyb, n, thresholds, levels, bracket, nlevels, out,
                                           nullptr);
  else if (out_kind == 4)
    k_colour_out<4><<<blocks, 256, 0, s>>>(xyb, n, thresholds, levels, bracket, nlevels, out,
                                           nullptr);
  else
    k_colour_out<3><<<blocks, 256, 0, s>>>(xyb, n, thresholds, levels, bracket, nlevels, out,
                                           pxyb);
}

// ---------------------------------------------------------------------------
// R5 — LF of a decoded frame (jpxl-decode vardct/lf.rs:448 dequantize_lf and
// :351 adaptive_smoothing, decode.rs:3246 over the whole frame): dequantize
// (m * q / 2^extra_precision), apply the LF CfL, then smooth interior cells.
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(256) k_lf_dequant(const int32_t* __restrict__ lfq, size_t nb,
                                                    float m0, float m1, float m2, float div,
                                                    float kx, float kb, float* __restrict__ out) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nb;
       i += (size_t)gridDim.x * blockDim.x) {
    const float dx = m0 * (float)lfq[i] / div;
    const float dy = m1 * (float)lfq[nb + i] / div;
    const float db = m2 * (float)lfq[2 * nb + i] / div;
    out[i] = dx + kx * dy;
    out[nb + i] = dy;
    out[2 * nb + i] = db + kb * dy;
  }
}

__global__ void __launch_bounds__(256) k_lf_smooth(const float* __restrict__ in, int bw, int bh,
                                                   float m0, float m1, float m2,
                                                   float* __restrict__ out) {
  const size_t nb = (size_t)bw * bh;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nb;
       i += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % bw), y = (int)(i / bw);
    if (x == 0 || y == 0 || x == bw - 1 || y == bh - 1) {
      for (int c = 0; c < 3; ++c) out[c * nb + i] = in[c * nb + i];
      continue;
    }
    float wa[3], sv[3];
    for (int c = 0; c < 3; ++c) {
      const float* p = in + c * nb;
      auto g = [&](int dx, int dy) { return p[(size_t)(y + dy) * bw + x + dx]; };
      sv[c] = g(0, 0);
      wa[c] = (0.052262735f * sv[c] + 0.2034514f * (((g(-1, 0) + g(1, 0)) + g(0, -1)) + g(0, 1))) +
              0.03348292f * (((g(-1, -1) + g(1, -1)) + g(-1, 1)) + g(1, 1));
    }
    const float m[3] = {m0, m1, m2};
    float gap = 0.5f;
    for (int c = 0; c < 3; ++c) gap = fmaxf(gap, fabsf(wa[c] - sv[c]) / m[c]);
    const float factor = fmaxf(3.0f - 4.0f * gap, 0.0f);
    for (int c = 0; c < 3; ++c) out[c * nb + i] = (wa[c] - sv[c]) * factor + sv[c];
  }
}

void launch_lf_prepare(const int32_t* lfq, int bw, int bh, const float m[3], float div, float kx,
                       float kb, bool smooth, float* tmp, float* out, int num_sms,
                       cudaStream_t s) {
  const size_t nb = (size_t)bw * bh;
  const int blocks = (int)std::max<size_t>(1, std::min<size_t>((nb + 255) / 256, num_sms * 4));
  k_lf_dequant<<<blocks, 256, 0, s>>>(lfq, nb, m[0], m[1], m[2], div, kx, kb, smooth ? tmp : out);
  if (smooth) k_lf_smooth<<<blocks, 256, 0, s>>>(tmp, bw, bh, m[0], m[1], m[2], out);
}

// The special transforms on given blocks, one thread per block (a
// diagnostic of jpxlg_diag_special_blocks): kind 1 DCT2x2, 2..9 as
// special_block.
template <int KIND>
__global__ void __launch_bounds__(64) k_special_diag(const float* __restrict__ coef, int n,
                                                     float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float b[64], o[64];
#pragma unroll
  for (int k = 0; k < 64; ++k) b[k] = coef[(size_t)i * 64 + k];
  if constexpr (KIND == 1) {
    dct2x2_block(b);
#pragma unroll
    for (int k = 0; k < 64; ++k) o[k] = b[k];
  } else {
    special_block<KIND>(b, o);
  }
#pragma unroll
  for (int k = 0; k < 64; ++k) out[(size_t)i * 64 + k] = o[k];
}

bool launch_special_diag(int kind, const float* coef, int n, float* out, cudaStream_t s) {
  const int blocks = (n + 63) / 64;
  switch (kind) {
    case 1: k_special_diag<1><<<blocks, 64, 0, s>>>(coef, n, out); return true;
    case 2: k_special_diag<2><<<blocks, 64, 0, s>>>(coef, n, out); return true;
    case 3: k_special_diag<3><<<blocks, 64, 0, s>>>(coef, n, out); return true;
    case 4: k_special_diag<4><<<blocks, 64, 0, s>>>(coef, n, out); return true;
    case 5: k_special_diag<5><<<blocks, 64, 0, s>>>(coef, n, out); return true;
    case 6: k_special_diag<6><<<blocks, 64, 0, s>>>(coef, n, out); return true;
    case 7: k_special_diag<7><<<blocks, 64, 0, s>>>(coef, n, out); return true;
    case 8: k_special_diag<8><<<blocks, 64, 0, s>>>(coef, n, out); return true;
    case 9: k_special_diag<9><<<blocks, 64, 0, s>>>(coef, n, out); return true;
    default: return false;
  }
}

void upload_afv(const double* basis, cudaStream_t s) {
  cudaMemcpyToSymbolAsync(g_afv, basis, sizeof(double) * 256, 0, cudaMemcpyHostToDevice, s);
}

void upload_dct64(const float* matrix, cudaStream_t s) {
  cudaMemcpyToSymbolAsync(g_dct64, matrix, sizeof(float) * 64 * 64, 0, cudaMemcpyHostToDevice, s);
}

void upload_render_constants(const float* opsin_m, const float* opsin_bias,
                             const float* opsin_bias_cbrt, cudaStream_t s) {
  cudaMemcpyToSymbolAsync(c_opsin_m, opsin_m, sizeof(float) * 9, 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_opsin_bias, opsin_bias, sizeof(float) * 3, 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_opsin_bias_cbrt, opsin_bias_cbrt, sizeof(float) * 3, 0,
                          cudaMemcpyHostToDevice, s);
}

}  // namespace jpxlg
