// jpxlg_common.cuh — device helpers shared by the sm_103a kernels of the
// lossy VarDCT pixel path: exact-parity cube roots, mirroring, the transform
// table, the DCT butterflies and the error word.
//
// Everything here is compiled with -fmad=false: a*b+c always rounds twice,
// exactly as the Rust reference (which never contracts), and __fmaf_rn is
// written out exactly where the reference calls mul_add.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "jpxlg_defs.cuh"

namespace jpxlg {

// ---- mirroring (18181-1 5.2 Mirror1D) ---------------------------------------
__device__ __forceinline__ int mirror1d(int c, int size) {
  // Bounded: a coordinate at most a few samples outside needs at most a few
  // reflections even for a one-sample plane.
  for (int i = 0; i < 64; ++i) {
    if (c < 0) c = -c - 1;
    else if (c >= size) c = 2 * size - 1 - c;
    else return c;
  }
  return 0;
}

// ---- exact-parity cube roots -----------------------------------------------
// The reference has two cube roots, each f64 iteration rounded once to f32:
// jpxl-core simd.rs:36 (estimate + 2 Halley steps) and jpxl-perceptual
// color.rs:46 (estimate + 4 Newton steps).  Both land within ~2^-24 ulp of the
// exact cube root, i.e. they return the correctly rounded cube root unless
// the exact root lies within that distance of a rounding midpoint.  The fast
// path below finds the correctly rounded root in f32 arithmetic (CUDA's
// cbrtf, then a double-float residual that places the exact root to within
// 2^-21 ulp); where the root lies within 2^-17 ulp of a midpoint, or the input
// is outside the verified range, it runs the reference's own f64 iteration,
// so the result is the reference's bit for bit either way.

static __device__ __noinline__ float cbrt_core_f64(float value) {
  const uint32_t B1 = 709958130u, B2 = 642849266u;
  uint32_t bits = __float_as_uint(value);
  uint32_t magnitude = bits & 0x7fffffffu;
  if (magnitude == 0 || magnitude >= 0x7f800000u) return value;
  uint32_t estimate;
  if (magnitude < 0x00800000u) {
    float scaled = value * 16777216.0f;
    estimate = (__float_as_uint(scaled) & 0x7fffffffu) / 3u + B2;
  } else {
    estimate = magnitude / 3u + B1;
  }
  double x = (double)value;
  double t = (double)__uint_as_float((bits & 0x80000000u) | estimate);
  for (int i = 0; i < 2; ++i) {
    double r = (t * t) * t;
    t = (t * ((x + x) + r)) / ((x + r) + r);
  }
  return (float)t;
}

static __device__ __noinline__ float cbrt_perceptual_f64(float value) {
  double x = (double)value;
  double a = fabs(x);
  unsigned long long ab = (unsigned long long)__double_as_longlong(a);
  double y = __longlong_as_double((long long)(ab / 3ull + (0x2A9F7893ull << 32)));
  for (int i = 0; i < 4; ++i) y -= (((y * y) * y) - a) / ((3.0 * y) * y);
  float root = (float)y;
  float signed_root = x < 0.0 ? -root : root;
  if (value == 0.0f || !isfinite(value)) return value;
  return signed_root;
}

// Correctly rounded cbrt of a > 0 in [2^-90, 2^90]; sets *ok = false where
// the decision is not certain to 2^-17 ulp.
__device__ __forceinline__ float cbrt_cr_fast(float a, bool* ok) {
  float y = cbrtf(a);
  uint32_t yb = __float_as_uint(y);
  float p = y * y;
  float e1 = __fmaf_rn(y, y, -p);   // y*y = p + e1 exactly
  float q = p * y;
  float e2 = __fmaf_rn(p, y, -q);   // p*y = q + e2 exactly
  float e3 = e1 * y;                // e1*y, rounded (relative 2^-48 of y^3)
  float d = (q - a) + (e2 + e3);    // y^3 - a; q - a is exact (Sterbenz)
  int e = (int)((yb >> 23) & 0xffu) - 127;
  float inv_ulp = __uint_as_float((uint32_t)(127 + 23 - e) << 23);  // 2^(23-e)
  // (cbrt(a) - y) in ulps of y.  The quotient needs ~2^-20 relative accuracy
  // only (|delta| < 2.5 against a 2^-17 decision margin), so the fast
  // division (at most 2 ulp off) serves.
  float delta = __fdividef(-d, 3.0f * p) * inv_ulp;
  float k = rintf(delta);
  float frac = fabsf(delta - k);
  *ok = frac < 0.5f - 7.62939453125e-06f && fabsf(delta) < 2.5f;  // 2^-17
  int ki = (int)k;
  uint32_t mant = yb & 0x7fffffu;
  if ((ki < 0 && mant < (uint32_t)(-ki)) || (ki > 0 && mant + (uint32_t)ki > 0x7fffffu))
    *ok = false;  // the step would cross a binade, where the ulp changes
  return __uint_as_float(yb + ki);
}

// jpxl-core simd.rs:36 reproducible_cbrt, bit for bit.
__device__ __forceinline__ float cbrt_core(float v) {
  float a = fabsf(v);
  if (a >= 8.0e-28f && a <= 1.2e27f) {
    bool ok;
    float r = cbrt_cr_fast(a, &ok);
    if (ok) return copysignf(r, v);
  }
  return cbrt_core_f64(v);
}

// jpxl-perceptual color.rs:46 reproducible_cbrt, bit for bit.
__device__ __forceinline__ float cbrt_perceptual(float v) {
  float a = fabsf(v);
  if (a >= 8.0e-28f && a <= 1.2e27f) {
    bool ok;
    float r = cbrt_cr_fast(a, &ok);
    if (ok) return copysignf(r, v);
  }
  return cbrt_perceptual_f64(v);
}

// ---- SSIMULACRA2 positive XYB (jpxl-perceptual color.rs:66) ------------------
// Opsin mix without FMA, the metric's reproducible cube root, then
// [14x + 0.42, y + 0.01, b - y + 0.55].
__device__ __forceinline__ void positive_xyb(float r, float g, float b, float* o) {
  float lm = 0.3f * r + 0.622f * g + 0.078f * b + 0.0037930734f;
  float mm = 0.23f * r + 0.692f * g + 0.078f * b + 0.0037930734f;
  float sm = 0.2434227f * r + 0.2047674f * g + 0.5518099f * b + 0.0037930734f;
  float lg = cbrt_perceptual(lm) - 0.1559542f;
  float mg = cbrt_perceptual(mm) - 0.1559542f;
  float sg = cbrt_perceptual(sm) - 0.1559542f;
  float x = 0.5f * (lg - mg);
  float y = 0.5f * (lg + mg);
  o[0] = x * 14.0f + 0.42f;
  o[1] = y + 0.01f;
  o[2] = (sg - y) + 0.55f;
}

// ---- paired f32 arithmetic (sm_100 family) ----------------------------------
// Two f32 lanes in one 64-bit register (lane 0 in the low word).  Each lane
// of add/sub.rn.f32x2 rounds exactly as the scalar f32 operation.
//
// Products need care: the assembler fuses a paired multiply with a following
// paired add into one rounding, whatever the rounding modifier or -fmad
// setting (measured on sm_103a: mul.rn.f32x2 then add.rn.f32x2 differed
// from the scalar mul-then-add in about one result in nine, and so did
// fma.rn.f32x2(a, b, -0.0) with the -0.0 as an immediate).  f2_mul is
// therefore fma.rn.f32x2(a, b, z) with z = (-0.0, -0.0) supplied at run time
// (a kernel argument), which the assembler cannot see through: one rounding
// of a*b, signed zeros included, exactly the scalar product.
typedef unsigned long long f2;
__device__ __forceinline__ f2 f2_pack(float lo, float hi) {
  f2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ float f2_lo(f2 v) {
  float a;
  asm("mov.b64 {%0, _}, %1;" : "=f"(a) : "l"(v));
  return a;
}
__device__ __forceinline__ float f2_hi(f2 v) {
  float b;
  asm("mov.b64 {_, %0}, %1;" : "=f"(b) : "l"(v));
  return b;
}
__device__ __forceinline__ f2 f2_add(f2 a, f2 b) {
  f2 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b) {
  f2 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
// a * b per lane; nz must be the run-time pair (-0.0f, -0.0f).
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b, f2 nz) {
  f2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(nz));
  return d;
}
// a * b + c per lane with one rounding (the paired __fmaf_rn).
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c) {
  f2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

// ---- double-float (f32 pair) sums --------------------------------------------
// Products of two f32 are split exactly (two_prod); sums keep hi + lo to
// about 2^-46 per addition, so a sum over n terms lies within
// n * 2^-46 * sum|t| of the exact sum, at f32 issue rates (GB300's FP64
// rate is a small fraction of its FP32 rate).  hi + lo converts to f64
// exactly.
struct DF {
  float hi, lo;
};
__device__ __forceinline__ DF df_two_prod(float a, float b) {
  float p = a * b;
  return {p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
  float s = a.hi + b.hi;
  float bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b.hi - bb);
  e = e + (a.lo + b.lo);
  float h = s + e;
  return {h, e - (h - s)};
}
// Fixed-order butterfly over a warp; every lane ends with the same sum.
__device__ __forceinline__ DF df_warp_sum(DF v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    DF w{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
    v = df_add(v, w);
  }
  return v;
}
__device__ __forceinline__ double df_value(DF v) { return (double)v.hi + (double)v.lo; }

// ---- reconstruct.rs:50 bias_adjust ------------------------------------------
// q -> q * bias for |q| <= 1, else q - 0.145 / q.  The expression is odd in q
// under round-to-nearest, so |q| < kBiasQuotN reads 0.145f / |q| from a table
// that the host fills with the same IEEE division, and the sign is applied
// last; larger |q| divide.
constexpr int kBiasQuotN = 256;
extern __device__ float g_bias_quot[kBiasQuotN];

__device__ __forceinline__ float bias_adjust_q(int32_t q, float bias) {
  const float f = (float)q;
  if (q >= -1 && q <= 1) return f * bias;
  const int32_t aq = q < 0 ? -q : q;
  const float af = (float)aq;
  const float t = aq < kBiasQuotN ? __ldg(&g_bias_quot[aq]) : 0.145f / af;
  const float r = af - t;
  return q < 0 ? -r : r;
}

// ---- DCT butterflies (jpxl-core dct.rs:235-465) -----------------------------
// Orthonormal DCT-IV leaves live in constant memory (filled by the host from
// the reference's first-row magnitudes); loops over them are unrolled, so
// every coefficient is a constant-bank operand.
extern __constant__ float c_iv4[16];
extern __constant__ float c_iv8[64];
extern __constant__ float c_iv16[256];

constexpr float kSqrtHalf = 0.707106769f;
constexpr float kCosPi8 = 0.9238795f;
constexpr float kSinPi8 = 0.38268343f;

template <int M>
__device__ __forceinline__ float iv_coef(int u, int n) {
  if constexpr (M == 4) return c_iv4[u * 4 + n];
  else if constexpr (M == 8) return c_iv8[u * 8 + n];
  else return c_iv16[u * 16 + n];
}

template <int M>
__device__ __forceinline__ void dct_iv(float* v) {
  if constexpr (M == 2) {
    float x0 = v[0], x1 = v[1];
    v[0] = kCosPi8 * x0 + kSinPi8 * x1;
    v[1] = kSinPi8 * x0 - kCosPi8 * x1;
  } else {
    float x[M];
#pragma unroll
    for (int i = 0; i < M; ++i) x[i] = v[i];
#pragma unroll
    for (int u = 0; u < M; ++u) {
      float acc = 0.0f;
#pragma unroll
      for (int n = 0; n < M; ++n) acc = acc + iv_coef<M>(u, n) * x[n];
      v[u] = acc;
    }
  }
}

__device__ __forceinline__ void dct_ii_2(float* v) {
  float x0 = v[0], x1 = v[1];
  v[0] = (x0 + x1) * kSqrtHalf;
  v[1] = (x0 - x1) * kSqrtHalf;
}

template <int N>
__device__ __forceinline__ void dct_ii(float* v) {
  if constexpr (N == 1) {
  } else if constexpr (N == 2) {
    dct_ii_2(v);
  } else {
    constexpr int H = N / 2;
    float even[H], odd[H];
#pragma unroll
    for (int k = 0; k < H; ++k) {
      even[k] = v[k] + v[N - 1 - k];
      odd[k] = v[k] - v[N - 1 - k];
    }
    dct_ii<H>(even);
    dct_iv<H>(odd);
#pragma unroll
    for (int k = 0; k < H; ++k) {
      v[2 * k] = even[k] * kSqrtHalf;
      v[2 * k + 1] = odd[k] * kSqrtHalf;
    }
  }
}

template <int N>
__device__ __forceinline__ void dct_iii(float* v) {
  if constexpr (N == 1) {
  } else if constexpr (N == 2) {
    dct_ii_2(v);
  } else {
    constexpr int H = N / 2;
    float even[H], odd[H];
#pragma unroll
    for (int k = 0; k < H; ++k) {
      even[k] = v[2 * k] * kSqrtHalf;
      odd[k] = v[2 * k + 1] * kSqrtHalf;
    }
    dct_iii<H>(even);
    dct_iv<H>(odd);
#pragma unroll
    for (int k = 0; k < H; ++k) {
      v[k] = even[k] + odd[k];
      v[N - 1 - k] = even[k] - odd[k];
    }
  }
}

// dct.rs:731/749: normative scaling after the butterfly.  The factors are
// 1/sqrtf(N) and sqrtf(N) in f32, as the reference computes them.
template <int N>
__device__ __forceinline__ float fwd_factor() {
  return 1.0f / sqrtf((float)N);
}
template <int N>
__device__ __forceinline__ void dct_1d(float* v) {
  dct_ii<N>(v);
  const float f = 1.0f / __fsqrt_rn((float)N);
#pragma unroll
  for (int i = 0; i < N; ++i) v[i] *= f;
}
template <int N>
__device__ __forceinline__ void idct_1d(float* v) {
  dct_iii<N>(v);
  const float f = __fsqrt_rn((float)N);
#pragma unroll
  for (int i = 0; i < N; ++i) v[i] *= f;
}

// ---- LF rectangles (dct.rs:956 on the LLF corner of a varblock) -------------
template <int N>
__device__ __forceinline__ void dct_small(float* v) {
  if (N == 2) dct_1d<2>(v);
  else if (N == 4) dct_1d<4>(v);
  else if (N == 8) dct_1d<8>(v);
}

// dct.rs:956 DCT_2D of an LF rectangle cy x cx (cy <= cx, both <= 8) in place.
__device__ __forceinline__ void dct2d_small(float* m, int rows, int cols) {
  float col[8], s[64];
  // column pass (length rows) on rows x cols
  for (int c = 0; c < cols; ++c) {
    for (int r = 0; r < rows; ++r) col[r] = m[r * cols + c];
    if (rows == 2) dct_small<2>(col);
    else if (rows == 4) dct_small<4>(col);
    else if (rows == 8) dct_small<8>(col);
    for (int r = 0; r < rows; ++r) m[r * cols + c] = col[r];
  }
  // transpose to cols x rows, column pass (length cols)
  for (int r = 0; r < rows; ++r)
    for (int c = 0; c < cols; ++c) s[c * rows + r] = m[r * cols + c];
  for (int r = 0; r < rows; ++r) {
    for (int c = 0; c < cols; ++c) col[c] = s[c * rows + r];
    if (cols == 2) dct_small<2>(col);
    else if (cols == 4) dct_small<4>(col);
    else if (cols == 8) dct_small<8>(col);
    for (int c = 0; c < cols; ++c) s[c * rows + r] = col[c];
  }
  // cols x rows result; landscape => transpose back when cols > rows
  if (cols <= rows) {
    for (int i = 0; i < rows * cols; ++i) m[i] = s[i];
  } else {
    for (int c = 0; c < cols; ++c)
      for (int r = 0; r < rows; ++r) m[r * cols + c] = s[c * rows + r];
  }
}


}  // namespace jpxlg
