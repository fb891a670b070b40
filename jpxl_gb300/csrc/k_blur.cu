// k_blur.cu — SSIMULACRA2's Gaussian (jpxl-perceptual blur.rs) evaluated to
// the reference's f32 outputs, and the candidate side of one scale.
//
// blur.rs runs along every row, then along every column of that result,
// three f64 two-pole resonators (feedback 2 cos(k pi / 10) and -1, k = 1, 3,
// 5) fed with s_j = f32(x[j-6] + x[j+4]), and rounds their summed output to
// f32 once per sample (blur.rs:164 step, :414 horizontal_padded, :574
// vertical_row).  Split s_j = (x[j-6] + x[j+4]) + e_j, with e_j the rounding
// error of the f32 pair sum (exact in f32).  The resonators fed with the
// exact pair sums have a finite response: the 9-tap symmetric FIR
// FIR_j = sum_d tap_d x[j+d], |d| <= 4 (the fifth harmonics cancel).  Fed
// with the e's they ring without damping for the rest of the line: R_j.  So
//
//     output_j = f32(FIR_j + R_j)
//
// up to the reference's own f64 noise (~1e-16 relative).  R is a size- and
// content-dependent ripple of order 1e-7 of the signal; a plain f32 FIR
// misses it and lands tens of ulps away, which SSIMULACRA2's variance
// differences (sigma - mu^2 with C2 = 0.0009) amplify into score errors of
// a tenth of a point on large near-identical pairs.  Here FIR_j is a
// double-float dot product (exact pair sums, exact products, compensated
// accumulation; taps as hi + lo from the f64 recursion's impulse response)
// and R_j comes from f32 resonators (R's own relative error of 1e-6 is far
// below an output ulp); one final f32 addition rounds FIR_j + R_j.
//
// Lines are split into segments.  Each segment runs its resonators from
// rest; a scan over the segments (after L steps the state is M^L times the
// entry state plus the segment's own response, M the resonator's 2x2 step
// matrix) gives each segment its entry state; each segment adds the
// homogeneous response of that state to its R from rest, and the FIR
// outputs, independent of one another, are formed in parallel.  Arithmetic
// is paired (two f32 lanes per instruction, each rounded as the scalar
// operation): rows two at a time in the row pass, columns two at a time in
// the column pass.
//   B1 k_blur_rows<NQ>     one CTA per row pair and channel, one segment per
//                          thread, the scan across the CTA's threads; NQ
//                          quantities x, x*x (and r*x), products rounded to
//                          f32 as blur.rs:395 forms them
//   B2 k_blur_col_out<NQ>  one CTA per 32-row segment of a 32-column strip
//                          and channel: the ripple from rest per column and
//                          quantity, the chained scan over the strip's
//                          segments (each CTA waits, boundedly, for the
//                          previous segment's published state; CTAs take
//                          their segments in the order they start), then the
//                          outputs; NQ = 2 writes mu and sigma11
//                          (reference.rs:90), NQ = 3 evaluates pool.rs:248's
//                          per-pixel terms on the blurred mu2, sigma22,
//                          sigma12 and writes one row of partial sums per
//                          tile
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

#include "jpxlg_common.cuh"
#include "jpxlg_internal.h"
#include "jpxlg_kernels.h"

namespace jpxlg {

struct BlurConsts {
  float a[3], b[3];    // MUL_IN and MUL_PREV (blur.rs:41/:47) in f32, for the ripple
  float th[5], tl[5];  // FIR taps (centre, +-1 .. +-4) as hi + lo
  // U[k][n] = sin((n+1) w_k) / sin(w_k), w_k = (2k+1) pi / 10: M_k^n is
  // [[U[n], -U[n-1]], [U[n-1], -U[n-2]]] (period 20 in n; U[-1] = 0).
  float U[3][20];
};
__constant__ BlurConsts c_blur;

// The constants as lane pairs for the paired forms, and the pair (+0, +0)
// for negations.
struct BlurPairs {
  f2 a[3], b[3], th[5], tl[5], nth[5], ntl[5], z;  // nth, ntl: the taps negated
};
__constant__ BlurPairs c_blur2;

// blur.rs:41 / :47.
static const double kMulIn[3] = {0.05529523572608661, -0.05883668702694998,
                                 0.012955819110517063};
static const double kMulPrev[3] = {1.902113032590307, 1.1755705045849463,
                                   1.2246467991473532e-16};

void upload_blur_consts(cudaStream_t s) {
  BlurConsts bc;
  for (int k = 0; k < 3; ++k) {
    bc.a[k] = (float)kMulIn[k];
    bc.b[k] = (float)kMulPrev[k];
  }
  // Tap d: the f64 recursion's response at output p + d to a unit sample at
  // p, the sample entering as the right (x[j+4]) and later the left
  // (x[j-6]) member of the pair sums.
  for (int d = 0; d <= 4; ++d) {
    double prev[3] = {0, 0, 0}, prev2[3] = {0, 0, 0}, out = 0.0;
    const int p = 16;
    for (int j = 0; j <= p + d; ++j) {
      const double s = (j + 4 == p ? 1.0 : 0.0) + (j - 6 == p ? 1.0 : 0.0);
      double o[3];
      for (int k = 0; k < 3; ++k) o[k] = s * kMulIn[k] + kMulPrev[k] * prev[k] - prev2[k];
      for (int k = 0; k < 3; ++k) {
        prev2[k] = prev[k];
        prev[k] = o[k];
      }
      out = (o[0] + o[1]) + o[2];
    }
    bc.th[d] = (float)out;
    bc.tl[d] = (float)(out - (double)bc.th[d]);
  }
  for (int k = 0; k < 3; ++k) {
    const double w = (2 * k + 1) * M_PI / 10.0;
    for (int m = 0; m < 20; ++m) bc.U[k][m] = (float)(std::sin((m + 1) * w) / std::sin(w));
  }
  cudaMemcpyToSymbolAsync(c_blur, &bc, sizeof(bc), 0, cudaMemcpyHostToDevice, s);
  BlurPairs bp;
  auto pair = [](float v) {
    uint32_t u;
    std::memcpy(&u, &v, 4);
    return ((unsigned long long)u << 32) | u;
  };
  for (int k = 0; k < 3; ++k) {
    bp.a[k] = pair(bc.a[k]);
    bp.b[k] = pair(bc.b[k]);
  }
  for (int d = 0; d < 5; ++d) {
    bp.th[d] = pair(bc.th[d]);
    bp.tl[d] = pair(bc.tl[d]);
    bp.nth[d] = pair(-bc.th[d]);
    bp.ntl[d] = pair(-bc.tl[d]);
  }
  bp.z = 0ull;
  cudaMemcpyToSymbolAsync(c_blur2, &bp, sizeof(bp), 0, cudaMemcpyHostToDevice, s);
}

// M_k^steps for the three resonators (row-major 2x2 acting on (o[j], o[j-1])),
// by repeated squaring in f64.
static void resonator_power(long long steps, float out[3][4]) {
  for (int k = 0; k < 3; ++k) {
    double r[4] = {1, 0, 0, 1};
    double m[4] = {kMulPrev[k], -1.0, 1.0, 0.0};
    long long e = steps;
    while (e > 0) {
      if (e & 1) {
        const double t[4] = {r[0] * m[0] + r[1] * m[2], r[0] * m[1] + r[1] * m[3],
                             r[2] * m[0] + r[3] * m[2], r[2] * m[1] + r[3] * m[3]};
        for (int i = 0; i < 4; ++i) r[i] = t[i];
      }
      const double t[4] = {m[0] * m[0] + m[1] * m[2], m[0] * m[1] + m[1] * m[3],
                           m[2] * m[0] + m[3] * m[2], m[2] * m[1] + m[3] * m[3]};
      for (int i = 0; i < 4; ++i) m[i] = t[i];
      e >>= 1;
    }
    for (int i = 0; i < 4; ++i) out[k][i] = (float)r[i];
  }
}

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// The ripple: three resonators fed with the pair-sum rounding errors.
struct Ripple {
  float p[3], q[3];  // o[j], o[j-1]
};

__device__ __forceinline__ float ripple_step(Ripple& r, float e) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float o = (e * c_blur.a[k] + c_blur.b[k] * r.p[k]) - r.q[k];
    r.q[k] = r.p[k];
    r.p[k] = o;
  }
  return (r.p[0] + r.p[1]) + r.p[2];
}

// The ripple's input at output j: what rounding added to the pair sum,
// f32(x[j-6] + x[j+4]) - (x[j-6] + x[j+4]) (two_sum's error with its sign
// turned).
__device__ __forceinline__ float pair_error(float left, float right) {
  float s, e;
  two_sum(left, right, s, e);
  return -e;
}

// ---- paired forms --------------------------------------------------------

__device__ __forceinline__ void two_sum2(f2 a, f2 b, f2& s, f2& e) {
  s = f2_add(a, b);
  const f2 bb = f2_sub(s, a);
  e = f2_add(f2_sub(a, f2_sub(s, bb)), f2_sub(b, bb));
}

// pair_error on two lanes: f32(l + r) - (l + r), i.e. two_sum's error negated
// term by term (negation commutes with rounding).
__device__ __forceinline__ f2 pair_error2(f2 l, f2 r) {
  const f2 s = f2_add(l, r);
  const f2 bb = f2_sub(s, l);
  return f2_add(f2_sub(f2_sub(s, bb), l), f2_sub(bb, r));
}

struct Ripple2 {
  f2 p[3], q[3];
};

__device__ __forceinline__ f2 ripple_step2(Ripple2& r, f2 e, f2 nz) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const f2 o = f2_sub(f2_add(f2_mul(e, c_blur2.a[k], nz), f2_mul(c_blur2.b[k], r.p[k], nz)),
                        r.q[k]);
    r.q[k] = r.p[k];
    r.p[k] = o;
  }
  return f2_add(f2_add(r.p[0], r.p[1]), r.p[2]);
}

// The double-float FIR on two lanes.  The low word is kept negated (cn = -c,
// exact since rounding is symmetric) so that every product error comes from
// one FMA with a negated tap: fma(-t, u, t*u rounded) = -(t*u - its rounding).
__device__ __forceinline__ f2 fir_exact2(f2 m4, f2 m3, f2 m2, f2 m1, f2 c0, f2 p1, f2 p2, f2 p3,
                                         f2 p4, f2 rip, f2 nz) {
  f2 S = f2_mul(c_blur2.th[0], c0, nz);
  f2 cn = f2_fma(c_blur2.ntl[0], c0, f2_fma(c_blur2.nth[0], c0, S));
  const f2 lo[4] = {m1, m2, m3, m4}, hi[4] = {p1, p2, p3, p4};
#pragma unroll
  for (int d = 1; d <= 4; ++d) {
    f2 u, ul;
    two_sum2(lo[d - 1], hi[d - 1], u, ul);
    const f2 p = f2_mul(c_blur2.th[d], u, nz);
    const f2 rn = f2_fma(c_blur2.nth[d], u, p);  // -(th*u - p)
    f2 q;
    two_sum2(S, p, S, q);
    cn = f2_sub(cn, q);
    cn = f2_add(cn, rn);
    cn = f2_fma(c_blur2.nth[d], ul, cn);
    cn = f2_fma(c_blur2.ntl[d], u, cn);
  }
  return f2_add(S, f2_sub(rip, cn));
}

// ---------------------------------------------------------------------------
// B1 — rows, two at a time (the lanes).
// ---------------------------------------------------------------------------

constexpr int kRowThreads = 128;
constexpr int kRowLevels = 7;  // log2(kRowThreads): Kogge-Stone levels

struct RowArgs {
  const float* x;  // [3][h][w]
  const float* r;  // [3][h][w] (NQ == 3: the reference side of r*x)
  float* out;      // [nch][NQ][h][w]
  int w, h, c0, seg;
  float nz;                    // -0.0f
  float pw[kRowLevels][3][4];  // M_k^(seg * 2^l)
};

template <int NQ>
__global__ void __launch_bounds__(kRowThreads, 6) k_blur_rows(RowArgs a) {
  extern __shared__ __align__(16) f2 bsm2[];
  f2* xl = bsm2;                                      // [w + 20]: x at i - 10, both rows
  f2* rl = NQ == 3 ? bsm2 + a.w + 20 : nullptr;       // [w + 20]: r likewise (NQ == 3)
  f2* rip = bsm2 + (NQ == 3 ? 2 : 1) * (a.w + 20);    // [w]: R of both rows
  __shared__ f2 carry[kRowThreads][6];
  const int y0 = 2 * blockIdx.x, ch = blockIdx.y, c = a.c0 + ch;
  const bool two = y0 + 1 < a.h;
  const size_t n = (size_t)a.w * a.h;
  const float* xr0 = a.x + n * c + (size_t)y0 * a.w;
  const float* xr1 = two ? xr0 + a.w : xr0;
  const float* rr0 = NQ == 3 ? a.r + n * c + (size_t)y0 * a.w : nullptr;
  const float* rr1 = NQ == 3 ? (two ? rr0 + a.w : rr0) : nullptr;
  const f2 nz = f2_pack(a.nz, a.nz);
  const int t = threadIdx.x;
  const int j0 = min(t * a.seg, a.w), j1 = min(j0 + a.seg, a.w);
  // Both rows of x (and r) once, zero outside the line.
#pragma unroll 8
  for (int i = t; i < a.w + 20; i += kRowThreads) {
    const int gx = i - 10;
    const bool in = gx >= 0 && gx < a.w;
    const float x0 = in ? xr0[gx] : 0.0f, x1 = in && two ? xr1[gx] : 0.0f;
    xl[i] = f2_pack(x0, x1);
    if (NQ == 3) {
      const float r0 = in ? rr0[gx] : 0.0f, r1 = in && two ? rr1[gx] : 0.0f;
      rl[i] = f2_pack(r0, r1);
    }
  }
  __syncthreads();
  // Quantities in the order x, r*x, x*x, each product line formed once in
  // place (r*x over r, then x*x over x) and rounded to f32 (blur.rs:395).
#pragma unroll
  for (int qi = 0; qi < NQ; ++qi) {
    const int q = NQ == 3 ? (qi == 0 ? 0 : (qi == 1 ? 2 : 1)) : qi;
    if (q != 0) {
      for (int i = t; i < a.w + 20; i += kRowThreads) {
        if (q == 2) rl[i] = f2_mul(rl[i], xl[i], nz);
        else xl[i] = f2_mul(xl[i], xl[i], nz);
      }
      __syncthreads();
    }
    const f2* line = q == 2 ? rl : xl;
    auto L = [&](int i) -> f2 { return line[i]; };
    // (1) the segment's ripple from rest, recorded.
    Ripple2 rp;
#pragma unroll
    for (int k = 0; k < 3; ++k) rp.p[k] = rp.q[k] = 0ull;
    // blur.rs:414 starts the recursion four samples before the line, fed
    // with 0 + x[0..3]: no rounding, so no ripple, for finite samples, and
    // NaN through the whole line for a non-finite one.
    if (t == 0)
#pragma unroll
      for (int j = -4; j < 0; ++j) ripple_step2(rp, pair_error2(L(j + 4), L(j + 14)), nz);
#pragma unroll 4
    for (int j = j0; j < j1; ++j) rip[j] = ripple_step2(rp, pair_error2(L(j + 4), L(j + 14)), nz);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      carry[t][2 * k] = rp.p[k];
      carry[t][2 * k + 1] = rp.q[k];
    }
    __syncthreads();
    // (2) inclusive scan over segments: S_t = sum_{u <= t} A^(t-u) B_u, per lane.
#pragma unroll 1
    for (int l = 0; l < kRowLevels; ++l) {
      const int d = 1 << l;
      f2 add[6] = {0, 0, 0, 0, 0, 0};
      if (t >= d) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const f2 op = carry[t - d][2 * k], oq = carry[t - d][2 * k + 1];
          const float* m = a.pw[l][k];
          add[2 * k] = f2_add(f2_mul(f2_pack(m[0], m[0]), op, nz),
                              f2_mul(f2_pack(m[1], m[1]), oq, nz));
          add[2 * k + 1] = f2_add(f2_mul(f2_pack(m[2], m[2]), op, nz),
                                  f2_mul(f2_pack(m[3], m[3]), oq, nz));
        }
      }
      __syncthreads();
      if (t >= d)
#pragma unroll
        for (int i = 0; i < 6; ++i) carry[t][i] = f2_add(carry[t][i], add[i]);
      __syncthreads();
    }
    // (3) add the homogeneous response of the entry state (p, q) = (o[j0-1],
    // o[j0-2]): o[j0+i] = U[i+1] p - U[i] q per resonator.
    if (t > 0) {
      f2 ep[3], eq[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        ep[k] = carry[t - 1][2 * k];
        eq[k] = carry[t - 1][2 * k + 1];
      }
#pragma unroll 4
      for (int j = j0; j < j1; ++j) {
        const int i = j - j0;
        f2 hom = 0ull;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const float u1 = c_blur.U[k][(i + 1) % 20], u0 = c_blur.U[k][i % 20];
          hom = f2_add(hom, f2_sub(f2_mul(f2_pack(u1, u1), ep[k], nz),
                                   f2_mul(f2_pack(u0, u0), eq[k], nz)));
        }
        rip[j] = f2_add(rip[j], hom);
      }
    }
    __syncthreads();
    // (4) the outputs, in parallel.
    float* o0 = a.out + (size_t)(ch * NQ + q) * n + (size_t)y0 * a.w;
    float* o1 = o0 + a.w;
#pragma unroll 2
    for (int j = t; j < a.w; j += kRowThreads) {
      const int i = j + 10;
      const f2 r = fir_exact2(L(i - 4), L(i - 3), L(i - 2), L(i - 1), L(i), L(i + 1), L(i + 2),
                              L(i + 3), L(i + 4), rip[j], nz);
      o0[j] = f2_lo(r);
      if (two) o1[j] = f2_hi(r);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// B2/B3 — columns (and the candidate's per-pixel terms).
// ---------------------------------------------------------------------------

constexpr int kColW = 32;      // columns per strip
constexpr int kColT = 32;      // rows per segment (and per output tile)

struct ColArgs {
  const float* hpl;  // [nch][NQ][h][w] row-pass planes
  float* carry;      // [2][nch][nseg][NQ * 6][w]: segment responses, then entry states
  float* mu;         // NQ == 2: [3][h][w] outputs
  float* s11;
  const float* mu1;  // NQ == 3: reference mu, sigma11, positive XYB; candidate XYB
  const float* s11r;
  const float* rx;
  const float* cx;
  DF* partial;  // NQ == 3: [nseg][strips][18]
  uint32_t* err;  // the context's device error word
  int w, h, c0, nseg, nch, strips;
  float nz;
  float pw[3][4];  // M_k^kColT
};

// The column pass's cross-segment state lives in the carry buffer:
// [nch][nseg][NQ * 6][w] inclusive states (the ripple's state after each
// segment, from the top of the plane), then the publication flags
// [nch][strips][nseg] and the work counter, zeroed before each launch.
__host__ __device__ inline size_t col_state_floats(int nch, int nseg, int w) {
  return (size_t)nch * nseg * 3 * 6 * w;
}
constexpr uint32_t kColWaitLimit = 1u << 20;  // polls of a predecessor's flag (about a second)

constexpr int kOutThreads = 256;

template <int NQ>
__global__ void __launch_bounds__(kOutThreads, 4) k_blur_col_out(ColArgs a) {
  __shared__ __align__(16) float tile[NQ][kColT + 10][kColW];  // rows r0-6 .. r0+kColT+3
  __shared__ __align__(16) float rp[NQ][kColT][kColW];
  __shared__ DF red[kOutThreads / 32][6];
  // Each half's end state from rest; once the segment's entry is known,
  // each half's entry state (read by the outputs as lane pairs).
  __shared__ __align__(16) float half_end[2][NQ][6][kColW];
  __shared__ float entry[NQ][6][kColW];        // the segment's entry state
  __shared__ int s_item, s_late;
  const int t = threadIdx.x;
  float* const incl = a.carry;  // inclusive states
  int* const flags = reinterpret_cast<int*>(a.carry + col_state_floats(a.nch, a.nseg, a.w));
  int* const counter = flags + (size_t)a.nch * a.strips * a.nseg;
  // Items in the order CTAs start (segments slowest), so that the segment a
  // CTA waits for belongs to a CTA that has already started.
  if (t == 0) {
    s_item = atomicAdd(counter, 1);
    s_late = 0;
  }
  __syncthreads();
  const int per_sg = a.strips * a.nch;
  const int sg = s_item / per_sg, ch = (s_item % per_sg) / a.strips, sx = s_item % a.strips;
  const int c = a.c0 + ch;
  const int x0 = sx * kColW, r0 = sg * kColT;
  const size_t n = (size_t)a.w * a.h;
  const float* H = a.hpl + (size_t)ch * NQ * n;
  {
    constexpr int kElems = (kColT + 10) * kColW;
    constexpr int kIt = (kElems + kOutThreads - 1) / kOutThreads;
    float v[NQ][kIt];
#pragma unroll
    for (int q = 0; q < NQ; ++q)
#pragma unroll
      for (int it = 0; it < kIt; ++it) {
        const int i = t + it * kOutThreads;
        const int ly = i / kColW, lx = i % kColW;
        const int gy = r0 - 6 + ly, gx = x0 + lx;
        v[q][it] = (i < kElems && gx < a.w && gy >= 0 && gy < a.h)
                       ? __ldg(H + (size_t)q * n + (size_t)gy * a.w + gx)
                       : 0.0f;
      }
#pragma unroll
    for (int q = 0; q < NQ; ++q)
#pragma unroll
      for (int it = 0; it < kIt; ++it) {
        const int i = t + it * kOutThreads;
        if (i < kElems) tile[q][i / kColW][i % kColW] = v[q][it];
      }
  }
  __syncthreads();
  // The ripple in two halves of kColT / 2 rows per column and quantity: each
  // half walks from rest, recording R from rest and its end state.
  constexpr int kHalf = kColT / 2;
  const bool walker = t < 2 * NQ * kColW;
  const int wq = (t / kColW) % NQ, wh = t / (NQ * kColW), wl = t % kColW;
  if (walker) {
    Ripple st = {{0, 0, 0}, {0, 0, 0}};
#pragma unroll 8
    for (int r = wh * kHalf; r < (wh + 1) * kHalf; ++r)
      rp[wq][r][wl] = ripple_step(st, pair_error(tile[wq][r][wl], tile[wq][r + 10][wl]));
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      half_end[wh][wq][2 * k][wl] = st.p[k];
      half_end[wh][wq][2 * k + 1][wl] = st.q[k];
    }
  }
  __syncthreads();
  // The chained scan over the column's segments: the entry state is the
  // previous segment's inclusive state (for the first segment, the state
  // blur.rs:574 reaches over its four warm-up rows, fed with 0 + rows 0..3:
  // zero ripple for finite samples); this segment's inclusive state is
  // M^kColT times the entry plus its own response from rest, M^kHalf times
  // the first half's end state plus the second's.  Published with a flag;
  // every wait is bounded and a wait that runs out raises kDevBlurTimeout.
  const bool scanner = t < NQ * kColW;
  const int sq = t / kColW, sl = t % kColW, sxc = x0 + sl;
  float* const my_incl = incl + ((size_t)(ch * a.nseg + sg) * NQ * 6 + sq * 6) * a.w + sxc;
  if (sg == 0) {
    if (scanner)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        float sp = 0.0f, sqq = 0.0f;
        for (int i = 0; i < 4 && i < a.h; ++i) {
          const float e = pair_error(0.0f, tile[sq][6 + i][sl]);
          const float o = (e * c_blur.a[k] + c_blur.b[k] * sp) - sqq;
          sqq = sp;
          sp = o;
        }
        entry[sq][2 * k][sl] = sp;
        entry[sq][2 * k + 1][sl] = sqq;
      }
  } else {
    int* const prev_flag = flags + ((size_t)ch * a.strips + sx) * a.nseg + (sg - 1);
    if (t == 0) {
      uint32_t it = 0;
      while (atomicAdd(prev_flag, 0) == 0 && it < kColWaitLimit) {
        __nanosleep(64);
        ++it;
      }
      if (it == kColWaitLimit) s_late = 1;
      __threadfence();
    }
    __syncthreads();
    if (scanner && sxc < a.w) {
      const float* pv = my_incl - (size_t)NQ * 6 * a.w;
#pragma unroll
      for (int k = 0; k < 6; ++k) entry[sq][k][sl] = __ldcg(pv + (size_t)k * a.w);
    } else if (scanner) {
#pragma unroll
      for (int k = 0; k < 6; ++k) entry[sq][k][sl] = 0.0f;
    }
  }
  if (scanner && sxc < a.w) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float* U = c_blur.U[k];
      const float u0 = U[kHalf % 20], u1 = U[(kHalf - 1) % 20], u2 = U[(kHalf - 2) % 20];
      const float p1 = half_end[0][sq][2 * k][sl], q1 = half_end[0][sq][2 * k + 1][sl];
      const float bp = (u0 * p1 - u1 * q1) + half_end[1][sq][2 * k][sl];
      const float bq = (u1 * p1 - u2 * q1) + half_end[1][sq][2 * k + 1][sl];
      const float* m = a.pw[k];
      const float sp = entry[sq][2 * k][sl], sqq = entry[sq][2 * k + 1][sl];
      my_incl[(size_t)(2 * k) * a.w] = (m[0] * sp + m[1] * sqq) + bp;
      my_incl[(size_t)(2 * k + 1) * a.w] = (m[2] * sp + m[3] * sqq) + bq;
      // Each half's entry state: the segment's entry for the first half,
      // M^kHalf times it plus the first half's end state for the second.
      half_end[1][sq][2 * k][sl] = (u0 * sp - u1 * sqq) + p1;
      half_end[1][sq][2 * k + 1][sl] = (u1 * sp - u2 * sqq) + q1;
      half_end[0][sq][2 * k][sl] = sp;
      half_end[0][sq][2 * k + 1][sl] = sqq;
    }
    __threadfence();
  }
  __syncthreads();
  if (t == 0) {
    atomicExch(flags + ((size_t)ch * a.strips + sx) * a.nseg + sg, 1);
    if (s_late) raise_error(a.err, kDevBlurTimeout);
  }
  // Outputs: columns 2j, 2j+1 (the lanes) of rows kR*b .. kR*b+kR-1.
  constexpr int kR = kColT / (kOutThreads / (kColW / 2));
  const f2 nz = f2_pack(a.nz, a.nz);
  const int jp = t % (kColW / 2), b = t / (kColW / 2);
  const int lx = 2 * jp, gx = x0 + lx;
  float acc[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
  for (int i = 0; i < kR; ++i) {
    const int r = kR * b + i, gy = r0 + r;
    // The reference side's mu, sigma11 and XYB and the candidate's XYB at
    // this row's two outputs, loaded before the FIRs so that their latency
    // overlaps the arithmetic.
    float pf[2][4];
    if (NQ == 3)
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const bool in = gy < a.h && gx + e < a.w;
        const size_t p = (size_t)c * n + (size_t)(in ? gy : 0) * a.w + (in ? gx + e : 0);
        pf[e][0] = in ? __ldg(a.mu1 + p) : 0.0f;
        pf[e][1] = in ? __ldg(a.s11r + p) : 0.0f;
        pf[e][2] = in ? __ldg(a.rx + p) : 0.0f;
        pf[e][3] = in ? __ldg(a.cx + p) : 0.0f;
      }
    f2 val[NQ];
    const int wh = r / kHalf, ir = r % kHalf;
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      // The ripple: its response from rest plus the homogeneous response of
      // its half's entry state through the U table, hom = sum over the
      // resonators of U[ir + 1] p - U[ir] q (accumulated from 0).
      f2 hom = 0ull;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float u1 = c_blur.U[k][(ir + 1) % 20], u0 = c_blur.U[k][ir % 20];
        const f2 ep = *reinterpret_cast<const f2*>(&half_end[wh][q][2 * k][lx]);
        const f2 eq = *reinterpret_cast<const f2*>(&half_end[wh][q][2 * k + 1][lx]);
        hom = f2_add(hom, f2_sub(f2_mul(f2_pack(u1, u1), ep, nz), f2_mul(f2_pack(u0, u0), eq, nz)));
      }
      const f2 rip = f2_add(*reinterpret_cast<const f2*>(&rp[q][r][lx]), hom);
      auto tv = [&](int ly) { return *reinterpret_cast<const f2*>(&tile[q][ly][lx]); };
      val[q] = fir_exact2(tv(r + 2), tv(r + 3), tv(r + 4), tv(r + 5), tv(r + 6), tv(r + 7),
                          tv(r + 8), tv(r + 9), tv(r + 10), rip, nz);
    }
    if (gy >= a.h || gx >= a.w) continue;
    const bool second = gx + 1 < a.w;
    const size_t p = (size_t)c * n + (size_t)gy * a.w + gx;
    if (NQ == 2) {
      a.mu[p] = f2_lo(val[0]);
      a.s11[p] = f2_lo(val[1]);
      if (second) {
        a.mu[p + 1] = f2_hi(val[0]);
        a.s11[p + 1] = f2_hi(val[1]);
      }
    } else {
      // pool.rs:248 accumulate_scalar, in the reference's operation order.
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        if (e == 1 && !second) break;
        const float m1 = pf[e][0];
        const float m2 = e ? f2_hi(val[0]) : f2_lo(val[0]);
        const float v11 = pf[e][1];
        const float s22 = e ? f2_hi(val[1]) : f2_lo(val[1]);
        const float s12 = e ? f2_hi(val[NQ - 1]) : f2_lo(val[NQ - 1]);
        const float mu11 = m1 * m1, mu22 = m2 * m2, mu12 = m1 * m2;
        const float md = m1 - m2;
        const float num_m = 1.0f - md * md;
        const float num_s = 2.0f * (s12 - mu12) + 0.0009f;
        const float den_s = (v11 - mu11) + (s22 - mu22) + 0.0009f;
        const float d = fmaxf(1.0f - (num_m * num_s) / den_s, 0.0f);
        const float d2 = d * d;
        // (1 + |i2-m2|) / (1 + |i1-m1|) - 1 as a difference over the
        // denominator (within the 0.01-point contract the fast division, at
        // most 2 ulp off, serves; identical images give a zero numerator).
        const float a1 = fabsf(pf[e][2] - m1), a2 = fabsf(pf[e][3] - m2);
        const float d1 = __fdividef(a2 - a1, 1.0f + a1);
        const float art = fmaxf(d1, 0.0f), lost = fmaxf(-d1, 0.0f);
        const float art2 = art * art, lost2 = lost * lost;
        acc[0] += d;
        acc[1] += d2 * d2;
        acc[2] += art;
        acc[3] += art2 * art2;
        acc[4] += lost;
        acc[5] += lost2 * lost2;
      }
    }
  }
  if (NQ == 3) {
    // threads, then warps in order, in double-float.
    const int lane = t % 32, wid = t / 32;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const DF s = df_warp_sum(DF{acc[k], 0.0f});
      if (lane == 0) red[wid][k] = s;
    }
    __syncthreads();
    if (t < 6) {
      DF s = red[0][t];
      for (int i = 1; i < kOutThreads / 32; ++i) s = df_add(s, red[i][t]);
      a.partial[((size_t)sg * a.strips + sx) * 18 + c * 6 + t] = s;
    }
  }
}

// ---------------------------------------------------------------------------
// Launches.
// ---------------------------------------------------------------------------

namespace {

int row_seg(int w) {
  int seg = (w + kRowThreads - 1) / kRowThreads;
  return seg | 1;  // odd: the threads' shared-memory strides fall on distinct banks
}

void fill_row_args(RowArgs& a, int w, int h) {
  a.w = w;
  a.h = h;
  a.seg = row_seg(w);
  a.nz = -0.0f;
  for (int l = 0; l < kRowLevels; ++l) resonator_power((long long)a.seg << l, a.pw[l]);
}

void fill_col_args(ColArgs& a, int w, int h, int nch, uint32_t* err) {
  a.w = w;
  a.h = h;
  a.nseg = (h + kColT - 1) / kColT;
  a.nch = nch;
  a.strips = (w + kColW - 1) / kColW;
  a.err = err;
  a.nz = -0.0f;
  resonator_power(kColT, a.pw);
}

// The column pass: the flags and work counter zeroed, then one CTA per
// 32 x 32 tile and channel.
template <int NQ>
void launch_columns(const ColArgs& ca, cudaStream_t s) {
  int* flags = reinterpret_cast<int*>(ca.carry + col_state_floats(ca.nch, ca.nseg, ca.w));
  cudaMemsetAsync(flags, 0, ((size_t)ca.nch * ca.strips * ca.nseg + 1) * sizeof(int), s);
  k_blur_col_out<NQ><<<ca.strips * ca.nseg * ca.nch, kOutThreads, 0, s>>>(ca);
}

}  // namespace

// x, r and R lines of a row pair.
size_t blur_row_smem(int w) { return (size_t)(3 * w + 40) * sizeof(f2); }


cudaError_t configure_blur_kernels() {
  const int smem = (int)blur_row_smem(kBlurMaxWidth);
  cudaError_t e = cudaFuncSetAttribute(k_blur_rows<2>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_blur_rows<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

int blur_partial_rows(int w, int h) {
  return ((w + kColW - 1) / kColW) * ((h + kColT - 1) / kColT);
}

size_t blur_carry_floats(int w, int h) {
  // the inclusive states of three channels, then the flags and the counter
  // (which the same count of floats again covers many times over)
  return (size_t)2 * 3 * ((h + kColT - 1) / kColT) * 3 * 6 * w;
}

void launch_ref_moments(const float* xyb, float* mu, float* s11, float* hpl, float* carry, int w,
                        int h, uint32_t* err, cudaStream_t s) {
  RowArgs ra{};
  ra.x = xyb;
  ra.out = hpl;
  ra.c0 = 0;
  fill_row_args(ra, w, h);
  k_blur_rows<2><<<dim3((h + 1) / 2, 3), kRowThreads, blur_row_smem(w), s>>>(ra);
  ColArgs ca{};
  ca.hpl = hpl;
  ca.carry = carry;
  ca.mu = mu;
  ca.s11 = s11;
  ca.c0 = 0;
  fill_col_args(ca, w, h, 3, err);
  launch_columns<2>(ca, s);
}

int launch_score_scale(const float* cand_xyb, const SsimScale& ref, float* hpl, float* carry,
                       int c0, int nch, DF* partial, uint32_t* err, cudaStream_t s,
                       ScaleHook hook, void* user) {
  const int w = ref.w, h = ref.h;
  if (hook) hook(user, 0);
  RowArgs ra{};
  ra.x = cand_xyb;
  ra.r = ref.xyb;
  ra.out = hpl;
  ra.c0 = c0;
  fill_row_args(ra, w, h);
  k_blur_rows<3><<<dim3((h + 1) / 2, nch), kRowThreads, blur_row_smem(w), s>>>(ra);
  if (hook) hook(user, 1);
  ColArgs ca{};
  ca.hpl = hpl;
  ca.carry = carry;
  ca.mu1 = ref.mu;
  ca.s11r = ref.s11;
  ca.rx = ref.xyb;
  ca.cx = cand_xyb;
  ca.partial = partial;
  ca.c0 = c0;
  fill_col_args(ca, w, h, nch, err);
  if (hook) hook(user, 2);
  launch_columns<3>(ca, s);
  if (hook) hook(user, 3);
  return blur_partial_rows(w, h);
}

}  // namespace jpxlg
