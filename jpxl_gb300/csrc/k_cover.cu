// k_cover.cu — sm_103a kernels of the encoder's cover selection
// (jpxl-encode-policy lib.rs:5260 select_blocks, :5115 tile_region_with,
// :4909 block_cost_bounded, :4685 score_channel_lanes) for a fixed quantizer
// with adaptive quantization off and the Legacy rate model:
//   C1 k_cover_score<N>  every candidate of one square shape: forward DCT of
//                        Y, X, B; quantization of the non-LLF cells (X and B
//                        against neutral chroma-from-luma, B minus Y's
//                        reconstruction); residual bits (exact) and each
//                        channel's squared error in double-float
//   C2 k_cover_decide    one thread per 32x32 region: the quadtree (DCT8 /
//                        DCT16 / DCT32, ties keep the split) on those costs
//
// The reference accumulates each candidate's weighted error in f64, cell by
// cell in row order, and prunes a merge once the running cost reaches the
// split's.  C1 sums in a fixed tree order instead; C2 carries a bound on the
// distance between the two sums (all terms are non-negative) through every
// comparison, and a region whose comparisons are not all settled by the
// bound is replayed in the reference's own order (sequential f64, row-wise
// pruning) from the stored candidate coefficients.  Replays are counted.
#include <cstdint>

#include "jpxlg_common.cuh"
#include "jpxlg_internal.h"
#include "jpxlg_kernels.h"
#include "jpxlg_quant.cuh"

namespace jpxlg {

// Shape s: 0 DCT8 (1 block), 1 DCT16 (2x2), 2 DCT32 (4x4).
__host__ __device__ constexpr int cover_blocks(int s) { return 1 << s; }

// C1 — candidates of shape N at every aligned position that fits the grid.
template <int N>
__global__ void __launch_bounds__(128) k_cover_score(CoverArgs a) {
  constexpr int S = N == 8 ? 0 : (N == 16 ? 1 : 2);
  constexpr int B = N / 8;
  constexpr int VPB = 128 / N;
  constexpr int n = B;  // LLF corner side
  __shared__ float T[VPB][N][N + 1];
  __shared__ float YR[VPB][N][N + 1];
  const Geo& geo = a.geo;
  const int pw = geo.bw / B, ph = geo.bh / B;
  const int g = threadIdx.x / N, j = threadIdx.x % N;
  const int ci = blockIdx.x * VPB + g;
  const bool active = ci < pw * ph;
  const int bx = active ? (ci % pw) * B : 0, by = active ? (ci / pw) * B : 0;
  const int x0 = bx * 8, y0 = by * 8;
  const size_t plane = (size_t)geo.w * geo.h;
  const size_t cplane = (size_t)geo.W8 * geo.H8;
  const int off = dq_offset(dq_slot(N == 8 ? 0 : (N == 16 ? 4 : 5)));
  uint32_t bits = 0;
  DF sse[3] = {};
  float v[N];
  // Channels in the reference's scoring order: Y (its reconstruction feeds
  // B's targets), X, B.
#pragma unroll 1
  for (int ci3 = 0; ci3 < 3; ++ci3) {
    const int c = ci3 == 0 ? 1 : (ci3 == 1 ? 0 : 2);
    // DCT_2D: column pass, then row pass (k_fdct_luma's order); thread j
    // ends with cells (k, j), k = 0..N-1.
#pragma unroll 1
    for (int pass = 0; pass < 2; ++pass) {
      if (active) {
        if (pass == 0) {
          const float* p = a.pre + plane * c;
          const int xx = min(x0 + j, geo.w - 1);
#pragma unroll
          for (int r = 0; r < N; ++r) v[r] = p[(size_t)min(y0 + r, geo.h - 1) * geo.w + xx];
        } else {
#pragma unroll
          for (int k = 0; k < N; ++k) v[k] = T[g][j][k];
        }
        dct_1d<N>(v);
        if (pass == 0) {
#pragma unroll
          for (int r = 0; r < N; ++r) T[g][r][j] = v[r];
        }
      }
      __syncthreads();
    }
    if (active) {
      float* coef = a.coef[S] + cplane * c;
      const float scale = a.scale[c];
      const float* m = a.dq + c * kDequantTableFloats + off;
      const float bias = c_quant_bias[c];
#pragma unroll 4
      for (int k = 0; k < N; ++k) {
        coef[(size_t)(y0 + k) * geo.W8 + x0 + j] = v[k];
        if (k < n && j < n) continue;
        const float target = c == 1 ? v[k] : (c == 0 ? v[k] - 0.0f * YR[g][k][j]
                                                      : v[k] - 1.0f * YR[g][k][j]);
        const float step = scale * __ldg(&m[k * N + j]);
        float recon;
        const int32_t q = choose(target, step, 1.0f / step, bias, a.err, &recon);
        if (c == 1) YR[g][k][j] = recon;
        bits += residual_bits(q);
        const float d = recon - target;
        sse[c] = df_add(sse[c], df_two_prod(d, d));
      }
    }
  }
  // Fold the group's N threads (xor butterflies stay inside a segment of N
  // lanes, N a power of two <= 32).
#pragma unroll
  for (int o = N / 2; o > 0; o >>= 1) {
    bits += __shfl_xor_sync(0xffffffffu, bits, o);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      DF u{__shfl_xor_sync(0xffffffffu, sse[c].hi, o), __shfl_xor_sync(0xffffffffu, sse[c].lo, o)};
      sse[c] = df_add(sse[c], u);
    }
  }
  if (active && j == 0) {
    a.bits[S][ci] = bits;
#pragma unroll
    for (int c = 0; c < 3; ++c) a.sse[S][(size_t)ci * 3 + c] = sse[c];
  }
}

// A cost with a bound on its distance from the reference's f64 value.
struct Cost {
  double v, e;
};

__device__ __forceinline__ Cost cover_rd(const CoverArgs& a, int s, int bx, int by) {
  const int B = cover_blocks(s);
  const int pw = a.geo.bw / B;
  const int ci = (by / B) * pw + bx / B;
  const double bits = (double)a.bits[s][ci];
  double t = 0.0;
  for (int c = 0; c < 3; ++c) t += a.w[s][c] * df_value(a.sse[s][(size_t)ci * 3 + c]);
  // At most 3 x 1024 non-negative terms: the double-float tree sums lie
  // within cells x 2^-44 of the exact sum, the reference's sequential f64
  // sum within cells x 2^-53, and the products by w and the three-channel
  // sum add a few 2^-53 more; 2^-40 per term covers all of it with margin.
  const double eps = (3.0 * 1024.0 + 64.0) * 9.094947017729282e-13;  // 2^-40
  return {bits + t, eps * t + 1e-300};
}

// A few ulps of an f64 sum of four values.
__device__ __forceinline__ double sum_slack(double v) { return 8.0 * 1.1102230246251565e-16 * fabs(v); }

// One node of the quadtree with bounds; returns false when a comparison is
// not settled.  blocks: up to 16 (shape, bx, by) chosen varblocks.
struct CoverPick {
  int n;
  uint8_t s[16];
  uint8_t bx[16], by[16];
};

__device__ bool cover_node(const CoverArgs& a, int bx, int by, int size, Cost* out,
                           CoverPick* pick) {
  const int bw = a.geo.bw, bh = a.geo.bh;
  if (bx >= bw || by >= bh) {
    *out = {0.0, 0.0};
    return true;
  }
  if (size == 1) {
    const Cost rd = cover_rd(a, 0, bx, by);
    *out = {rd.v + 2.0 + 0.0, rd.e + sum_slack(rd.v + 2.0)};
    pick->s[pick->n] = 0;
    pick->bx[pick->n] = (uint8_t)(bx & 3);
    pick->by[pick->n] = (uint8_t)(by & 3);
    ++pick->n;
    return true;
  }
  const int half = size / 2;
  const int first = pick->n;
  Cost split{0.0, 0.0};
  const int qx[4] = {bx, bx + half, bx, bx + half}, qy[4] = {by, by, by + half, by + half};
  for (int i = 0; i < 4; ++i) {
    Cost c;
    if (!cover_node(a, qx[i], qy[i], half, &c, pick)) return false;
    split.v += c.v;
    split.e += c.e;
  }
  split.e += sum_slack(split.v);
  const bool fits = bx + size <= bw && by + size <= bh;
  if (fits) {
    const double fixed = 34.0 + 0.0;
    if (fabs(fixed - split.v) <= split.e) return false;
    if (!(fixed >= split.v)) {
      const int s = size == 2 ? 1 : 2;
      const Cost rd = cover_rd(a, s, bx, by);
      const Cost single{rd.v + fixed, rd.e + sum_slack(rd.v + fixed)};
      // Reference: kept only if not pruned (rd < split - fixed) and
      // single < split; both are this comparison up to rounding.
      if (fabs(single.v - split.v) <= single.e + split.e) return false;
      if (single.v < split.v) {
        pick->n = first;
        pick->s[pick->n] = (uint8_t)s;
        pick->bx[pick->n] = (uint8_t)(bx & 3);
        pick->by[pick->n] = (uint8_t)(by & 3);
        ++pick->n;
        *out = single;
        return true;
      }
    }
  }
  *out = split;
  return true;
}

// ---- the reference's own order, for regions the bound does not settle ----

// lib.rs:4685 for one channel of a stored candidate: rows, non-LLF columns,
// f64 accumulation cell by cell, the cutoff tested after each row.  B's
// targets subtract Y's reconstruction, recomputed cell by cell.
__device__ bool exact_channel(const CoverArgs& a, int s, int bx, int by, int c, double cutoff,
                              bool has_cutoff, uint64_t* bits, double* sse) {
  const int N = 8 << s, n = 1 << s;
  const size_t cplane = (size_t)a.geo.W8 * a.geo.H8;
  const float* coef = a.coef[s] + cplane * c;
  const float* coef_y = a.coef[s] + cplane;
  const int off = dq_offset(dq_slot(s == 0 ? 0 : (s == 1 ? 4 : 5)));
  const float* m = a.dq + c * kDequantTableFloats + off;
  const float* my = a.dq + kDequantTableFloats + off;
  const double flat_weight = a.lambda[c] * ((double)(N * N) * 1.0);
  for (int row = 0; row < N; ++row) {
    for (int col = row < n ? n : 0; col < N; ++col) {
      const size_t ix = (size_t)(by * 8 + row) * a.geo.W8 + bx * 8 + col;
      float target = coef[ix];
      if (c != 1) {
        float ry;
        const float sy = a.scale[1] * my[row * N + col];
        choose(coef_y[ix], sy, 1.0f / sy, c_quant_bias[1], nullptr, &ry);
        target = c == 0 ? target - 0.0f * ry : target - 1.0f * ry;
      }
      const float step = a.scale[c] * m[row * N + col];
      float recon;
      const int32_t q = choose(target, step, 1.0f / step, c_quant_bias[c], nullptr, &recon);
      *bits += residual_bits(q);
      const double d = (double)(recon - target);
      *sse += flat_weight * (d * d);
    }
    if (has_cutoff && (double)*bits * 1.0 + *sse >= cutoff) return false;
  }
  return true;
}

__device__ bool exact_cost(const CoverArgs& a, int s, int bx, int by, double cutoff,
                           bool has_cutoff, double* cost) {
  uint64_t bits = 0;
  double sse = 0.0;
  if (!exact_channel(a, s, bx, by, 1, cutoff, has_cutoff, &bits, &sse)) return false;
  if (!exact_channel(a, s, bx, by, 0, cutoff, has_cutoff, &bits, &sse)) return false;
  if (!exact_channel(a, s, bx, by, 2, cutoff, has_cutoff, &bits, &sse)) return false;
  *cost = (double)bits * 1.0 + sse;
  return true;
}

__device__ double exact_node(const CoverArgs& a, int bx, int by, int size, CoverPick* pick) {
  const int bw = a.geo.bw, bh = a.geo.bh;
  if (bx >= bw || by >= bh) return 0.0;
  if (size == 1) {
    double rd = 0.0;
    exact_cost(a, 0, bx, by, 0.0, false, &rd);
    pick->s[pick->n] = 0;
    pick->bx[pick->n] = (uint8_t)(bx & 3);
    pick->by[pick->n] = (uint8_t)(by & 3);
    ++pick->n;
    return rd + 2.0 + 0.0;
  }
  const int half = size / 2;
  const int first = pick->n;
  double split = 0.0;
  const int qx[4] = {bx, bx + half, bx, bx + half}, qy[4] = {by, by, by + half, by + half};
  for (int i = 0; i < 4; ++i) split += exact_node(a, qx[i], qy[i], half, pick);
  if (bx + size <= bw && by + size <= bh) {
    const double fixed = 34.0 + 0.0;
    if (fixed >= split) return split;
    const double cutoff = split - fixed;
    const int s = size == 2 ? 1 : 2;
    double rd;
    if (exact_cost(a, s, bx, by, cutoff, true, &rd)) {
      const double single = rd + fixed;
      if (single < split) {
        pick->n = first;
        pick->s[pick->n] = (uint8_t)s;
        pick->bx[pick->n] = (uint8_t)(bx & 3);
        pick->by[pick->n] = (uint8_t)(by & 3);
        ++pick->n;
        return single;
      }
    }
  }
  return split;
}

// C2 — one thread per aligned 4x4-block region.
__global__ void __launch_bounds__(128) k_cover_decide(CoverArgs a) {
  const int rw = (a.geo.bw + 3) / 4, rh = (a.geo.bh + 3) / 4;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rw * rh) return;
  const int bx0 = (r % rw) * 4, by0 = (r / rw) * 4;
  CoverPick pick;
  pick.n = 0;
  Cost total;
  if (!cover_node(a, bx0, by0, 4, &total, &pick)) {
    atomicAdd(a.fallbacks, 1u);
    pick.n = 0;
    exact_node(a, bx0, by0, 4, &pick);
  }
  static const uint8_t kSel[3] = {0, 4, 5};
  for (int i = 0; i < pick.n; ++i) {
    const int s = pick.s[i], B = cover_blocks(s);
    const int bx = bx0 + pick.bx[i], by = by0 + pick.by[i];
    for (int dy = 0; dy < B; ++dy)
      for (int dx = 0; dx < B; ++dx)
        a.map[(size_t)(by + dy) * a.geo.bw + bx + dx] =
            (uint8_t)(kSel[s] | ((dx == 0 && dy == 0) ? 0x80 : 0));
  }
}

size_t cover_scratch_bytes(const Geo& g) {
  size_t total = 0;
  for (int s = 0; s < 3; ++s) {
    const size_t cands = (size_t)(g.bw >> s) * (g.bh >> s);
    total += ((cands * sizeof(uint32_t) + 255) / 256) * 256;
    total += ((cands * 3 * sizeof(DF) + 255) / 256) * 256;
    total += ((3 * (size_t)g.W8 * g.H8 * sizeof(float) + 255) / 256) * 256;
  }
  return total;
}

void cover_bind_scratch(CoverArgs* a, void* scratch) {
  char* p = (char*)scratch;
  for (int s = 0; s < 3; ++s) {
    const size_t cands = (size_t)(a->geo.bw >> s) * (a->geo.bh >> s);
    a->bits[s] = (uint32_t*)p;
    p += ((cands * sizeof(uint32_t) + 255) / 256) * 256;
    a->sse[s] = (DF*)p;
    p += ((cands * 3 * sizeof(DF) + 255) / 256) * 256;
    a->coef[s] = (float*)p;
    p += ((3 * (size_t)a->geo.W8 * a->geo.H8 * sizeof(float) + 255) / 256) * 256;
  }
}

int launch_cover(const CoverArgs& a, cudaStream_t s) {
  const int bw = a.geo.bw, bh = a.geo.bh;
  int k = 0;
  const int n8 = bw * bh, n16 = (bw / 2) * (bh / 2), n32 = (bw / 4) * (bh / 4);
  if (n8) { k_cover_score<8><<<(n8 + 15) / 16, 128, 0, s>>>(a); ++k; }
  if (n16) { k_cover_score<16><<<(n16 + 7) / 8, 128, 0, s>>>(a); ++k; }
  if (n32) { k_cover_score<32><<<(n32 + 3) / 4, 128, 0, s>>>(a); ++k; }
  const int regions = ((bw + 3) / 4) * ((bh + 3) / 4);
  k_cover_decide<<<(regions + 127) / 128, 128, 0, s>>>(a);
  return k + 1;
}

}  // namespace jpxlg
