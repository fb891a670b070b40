// k_encode.cu — sm_103a kernels of the encoder's transform path:
//   K1 k_srgb_to_xyb       RGB8/RGB16 -> LUT -> linear -> XYB planes
//   K2 k_precondition      12 fused Jacobi steps of the inverse Gaborish
//   K3 k_fdct_luma<N>      gather + DCT_2D + LF samples + luma quantization
//   K4 k_cfl_*             chroma-from-luma factor estimation
//   K5 k_quant_chroma<N>   X/B quantization against reconstructed luma
// Each kernel restates the reference arithmetic it replaces (cited per
// kernel) in the reference's operation order; the build uses -fmad=false.
#include <algorithm>
#include <cstdint>

#include "jpxlg_common.cuh"
#include "jpxlg_internal.h"
#include "jpxlg_kernels.h"
#include "jpxlg_quant.cuh"

namespace jpxlg {

__constant__ float c_iv4[16];
__constant__ float c_iv8[64];
__constant__ float c_iv16[256];
__constant__ float c_scale_f[32];  // [lf count 1,2,4,8][c < 8]

// ---------------------------------------------------------------------------
// K1 — jpxl-encode-policy source.rs:226 (RGB8) / :355 (RGB16): code point ->
// linear through the host-built table, then jpxl-core color.rs:84 opsin mix
// (no FMA), reproducible cube root, opponent rotation.
// ---------------------------------------------------------------------------

__device__ __forceinline__ void xyb_of(float r, float g, float b, float* x, float* y, float* s) {
  float lm = 0.3f * r + 0.622f * g + 0.078f * b + 0.0037930734f;
  float mm = 0.23f * r + 0.692f * g + 0.078f * b + 0.0037930734f;
  float sm = 0.2434227f * r + 0.2047674f * g + 0.5518099f * b + 0.0037930734f;
  float lg = cbrt_core(lm) - 0.1559542f;
  float mg = cbrt_core(mm) - 0.1559542f;
  float sg = cbrt_core(sm) - 0.1559542f;
  *x = 0.5f * (lg - mg);
  *y = 0.5f * (lg + mg);
  *s = sg;
}

template <typename T>
__global__ void __launch_bounds__(256) k_srgb_to_xyb(const T* __restrict__ rgb, size_t n,
                                                     const float* __restrict__ lut,
                                                     float* __restrict__ px,
                                                     float* __restrict__ py,
                                                     float* __restrict__ pb,
                                                     uint32_t* __restrict__ not_gray) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  bool color = false;
  for (; i < n; i += stride) {
    uint32_t cr = rgb[3 * i], cg = rgb[3 * i + 1], cb = rgb[3 * i + 2];
    color |= (cr != cg) || (cg != cb);
    float x, y, b;
    xyb_of(__ldg(&lut[cr]), __ldg(&lut[cg]), __ldg(&lut[cb]), &x, &y, &b);
    px[i] = x;
    py[i] = y;
    pb[i] = b;
  }
  if (__any_sync(0xffffffffu, color) && (threadIdx.x & 31) == 0) atomicOr(not_gray, 1u);
}

void launch_srgb_to_xyb(const void* rgb, int bits, size_t n, const float* lut, float* x, float* y,
                        float* b, uint32_t* not_gray, int num_sms, cudaStream_t s) {
  int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)num_sms * 8);
  if (blocks < 1) blocks = 1;
  if (bits == 8)
    k_srgb_to_xyb<uint8_t><<<blocks, 256, 0, s>>>((const uint8_t*)rgb, n, lut, x, y, b, not_gray);
  else
    k_srgb_to_xyb<uint16_t><<<blocks, 256, 0, s>>>((const uint16_t*)rgb, n, lut, x, y, b,
                                                   not_gray);
}

// ---------------------------------------------------------------------------
// K2 — jpxl-encode vardct/gaborish.rs:218 precondition_xyb_planes: twelve
// Jacobi steps x <- x + (f - Kx) * (1/centre) (tail: / centre) against the
// encoder's non-FMA J.1 kernel.  All twelve steps run on one register-resident
// tile with a 12-sample halo, so the plane is read once and written once.
//
// Bit parity with the reference's position-dependent arithmetic:
//   * a pixel on the frame border sums its nine mirrored taps sequentially
//     (dy outer, dx inner), acc += w*s;
//   * an interior pixel in the SIMD groups of four that start at x = 1
//     (x - 1 < 4*floor((w-2)/4)) evaluates mid*c + (N+S+W+E)*e + (NW+NE+SW+SE)*k;
//   * remaining interior pixels sum the nine taps sequentially;
//   * the update multiplies by 1/centre for flat indices below 4*floor(n/4)
//     and divides by centre above.
// Border cells read their taps at mirrored frame coordinates, so no cell
// outside the frame is ever read after the load.
// ---------------------------------------------------------------------------

// Tiling.  A CTA owns a 128 x 128 tile of one plane with a 12-sample halo
// (104 x 104 outputs).  Lane l of warp v holds columns 4l .. 4l+3 of tile
// rows 4v .. 4v+3 in registers for all twelve steps: west and east
// neighbours come from the adjacent lanes by shuffle, the rows above and
// below the warp's four from the neighbouring warps through shared memory
// (double-buffered, one barrier per step), and the source plane F from
// shared memory.  Every step updates the whole tile; a cell k samples from
// the tile's edge is exact for k steps, so after twelve the inner 104 x 104
// are, and no cell of the edge ring is ever read by one nearer the centre
// than itself.
//
// Two kinds of tile cover a frame: those whose haloed extent has no cell of
// another rule (kEdge false), and the ring of tiles around them (kEdge
// true).  A ring tile keeps each step's input in shared memory and, after
// the paired update of every cell, the CTA's threads share out the cells of
// another rule (frame border and columns past the groups of four: the
// sequential nine-tap sum; the last n % 4 cells of the plane: the division
// by the centre weight) and recompute them from their nine taps at mirrored
// frame coordinates (always among the cell's own 3 x 3 neighbourhood).  One
// launch holds both: the ring's CTAs first (they take longer), then the
// interior's, which fill the SMs around them.
constexpr int kPreOut = 104;
constexpr int kPreHalo = 12;
constexpr int kPreW = kPreOut + 2 * kPreHalo;  // 128: 32 lanes x 4 columns
constexpr int kPreWarps = kPreW / 4;            // 32 warps of four rows
constexpr int kPreThreads = 32 * kPreWarps;
static_assert(kPreW == 128 && kPreHalo >= 12, "tile of the inverse Gaborish");
// Tile rows in shared memory are kPreP floats apart: 16-byte aligned for the
// rows' float4 accesses, and a column's 32 consecutive rows spread over 8
// banks for the ring's per-cell accesses (a pitch of 128 puts them all in
// one).
constexpr int kPreP = kPreW + 4;
// F (the source tile, [kPreW][kPreP]), then the interior kernel's published
// rows [2 parities][kPreWarps][first, last][kPreW], or the ring kernel's
// step inputs [2 parities][kPreW][kPreP].
constexpr size_t kPreSmem = (size_t)(kPreW * kPreP + 2 * kPreWarps * 2 * kPreW) * sizeof(float);
constexpr size_t kPreRingSmem = (size_t)3 * kPreW * kPreP * sizeof(float);

struct EncKernel {
  float centre, edge, corner, inv_c;
  float neg_zero;  // -0.0f, the run-time addend of the paired products
};

// The tiles of a frame: a rectangle [fx0, fx1) x [fy0, fy1) of tiles with no
// cell of another rule (kEdge false) and the ring around it (kEdge true).
struct PreTiles {
  int tx, ty;  // tiles across and down
  int fx0, fx1, fy0, fy1;
};

// The update of the last n % 4 samples of the plane divides by the centre
// weight; out of line so that the division is not evaluated for every cell.
static __device__ __noinline__ float precondition_tail(float mm, float fv, float kx, float centre) {
  return mm + (fv - kx) / centre;
}

// The three rows around a row of four cells, as lane pairs.  Columns are
// paired (0, 1) and (2, 3); W*, C*, E* are the pairs one column to the
// left of pair 0, between the pairs, and one column to the right of pair 1.
struct PreRows {
  f2 Mn0, Mn1, Mm0, Mm1, Ms0, Ms1;
  f2 Wn, Cn, En, Wm, Cm, Em, Ws, Cs, Es;
};
__device__ __forceinline__ PreRows pre_rows(const float4& n, float nW, float nE, const float4& m,
                                            float mW, float mE, const float4& s, float sW,
                                            float sE) {
  PreRows q;
  q.Mn0 = f2_pack(n.x, n.y);
  q.Mn1 = f2_pack(n.z, n.w);
  q.Mm0 = f2_pack(m.x, m.y);
  q.Mm1 = f2_pack(m.z, m.w);
  q.Ms0 = f2_pack(s.x, s.y);
  q.Ms1 = f2_pack(s.z, s.w);
  q.Wn = f2_pack(nW, n.x);
  q.Cn = f2_pack(n.y, n.z);
  q.En = f2_pack(n.w, nE);
  q.Wm = f2_pack(mW, m.x);
  q.Cm = f2_pack(m.y, m.z);
  q.Em = f2_pack(m.w, mE);
  q.Ws = f2_pack(sW, s.x);
  q.Cs = f2_pack(s.y, s.z);
  q.Es = f2_pack(s.w, sE);
  return q;
}

// Interior rule: mm*c + (((N + S) + W) + E)*e + (((NW + NE) + SW) + SE)*k.
__device__ __forceinline__ void pre_kx_interior(const PreRows& q, f2 c2, f2 e2, f2 k2, f2 nz,
                                                f2& kxa, f2& kxb) {
  const f2 s1a = f2_add(f2_add(f2_add(q.Mn0, q.Ms0), q.Wm), q.Cm);
  const f2 s2a = f2_add(f2_add(f2_add(q.Wn, q.Cn), q.Ws), q.Cs);
  const f2 s1b = f2_add(f2_add(f2_add(q.Mn1, q.Ms1), q.Cm), q.Em);
  const f2 s2b = f2_add(f2_add(f2_add(q.Cn, q.En), q.Cs), q.Es);
  kxa = f2_add(f2_add(f2_mul(q.Mm0, c2, nz), f2_mul(s1a, e2, nz)), f2_mul(s2a, k2, nz));
  kxb = f2_add(f2_add(f2_mul(q.Mm1, c2, nz), f2_mul(s1b, e2, nz)), f2_mul(s2b, k2, nz));
}

// mm + (f - kx) * (1/c).
__device__ __forceinline__ float4 pre_update(const PreRows& q, const float4& f, f2 kxa, f2 kxb,
                                             f2 i2, f2 nz) {
  const f2 ya = f2_add(q.Mm0, f2_mul(f2_sub(f2_pack(f.x, f.y), kxa), i2, nz));
  const f2 yb = f2_add(q.Mm1, f2_mul(f2_sub(f2_pack(f.z, f.w), kxb), i2, nz));
  return make_float4(f2_lo(ya), f2_hi(ya), f2_lo(yb), f2_hi(yb));
}

// A ring tile's cell of another rule, found once: its tile position and the
// tile rows and columns of its mirrored taps (7 bits each) and its rule.
struct PreSpecial {
  uint32_t a;  // tx | xm << 7 | xp << 14 | ty << 21
  uint32_t b;  // ym | yp << 7 | seq << 14 | div << 15 | valid << 16
};
__device__ __forceinline__ PreSpecial pre_special(int ty, int tx, int cx, int cy, int gx0, int gy0,
                                                  int w, int h, bool seq, bool div) {
  auto clampt = [](int v) { return min(max(v, 0), kPreW - 1); };
  const int xm = clampt(mirror1d(cx - 1, w) - gx0), xp = clampt(mirror1d(cx + 1, w) - gx0);
  const int ym = clampt(mirror1d(cy - 1, h) - gy0), yp = clampt(mirror1d(cy + 1, h) - gy0);
  return {(uint32_t)tx | (uint32_t)xm << 7 | (uint32_t)xp << 14 | (uint32_t)ty << 21,
          (uint32_t)ym | (uint32_t)yp << 7 | (uint32_t)seq << 14 | (uint32_t)div << 15 | 1u << 16};
}
// Its update from the step's input S into Sn.
__device__ __forceinline__ void pre_special_step(const PreSpecial& c, const float* S, const float* F,
                                                 float* Sn, const EncKernel& k) {
  const int tx = c.a & 127, xm = (c.a >> 7) & 127, xp = (c.a >> 14) & 127, y0 = (c.a >> 21) * kPreP;
  const int ym = (c.b & 127) * kPreP, yp = ((c.b >> 7) & 127) * kPreP;
  const float nw = S[ym + xm], nn = S[ym + tx], ne = S[ym + xp];
  const float ww = S[y0 + xm], mm = S[y0 + tx], ee = S[y0 + xp];
  const float sw = S[yp + xm], ss = S[yp + tx], se = S[yp + xp];
  float kx;
  if (!((c.b >> 14) & 1u)) {
    kx = mm * k.centre + (nn + ss + ww + ee) * k.edge + (nw + ne + sw + se) * k.corner;
  } else {
    // nine taps in order: dy = -1, 0, 1 outer, dx inner
    float acc = 0.0f;
    acc += k.corner * nw;
    acc += k.edge * nn;
    acc += k.corner * ne;
    acc += k.edge * ww;
    acc += k.centre * mm;
    acc += k.edge * ee;
    acc += k.corner * sw;
    acc += k.edge * ss;
    acc += k.corner * se;
    kx = acc;
  }
  const float fv = F[y0 + tx];
  Sn[y0 + tx] = ((c.b >> 15) & 1u) ? precondition_tail(mm, fv, kx, k.centre)
                                    : mm + (fv - kx) * k.inv_c;
}

// The cells of another rule in a ring tile with frame origin (gx0, gy0):
// the special rows (frame row 0 and rows [rb, h)) across the tile's
// in-frame columns, then the special columns (0 and [cb, w)) down its other
// in-frame rows; rb and cb as the reference's groups of four and division
// tail place them.
struct PreRingCells {
  int cx0, ncin, rB0, nr0, nrin, cB0, nrow_cells, count, groups;
  bool r0, c0;
  size_t bulk;
  __device__ __forceinline__ PreSpecial special(int i, int w, int h, int gx0, int gy0) const {
    int ty, tx;
    if (i < nrow_cells) {
      const int rr = i / ncin;
      tx = cx0 + (i - rr * ncin);
      ty = r0 ? (rr == 0 ? -gy0 : rB0 + rr - 1) : rB0 + rr;
    } else {
      const int j = i - nrow_cells;
      const int ci = j / nrin;
      ty = nr0 + (j - ci * nrin);
      tx = c0 ? (ci == 0 ? -gx0 : cB0 + ci - 1) : cB0 + ci;
    }
    const int cx = gx0 + tx, cy = gy0 + ty;
    const bool border = cx == 0 || cx == w - 1 || cy == 0 || cy == h - 1;
    return pre_special(ty, tx, cx, cy, gx0, gy0, w, h, border || cx - 1 >= 4 * groups,
                       (size_t)cy * w + cx >= bulk);
  }
};
__device__ __forceinline__ PreRingCells pre_ring_cells(int w, int h, int gx0, int gy0) {
  PreRingCells g;
  const size_t plane = (size_t)w * h;
  g.groups = (w >= 3 && h >= 3) ? (w - 2) / 4 : 0;
  g.bulk = plane - plane % 4;
  const int bulk_row = (int)(g.bulk / (size_t)w);
  const int rb = max(g.bulk == plane ? h - 1 : min(h - 1, bulk_row), 1);
  const int cb = max(min(w - 1, 4 * g.groups + 1), 1);
  g.cx0 = max(0, -gx0);
  g.ncin = max(0, min(kPreW, w - gx0) - g.cx0);
  const int ry0 = max(0, -gy0), ry1 = min(kPreW, h - gy0), cx1 = g.cx0 + g.ncin;
  g.r0 = -gy0 >= ry0 && -gy0 < ry1;
  g.rB0 = max(ry0, rb - gy0);
  const int nsr = (g.r0 ? 1 : 0) + max(0, ry1 - g.rB0);
  g.nr0 = max(ry0, 1 - gy0);
  g.nrin = max(0, min(ry1, rb - gy0) - g.nr0);
  g.c0 = -gx0 >= g.cx0 && -gx0 < cx1;
  g.cB0 = max(g.cx0, cb - gx0);
  const int nsc = (g.c0 ? 1 : 0) + max(0, cx1 - g.cB0);
  g.nrow_cells = nsr * g.ncin;
  g.count = g.nrow_cells + nsc * g.nrin;
  return g;
}

__device__ __forceinline__ int pre_clamp(int c, int size) { return min(max(c, 0), size - 1); }

// One tile: item is the tile's index among the interior tiles (row-major
// over the rectangle) or among the ring tiles.
template <bool kEdge>
__device__ __forceinline__ void precondition_tile(const float* __restrict__ in,
                                                  float* __restrict__ out, int w, int h,
                                                  const EncKernel& k, const PreTiles& pt,
                                                  int item) {
  extern __shared__ __align__(16) float pre_smem[];
  float* const F = pre_smem;                   // [kPreW][kPreP]
  float* const xb = pre_smem + kPreW * kPreP;  // published rows, or the ring's step inputs
  const size_t plane = (size_t)w * h;
  in += plane * blockIdx.z;
  out += plane * blockIdx.z;
  int tile_x, tile_y;
  if (!kEdge) {
    const int nfx = pt.fx1 - pt.fx0;
    tile_y = pt.fy0 + item / nfx;
    tile_x = pt.fx0 + item % nfx;
  } else {
    // Ring tiles: the rows above the rectangle, the rows below it, then the
    // tiles left and right of it on its rows.
    int i = item;
    const int top = pt.fy0 * pt.tx, bottom = (pt.ty - pt.fy1) * pt.tx;
    if (i < top) {
      tile_y = i / pt.tx;
      tile_x = i - tile_y * pt.tx;
    } else if (i < top + bottom) {
      i -= top;
      tile_y = pt.fy1 + i / pt.tx;
      tile_x = i - (tile_y - pt.fy1) * pt.tx;
    } else {
      i -= top + bottom;
      const int side = pt.fx0 + (pt.tx - pt.fx1);
      tile_y = pt.fy0 + i / side;
      const int c = i - (tile_y - pt.fy0) * side;
      tile_x = c < pt.fx0 ? c : pt.fx1 + (c - pt.fx0);
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int tx0 = tile_x * kPreOut, ty0 = tile_y * kPreOut;
  const int gx0 = tx0 - kPreHalo, gy0 = ty0 - kPreHalo;
  const int lx = 4 * lane, ly = 4 * warp;  // the thread's first column and row in the tile
  const int gx = gx0 + lx, gy = gy0 + ly;  // ... in the frame
  // Load: tiles inside the frame with 16-byte aligned rows take 16-byte
  // loads; others clamp each coordinate (cells outside the frame are never
  // read by a cell inside it, so their values do not matter).
  const bool vec = gx0 >= 0 && gy0 >= 0 && gx0 + kPreW <= w && gy0 + kPreW <= h && (w % 4) == 0 &&
                   ((reinterpret_cast<uintptr_t>(in) & 15) == 0);
  float4 X[4];
  if (vec) {
#pragma unroll
    for (int r = 0; r < 4; ++r)
      X[r] = __ldg(reinterpret_cast<const float4*>(in + (size_t)(gy + r) * w + gx));
  } else {
    const int c0 = pre_clamp(gx, w), c1 = pre_clamp(gx + 1, w), c2 = pre_clamp(gx + 2, w),
              c3 = pre_clamp(gx + 3, w);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const float* row = in + (size_t)pre_clamp(gy + r, h) * w;
      X[r] = make_float4(__ldg(row + c0), __ldg(row + c1), __ldg(row + c2), __ldg(row + c3));
    }
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) *reinterpret_cast<float4*>(F + (ly + r) * kPreP + lx) = X[r];
  const f2 c2 = f2_pack(k.centre, k.centre), e2 = f2_pack(k.edge, k.edge);
  const f2 k2 = f2_pack(k.corner, k.corner), i2 = f2_pack(k.inv_c, k.inv_c);
  const f2 nz = f2_pack(k.neg_zero, k.neg_zero);
  const unsigned full = 0xffffffffu;
  if (!kEdge) {
    // The rows just above and below the warp's: the last row of the warp
    // above and the first of the warp below (the tile's edge rows for the
    // first and last warps, never read by an exact cell).
    const int row_up = (2 * max(warp - 1, 0) + 1) * kPreW + lx;
    const int row_down = (2 * min(warp + 1, kPreWarps - 1)) * kPreW + lx;
#pragma unroll 1
    for (int it = 0; it < 12; ++it) {
      float* const S = xb + (it & 1) * (kPreWarps * 2 * kPreW);
      *reinterpret_cast<float4*>(S + (2 * warp) * kPreW + lx) = X[0];
      *reinterpret_cast<float4*>(S + (2 * warp + 1) * kPreW + lx) = X[3];
      __syncthreads();
      float4 prev = *reinterpret_cast<const float4*>(S + row_up);
      float pW = __shfl_up_sync(full, prev.w, 1), pE = __shfl_down_sync(full, prev.x, 1);
      float mW = __shfl_up_sync(full, X[0].w, 1), mE = __shfl_down_sync(full, X[0].x, 1);
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const float4 nxt =
            r < 3 ? X[r + 1 < 4 ? r + 1 : 3] : *reinterpret_cast<const float4*>(S + row_down);
        const float sW = __shfl_up_sync(full, nxt.w, 1), sE = __shfl_down_sync(full, nxt.x, 1);
        const float4 f = *reinterpret_cast<const float4*>(F + (ly + r) * kPreP + lx);
        f2 kxa, kxb;
        const PreRows q = pre_rows(prev, pW, pE, X[r], mW, mE, nxt, sW, sE);
        pre_kx_interior(q, c2, e2, k2, nz, kxa, kxb);
        const float4 y = pre_update(q, f, kxa, kxb, i2, nz);
        prev = X[r];
        pW = mW;
        pE = mE;
        X[r] = y;
        mW = sW;
        mE = sE;
      }
    }
  } else {
    // Ring tiles keep the step's input in shared memory and write the
    // step's output to the other buffer; each thread first finds its cell
    // of another rule, if it has one.
    const PreRingCells rc = pre_ring_cells(w, h, gx0, gy0);
    PreSpecial mine{0u, 0u};
    if ((int)threadIdx.x < rc.count) mine = rc.special(threadIdx.x, w, h, gx0, gy0);
#pragma unroll
    for (int r = 0; r < 4; ++r) *reinterpret_cast<float4*>(xb + (ly + r) * kPreP + lx) = X[r];
    const int row_up = max(ly - 1, 0) * kPreP + lx;
#pragma unroll 1
    for (int it = 0; it < 12; ++it) {
      const float* const S = xb + (it & 1) * (kPreW * kPreP);
      float* const Sn = xb + ((it + 1) & 1) * (kPreW * kPreP);
      __syncthreads();
      // A warp whose four rows have all left the exact region [1 + it,
      // 127 - it) rests; its rows in the step buffers are read only by
      // cells that are no longer exact either.
      if (!(4 * warp + 3 < 1 + it || 4 * warp >= kPreW - 1 - it)) {
        float4 prev = *reinterpret_cast<const float4*>(S + row_up);
        float4 cur = *reinterpret_cast<const float4*>(S + ly * kPreP + lx);
        float pW = __shfl_up_sync(full, prev.w, 1), pE = __shfl_down_sync(full, prev.x, 1);
        float mW = __shfl_up_sync(full, cur.w, 1), mE = __shfl_down_sync(full, cur.x, 1);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const float4 nxt =
              *reinterpret_cast<const float4*>(S + min(ly + r + 1, kPreW - 1) * kPreP + lx);
          const float sW = __shfl_up_sync(full, nxt.w, 1), sE = __shfl_down_sync(full, nxt.x, 1);
          const float4 f = *reinterpret_cast<const float4*>(F + (ly + r) * kPreP + lx);
          f2 kxa, kxb;
          const PreRows q = pre_rows(prev, pW, pE, cur, mW, mE, nxt, sW, sE);
          pre_kx_interior(q, c2, e2, k2, nz, kxa, kxb);
          *reinterpret_cast<float4*>(Sn + (ly + r) * kPreP + lx) = pre_update(q, f, kxa, kxb, i2, nz);
          prev = cur;
          pW = mW;
          pE = mE;
          cur = nxt;
          mW = sW;
          mE = sE;
        }
      }
      __syncthreads();
      if (mine.b) pre_special_step(mine, S, F, Sn, k);
      // More cells than threads (none for frames at least 4 samples wide).
      if (rc.count > kPreThreads) {
        const PreRingCells more = pre_ring_cells(w, h, gx0, gy0);
        for (int i = threadIdx.x + kPreThreads; i < more.count; i += kPreThreads)
          pre_special_step(more.special(i, w, h, gx0, gy0), S, F, Sn, k);
      }
    }
    __syncthreads();
    // Twelve steps end in buffer 0; each thread reads back its own rows.
#pragma unroll
    for (int r = 0; r < 4; ++r) X[r] = *reinterpret_cast<const float4*>(xb + (ly + r) * kPreP + lx);
  }
  // The inner 104 x 104: lanes 3 .. 28 of warps 3 .. 28.
  const int oh = kPreHalo / 4;
  if (lane >= oh && lane < 32 - oh && warp >= oh && warp < kPreWarps - oh) {
    const bool vec_out =
        gx + 3 < w && (w % 4) == 0 && ((reinterpret_cast<uintptr_t>(out) & 15) == 0);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      if (gy + r >= h) break;
      float* row = out + (size_t)(gy + r) * w;
      if (vec_out) {
        *reinterpret_cast<float4*>(row + gx) = X[r];
      } else {
        if (gx < w) row[gx] = X[r].x;
        if (gx + 1 < w) row[gx + 1] = X[r].y;
        if (gx + 2 < w) row[gx + 2] = X[r].z;
        if (gx + 3 < w) row[gx + 3] = X[r].w;
      }
    }
  }
}

// Both kinds of tile in one launch: the ring tiles at blockIdx.x < nedge,
// then the interior tiles.
__global__ void __launch_bounds__(kPreThreads, 1) k_precondition(const float* __restrict__ in,
                                                              float* __restrict__ out, int w,
                                                              int h, EncKernel k, PreTiles pt,
                                                              int nedge) {
  const int i = (int)blockIdx.x;
  if (i < nedge) precondition_tile<true>(in, out, w, h, k, pt, i);
  else precondition_tile<false>(in, out, w, h, k, pt, i - nedge);
}

int launch_precondition(const float* in, float* out, int w, int h, cudaStream_t s) {
  const float w1 = 0.115169525f, w2 = 0.061248592f;
  // gaborish.rs:31 GaborKernel::new, normalised without FMA.
  float unnorm = 1.0f + 4.0f * w1 + 4.0f * w2;
  float scale = 1.0f / unnorm;
  EncKernel k{scale, w1 * scale, w2 * scale, 1.0f / scale, -0.0f};
  PreTiles pt{(w + kPreOut - 1) / kPreOut, (h + kPreOut - 1) / kPreOut, 0, 0, 0, 0};
  // Columns and rows of cells with another rule: 0, [cb, w) and 0, [rb, h)
  // (the frame border, the columns past the groups of four, the rows of
  // the division tail).  A tile is in the rectangle when its haloed extent
  // [t*104 - 12, t*104 + 116) lies inside [1, cb) and [1, rb).
  const long long n = (long long)w * h;
  const int groups = (w >= 3 && h >= 3) ? (w - 2) / 4 : 0;
  const int cb = std::max(std::min(w - 1, 4 * groups + 1), 1);
  const int row_end = n % 4 == 0 ? h - 1 : (int)std::min<long long>(h - 1, (n - n % 4) / w);
  const int rb = std::max(row_end, 1);
  const int reach = kPreW - kPreHalo;  // 116
  const int fx1 = cb >= reach ? std::min((cb - reach) / kPreOut + 1, pt.tx) : 0;
  const int fy1 = rb >= reach ? std::min((rb - reach) / kPreOut + 1, pt.ty) : 0;
  if (fx1 > 1 && fy1 > 1) {
    pt.fx0 = 1;
    pt.fx1 = fx1;
    pt.fy0 = 1;
    pt.fy1 = fy1;
  }
  const int nfast = (pt.fx1 - pt.fx0) * (pt.fy1 - pt.fy0);
  const int nedge = pt.tx * pt.ty - nfast;
  k_precondition<<<dim3(nedge + nfast, 1, 3), kPreThreads, kPreRingSmem, s>>>(in, out, w, h, k,
                                                                             pt, nedge);
  return 1;
}

// ---------------------------------------------------------------------------
// Shared quantization rules (jpxl-encode-policy quantize.rs)
// ---------------------------------------------------------------------------

__constant__ float c_quant_bias[3] = {1.0f - 0.054650073f, 1.0f - 0.0700545f,
                                      1.0f - 0.049935103f};

__device__ float g_bias_quot[kBiasQuotN];

// quantize.rs:199 LfQuantizer::quantize with extra_precision 0.
__device__ __forceinline__ int32_t lf_quantize(float target, float m, uint32_t* err) {
  if (!(isfinite(m) && m > 0.0f)) {
    raise_error(err, kDevBadStep);
    return 0;
  }
  float scaled = target * 1.0f / m;
  int32_t q;
  if (!clamp_round(scaled, &q)) {
    raise_error(err, kDevQuantRange);
    return 0;
  }
  return q;
}

// forward.rs:779 lf_from_llf_into for an n x n (n = 1, 2, 4) LLF corner:
// divide by scale_f(y)*scale_f(x), then IDCT_2D.
__device__ __forceinline__ void lf_from_llf(const float* llf, int n, float* lf) {
  const float* sf = &c_scale_f[(n == 1 ? 0 : (n == 2 ? 1 : 2)) * 8];
  float work[16];
  for (int y = 0; y < n; ++y)
    for (int x = 0; x < n; ++x) work[y * n + x] = llf[y * n + x] / (sf[y] * sf[x]);
  if (n == 1) {
    lf[0] = work[0];  // a 1x1 IDCT_2D multiplies by sqrt(1) twice
    lf[0] = lf[0] * 1.0f * 1.0f;
    return;
  }
  // dct.rs:982 idct_2d_in_place on an n x n square: scratch = work;
  // column pass; transpose; column pass.
  float col[4], t[16];
  for (int c = 0; c < n; ++c) {
    for (int r = 0; r < n; ++r) col[r] = work[r * n + c];
    if (n == 2) idct_1d<2>(col); else idct_1d<4>(col);
    for (int r = 0; r < n; ++r) work[r * n + c] = col[r];
  }
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) t[c * n + r] = work[r * n + c];
  for (int c = 0; c < n; ++c) {
    for (int r = 0; r < n; ++r) col[r] = t[r * n + c];
    if (n == 2) idct_1d<2>(col); else idct_1d<4>(col);
    for (int r = 0; r < n; ++r) lf[r * n + c] = col[r];
  }
}

// ---------------------------------------------------------------------------
// K3 — forward transform of every square varblock of size N (policy
// lib.rs:3008 gather_square with edge replication; forward.rs:451
// forward_dct_rc = dct.rs:956 DCT_2D), LF samples (lib.rs:3100
// lf_samples_of), and the luma half of lib.rs:3237 quantize_square_varblock:
// LF quantize + reconstruct, HF choose + reconstruct.
//
// N threads per varblock: thread j transforms column j, then (after a shared
// memory transpose) row j, ending with column j of the coefficient matrix,
// which it writes to column bx*8+j of the coefficient image (coalesced).
// ---------------------------------------------------------------------------

template <int N, bool FROM_IMAGE = false>
__global__ void __launch_bounds__(128) k_fdct_luma(EncArgs a, const uint32_t* __restrict__ list,
                                                   int count) {
  constexpr int VPB = 128 / N;  // varblocks per CTA
  constexpr int n = N / 8;
  __shared__ float T[VPB][N][N + 1];
  __shared__ float LL[VPB][3][16];
  const int g = threadIdx.x / N, j = threadIdx.x % N;
  const int vi = blockIdx.x * VPB + g;
  const bool active = vi < count;
  uint32_t packed = active ? list[vi] : 0u;
  const int bx = packed & 0xffff, by = packed >> 16;
  const int x0 = bx * 8, y0 = by * 8;
  const Geo& geo = a.geo;
  const size_t plane = (size_t)geo.w * geo.h;
  const size_t cplane = (size_t)geo.W8 * geo.H8;
  // Six passes (three channels x column and row transforms) through one copy
  // of the transform: the loop stays rolled so that a 32-point transform is
  // not inlined six times past the instruction cache.  Luma runs last, so
  // its coefficients are in v when the loop ends.
  float v[N];
  if constexpr (FROM_IMAGE) {
    // The split-precision forward transform has written all three channels'
    // coefficients: column j of the luma matrix, and the LLF corners.
    if (active) {
#pragma unroll
      for (int k = 0; k < N; ++k) v[k] = a.coeff[cplane + (size_t)(y0 + k) * geo.W8 + x0 + j];
      if (j < n) {
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
          for (int k = 0; k < n; ++k)
            LL[g][c][k * n + j] = a.coeff[cplane * c + (size_t)(y0 + k) * geo.W8 + x0 + j];
      }
    }
    __syncthreads();
  }
#pragma unroll 1
  for (int pass = 0; pass < (FROM_IMAGE ? 0 : 6); ++pass) {
    const int c = pass < 2 ? 0 : (pass < 4 ? 2 : 1);
    if (active) {
      if ((pass & 1) == 0) {
        const float* p = a.pre + plane * c;
        const int xx = min(x0 + j, geo.w - 1);
#pragma unroll
        for (int r = 0; r < N; ++r) v[r] = p[(size_t)min(y0 + r, geo.h - 1) * geo.w + xx];
      } else {
#pragma unroll
        for (int k = 0; k < N; ++k) v[k] = T[g][j][k];
      }
      dct_1d<N>(v);
      if ((pass & 1) == 0) {
#pragma unroll
        for (int r = 0; r < N; ++r) T[g][r][j] = v[r];
      } else {
#pragma unroll
        for (int k = 0; k < N; ++k) a.coeff[cplane * c + (size_t)(y0 + k) * geo.W8 + x0 + j] = v[k];
        if (j < n) {
#pragma unroll
          for (int k = 0; k < n; ++k) LL[g][c][k * n + j] = v[k];
        }
      }
    }
    __syncthreads();
  }
  if (!active) return;
  // LF samples of all three channels and the luma LF quantization.
  const size_t bplane = (size_t)geo.bw * geo.bh;
  if (j < 3) {
    float lf[16];
    lf_from_llf(LL[g][j], n, lf);
    for (int i = 0; i < n * n; ++i) {
      size_t bi = (size_t)(by + i / n) * geo.bw + bx + i % n;
      a.lfs[bplane * j + bi] = lf[i];
      if (j == 1) {
        int32_t q = lf_quantize(lf[i], a.qs.m_dc[1], a.err);
        a.lfq[bplane + bi] = q;
        a.dylf[bi] = a.qs.m_dc[1] * (float)q / 1.0f;
      }
    }
  }
  // Luma HF: cells (k, j) of column j; the n x n LLF corner stays zero.
  const float mul =
      hf_multiplier(a.mul_table, a.qs.global_scale, a.hf_mul[(size_t)by * geo.bw + bx]);
  const float scale = mul * a.qs.qm[1];
  const float* m = a.dq + kDequantTableFloats + dq_offset(dq_slot(N == 8 ? 0 : (N == 16 ? 4 : 5)));
  const float bias = c_quant_bias[1];
  // The luma coefficients go through this thread's own row of T so that the
  // quantization loop need not be unrolled N times.
#pragma unroll
  for (int k = 0; k < N; ++k) T[g][j][k] = v[k];
#pragma unroll 2
  for (int k = 0; k < N; ++k) {
    const int cell = k * N + j;
    const size_t ci = (size_t)(y0 + k) * geo.W8 + x0 + j;
    int32_t q = 0;
    float recon;
    const float step = scale * __ldg(&m[cell]);
    if (k < n && j < n) {
      recon = bias_adjust(0, bias) * step;
    } else {
      q = choose(T[g][j][k], step, 1.0f / step, bias, a.err, &recon);
    }
    a.qcoeff[cplane + ci] = q;
    a.dyhf[ci] = recon;
  }
}

// ---------------------------------------------------------------------------
// K4 — chroma-from-luma estimation (policy lib.rs:3437 estimate_cfl).
//
// Decisions depend on f64 regression sums that the reference accumulates in
// one fixed sequential order.  The kernels sum in a fixed tree order instead
// and bound the difference: both orders lie within n*u*sum|t| of the exact
// sum (u = 2^-53), which bounds how far the least-squares seed
// round((s_yc/s_yy - base)*84) and the energy comparisons that confirm it
// can move.  Where the seed is more than that bound away from a decision
// boundary the tree result is the reference's; otherwise the tile (or the
// frame-wide LF pair) is recomputed sequentially in the reference's own
// order.  Residual bit costs are integer sums, exact in any order.
// ---------------------------------------------------------------------------

struct RegSums {
  double s_yy, s_yc, s_cc, a_yc;
  double n;
};

// quantize.rs:1640 best_factor on given sums; *robust = the result is
// certainly the one the reference's sequential sums give (bound `slack` on
// the absolute error of each sum, relative to its magnitude sum).
__device__ int best_factor(const RegSums& s, float base, double slack_yy, double slack_yc,
                           double slack_cc, bool* robust) {
  *robust = true;
  if (s.s_yy <= 0.0) {
    // s_yy is a sum of squares: the reference's is <= 0 only when every term
    // is zero, which the tree sum sees identically.
    return 0;
  }
  const double cf = 84.0;
  double k_ls = s.s_yc / s.s_yy;
  double star = (k_ls - (double)base) * cf;
  double centre_d = round(star);
  // Error of star from the sum differences (first order), with margin.
  double dk = (slack_yc + fabs(k_ls) * slack_yy) / s.s_yy;
  double dstar = cf * dk * 1.01 + 1e-12 * (1.0 + fabs(star));
  // Energy comparisons between neighbouring candidates are decided by
  // |j + 0.5 - star| * 2 s_yy / 84^2 against the f64 rounding of the
  // energies themselves (a few ulps of s_cc + 2|k s_yc| + k^2 s_yy).
  double kk = fabs(k_ls) + 2.0;
  double e_round = 8.0 * 1.1102230246251565e-16 *
                   (s.s_cc + slack_cc + 2.0 * kk * (fabs(s.s_yc) + slack_yc) + kk * kk * (s.s_yy + slack_yy));
  double tie = e_round * cf * cf / (2.0 * s.s_yy);
  double frac = star - floor(star);
  double dist = fabs(frac - 0.5);
  if (dist <= dstar + tie || !isfinite(star)) *robust = false;
  long long centre = (long long)centre_d;
  // candidates centre-2..centre+2 clamped to [-128,127], then 0; with a
  // robust star the nearest candidate wins outright.
  int best = 0;
  double best_e = 0.0;
  bool have = false;
  auto consider = [&](int cand) {
    double k = (double)((float)base + (float)cand / 84.0f);
    double e = s.s_cc - 2.0 * k * s.s_yc + k * k * s.s_yy;
    int ac = cand < 0 ? -cand : cand, ab = best < 0 ? -best : best;
    if (!have || e < best_e || (e == best_e && ac < ab)) {
      have = true;
      best = cand;
      best_e = e;
    }
  };
  for (int d = -2; d <= 2; ++d) {
    long long c = centre + d;
    c = c < -128 ? -128 : (c > 127 ? 127 : c);
    consider((int)c);
  }
  consider(0);
  return best;
}

__device__ __forceinline__ uint32_t factor_bits(int32_t f) {
  if (f == 0) return 0;
  uint32_t af = (uint32_t)(f < 0 ? -f : f);
  return (32u - __clz(af)) + 2u;
}

// Whether coefficient-image cell (px, py) is in the n x n LLF corner of its
// varblock; *lg = log2 of the varblock side in blocks (DCT8 0, DCT16 1,
// DCT32 2).  Square varblocks only (the encoder's cover); origins are
// naturally aligned, so positions within the varblock are masks.
__device__ __forceinline__ bool cell_is_llf(const uint8_t* map, int bw, int px, int py, int* lg) {
  const int sel = map[(size_t)(py >> 3) * bw + (px >> 3)] & 0x1f;
  const int l = sel == 0 ? 0 : (sel == 4 ? 1 : 2);
  *lg = l;
  const int mask = (8 << l) - 1;
  return (px & mask) < (1 << l) && (py & mask) < (1 << l);
}

constexpr int kCflThreads = 256;

// Per 64x64 tile in three kernels: (1) the HF regression sums (X and B
// against source Y) in double-float, one CTA per tile; (2) the seeds, one
// thread per tile and channel, so that the f64 arithmetic of best_factor and
// its robustness bound overlaps across tiles instead of holding a CTA at a
// barrier; (3) the residual bit costs of the candidate windows and the
// choice, one CTA per tile.

// (1) sums[tile][8]: s_yy, s_yx, s_xx, s_yb, s_bb, sum|yx|, sum|yb|, count.
__global__ void __launch_bounds__(kCflThreads) k_cfl_tile_sums(EncArgs a, DF* __restrict__ sums) {
  __shared__ DF s_part[kCflThreads / 32][8];
  const Geo& geo = a.geo;
  const int tx = blockIdx.x, ty = blockIdx.y;
  const int tile = ty * geo.tw + tx;
  if (*a.not_gray == 0u || !a.cfl_enabled) return;
  const size_t cplane = (size_t)geo.W8 * geo.H8;
  const int px0 = tx * 64, py0 = ty * 64;
  const int pw = min(64, geo.W8 - px0), ph = min(64, geo.H8 - py0);
  // Thread t covers column (t % 64) of rows t/64, t/64 + 4, ... of the tile:
  // coalesced rows, no divisions.
  DF syy{0, 0}, syx{0, 0}, sxx{0, 0}, syb{0, 0}, sbb{0, 0};
  float ayx = 0.0f, ayb = 0.0f, cnt = 0.0f;
  {
    const int col = threadIdx.x % 64;
    if (col < pw) {
      const int px = px0 + col;
      for (int row = threadIdx.x / 64; row < ph; row += kCflThreads / 64) {
        const int py = py0 + row;
        int lg;
        if (cell_is_llf(a.block_map, geo.bw, px, py, &lg)) continue;
        size_t ci = (size_t)py * geo.W8 + px;
        float y = a.coeff[cplane + ci];
        float x = a.coeff[ci];
        float b = a.coeff[2 * cplane + ci];
        syy = df_add(syy, df_two_prod(y, y));
        syx = df_add(syx, df_two_prod(y, x));
        sxx = df_add(sxx, df_two_prod(x, x));
        syb = df_add(syb, df_two_prod(y, b));
        sbb = df_add(sbb, df_two_prod(b, b));
        ayx += fabsf(y * x);
        ayb += fabsf(y * b);
        cnt += 1.0f;
      }
    }
  }
  // One fixed-order reduction: a butterfly per warp, then the warps in order.
  DF v[8] = {syy, syx, sxx, syb, sbb, DF{ayx, 0.0f}, DF{ayb, 0.0f}, DF{cnt, 0.0f}};
  const int lane = threadIdx.x % 32, wid = threadIdx.x / 32;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const DF t = df_warp_sum(v[q]);
    if (lane == 0) s_part[wid][q] = t;
  }
  __syncthreads();
  if (threadIdx.x < 8) {
    DF t = s_part[0][threadIdx.x];
    for (int i = 1; i < kCflThreads / 32; ++i) t = df_add(t, s_part[i][threadIdx.x]);
    sums[(size_t)tile * 8 + threadIdx.x] = t;
  }
}

// (2) seeds[tile][2] from the sums; a seed the bound cannot settle is
// recomputed from the tile's coefficients in the reference's order
// (varblocks in raster order of their origins within the tile, then
// coefficient rows and columns).
__global__ void __launch_bounds__(128) k_cfl_tile_seeds(EncArgs a, const DF* __restrict__ sums,
                                                        int* __restrict__ seeds) {
  const Geo& geo = a.geo;
  const int ntiles = geo.tw * geo.th;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 2 * ntiles) return;
  const int tile = i >> 1, ch = i & 1;
  if (*a.not_gray == 0u || !a.cfl_enabled) {
    seeds[i] = 0;
    return;
  }
  const DF* t = sums + (size_t)tile * 8;
  const double t_syy = df_value(t[0]), t_syc = df_value(t[ch == 0 ? 1 : 3]);
  const double t_scc = df_value(t[ch == 0 ? 2 : 4]), t_ayc = df_value(t[ch == 0 ? 5 : 6]);
  const double t_cnt = df_value(t[7]);
  // Distance of the double-float tree sum and of the reference's sequential
  // f64 sum from the exact sum, relative to sum|t| (the |t| sums are f32
  // estimates; the factor 2 covers their error).
  const double gam = 2.0 * (t_cnt + 64.0) * (2.2737367544323206e-13 + 1.1102230246251565e-16);
  const float base = ch == 0 ? 0.0f : 1.0f;
  int seed = 0;
  bool robust = true;
  if (t_cnt > 0.0) {
    RegSums r{t_syy, t_syc, t_scc, t_ayc, t_cnt};
    seed = best_factor(r, base, gam * t_syy, gam * t_ayc, gam * t_scc, &robust);
  }
  if (!robust) {
    atomicAdd(a.cfl_fallbacks, 1u);
    const size_t cplane = (size_t)geo.W8 * geo.H8;
    const int tx = tile % geo.tw, ty = tile / geo.tw;
    const int px0 = tx * 64, py0 = ty * 64;
    const int pw = min(64, geo.W8 - px0), ph = min(64, geo.H8 - py0);
    const float* cc = a.coeff + (ch == 0 ? 0 : 2 * cplane);
    RegSums r{0, 0, 0, 0, 0};
    for (int by = py0 / 8; by < (py0 + ph) / 8; ++by)
      for (int bx = px0 / 8; bx < (px0 + pw) / 8; ++bx) {
        uint8_t e = a.block_map[(size_t)by * geo.bw + bx];
        if (!(e & 0x80)) continue;
        int sel = e & 0x1f;
        int nb = sel == 0 ? 1 : (sel == 4 ? 2 : 4), side = nb * 8;
        for (int row = 0; row < side; ++row)
          for (int col = (row < nb ? nb : 0); col < side; ++col) {
            size_t ci = (size_t)(by * 8 + row) * geo.W8 + bx * 8 + col;
            double y = (double)a.coeff[cplane + ci];
            double c = (double)cc[ci];
            r.s_yy += y * y;
            r.s_yc += y * c;
            r.s_cc += c * c;
            r.n += 1.0;
          }
      }
    bool unused;
    seed = r.n > 0 ? best_factor(r, base, 0, 0, 0, &unused) : 0;
  }
  seeds[i] = seed;
}

// (3) Residual bits of every candidate through the DCT8x8 baseline quantizer
// (cells folded onto the 8x8 grid, lib.rs:3585), then the choice.
__global__ void __launch_bounds__(kCflThreads, 4) k_cfl_tile_bits(EncArgs a,
                                                               const int* __restrict__ seeds) {
  __shared__ uint32_t s_bits[kCflThreads / 32][8];
  __shared__ float s_step[2][64], s_rstep[2][64];
  const Geo& geo = a.geo;
  const int tx = blockIdx.x, ty = blockIdx.y;
  const int tile = ty * geo.tw + tx;
  if (*a.not_gray == 0u || !a.cfl_enabled) {
    if (threadIdx.x == 0) {
      a.cfl_x[tile] = 0;
      a.cfl_b[tile] = 0;
    }
    return;
  }
  const size_t cplane = (size_t)geo.W8 * geo.H8;
  const int px0 = tx * 64, py0 = ty * 64;
  const int pw = min(64, geo.W8 - px0), ph = min(64, geo.H8 - py0);
  // lib.rs:3735 factor_candidates(seed, -128, 127): seed-1, seed, seed+1
  // clamped and de-duplicated, then 0 if absent (every thread forms both).
  int cands[2][4], ncand[2];
  const int seed[2] = {seeds[2 * tile], seeds[2 * tile + 1]};
#pragma unroll
  for (int ch = 0; ch < 2; ++ch) {
    int nc = 0;
    for (int d = -1; d <= 1; ++d) {
      int v = min(max(seed[ch] + d, -128), 127);
      bool dup = false;
      for (int i = 0; i < nc; ++i) dup |= cands[ch][i] == v;
      if (!dup) cands[ch][nc++] = v;
    }
    bool has0 = false;
    for (int i = 0; i < nc; ++i) has0 |= cands[ch][i] == 0;
    if (!has0) cands[ch][nc++] = 0;
    ncand[ch] = nc;
  }
  // Steps of the 64 folded cells and their reciprocals, per channel.
  if (threadIdx.x < 128) {
    const int ch = threadIdx.x / 64, cell = threadIdx.x % 64;
    const float scale = a.base_mul * a.qs.qm[ch == 0 ? 0 : 2];
    const float st = scale * a.dq[(ch == 0 ? 0 : 2) * kDequantTableFloats + cell];
    s_step[ch][cell] = st;
    s_rstep[ch][cell] = 1.0f / st;
  }
  __syncthreads();
  uint32_t bits[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
  float kx[4], kb[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    kx[i] = 0.0f + (float)cands[0][i < ncand[0] ? i : 0] / 84.0f;
    kb[i] = 1.0f + (float)cands[1][i < ncand[1] ? i : 0] / 84.0f;
  }
  const bool need_x = seed[0] != 0, need_b = seed[1] != 0;
  const int ncx = need_x ? ncand[0] : 0, ncb = need_b ? ncand[1] : 0;
  if (need_x || need_b) {
    const int col = threadIdx.x % 64;
    if (col < pw) {
      const int px = px0 + col;
      // Each row's block-map entry and three samples are loaded a row ahead
      // of its quantizer evaluations, so that their latency overlaps them.
      struct Cell {
        uint8_t sel;
        float dy, x, b;
      };
      auto fetch = [&](int row) {
        const int py = py0 + row;
        const size_t ci = (size_t)py * geo.W8 + px;
        return Cell{a.block_map[(size_t)(py >> 3) * geo.bw + (px >> 3)], a.dyhf[ci], a.coeff[ci],
                    a.coeff[2 * cplane + ci]};
      };
      int row = threadIdx.x / 64;
      Cell nxt = row < ph ? fetch(row) : Cell{0, 0.0f, 0.0f, 0.0f};
      for (; row < ph; row += kCflThreads / 64) {
        const int py = py0 + row;
        const Cell cur = nxt;
        if (row + kCflThreads / 64 < ph) nxt = fetch(row + kCflThreads / 64);
        // cell_is_llf on the prefetched block-map entry.
        const int sel = cur.sel & 0x1f;
        const int lg = sel == 0 ? 0 : (sel == 4 ? 1 : 2);
        const int mask = (8 << lg) - 1;
        if ((px & mask) < (1 << lg) && (py & mask) < (1 << lg)) continue;
        const int cell8 = ((py & mask) >> lg) * 8 + ((px & mask) >> lg);
        const float dy = cur.dy, x = cur.x, b = cur.b;
        const float step_x = s_step[0][cell8], rstep_x = s_rstep[0][cell8];
        const float step_b = s_step[1][cell8], rstep_b = s_rstep[1][cell8];
        float rc;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          if (c < ncx)
            bits[0][c] += residual_bits(
                choose(x - kx[c] * dy, step_x, rstep_x, c_quant_bias[0], a.err, &rc));
          if (c < ncb)
            bits[1][c] += residual_bits(
                choose(b - kb[c] * dy, step_b, rstep_b, c_quant_bias[2], a.err, &rc));
        }
      }
    }
  }
  // Integer sums (exact in any order): butterflies, then warps in order.
  // A tile holds at most 4096 cells of at most 22 bits, so 32 bits suffice.
  {
    uint32_t v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      v[q] = bits[q / 4][q % 4];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
    }
    const int lane = threadIdx.x % 32, wid = threadIdx.x / 32;
    if (lane == 0)
#pragma unroll
      for (int q = 0; q < 8; ++q) s_bits[wid][q] = v[q];
    __syncthreads();
  }
  if (threadIdx.x % 32 == 0 && threadIdx.x < 64) {
    const int ch = threadIdx.x / 32;
    unsigned long long tot[4];
    for (int c = 0; c < 4; ++c) {
      unsigned long long t = 0;
      for (int i = 0; i < kCflThreads / 32; ++i) t += s_bits[i][ch * 4 + c];
      tot[c] = t;
    }
    int result = 0;
    if (seed[ch] != 0) {
      // lib.rs:3966 refine_hf_factor: cost(0) first, then each non-zero
      // candidate needs residual + factor bits strictly below (ties to the
      // smaller magnitude).
      unsigned long long best_cost = 0;
      for (int c = 0; c < ncand[ch]; ++c)
        if (cands[ch][c] == 0) best_cost = tot[c];
      int best_f = 0;
      for (int c = 0; c < ncand[ch]; ++c) {
        int f = cands[ch][c];
        if (f == 0) continue;
        unsigned long long fb = factor_bits(f);
        unsigned long long cutoff = best_cost > fb ? best_cost - fb : 0;
        if (tot[c] > cutoff) continue;
        unsigned long long cost = tot[c] + fb;
        int af = f < 0 ? -f : f, ab = best_f < 0 ? -best_f : best_f;
        if (cost < best_cost || (cost == best_cost && af < ab)) {
          best_cost = cost;
          best_f = f;
        }
      }
      result = best_f;
    }
    if (ch == 0) a.cfl_x[tile] = (int8_t)result;
    else a.cfl_b[tile] = (int8_t)result;
  }
}

// Frame-wide LF pair (lib.rs:3831 refine_lf_factors) in four kernels: the
// regression sums of every LF sample as per-CTA double-float partials across
// the GPU; one CTA folding them in a fixed order into the two seeds (with the
// sequential fallback in the reference's LF-group / band / varblock / cell
// order when a seed is not robust); the residual bit costs of both candidate
// windows as per-CTA partials; one CTA folding those and making the joint
// choice.
constexpr int kLfThreads = 256;

__device__ void lf_candidates(int seed, int* c, int* nc_out) {
  int nc = 0;
  for (int d = -1; d <= 1; ++d) {
    int v = min(max(seed + d, -128), 127);
    bool dup = false;
    for (int i = 0; i < nc; ++i) dup |= c[i] == v;
    if (!dup) c[nc++] = v;
  }
  bool has0 = false;
  for (int i = 0; i < nc; ++i) has0 |= c[i] == 0;
  if (!has0) c[nc++] = 0;
  *nc_out = nc;
}

__device__ __forceinline__ bool cfl_off(const EncArgs& a) {
  return *a.not_gray == 0u || !a.cfl_enabled;
}

// Partial sums per CTA: [kLfCtas][7] double-float (yy, yx, xx, yb, bb, |yx|, |yb|).
__global__ void __launch_bounds__(kLfThreads) k_cfl_lf_sums(EncArgs a, DF* part) {
  __shared__ DF s_w[kLfThreads / 32][7];
  if (cfl_off(a)) return;
  const size_t nb = (size_t)a.geo.bw * a.geo.bh;
  DF v[7] = {};
  for (size_t i = (size_t)blockIdx.x * kLfThreads + threadIdx.x; i < nb;
       i += (size_t)kLfCtas * kLfThreads) {
    const float y = a.lfs[nb + i], x = a.lfs[i], b = a.lfs[2 * nb + i];
    v[0] = df_add(v[0], df_two_prod(y, y));
    v[1] = df_add(v[1], df_two_prod(y, x));
    v[2] = df_add(v[2], df_two_prod(x, x));
    v[3] = df_add(v[3], df_two_prod(y, b));
    v[4] = df_add(v[4], df_two_prod(b, b));
    v[5].hi += fabsf(y * x);
    v[6].hi += fabsf(y * b);
  }
  const int lane = threadIdx.x % 32, wid = threadIdx.x / 32;
#pragma unroll
  for (int q = 0; q < 7; ++q) {
    DF t = df_warp_sum(v[q]);
    if (lane == 0) s_w[wid][q] = t;
  }
  __syncthreads();
  if (threadIdx.x < 7) {
    DF t = s_w[0][threadIdx.x];
    for (int i = 1; i < kLfThreads / 32; ++i) t = df_add(t, s_w[i][threadIdx.x]);
    part[blockIdx.x * 7 + threadIdx.x] = t;
  }
}

__global__ void __launch_bounds__(64) k_cfl_lf_seed(EncArgs a, const DF* part, int* seeds) {
  __shared__ double s_t[7];
  const Geo& geo = a.geo;
  if (cfl_off(a)) {
    if (threadIdx.x == 0) {
      seeds[0] = 0;
      seeds[1] = 0;
    }
    return;
  }
  if (threadIdx.x < 7) {
    DF t = part[threadIdx.x];
    for (int c = 1; c < kLfCtas; ++c) t = df_add(t, part[c * 7 + threadIdx.x]);
    s_t[threadIdx.x] = df_value(t);
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  const size_t nb = (size_t)geo.bw * geo.bh;
  const double* t = s_t;
  const double n = (double)nb;
  const double gam = 2.0 * (n + 64.0) * (2.2737367544323206e-13 + 1.1102230246251565e-16);
  bool rx, rb;
  RegSums sx{t[0], t[1], t[2], t[5], n}, sb{t[0], t[3], t[4], t[6], n};
  int seed_x = best_factor(sx, 0.0f, gam * t[0], gam * t[5], gam * t[2], &rx);
  int seed_b = best_factor(sb, 1.0f, gam * t[0], gam * t[6], gam * t[4], &rb);
  if (!rx || !rb) {
    atomicAdd(a.cfl_fallbacks, 1u);
    RegSums qx{0, 0, 0, 0, n}, qb{0, 0, 0, 0, n};
    const int G = 256;
    const int gw = (geo.bw + G - 1) / G, gh = (geo.bh + G - 1) / G;
    for (int gy = 0; gy < gh; ++gy)
      for (int gx = 0; gx < gw; ++gx) {
        int by0 = gy * G, bx0 = gx * G;
        int gbh = min(G, geo.bh - by0), gbw = min(G, geo.bw - bx0);
        for (int trow = 0; trow < (gbh + 7) / 8; ++trow)
          for (int by = by0 + trow * 8; by < min(by0 + trow * 8 + 8, by0 + gbh); ++by)
            for (int bx = bx0; bx < bx0 + gbw; ++bx) {
              uint8_t e = a.block_map[(size_t)by * geo.bw + bx];
              if (!(e & 0x80)) continue;
              int sel = e & 0x1f, nbk = sel == 0 ? 1 : (sel == 4 ? 2 : 4);
              for (int i = 0; i < nbk * nbk; ++i) {
                size_t bi = (size_t)(by + i / nbk) * geo.bw + bx + i % nbk;
                double y = a.lfs[nb + bi], x = a.lfs[bi], b = a.lfs[2 * nb + bi];
                qx.s_yy += y * y; qx.s_yc += y * x; qx.s_cc += x * x;
                qb.s_yy += y * y; qb.s_yc += y * b; qb.s_cc += b * b;
              }
            }
      }
    bool r;
    seed_x = best_factor(qx, 0.0f, 0, 0, 0, &r);
    seed_b = best_factor(qb, 1.0f, 0, 0, 0, &r);
  }
  seeds[0] = seed_x;
  seeds[1] = seed_b;
}

// Residual bits of every candidate per CTA: [kLfCtas][8] (X candidates 0..3,
// B candidates 0..3).  At most 2^16 * 22 bits per CTA fit in 32 bits for
// frames up to 2^28 LF samples.
__global__ void __launch_bounds__(kLfThreads) k_cfl_lf_bits(EncArgs a, const int* seeds,
                                                            uint32_t* part) {
  __shared__ uint32_t s_w[kLfThreads / 32][8];
  if (cfl_off(a)) return;
  const size_t nb = (size_t)a.geo.bw * a.geo.bh;
  int cand[2][4], ncand[2];
  lf_candidates(seeds[0], cand[0], &ncand[0]);
  lf_candidates(seeds[1], cand[1], &ncand[1]);
  uint32_t bits[8] = {};
  float k[2][4];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    k[0][c] = 0.0f + (float)cand[0][c < ncand[0] ? c : 0] / 84.0f;
    k[1][c] = 1.0f + (float)cand[1][c < ncand[1] ? c : 0] / 84.0f;
  }
  for (size_t i = (size_t)blockIdx.x * kLfThreads + threadIdx.x; i < nb;
       i += (size_t)kLfCtas * kLfThreads) {
    const float dy = a.dylf[i], x = a.lfs[i], b = a.lfs[2 * nb + i];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      if (c < ncand[0]) bits[c] += residual_bits(lf_quantize(x - k[0][c] * dy, a.qs.m_dc[0], a.err));
      if (c < ncand[1]) bits[4 + c] += residual_bits(lf_quantize(b - k[1][c] * dy, a.qs.m_dc[2], a.err));
    }
  }
  const int lane = threadIdx.x % 32, wid = threadIdx.x / 32;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    uint32_t t = bits[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) s_w[wid][q] = t;
  }
  __syncthreads();
  if (threadIdx.x < 8) {
    uint32_t t = 0;
    for (int i = 0; i < kLfThreads / 32; ++i) t += s_w[i][threadIdx.x];
    part[blockIdx.x * 8 + threadIdx.x] = t;
  }
}

__global__ void __launch_bounds__(32) k_cfl_lf_pick(EncArgs a, const int* seeds,
                                                    const uint32_t* part) {
  __shared__ unsigned long long s_cost[8];
  int* out = a.lf_factors;
  if (cfl_off(a)) {
    if (threadIdx.x == 0) {
      out[0] = 0;
      out[1] = 0;
    }
    return;
  }
  if (threadIdx.x < 8) {
    unsigned long long t = 0;
    for (int c = 0; c < kLfCtas; ++c) t += part[c * 8 + threadIdx.x];
    s_cost[threadIdx.x] = t;
  }
  __syncwarp();
  if (threadIdx.x != 0) return;
  int cand[2][4], ncand[2];
  lf_candidates(seeds[0], cand[0], &ncand[0]);
  lf_candidates(seeds[1], cand[1], &ncand[1]);
  const unsigned long long* cost0 = s_cost;
  const unsigned long long* cost1 = s_cost + 4;
  unsigned long long nx = 0, nbb = 0;
  for (int c = 0; c < ncand[0]; ++c) if (cand[0][c] == 0) { nx = cost0[c]; break; }
  for (int c = 0; c < ncand[1]; ++c) if (cand[1][c] == 0) { nbb = cost1[c]; break; }
  int bx = 0, bbf = 0;
  unsigned long long best = nx + nbb;
  for (int i = 0; i < ncand[0]; ++i)
    for (int j = 0; j < ncand[1]; ++j) {
      int fx = cand[0][i], fb = cand[1][j];
      unsigned long long c = cost0[i] + cost1[j];
      if (fx != 0 || fb != 0) c += 50ull + factor_bits(fx) + factor_bits(fb);
      int mag = abs(fx) + abs(fb), bmag = abs(bx) + abs(bbf);
      if (c < best || (c == best && mag < bmag)) {
        bx = fx;
        bbf = fb;
        best = c;
      }
    }
  out[0] = bx;
  out[1] = bbf;
}

// ---------------------------------------------------------------------------
// K5 — chroma half of lib.rs:3237 quantize_square_varblock: LF targets
// c - k_lf*dY_lf, HF targets c - k_hf*dY_hf (no FMA), nearest choice.
// ---------------------------------------------------------------------------

template <int N>
__global__ void __launch_bounds__(128) k_quant_chroma(EncArgs a, const uint32_t* __restrict__ list,
                                                      int count) {
  constexpr int VPB = 128 / N;
  constexpr int n = N / 8;
  const int g = threadIdx.x / N, j = threadIdx.x % N;
  const int vi = blockIdx.x * VPB + g;
  if (vi >= count) return;
  const uint32_t packed = list[vi];
  const int bx = packed & 0xffff, by = packed >> 16;
  const int x0 = bx * 8, y0 = by * 8;
  const Geo& geo = a.geo;
  const size_t cplane = (size_t)geo.W8 * geo.H8;
  const size_t bplane = (size_t)geo.bw * geo.bh;
  const int tile = (by / 8) * geo.tw + bx / 8;
  const int fx = a.lf_factors[0], fb = a.lf_factors[1];
  const float k_lf[3] = {0.0f + (float)fx / 84.0f, 0.0f, 1.0f + (float)fb / 84.0f};
  const float k_hf[3] = {0.0f + (float)a.cfl_x[tile] / 84.0f, 0.0f,
                         1.0f + (float)a.cfl_b[tile] / 84.0f};
  // LF: n*n samples, thread j < n*n takes sample j.
  if (j < n * n) {
    size_t bi = (size_t)(by + j / n) * geo.bw + bx + j % n;
    float dy = a.dylf[bi];
    for (int c = 0; c <= 2; c += 2) {
      float target = a.lfs[bplane * c + bi] - k_lf[c] * dy;
      a.lfq[bplane * c + bi] = lf_quantize(target, a.qs.m_dc[c], a.err);
    }
  }
  const float mul =
      hf_multiplier(a.mul_table, a.qs.global_scale, a.hf_mul[(size_t)by * geo.bw + bx]);
  const int off = dq_offset(dq_slot(N == 8 ? 0 : (N == 16 ? 4 : 5)));
  for (int c = 0; c <= 2; c += 2) {
    const float scale = mul * a.qs.qm[c];
    const float* m = a.dq + c * kDequantTableFloats + off;
    const float bias = c_quant_bias[c];
#pragma unroll 4
    for (int k = 0; k < N; ++k) {
      const size_t ci = (size_t)(y0 + k) * geo.W8 + x0 + j;
      int32_t q = 0;
      if (!(k < n && j < n)) {
        float target = a.coeff[cplane * c + ci] - k_hf[c] * a.dyhf[ci];
        float rc;
        const float step = scale * __ldg(&m[k * N + j]);
        q = choose(target, step, 1.0f / step, bias, a.err, &rc);
      }
      a.qcoeff[cplane * c + ci] = q;
    }
  }
}

int launch_fdct_luma(const EncArgs& a, const uint32_t* const* lists, const int* counts,
                     const cudaStream_t* s) {
  // square classes: 0 -> DCT8, 1 -> DCT16, 2 -> DCT32, each on its stream
  int k = 0;
  if (counts[0]) { k_fdct_luma<8><<<(counts[0] + 15) / 16, 128, 0, s[0]>>>(a, lists[0], counts[0]); ++k; }
  if (counts[1]) { k_fdct_luma<16><<<(counts[1] + 7) / 8, 128, 0, s[1]>>>(a, lists[1], counts[1]); ++k; }
  if (counts[2]) { k_fdct_luma<32><<<(counts[2] + 3) / 4, 128, 0, s[2]>>>(a, lists[2], counts[2]); ++k; }
  return k;
}

int launch_luma_from_image(const EncArgs& a, const uint32_t* const* lists, const int* counts,
                           const cudaStream_t* s) {
  int k = 0;
  if (counts[0]) { k_fdct_luma<8, true><<<(counts[0] + 15) / 16, 128, 0, s[0]>>>(a, lists[0], counts[0]); ++k; }
  if (counts[1]) { k_fdct_luma<16, true><<<(counts[1] + 7) / 8, 128, 0, s[1]>>>(a, lists[1], counts[1]); ++k; }
  if (counts[2]) { k_fdct_luma<32, true><<<(counts[2] + 3) / 4, 128, 0, s[2]>>>(a, lists[2], counts[2]); ++k; }
  return k;
}

int launch_cfl(const EncArgs& a, int* lf_seeds, void* lf_scratch, void* tile_scratch,
               cudaStream_t s, cudaStream_t lf_s) {
  dim3 tiles(a.geo.tw, a.geo.th);
  const int ntiles = a.geo.tw * a.geo.th;
  DF* tile_sums = (DF*)tile_scratch;
  int* tile_seeds = (int*)((char*)tile_scratch + (size_t)ntiles * 8 * sizeof(DF));
  k_cfl_tile_sums<<<tiles, kCflThreads, 0, s>>>(a, tile_sums);
  k_cfl_tile_seeds<<<(2 * ntiles + 127) / 128, 128, 0, s>>>(a, tile_sums, tile_seeds);
  k_cfl_tile_bits<<<tiles, kCflThreads, 0, s>>>(a, tile_seeds);
  DF* sums = (DF*)lf_scratch;
  uint32_t* bits = (uint32_t*)((char*)lf_scratch + kLfCtas * 7 * sizeof(DF));
  // The LF factors' chain reads only the LF planes: on its own stream.
  k_cfl_lf_sums<<<kLfCtas, kLfThreads, 0, lf_s>>>(a, sums);
  k_cfl_lf_seed<<<1, 64, 0, lf_s>>>(a, sums, lf_seeds);
  k_cfl_lf_bits<<<kLfCtas, kLfThreads, 0, lf_s>>>(a, lf_seeds, bits);
  k_cfl_lf_pick<<<1, 32, 0, lf_s>>>(a, lf_seeds, bits);
  return 7;
}

int launch_quant_chroma(const EncArgs& a, const uint32_t* const* lists, const int* counts,
                        const cudaStream_t* s) {
  int k = 0;
  if (counts[0]) { k_quant_chroma<8><<<(counts[0] + 15) / 16, 128, 0, s[0]>>>(a, lists[0], counts[0]); ++k; }
  if (counts[1]) { k_quant_chroma<16><<<(counts[1] + 7) / 8, 128, 0, s[1]>>>(a, lists[1], counts[1]); ++k; }
  if (counts[2]) { k_quant_chroma<32><<<(counts[2] + 3) / 4, 128, 0, s[2]>>>(a, lists[2], counts[2]); ++k; }
  return k;
}

__global__ void k_mul_table(uint32_t global_scale, float* table) {
  const int h = threadIdx.x;
  if (h < kMulTableN) table[h] = hf_multiplier_f64(global_scale, (uint32_t)h);
}

void launch_mul_table(uint32_t global_scale, float* table, cudaStream_t s) {
  k_mul_table<<<1, kMulTableN, 0, s>>>(global_scale, table);
}

cudaError_t configure_encode_kernels() {
  return cudaFuncSetAttribute(k_precondition, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)kPreRingSmem);
}

void upload_dct_constants(const float* iv4, const float* iv8, const float* iv16,
                          const float* scale_f, cudaStream_t s) {
  cudaMemcpyToSymbolAsync(c_iv4, iv4, sizeof(float) * 16, 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_iv8, iv8, sizeof(float) * 64, 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_iv16, iv16, sizeof(float) * 256, 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_scale_f, scale_f, sizeof(float) * 32, 0, cudaMemcpyHostToDevice, s);
  // 0.145f / q in IEEE single precision, as bias_adjust divides on the device.
  static float quot[kBiasQuotN];
  quot[0] = 0.0f;
  for (int q = 1; q < kBiasQuotN; ++q) quot[q] = 0.145f / (float)q;
  cudaMemcpyToSymbolAsync(g_bias_quot, quot, sizeof quot, 0, cudaMemcpyHostToDevice, s);
}

}  // namespace jpxlg
