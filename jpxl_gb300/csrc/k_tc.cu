// k_tc.cu — the split-precision form of the path's transforms, on the
// tcgen05 tensor cores:
//   T1 k_fdct_tc<N, TERMS>    forward DCT_2D of the encoder's square varblocks
//                             (jpxl-core forward.rs:451 forward_dct_rc ->
//                             dct.rs:956, with the edge replication of policy
//                             lib.rs:3008 gather_square) into the coefficient
//                             image, all three channels
//   T2 k_render_tc<N, TERMS>  the render's dequantize, HF CfL, LLF and
//                             IDCT_2D (plan-render lib.rs:853-1136,
//                             varblock.rs:817, dct.rs:982) with the in-frame
//                             scatter and the per-block EPF sigma
//                             (restoration.rs:338), square varblocks
//
// Each 2-D transform is two batched dense contractions issued by
// tcgen05.mma (kind::f16, bf16 operands from shared memory, FP32
// accumulators in TMEM).  Every f32 operand is split into TERMS bf16 terms
// (x = t0 + t1 [+ t2], each term the bf16 rounding of what the previous ones
// leave); TERMS = 2 takes the three products t1*u0 + t0*u1 + t0*u0 (BF16x3),
// TERMS = 3 the six with term order <= 2 (BF16x6), smallest first.  The bf16
// products are exact in FP32, so the result carries FP32-level error (three
// terms) or about 2^-16 relative error (two terms); neither follows the
// reference's butterfly roundings, so coefficients differ from the
// reference's in their last bits and quantized integers can differ at
// decision boundaries: the FP32 kernels stay the bit-exact form.
//
// Tile: 128 rows = 128/N varblocks of one size N, one row of one varblock
// per thread (thread t = (b, r): block b = t / N, row r = t % N).
//   pass 1  A1 = the N x N transform matrix stacked 128/N times (constant),
//           B1 = the tile's data rows (row t from thread t, K-major), so
//           D1[(j, r)][(b, r')] = sum_k M[r][k] X_b[r'][k] for every block
//           pair; thread (j, r) reads its own block's N columns (b = j).
//   pass 2  A2 = those rows (written by the thread that read them, into the
//           B1 buffer, which pass 1 has finished with), B2 = the transform
//           matrix (constant); D2[(j, r)][k] is row r of block j's result.
// No transpose goes through shared memory: every operand row is written as
// 16-byte K-major chunks by the thread that owns it.  Forward (M = D): X
// rows are sample rows y, D2 rows are landscape coefficient rows v.  Inverse
// (M = I): X rows are landscape coefficient rows v, D2 rows are sample rows
// y.  Square shapes keep the coefficient matrix in the transposed
// (horizontal-frequency-first) layout of dct.rs:956, which is what these two
// passes produce and consume.
//
// Shared-memory operands use the no-swizzle K-major canonical layout: core
// matrices of 8 rows x 16 bytes (128 contiguous bytes), the K-direction
// core-matrix stride in the descriptor's leading-byte-offset field and the
// 8-row-group stride (128 bytes) in its stride-byte-offset field.  The
// kernels are persistent (grid-stride over tiles); each CTA allocates 128
// TMEM columns once, loads the constant operands once, and frees the TMEM on
// every exit path.  Every wait on the MMA's mbarrier is bounded; a wait that
// runs out raises kDevTcTimeout in the error word, waits once more (bounded)
// for the MMAs in flight and returns after freeing the TMEM.
//
// This unit is compiled as whole-program device code, without the
// relocatable device code of the library's other units: on sm_103a with
// CUDA 13.0, the same tcgen05 sequence compiled with -rdc=true produced
// wrong accumulators (measured: every element of a 128x128x32 product), and
// correct ones without.  It therefore refers to no device symbol of another
// unit: its constants are its own, and the render's LLF rectangles and EPF
// sigma come from k_llf_sigma (k_render.cu) through a buffer.
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>

#include "jpxlg_defs.cuh"
#include "jpxlg_internal.h"
#include "jpxlg_kernels.h"

namespace jpxlg {

// color.rs:591 quant biases (the same literals as the encoder's table).
__constant__ float c_tc_bias[3] = {1.0f - 0.054650073f, 1.0f - 0.0700545f,
                                   1.0f - 0.049935103f};

// Normative transform matrices of sizes 8, 16, 32 (row-major, f32 of the
// f64 cosines): [0] inverse I[i][u] = (u ? sqrt2 : 1) cos(pi (2i+1) u / 2N)
// (dct.rs:749 idct_1d), [1] forward D[u][i] = I[i][u] / N (dct.rs:731).
__device__ float g_tc_basis[2][3][32 * 32];

namespace tc {

constexpr int kThreads = 128;
constexpr uint32_t kWaitLimit = 1u << 24;
constexpr int kTmemCols = 128;  // pass 1's accumulator, reused by pass 2

template <int N, int TERMS>
struct Tile {
  static constexpr int kVpt = 128 / N;           // varblocks per tile
  static constexpr int kKp = N < 16 ? 16 : N;    // contraction length padded to a bf16 MMA's 16
  static constexpr int kNp = N < 16 ? 16 : N;    // pass-2 width (M = 128 needs a multiple of 16)
  static constexpr int kOpTerm = 128 * kKp * 2;  // bytes of one term of a 128-row operand
  static constexpr int kB2Term = kNp * kKp * 2;
  static constexpr int kA1 = 0;
  static constexpr int kB1 = TERMS * kOpTerm;
  static constexpr int kB2 = 2 * TERMS * kOpTerm;
  static constexpr int kBytes = kB2 + TERMS * kB2Term;
  static constexpr uint32_t kLbo128 = (128 / 8) * 128;  // K-direction core-matrix stride
  static constexpr uint32_t kLboB2 = (kNp / 8) * 128;
  static constexpr int kSizeIdx = N == 8 ? 0 : (N == 16 ? 1 : 2);
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Byte offset of (row, k) in a K-major operand of `rows` rows (k % 8 == 0).
__device__ __forceinline__ uint32_t kmaj_off(int row, int k, int rows) {
  return (uint32_t)(((k >> 3) * (rows >> 3) + (row >> 3)) * 128 + (row & 7) * 16);
}

// Shared-memory matrix descriptor: start address, leading-byte offset (the
// K-direction core-matrix stride), stride-byte offset (8-row groups), the
// descriptor version of this architecture family (bit 46), no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// Instruction descriptor, kind::f16: FP32 accumulator, bf16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(mbar))
      : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity) {
  uint32_t done = 0;
  for (uint32_t it = 0; it < kWaitLimit && !done; ++it) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(mbar)), "r"(parity)
        : "memory");
  }
  return done != 0;
}

__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* slot) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(slot)),
               "r"(kTmemCols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr),
               "r"(kTmemCols)
               : "memory");
}

// N consecutive TMEM columns of this warp's 32 lanes (one row per thread).
// The load and its wait are one asm statement: the destination registers of
// tcgen05.ld are undefined until tcgen05.wait::ld, and an output register
// read by a plain move could otherwise be scheduled between the two.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr)
      : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7])
      : "r"(taddr)
      : "memory");
}

// Splits x[0..N) (zero beyond N up to the padded length KP) into TERMS bf16
// terms and stores row `row` of a K-major operand of `rows` rows whose terms
// lie term_bytes apart.
template <int N, int TERMS, int KP>
__device__ __forceinline__ void store_row(uint8_t* region, int term_bytes, int row, int rows,
                                          const float* x) {
#pragma unroll
  for (int kc = 0; kc < KP / 8; ++kc) {
    uint32_t w[TERMS][4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int k0 = kc * 8 + 2 * i;
      float lo = k0 < N ? x[k0] : 0.0f;
      float hi = k0 + 1 < N ? x[k0 + 1] : 0.0f;
#pragma unroll
      for (int t = 0; t < TERMS; ++t) {
        const __nv_bfloat16 bl = __float2bfloat16_rn(lo), bh = __float2bfloat16_rn(hi);
        w[t][i] = (uint32_t)__bfloat16_as_ushort(bl) | ((uint32_t)__bfloat16_as_ushort(bh) << 16);
        lo = lo - __bfloat162float(bl);
        hi = hi - __bfloat162float(bh);
      }
    }
    const uint32_t off = kmaj_off(row, kc * 8, rows);
#pragma unroll
    for (int t = 0; t < TERMS; ++t)
      *reinterpret_cast<uint4*>(region + t * term_bytes + off) =
          make_uint4(w[t][0], w[t][1], w[t][2], w[t][3]);
  }
}

// The products of one contraction, smallest terms first: A term pa[p] times
// B term pb[p].  Issued by one thread.
template <int TERMS>
__device__ __forceinline__ void issue_split(uint32_t tmem, uint32_t a_base, uint32_t a_term,
                                            uint32_t a_lbo, uint32_t b_base, uint32_t b_term,
                                            uint32_t b_lbo, int ksteps, uint32_t idesc) {
  const int np = TERMS == 2 ? 3 : 6;
  const int pa[6] = {TERMS == 2 ? 1 : 2, TERMS == 2 ? 0 : 1, 0, 1, 0, 0};
  const int pb[6] = {0, 1, TERMS == 2 ? 0 : 2, 0, 1, 0};
  uint32_t acc = 0;
  for (int p = 0; p < np; ++p)
    for (int ks = 0; ks < ksteps; ++ks) {
      const uint64_t da = sdesc(a_base + pa[p] * a_term + ks * 2 * a_lbo, a_lbo, 128);
      const uint64_t db = sdesc(b_base + pb[p] * b_term + ks * 2 * b_lbo, b_lbo, 128);
      mma_bf16(tmem, da, db, idesc, acc);
      acc = 1;
    }
}

// reconstruct.rs:50 bias_adjust: q * bias for |q| <= 1, else q - 0.145 / q,
// the quotient by the same IEEE division the library's table holds.
__device__ __forceinline__ float bias_adjust(int32_t q, float bias) {
  const float f = (float)q;
  if (q >= -1 && q <= 1) return f * bias;
  const int32_t aq = q < 0 ? -q : q;
  const float af = (float)aq;
  const float r = af - 0.145f / af;
  return q < 0 ? -r : r;
}

// CTA-wide state of a persistent tile loop.
struct State {
  uint32_t tmem;
  uint32_t phase;
  bool ok;
};

// Loads the constant operands: A1 row t = M[t % N], B2 row r = M[r] (zero
// rows past N); M = the inverse (dir 0) or forward (dir 1) matrix.
template <int N, int TERMS>
__device__ __forceinline__ void load_basis(uint8_t* smem, int dir) {
  using T = Tile<N, TERMS>;
  const float* m = g_tc_basis[dir][T::kSizeIdx];
  const int t = threadIdx.x;
  float row[N];
#pragma unroll
  for (int k = 0; k < N; ++k) row[k] = m[(t % N) * N + k];
  store_row<N, TERMS, T::kKp>(smem + T::kA1, T::kOpTerm, t, 128, row);
  if (t < T::kNp) {
#pragma unroll
    for (int k = 0; k < N; ++k) row[k] = t < N ? m[t * N + k] : 0.0f;
    store_row<N, TERMS, T::kKp>(smem + T::kB2, T::kB2Term, t, T::kNp, row);
  }
}

// Both passes for the tile's rows: row[] holds this thread's data row on
// entry and its result row on return.  Collective over the CTA.
template <int N, int TERMS>
__device__ __forceinline__ void transform_rows(uint8_t* smem, uint64_t* mbar, State& st,
                                               float* row) {
  using T = Tile<N, TERMS>;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  const uint32_t s0 = smem_u32(smem);
  // pass 1
  store_row<N, TERMS, T::kKp>(smem + T::kB1, T::kOpTerm, t, 128, row);
  fence_async_smem();
  before_sync();
  __syncthreads();
  after_sync();
  if (t == 0) {
    issue_split<TERMS>(st.tmem, s0 + T::kA1, T::kOpTerm, T::kLbo128, s0 + T::kB1, T::kOpTerm,
                       T::kLbo128, T::kKp / 16, idesc_bf16(128, 128));
    mma_commit(mbar);
  }
  bool ok = mbar_wait(mbar, st.phase);
  st.phase ^= 1u;
  if (__syncthreads_or(!ok)) {
    st.ok = false;
    return;
  }
  after_sync();
  {
    // This warp's 32 columns hold its lanes' blocks (warp w: blocks
    // 32w/N .. 32(w+1)/N - 1); each lane keeps its own block's N.
    uint32_t r[32];
    tmem_ld32(st.tmem + lane_base + (uint32_t)(warp * 32), r);
    const int off = lane - lane % N;
#pragma unroll
    for (int s = 0; s < 32 / N; ++s)
      if (off == s * N) {
#pragma unroll
        for (int i = 0; i < N; ++i) row[i] = __uint_as_float(r[s * N + i]);
      }
  }
  // pass 2: A2 is written into B1's buffer, which pass 1 has consumed.
  store_row<N, TERMS, T::kKp>(smem + T::kB1, T::kOpTerm, t, 128, row);
  fence_async_smem();
  before_sync();
  __syncthreads();
  after_sync();
  if (t == 0) {
    issue_split<TERMS>(st.tmem, s0 + T::kB1, T::kOpTerm, T::kLbo128, s0 + T::kB2, T::kB2Term,
                       T::kLboB2, T::kKp / 16, idesc_bf16(128, T::kNp));
    mma_commit(mbar);
  }
  ok = mbar_wait(mbar, st.phase);
  st.phase ^= 1u;
  if (__syncthreads_or(!ok)) {
    st.ok = false;
    return;
  }
  after_sync();
  {
    uint32_t r[N];
    if constexpr (N == 32) tmem_ld32(st.tmem + lane_base, r);
    else if constexpr (N == 16) tmem_ld16(st.tmem + lane_base, r);
    else tmem_ld8(st.tmem + lane_base, r);
#pragma unroll
    for (int i = 0; i < N; ++i) row[i] = __uint_as_float(r[i]);
  }
  before_sync();
}

__device__ __forceinline__ void begin(uint32_t* slot, uint64_t* mbar) {
  if ((threadIdx.x >> 5) == 0) tmem_alloc(slot);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(1)
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
}

// Frees the TMEM on every exit path; after a timed-out wait, first gives the
// MMAs in flight one more bounded wait.
__device__ __forceinline__ void end(State& st, uint64_t* mbar, uint32_t* err) {
  if (!st.ok) {
    if (threadIdx.x == 0) raise_error(err, kDevTcTimeout);
    mbar_wait(mbar, st.phase ^ 1u);
  }
  before_sync();
  __syncthreads();
  after_sync();
  if ((threadIdx.x >> 5) == 0) tmem_free(st.tmem);
}

}  // namespace tc

namespace {

using namespace tc;

// ---------------------------------------------------------------------------
// T1 — forward DCT_2D of the square varblocks of size N into the
// coefficient image (all three channels).
// ---------------------------------------------------------------------------
template <int N, int TERMS>
__global__ void __launch_bounds__(kThreads) k_fdct_tc(EncArgs a, const uint32_t* __restrict__ list,
                                                       int count, int ntiles) {
  using T = Tile<N, TERMS>;
  extern __shared__ __align__(128) uint8_t smem[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_slot;
  const int t = threadIdx.x;
  const int b = t / N, r = t % N;
  begin(&tmem_slot, &mbar);
  load_basis<N, TERMS>(smem, 1);
  before_sync();
  __syncthreads();
  after_sync();
  State st{tmem_slot, 0u, true};
  const Geo& geo = a.geo;
  const size_t plane = (size_t)geo.w * geo.h;
  const size_t cplane = (size_t)geo.W8 * geo.H8;
  // The varblock of this thread's row in a tile, and its sample row r of one
  // channel, edges replicated (lib.rs:3008); zeros past the list's end.
  struct Src {
    bool active;
    int x0, y0;
  };
  auto locate = [&](int tile) {
    const int vi = tile * T::kVpt + b;
    const bool active = vi < count;
    const uint32_t packed = active ? __ldg(&list[vi]) : 0u;
    return Src{active, (int)(packed & 0xffff) * 8, (int)(packed >> 16) * 8};
  };
  // Rows inside the frame of a plane with 16-byte aligned rows take 16-byte
  // loads.
  const bool rows16 = (geo.w & 3) == 0 && (reinterpret_cast<uintptr_t>(a.pre) & 15) == 0;
  auto load_row = [&](const Src& src, int c, float* row) {
    if (src.active) {
      const int yy = min(src.y0 + r, geo.h - 1);
      const float* p = a.pre + plane * c + (size_t)yy * geo.w;
      if (rows16 && src.x0 + N <= geo.w) {
        const float4* p4 = reinterpret_cast<const float4*>(p + src.x0);
#pragma unroll
        for (int x = 0; x < N; x += 4) {
          const float4 v = __ldg(p4 + x / 4);
          row[x] = v.x;
          row[x + 1] = v.y;
          row[x + 2] = v.z;
          row[x + 3] = v.w;
        }
      } else {
#pragma unroll
        for (int x = 0; x < N; ++x) row[x] = __ldg(&p[min(src.x0 + x, geo.w - 1)]);
      }
    } else {
#pragma unroll
      for (int x = 0; x < N; ++x) row[x] = 0.0f;
    }
  };
  // (tile, channel) steps in order; the next step's row is loaded before
  // this step's transform, so that its latency overlaps the MMAs, and the
  // next tile's varblock a tile ahead, so that those loads never wait on it.
  const Src none{false, 0, 0};
  int tile = blockIdx.x, c = 0;
  Src cur = tile < ntiles ? locate(tile) : none;
  Src after = tile + (int)gridDim.x < ntiles ? locate(tile + gridDim.x) : none;
  float nxt[N];
  if (tile < ntiles) load_row(cur, 0, nxt);
  while (tile < ntiles && st.ok) {
    float row[N];
#pragma unroll
    for (int x = 0; x < N; ++x) row[x] = nxt[x];
    const Src here = cur;
    const int ch = c;
    if (++c == 3) {
      c = 0;
      tile += gridDim.x;
      cur = after;
      if (tile + (int)gridDim.x < ntiles) after = locate(tile + gridDim.x);
    }
    if (tile < ntiles) load_row(cur, c, nxt);
    transform_rows<N, TERMS>(smem, &mbar, st, row);
    if (!st.ok) break;
    if (here.active) {
      // landscape coefficient row r of the varblock
      float* o = a.coeff + cplane * ch + (size_t)(here.y0 + r) * geo.W8 + here.x0;
#pragma unroll
      for (int u = 0; u < N; u += 4)
        *reinterpret_cast<float4*>(o + u) = make_float4(row[u], row[u + 1], row[u + 2], row[u + 3]);
    }
  }
  end(st, &mbar, a.err);
}

// ---------------------------------------------------------------------------
// T2 — render of the square varblocks of size N: dequantize, HF CfL, LLF,
// IDCT_2D, scatter, sigma.
// ---------------------------------------------------------------------------
template <int N, int TERMS>
__global__ void __launch_bounds__(kThreads) k_render_tc(RenderArgs a,
                                                        const uint32_t* __restrict__ list,
                                                        int count, int ntiles,
                                                        const float* __restrict__ llf) {
  using T = Tile<N, TERMS>;
  constexpr int n = N / 8;  // LLF corner side in blocks
  extern __shared__ __align__(128) uint8_t smem[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_slot;
  __shared__ float s_mul[T::kVpt], s_kx[T::kVpt], s_kb[T::kVpt];
  const int t = threadIdx.x;
  const int b = t / N, r = t % N;
  begin(&tmem_slot, &mbar);
  load_basis<N, TERMS>(smem, 0);
  before_sync();
  __syncthreads();
  after_sync();
  State st{tmem_slot, 0u, true};
  const Geo& geo = a.geo;
  const size_t cplane = (size_t)geo.W8 * geo.H8;
  const size_t plane = (size_t)geo.w * geo.h;
  constexpr int slot = N == 8 ? 0 : (N == 16 ? 1 : 2);  // compact dequant slots 0..2
  const int dq_off = dq_offset(slot);
  // Per-tile scalars (HF multiplier, CfL factors) of the tile's varblocks,
  // loaded by thread t < kVpt for varblock t.
  auto tile_scalars = [&](int tile, float& mul, float& kx, float& kb) {
    const int vi = tile * T::kVpt + t;
    if (t < T::kVpt && vi < count) {
      const uint32_t packed = __ldg(&list[vi]);
      const int bx = packed & 0xffff, by = packed >> 16;
      mul = hf_multiplier(a.mul_table, a.qs.global_scale,
                          a.hf_mul[(size_t)by * geo.bw + bx]);  // reconstruct.rs:27
      const int tile64 = (by / 8) * geo.tw + bx / 8;
      kx = 0.0f + (float)a.cfl_x[tile64] / 84.0f;  // reconstruct.rs:96
      kb = 1.0f + (float)a.cfl_b[tile64] / 84.0f;
    }
  };
  // This thread's quantized row r of channel c of its varblock in a tile,
  // and in the LLF rows the channel's LLF values.
  struct QRow {
    int q[N];
    float l[n];
    bool active;
    int x0, y0;
  };
  // The list entry of this thread's varblock in a tile (0 past the end),
  // fetched a tile ahead of its rows.
  auto entry = [&](int tile) {
    const int vi = tile * T::kVpt + b;
    return vi < count ? __ldg(&list[vi]) : 0u;
  };
  auto load_q = [&](int tile, int c, uint32_t packed, QRow& qr) {
    const int vi = tile * T::kVpt + b;
    qr.active = vi < count;
    qr.x0 = (int)(packed & 0xffff) * 8;
    qr.y0 = (int)(packed >> 16) * 8;
    if (!qr.active) return;
    const int4* q4 =
        reinterpret_cast<const int4*>(a.qcoeff + cplane * c + (size_t)(qr.y0 + r) * geo.W8 + qr.x0);
#pragma unroll
    for (int u4 = 0; u4 < N / 4; ++u4) {
      const int4 v = __ldg(&q4[u4]);
      qr.q[4 * u4] = v.x;
      qr.q[4 * u4 + 1] = v.y;
      qr.q[4 * u4 + 2] = v.z;
      qr.q[4 * u4 + 3] = v.w;
    }
    if (r < n) {
      const float* lc = llf + (size_t)vi * 48 + c * 16 + r * n;
#pragma unroll
      for (int u = 0; u < n; ++u) qr.l[u] = __ldg(&lc[u]);
    }
  };
  auto channel_of = [](int ci) { return ci == 0 ? 1 : (ci == 1 ? 0 : 2); };  // luma first: CfL needs it
  // (tile, channel) steps in order; the next step's quantized row (and, at
  // a tile's last channel, the next tile's scalars) is loaded before this
  // step's transform, so that its latency overlaps the MMAs.
  int tile = blockIdx.x, ci = 0;
  float pm = 0.0f, pkx = 0.0f, pkb = 0.0f;
  QRow nq;
  uint32_t ent = 0u, ent_after = 0u;  // list entries of this tile and the next
  if (tile < ntiles) {
    ent = entry(tile);
    if (tile + (int)gridDim.x < ntiles) ent_after = entry(tile + gridDim.x);
    tile_scalars(tile, pm, pkx, pkb);
    load_q(tile, channel_of(0), ent, nq);
  }
  float dY[N];
  while (tile < ntiles && st.ok) {
    if (ci == 0) {
      if (t < T::kVpt) {
        s_mul[t] = pm;
        s_kx[t] = pkx;
        s_kb[t] = pkb;
      }
      __syncthreads();
    }
    const QRow q = nq;
    const int c = channel_of(ci);
    int ntile = tile, nci = ci + 1;
    if (nci == 3) {
      nci = 0;
      ntile += gridDim.x;
    }
    if (nci == 0) {
      ent = ent_after;
      if (ntile + (int)gridDim.x < ntiles) ent_after = entry(ntile + gridDim.x);
    }
    if (ntile < ntiles) {
      load_q(ntile, channel_of(nci), ent, nq);
      if (nci == 0) tile_scalars(ntile, pm, pkx, pkb);
    }
    float row[N];
    if (q.active) {
      // landscape row r (plan-render lib.rs:913: adjusted * (mul*qm) *
      // matrix, left to right), the HF CfL (lib.rs:1344), the LLF corner.
      const float scale = s_mul[b] * a.qs.qm[c];
      const float bias = c_tc_bias[c];
      const float kc = c == 0 ? s_kx[b] : s_kb[b];
      const float* m = a.dq + c * kDequantTableFloats + dq_off + r * N;
#pragma unroll
      for (int u4 = 0; u4 < N / 4; ++u4) {
        const float4 mm = __ldg(reinterpret_cast<const float4*>(m) + u4);
        const float ms[4] = {mm.x, mm.y, mm.z, mm.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int u = u4 * 4 + i;
          float d = bias_adjust(q.q[u], bias) * scale * ms[i];
          if (c == 1) dY[u] = d;
          else d = d + kc * dY[u];
          if (r < n && u < n) d = q.l[u < n ? u : 0];
          row[u] = d;
        }
      }
    } else {
#pragma unroll
      for (int u = 0; u < N; ++u) row[u] = 0.0f;
    }
    transform_rows<N, TERMS>(smem, &mbar, st, row);
    if (!st.ok) break;
    if (q.active) {
      const int fy = q.y0 + r;
      if (fy < geo.h) {
        float* o = a.planes + plane * c + (size_t)fy * geo.w + q.x0;
        if (q.x0 + N <= geo.w && (geo.w & 3) == 0) {
#pragma unroll
          for (int x = 0; x < N; x += 4)
            *reinterpret_cast<float4*>(o + x) =
                make_float4(row[x], row[x + 1], row[x + 2], row[x + 3]);
        } else {
#pragma unroll
          for (int x = 0; x < N; ++x)
            if (q.x0 + x < geo.w) o[x] = row[x];
        }
      }
    }
    if (nci == 0) __syncthreads();  // s_* are rewritten at the next tile's start
    tile = ntile;
    ci = nci;
  }
  end(st, &mbar, a.err);
}

// Persistent CTAs per SM of the tensor-core kernels: at most four, whose
// 128-column TMEM allocations fill an SM's 512; a tunable (tc_ctas_per_sm).
std::atomic<int> g_tc_ctas_per_sm{4};

template <typename K>
cudaError_t set_smem(K kernel, int bytes) {
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

template <int N, int TERMS>
int launch_fdct_one(const EncArgs& a, const uint32_t* list, int count, int num_sms,
                    cudaStream_t s) {
  const int ntiles = (count + Tile<N, TERMS>::kVpt - 1) / Tile<N, TERMS>::kVpt;
  const int grid = std::min(ntiles, num_sms * g_tc_ctas_per_sm.load());
  k_fdct_tc<N, TERMS><<<grid, kThreads, Tile<N, TERMS>::kBytes, s>>>(a, list, count, ntiles);
  return 1;
}

template <int N, int TERMS>
int launch_render_one(const RenderArgs& a, const uint32_t* list, int count, const float* llf,
                      int num_sms, cudaStream_t s) {
  const int ntiles = (count + Tile<N, TERMS>::kVpt - 1) / Tile<N, TERMS>::kVpt;
  const int grid = std::min(ntiles, num_sms * g_tc_ctas_per_sm.load());
  k_render_tc<N, TERMS><<<grid, kThreads, Tile<N, TERMS>::kBytes, s>>>(a, list, count, ntiles,
                                                                         llf);
  return 1;
}

}  // namespace

int tc_ctas_per_sm(int value) {
  const int old = g_tc_ctas_per_sm.load();
  if (value >= 1 && value <= 4) g_tc_ctas_per_sm.store(value);
  return old;
}

cudaError_t configure_tc_kernels() {
  cudaError_t e = cudaSuccess;
#define JPXLG_TC_ATTR(N, T)                                                          \
  if (e == cudaSuccess) e = set_smem(k_fdct_tc<N, T>, Tile<N, T>::kBytes);          \
  if (e == cudaSuccess) e = set_smem(k_render_tc<N, T>, Tile<N, T>::kBytes);
  JPXLG_TC_ATTR(8, 2)
  JPXLG_TC_ATTR(16, 2)
  JPXLG_TC_ATTR(32, 2)
  JPXLG_TC_ATTR(8, 3)
  JPXLG_TC_ATTR(16, 3)
  JPXLG_TC_ATTR(32, 3)
#undef JPXLG_TC_ATTR
  return e;
}

void upload_tc_basis(cudaStream_t s) {
  static float host[2][3][32 * 32];
  static bool ready = false;
  if (!ready) {
    for (int k = 0; k < 3; ++k) {
      const int n = 8 << k;
      for (int i = 0; i < n; ++i)
        for (int u = 0; u < n; ++u) {
          const double cu = u == 0 ? 1.0 : std::sqrt(2.0);
          const double c = cu * std::cos(M_PI * (2.0 * i + 1.0) * u / (2.0 * n));
          host[0][k][i * n + u] = (float)c;        // I[i][u]
          host[1][k][u * n + i] = (float)(c / n);  // D[u][i]
        }
    }
    ready = true;
  }
  cudaMemcpyToSymbolAsync(g_tc_basis, host, sizeof(host), 0, cudaMemcpyHostToDevice, s);
}

int launch_fdct_tc(const EncArgs& a, const uint32_t* const* lists, const int* counts, int terms,
                   int num_sms, const cudaStream_t* s) {
  int k = 0;
  // shape classes 0, 1, 2 are DCT8, DCT16, DCT32, each on its stream
  if (terms == 2) {
    if (counts[0]) k += launch_fdct_one<8, 2>(a, lists[0], counts[0], num_sms, s[0]);
    if (counts[1]) k += launch_fdct_one<16, 2>(a, lists[1], counts[1], num_sms, s[1]);
    if (counts[2]) k += launch_fdct_one<32, 2>(a, lists[2], counts[2], num_sms, s[2]);
  } else {
    if (counts[0]) k += launch_fdct_one<8, 3>(a, lists[0], counts[0], num_sms, s[0]);
    if (counts[1]) k += launch_fdct_one<16, 3>(a, lists[1], counts[1], num_sms, s[1]);
    if (counts[2]) k += launch_fdct_one<32, 3>(a, lists[2], counts[2], num_sms, s[2]);
  }
  return k;
}

int launch_render_tc(const RenderArgs& a, const uint32_t* const* lists, const int* counts,
                     const float* const* llf, int terms, int num_sms, const cudaStream_t* s) {
  int k = 0;
  if (terms == 2) {
    if (counts[0]) k += launch_render_one<8, 2>(a, lists[0], counts[0], llf[0], num_sms, s[0]);
    if (counts[1]) k += launch_render_one<16, 2>(a, lists[1], counts[1], llf[1], num_sms, s[1]);
    if (counts[2]) k += launch_render_one<32, 2>(a, lists[2], counts[2], llf[2], num_sms, s[2]);
  } else {
    if (counts[0]) k += launch_render_one<8, 3>(a, lists[0], counts[0], llf[0], num_sms, s[0]);
    if (counts[1]) k += launch_render_one<16, 3>(a, lists[1], counts[1], llf[1], num_sms, s[1]);
    if (counts[2]) k += launch_render_one<32, 3>(a, lists[2], counts[2], llf[2], num_sms, s[2]);
  }
  return k;
}

}  // namespace jpxlg
