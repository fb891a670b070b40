// jpxlg_api.cu — the C ABI (include/jpxlg.h): contexts, layouts, workspace
// and the host orchestration of the sm_103a kernels.  Host code only; the
// kernels live in k_encode.cu, k_render.cu and k_ssim.cu.
#include <limits>
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/jpxlg.h"
#include "codestream.h"
#include "jpxlg_common.cuh"
#include "jpxlg_internal.h"
#include "jpxlg_kernels.h"

using namespace jpxlg;

namespace {

// A grow-only device buffer.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t n) {
    if (n <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <typename T>
  T* as() const { return (T*)p; }
};

struct DepthTable {
  float* thr = nullptr;
  float* lev = nullptr;
  // Entry i: (threshold i-1 or -inf, threshold i or +inf, level i's value,
  // 0): a level estimate is confirmed and resolved by one 16-byte load.
  float4* bracket = nullptr;
  int levels = 0;
};

}  // namespace

struct jpxlg_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  // Side streams for the shape classes of a launch (ClassStreams below),
  // forked from and joined back into `stream` with events.
  cudaStream_t side[2] = {nullptr, nullptr};
  cudaEvent_t fork_ev = nullptr;
  cudaEvent_t join_ev[2] = {nullptr, nullptr};
  std::string last_error;
  uint64_t launches = 0;
  // tables
  float* d_dq = nullptr;
  std::map<int, float*> lut;          // sRGB -> linear per source depth
  std::map<int, DepthTable> depth;    // output depth classifiers
  // small device words
  uint32_t* d_words = nullptr;  // [0] err, [1] not_gray, [2] cfl fallbacks
  int* d_lf = nullptr;          // [0..1] unbiased LF factors, [2..3] biased
  float* d_mul = nullptr;       // hf multipliers of the current call's global_scale
  uint32_t* h_words = nullptr;  // pinned mirror
  double* h_score = nullptr;    // pinned score out (2 + 108)
  // workspace
  DevBuf rgb, xyb, pre, coeff, dyhf, qcoeff, lfs, dylf, lfq, cflx, cflb;
  DevBuf planes, aux, sigma, out, llf;
  DevBuf lf_part, lf_seed, cfl_tile, cover, cover_map;
  DevBuf pyr, partial, score, cxyb, hpl, bcarry;
  DevBuf pair_ref;  // the reference side of jpxlg_score_pair, kept across calls
  // stage timers
  struct Mark {
    int stage;
    cudaEvent_t a, b;
    uint64_t launches;
  };
  bool timing = false;
  std::vector<Mark> marks;
  std::vector<cudaEvent_t> event_pool;
  int open_stage = -1;
  cudaEvent_t open_event = nullptr;
  uint64_t open_launches = 0;
  double stage_ms[JPXLG_STAGE_COUNT] = {};
  uint64_t stage_launches[JPXLG_STAGE_COUNT] = {};
};

struct jpxlg_layout {
  jpxlg_ctx* ctx = nullptr;  // creating context (device checks at creation time only)
  int device = 0;
  Geo geo;
  uint8_t* d_map = nullptr;
  uint32_t* d_hf_mul = nullptr;
  uint8_t* d_sharp = nullptr;
  uint32_t* d_lists = nullptr;
  const uint32_t* lists[kNumShapes] = {};
  int counts[kNumShapes] = {};
  uint32_t base_hf_mul = 1;
  bool all_square = true;
};

struct jpxlg_ref {
  jpxlg_ctx* ctx = nullptr;
  int device = 0;
  int w = 0, h = 0, nscales = 0;
  SsimScale scales[6];
  void* block = nullptr;  // one allocation holding every scale's planes
};

namespace {

int fail(jpxlg_ctx* ctx, int code, const char* fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    ctx->last_error = buf;
  }
  return code;
}

// A failed runtime call returns JPXLG_ERR_CUDA.  A non-sticky error (a
// failed allocation) also stays in the runtime's last-error slot, where the
// next launch check would find it: it is read off here, so that the context
// stays usable.
#define CK(call)                                                                     \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) {                                                         \
      cudaGetLastError();                                                            \
      return fail(ctx, JPXLG_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));     \
    }                                                                                \
  } while (0)

cudaEvent_t pool_event(jpxlg_ctx* ctx) {
  if (!ctx->event_pool.empty()) {
    cudaEvent_t e = ctx->event_pool.back();
    ctx->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Stage boundaries: an event before the stage's first launch and one after
// its last, on the context's stream.
void stage_begin(jpxlg_ctx* ctx, int stage) {
  if (!ctx->timing) return;
  ctx->open_stage = stage;
  ctx->open_event = pool_event(ctx);
  ctx->open_launches = ctx->launches;
  cudaEventRecord(ctx->open_event, ctx->stream);
}

void stage_end(jpxlg_ctx* ctx) {
  if (!ctx->timing || ctx->open_stage < 0) return;
  cudaEvent_t b = pool_event(ctx);
  cudaEventRecord(b, ctx->stream);
  ctx->marks.push_back({ctx->open_stage, ctx->open_event, b, ctx->launches - ctx->open_launches});
  ctx->open_stage = -1;
}

// The blur kernels of one SSIMULACRA2 scale, each under its own stage: the
// row pass, the column ripple, the column outputs; the rest of the metric
// (positive XYB, downscaling, the final sums) stays under JPXLG_STAGE_SSIM.
void ssim_stage_hook(void* user, int part) {
  jpxlg_ctx* ctx = static_cast<jpxlg_ctx*>(user);
  static const int kNext[4] = {JPXLG_STAGE_SSIM_ROWS, JPXLG_STAGE_SSIM_COL_RIPPLE,
                               JPXLG_STAGE_SSIM_COL_OUT, JPXLG_STAGE_SSIM};
  static const int kLaunched[4] = {0, 1, 0, 1};  // the kernels since the previous part
  ctx->launches += kLaunched[part];
  stage_end(ctx);
  stage_begin(ctx, kNext[part]);
}

int after_launch(jpxlg_ctx* ctx, uint64_t n) {
  ctx->launches += n;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(ctx, JPXLG_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(e));
  return JPXLG_OK;
}

// A stream per shape class for one launch of independent per-class kernels:
// the class with the most varblocks stays on the context's stream, the
// others alternate over the two side streams, forked from the context's
// stream here and joined back by class_join.  A small class (a handful of
// DCT32 varblocks is one CTA that runs for tens of microseconds on its
// latency chains) then overlaps the large one instead of following it.
struct ClassStreams {
  cudaStream_t s[kNumShapes];
  bool used[2] = {false, false};
};

ClassStreams class_fork(jpxlg_ctx* ctx, const int* counts, int n) {
  ClassStreams cs;
  int biggest = -1;
  for (int i = 0; i < n; ++i)
    if (counts[i] && (biggest < 0 || counts[i] > counts[biggest])) biggest = i;
  int side = 0;
  for (int i = 0; i < kNumShapes; ++i) {
    cs.s[i] = ctx->stream;
    if (i < n && counts[i] && i != biggest && ctx->side[0]) {
      cs.s[i] = ctx->side[side];
      cs.used[side] = true;
      side ^= 1;
    }
  }
  if (cs.used[0] || cs.used[1]) {
    cudaEventRecord(ctx->fork_ev, ctx->stream);
    for (int k = 0; k < 2; ++k)
      if (cs.used[k]) cudaStreamWaitEvent(ctx->side[k], ctx->fork_ev, 0);
  }
  return cs;
}

void class_join(jpxlg_ctx* ctx, const ClassStreams& cs) {
  for (int k = 0; k < 2; ++k)
    if (cs.used[k]) {
      cudaEventRecord(ctx->join_ev[k], ctx->side[k]);
      cudaStreamWaitEvent(ctx->stream, ctx->join_ev[k], 0);
    }
}

// Reads and clears the device error word after the stream drains.
int sync_and_check(jpxlg_ctx* ctx) {
  CK(cudaMemcpyAsync(ctx->h_words, ctx->d_words, 3 * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  uint32_t err = ctx->h_words[0];
  if (err) {
    CK(cudaMemsetAsync(ctx->d_words, 0, sizeof(uint32_t), ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (err & kDevQuantRange)
      return fail(ctx, JPXLG_ERR_QUANT, "a quantization target outside the working range");
    if (err & kDevBadStep) return fail(ctx, JPXLG_ERR_QUANT, "a degenerate quantization step");
    if (err & kDevTcTimeout)
      return fail(ctx, JPXLG_ERR_CUDA, "a tensor-core transform timed out waiting for its MMA");
    if (err & kDevBlurTimeout)
      return fail(ctx, JPXLG_ERR_CUDA, "the blur's column scan timed out waiting for a segment");
    return fail(ctx, JPXLG_ERR_BLOCK_MAP, "a block-map entry the kernels cannot place");
  }
  return JPXLG_OK;
}

const float* get_lut(jpxlg_ctx* ctx, int bits) {
  auto it = ctx->lut.find(bits);
  if (it != ctx->lut.end()) return it->second;
  int n = bits == 8 ? 256 : 65536;
  std::vector<float> h(n);
  build_srgb_lut(bits, h.data());
  float* d = nullptr;
  if (cudaMalloc(&d, n * sizeof(float)) != cudaSuccess) return nullptr;
  cudaMemcpy(d, h.data(), n * sizeof(float), cudaMemcpyHostToDevice);
  ctx->lut[bits] = d;
  return d;
}

const DepthTable* get_depth(jpxlg_ctx* ctx, int bits) {
  auto it = ctx->depth.find(bits);
  if (it != ctx->depth.end()) return &it->second;
  int levels = bits >= 32 ? 65536 : (1 << std::min(std::max(bits, 1), 16));
  std::vector<float> thr(levels), lev(levels);
  build_depth_thresholds(bits, thr.data(), lev.data());
  DepthTable t;
  t.levels = levels;
  if (cudaMalloc(&t.thr, levels * sizeof(float)) != cudaSuccess) return nullptr;
  if (cudaMalloc(&t.lev, levels * sizeof(float)) != cudaSuccess) return nullptr;
  cudaMemcpy(t.thr, thr.data(), levels * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemcpy(t.lev, lev.data(), levels * sizeof(float), cudaMemcpyHostToDevice);
  // levels - 1 thresholds bracket the levels 0 .. levels - 1.
  std::vector<float4> br(levels);
  const float inf = std::numeric_limits<float>::infinity();
  for (int i = 0; i < levels; ++i)
    br[i] = make_float4(i == 0 ? -inf : thr[i - 1], i == levels - 1 ? inf : thr[i], lev[i], 0.0f);
  if (cudaMalloc(&t.bracket, levels * sizeof(float4)) != cudaSuccess) return nullptr;
  cudaMemcpy(t.bracket, br.data(), levels * sizeof(float4), cudaMemcpyHostToDevice);
  ctx->depth[bits] = t;
  return &ctx->depth[bits];
}

QuantScalars scalars_of(const jpxlg_params* p) {
  QuantScalars q;
  q.global_scale = p->global_scale;
  host_lf_multipliers(p->global_scale, p->quant_lf, q.m_dc);
  q.qm[0] = host_qm_multiplier(p->x_qm_scale);
  q.qm[1] = 1.0f;
  q.qm[2] = host_qm_multiplier(p->b_qm_scale);
  return q;
}

int check_params(jpxlg_ctx* ctx, const jpxlg_params* p) {
  if (!p) return fail(ctx, JPXLG_ERR_ARGUMENT, "null params");
  if (p->global_scale == 0 || p->quant_lf == 0)
    return fail(ctx, JPXLG_ERR_ARGUMENT, "global_scale and quant_lf must be positive");
  if (p->x_qm_scale > 7 || p->b_qm_scale > 7)
    return fail(ctx, JPXLG_ERR_ARGUMENT, "qm scales are u(3)");
  if (p->epf_iters > 3) return fail(ctx, JPXLG_ERR_ARGUMENT, "epf_iters outside 0..=3");
  if (p->precision > JPXLG_PRECISION_BF16X6)
    return fail(ctx, JPXLG_ERR_ARGUMENT, "precision must be a JPXLG_PRECISION_* value");
  return JPXLG_OK;
}

// The transform frame of policy lib.rs:605: XYB planes of the source
// (K1), preconditioned by the inverse Gaborish (K2) when the decoder will
// run Gaborish.  Also resets and sets the context's not-grey word.
int transform_frame(jpxlg_ctx* ctx, const Geo& g, const void* rgb_dev, int bits,
                    const jpxlg_params* p, const float** pre_out) {
  const size_t n = (size_t)g.w * g.h;
  CK(ctx->xyb.ensure(3 * n * sizeof(float)));
  const float* lut = get_lut(ctx, bits);
  if (!lut) return fail(ctx, JPXLG_ERR_CUDA, "transfer table allocation failed");
  CK(cudaMemsetAsync(ctx->d_words + 1, 0, sizeof(uint32_t), ctx->stream));
  float* xyb = ctx->xyb.as<float>();
  stage_begin(ctx, JPXLG_STAGE_XYB);
  launch_srgb_to_xyb(rgb_dev, bits, n, lut, xyb, xyb + n, xyb + 2 * n, ctx->d_words + 1,
                     ctx->num_sms, ctx->stream);
  int rc = after_launch(ctx, 1);
  stage_end(ctx);
  if (rc) return rc;
  const float* pre = xyb;
  if (p->gaborish) {
    CK(ctx->pre.ensure(3 * n * sizeof(float)));
    stage_begin(ctx, JPXLG_STAGE_PRECONDITION);
    rc = after_launch(ctx, launch_precondition(xyb, ctx->pre.as<float>(), g.w, g.h, ctx->stream));
    stage_end(ctx);
    if (rc) return rc;
    pre = ctx->pre.as<float>();
  }
  *pre_out = pre;
  return JPXLG_OK;
}

// Encode into plan buffers that live on the device.
int encode_device(jpxlg_ctx* ctx, const jpxlg_layout* L, const void* rgb_dev, int bits,
                  const jpxlg_params* p, int32_t* qcoeff, int32_t* lfq, int8_t* cflx,
                  int8_t* cflb, int32_t* lf_factors_biased) {
  const Geo& g = L->geo;
  if (!L->all_square)
    return fail(ctx, JPXLG_ERR_BLOCK_MAP,
                "the encoder covers frames with DCT8, DCT16 and DCT32 varblocks only");
  const size_t n = (size_t)g.w * g.h, n8 = (size_t)g.W8 * g.H8, nb = (size_t)g.bw * g.bh;
  CK(ctx->xyb.ensure(3 * n * sizeof(float)));
  CK(ctx->coeff.ensure(3 * n8 * sizeof(float)));
  CK(ctx->dyhf.ensure(n8 * sizeof(float)));
  CK(ctx->lfs.ensure(3 * nb * sizeof(float)));
  CK(ctx->dylf.ensure(nb * sizeof(float)));
  CK(ctx->lf_seed.ensure(4 * sizeof(int)));
  CK(ctx->lf_part.ensure(kCflScratchBytes));
  CK(ctx->cfl_tile.ensure(cfl_tile_scratch_bytes(g.tw * g.th)));
  const float* pre = nullptr;
  int rc = transform_frame(ctx, g, rgb_dev, bits, p, &pre);
  if (rc) return rc;
  EncArgs a;
  a.geo = g;
  a.qs = scalars_of(p);
  a.pre = pre;
  a.dq = ctx->d_dq;
  a.mul_table = ctx->d_mul;
  a.hf_mul = L->d_hf_mul;
  a.block_map = L->d_map;
  a.coeff = ctx->coeff.as<float>();
  a.dyhf = ctx->dyhf.as<float>();
  a.qcoeff = qcoeff;
  a.lfs = ctx->lfs.as<float>();
  a.dylf = ctx->dylf.as<float>();
  a.lfq = lfq;
  a.cfl_x = cflx;
  a.cfl_b = cflb;
  a.lf_factors = ctx->d_lf;
  a.not_gray = ctx->d_words + 1;
  a.cfl_enabled = p->cfl;
  a.base_mul = host_hf_multiplier(p->global_scale, L->base_hf_mul);
  a.err = ctx->d_words;
  a.cfl_fallbacks = ctx->d_words + 2;
  // square classes only: DCT8, DCT16, DCT32 are shape classes 0..2
  stage_begin(ctx, JPXLG_STAGE_FDCT_LUMA);
  launch_mul_table(p->global_scale, ctx->d_mul, ctx->stream);
  {
    const ClassStreams cs = class_fork(ctx, L->counts, 3);
    if (p->precision == JPXLG_PRECISION_FP32) {
      rc = after_launch(ctx, 1 + launch_fdct_luma(a, L->lists, L->counts, cs.s));
    } else {
      // split-precision forward transform of all three channels on the
      // tensor cores, then the luma quantization from the coefficient image
      const int terms = p->precision == JPXLG_PRECISION_BF16X3 ? 2 : 3;
      int k = 1 + launch_fdct_tc(a, L->lists, L->counts, terms, ctx->num_sms, cs.s);
      rc = after_launch(ctx, k + launch_luma_from_image(a, L->lists, L->counts, cs.s));
    }
    class_join(ctx, cs);
  }
  stage_end(ctx);
  if (rc) return rc;
  stage_begin(ctx, JPXLG_STAGE_CFL);
  {
    const int chains[2] = {2, 1};  // the tile chain on the context's stream, the LF one beside
    const ClassStreams cs = class_fork(ctx, chains, 2);
    rc = after_launch(ctx, launch_cfl(a, ctx->lf_seed.as<int>(), ctx->lf_part.p,
                                      ctx->cfl_tile.p, cs.s[0], cs.s[1]));
    class_join(ctx, cs);
  }
  stage_end(ctx);
  if (rc) return rc;
  stage_begin(ctx, JPXLG_STAGE_QUANT_CHROMA);
  {
    const ClassStreams cs = class_fork(ctx, L->counts, 3);
    rc = after_launch(ctx, launch_quant_chroma(a, L->lists, L->counts, cs.s));
    class_join(ctx, cs);
  }
  stage_end(ctx);
  if (rc) return rc;
  // biased copy of the LF factors for the plan
  if (lf_factors_biased) {
    // d_lf[0..1] unbiased; the plan stores factor + 128.
    CK(cudaMemcpyAsync(ctx->h_words + 4, ctx->d_lf, 2 * sizeof(int), cudaMemcpyDeviceToHost,
                       ctx->stream));
  }
  return JPXLG_OK;
}

int render_device(jpxlg_ctx* ctx, const jpxlg_layout* L, const int32_t* qcoeff,
                  const int32_t* lfq, const int8_t* cflx, const int8_t* cflb, int fx_biased,
                  int fb_biased, const int* lf_dev_unbiased, const jpxlg_params* p, int out_kind,
                  int bits, void* out_dev, float* pxyb_dev = nullptr,
                  const float* lf_float = nullptr) {
  const Geo& g = L->geo;
  const size_t n = (size_t)g.w * g.h, nb = (size_t)g.bw * g.bh;
  if (p->precision != JPXLG_PRECISION_FP32 && (uintptr_t)qcoeff % 16 != 0)
    return fail(ctx, JPXLG_ERR_ARGUMENT,
                "the split-precision render reads 16-byte aligned coefficient planes");
  CK(ctx->planes.ensure(3 * n * sizeof(float)));
  CK(ctx->aux.ensure(3 * n * sizeof(float)));
  CK(ctx->sigma.ensure(nb * sizeof(float)));
  RenderArgs a;
  a.geo = g;
  a.qs = scalars_of(p);
  a.dq = ctx->d_dq;
  a.mul_table = ctx->d_mul;
  a.hf_mul = L->d_hf_mul;
  a.sharpness = L->d_sharp;
  a.qcoeff = qcoeff;
  a.lfq = lfq;
  a.cfl_x = cflx;
  a.cfl_b = cflb;
  a.k_x_lf = 0.0f + (float)(fx_biased - 128) / 84.0f;
  a.k_b_lf = 1.0f + (float)(fb_biased - 128) / 84.0f;
  a.lf_factors_dev = lf_dev_unbiased;
  a.planes = ctx->planes.as<float>();
  a.sigma = ctx->sigma.as<float>();
  a.lf_float = lf_float;
  a.err = ctx->d_words;
  stage_begin(ctx, JPXLG_STAGE_RENDER_VARBLOCKS);
  launch_mul_table(p->global_scale, ctx->d_mul, ctx->stream);
  uint64_t k = 1;
  const ClassStreams cs = class_fork(ctx, L->counts, kNumShapes);
  if (p->precision == JPXLG_PRECISION_FP32) {
    launch_render_varblocks(a, L->lists, L->counts, cs.s);
    for (int i = 0; i < kNumShapes; ++i) k += L->counts[i] ? 1 : 0;
  } else {
    // square classes on the tensor cores; any other shape through the FP32
    // kernels (a decoded stream's cover)
    const int terms = p->precision == JPXLG_PRECISION_BF16X3 ? 2 : 3;
    CK(ctx->llf.ensure(48 * sizeof(float) *
                       (size_t)std::max(1, L->counts[0] + L->counts[1] + L->counts[2])));
    float* llf[3] = {ctx->llf.as<float>(), ctx->llf.as<float>() + 48 * (size_t)L->counts[0],
                     ctx->llf.as<float>() + 48 * (size_t)(L->counts[0] + L->counts[1])};
    k += launch_llf_sigma(a, L->lists, L->counts, llf, cs.s);
    const float* cllf[3] = {llf[0], llf[1], llf[2]};
    k += launch_render_tc(a, L->lists, L->counts, cllf, terms, ctx->num_sms, cs.s);
    int rest[kNumShapes];
    for (int i = 0; i < kNumShapes; ++i) rest[i] = i < 3 ? 0 : L->counts[i];
    launch_render_varblocks(a, L->lists, rest, cs.s);
    for (int i = 3; i < kNumShapes; ++i) k += rest[i] ? 1 : 0;
  }
  class_join(ctx, cs);
  int rc = after_launch(ctx, k);
  stage_end(ctx);
  if (rc) return rc;
  float* cur = ctx->planes.as<float>();
  float* nxt = ctx->aux.as<float>();
  if (p->gaborish) {
    stage_begin(ctx, JPXLG_STAGE_GABORISH);
    launch_gaborish(cur, nxt, g.w, g.h, ctx->stream);
    std::swap(cur, nxt);
    rc = after_launch(ctx, 1);
    stage_end(ctx);
    if (rc) return rc;
  }
  static const int steps_for[4][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 2, -1}, {0, 1, 2}};
  if (p->epf_iters) stage_begin(ctx, JPXLG_STAGE_EPF);
  for (int s = 0; s < 3; ++s) {
    int step = steps_for[p->epf_iters][s];
    if (step < 0) break;
    launch_epf_step(step, cur, nxt, ctx->sigma.as<float>(), g.w, g.h, ctx->stream);
    std::swap(cur, nxt);
    if ((rc = after_launch(ctx, 1))) return rc;
  }
  if (p->epf_iters) stage_end(ctx);
  if (out_kind == JPXLG_OUT_XYB) {
    CK(cudaMemcpyAsync(out_dev, cur, 3 * n * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
    return JPXLG_OK;
  }
  int b = out_kind == JPXLG_OUT_SRGB8 ? 8 : bits;
  const DepthTable* dt = nullptr;
  if (out_kind != JPXLG_OUT_LINEAR && out_kind != JPXLG_OUT_SRGB_FLOAT) {
    dt = get_depth(ctx, b);
    if (!dt) return fail(ctx, JPXLG_ERR_CUDA, "depth table allocation failed");
  }
  stage_begin(ctx, JPXLG_STAGE_COLOUR);
  launch_colour_out(cur, g.w, g.h, out_kind, dt ? dt->thr : nullptr, dt ? dt->lev : nullptr,
                    dt ? dt->bracket : nullptr, dt ? dt->levels : 0, out_dev, pxyb_dev,
                    ctx->num_sms, ctx->stream);
  rc = after_launch(ctx, 1);
  stage_end(ctx);
  return rc;
}

// Candidate side of SSIMULACRA2 against `ref`: cand_dev is the candidate's
// linear RGB; cand_xyb (optional) its positive XYB, when the producer of the
// pixels already formed it.  Each pyramid level keeps linear RGB (for the
// next level) and positive XYB (for the tile kernel).
int score_device(jpxlg_ctx* ctx, const jpxlg_ref* ref, const float* cand_dev,
                 const float* cand_xyb, double* out_dev) {
  const int w = ref->w, h = ref->h;
  size_t pyr = 0;
  for (int s = 1; s < ref->nscales; ++s) pyr += 6 * (size_t)ref->scales[s].w * ref->scales[s].h;
  CK(ctx->pyr.ensure(std::max<size_t>(pyr, 1) * sizeof(float)));
  size_t ctas_total = 0;
  for (int s = 0; s < ref->nscales; ++s)
    ctas_total += (size_t)blur_partial_rows(ref->scales[s].w, ref->scales[s].h);
  CK(ctx->partial.ensure(ctas_total * 18 * sizeof(DF)));
  CK(ctx->hpl.ensure(9 * (size_t)w * h * sizeof(float)));
  CK(ctx->bcarry.ensure(blur_carry_floats(w, h) * sizeof(float)));
  int ctas[6], pixels[6];
  stage_begin(ctx, JPXLG_STAGE_SSIM);
  uint64_t k = 0;
  if (!cand_xyb) {
    CK(ctx->cxyb.ensure(3 * (size_t)w * h * sizeof(float)));
    launch_positive_xyb(cand_dev, ctx->cxyb.as<float>(), (size_t)w * h, ctx->num_sms, ctx->stream);
    ++k;
    cand_xyb = ctx->cxyb.as<float>();
  }
  const float* cur = cand_dev;
  const float* cur_xyb = cand_xyb;
  float* next = ctx->pyr.as<float>();
  DF* part = ctx->partial.as<DF>();
  for (int s = 0; s < ref->nscales; ++s) {
    const SsimScale& rs = ref->scales[s];
    if (s > 0) {
      const size_t ns = (size_t)rs.w * rs.h;
      launch_downscale3(cur, ref->scales[s - 1].w, ref->scales[s - 1].h, next, next + 3 * ns,
                        ctx->stream);
      ++k;
      cur = next;
      cur_xyb = next + 3 * ns;
      next += 6 * ns;
    }
    ctas[s] = launch_score_scale(cur_xyb, rs, ctx->hpl.as<float>(), ctx->bcarry.as<float>(), 0,
                                 3, part, ctx->d_words, ctx->stream, ssim_stage_hook,
                                 ctx);  // the hook counts its kernels
    pixels[s] = rs.w * rs.h;
    part += (size_t)ctas[s] * 18;
  }
  k += launch_score_finish(ctx->partial.as<DF>(), ctas, ref->nscales, pixels, out_dev,
                           ctx->stream);
  int rc = after_launch(ctx, k);
  stage_end(ctx);
  return rc;
}

}  // namespace

extern "C" {

int jpxlg_ctx_create(int device, uint32_t flags, jpxlg_ctx** out) {
  (void)flags;
  if (!out) return JPXLG_ERR_ARGUMENT;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return JPXLG_ERR_NO_DEVICE;
  if (device < 0) cudaGetDevice(&device);
  if (device >= count) return JPXLG_ERR_NO_DEVICE;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return JPXLG_ERR_NO_DEVICE;
  if (prop.major != 10 || prop.minor != 3) return JPXLG_ERR_NO_DEVICE;  // built for sm_103a only
  std::unique_ptr<jpxlg_ctx> ctx(new jpxlg_ctx);
  ctx->device = device;
  ctx->num_sms = prop.multiProcessorCount;
  jpxlg_ctx* c = ctx.get();
#define CKC(call)                                 \
  do {                                            \
    if ((call) != cudaSuccess) return JPXLG_ERR_CUDA; \
  } while (0)
  CKC(cudaSetDevice(device));
  CKC(configure_encode_kernels());
  CKC(configure_blur_kernels());
  CKC(configure_tc_kernels());
  CKC(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking));
  c->stream = c->own_stream;
  for (int k = 0; k < 2; ++k) {
    CKC(cudaStreamCreateWithFlags(&c->side[k], cudaStreamNonBlocking));
    CKC(cudaEventCreateWithFlags(&c->join_ev[k], cudaEventDisableTiming));
  }
  CKC(cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming));
  CKC(cudaMalloc(&c->d_words, 8 * sizeof(uint32_t)));
  CKC(cudaMemset(c->d_words, 0, 8 * sizeof(uint32_t)));
  CKC(cudaMalloc(&c->d_lf, 4 * sizeof(int)));
  CKC(cudaMalloc(&c->d_mul, kMulTableN * sizeof(float)));
  CKC(cudaMemset(c->d_lf, 0, 4 * sizeof(int)));
  CKC(cudaMallocHost(&c->h_words, 16 * sizeof(uint32_t)));
  CKC(cudaMallocHost(&c->h_score, 128 * sizeof(double)));
  std::vector<float> dq(3 * kDequantTableFloats);
  build_dequant_tables(dq.data());
  CKC(cudaMalloc(&c->d_dq, dq.size() * sizeof(float)));
  CKC(cudaMemcpy(c->d_dq, dq.data(), dq.size() * sizeof(float), cudaMemcpyHostToDevice));
  float iv4[16], iv8[64], iv16[256], sf[32], om[9], ob[3], oc[3];
  build_iv_tables(iv4, iv8, iv16);
  build_scale_f(sf);
  std::vector<float> dct64(64 * 64);
  build_dct64_matrix(dct64.data());
  upload_dct64(dct64.data(), c->stream);
  upload_afv(&kAfvBasis[0][0], c->stream);
  build_opsin_inverse(om, ob, oc);
  upload_dct_constants(iv4, iv8, iv16, sf, c->stream);
  upload_blur_consts(c->stream);
  upload_render_constants(om, ob, oc, c->stream);
  upload_tc_basis(c->stream);
  CKC(cudaStreamSynchronize(c->stream));
#undef CKC
  *out = ctx.release();
  return JPXLG_OK;
}

int jpxlg_ctx_destroy(jpxlg_ctx* ctx) {
  if (!ctx) return JPXLG_ERR_ARGUMENT;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (auto& kv : ctx->lut) cudaFree(kv.second);
  for (auto& kv : ctx->depth) {
    cudaFree(kv.second.thr);
    cudaFree(kv.second.lev);
    cudaFree(kv.second.bracket);
  }
  DevBuf* bufs[] = {&ctx->rgb,    &ctx->xyb,   &ctx->pre,     &ctx->coeff,   &ctx->dyhf,
                    &ctx->qcoeff, &ctx->lfs,   &ctx->dylf,    &ctx->lfq,     &ctx->cflx,
                    &ctx->cflb,   &ctx->planes, &ctx->aux,    &ctx->sigma,   &ctx->out,
                    &ctx->lf_part, &ctx->lf_seed, &ctx->cfl_tile, &ctx->cover,
                    &ctx->cover_map, &ctx->pyr,  &ctx->pair_ref, &ctx->partial,
                    &ctx->score,  &ctx->cxyb,   &ctx->hpl,   &ctx->bcarry, &ctx->llf};
  for (DevBuf* b : bufs) b->release();
  for (auto& m : ctx->marks) {
    cudaEventDestroy(m.a);
    cudaEventDestroy(m.b);
  }
  for (cudaEvent_t e : ctx->event_pool) cudaEventDestroy(e);
  cudaFree(ctx->d_dq);
  cudaFree(ctx->d_words);
  cudaFree(ctx->d_lf);
  cudaFree(ctx->d_mul);
  cudaFreeHost(ctx->h_words);
  cudaFreeHost(ctx->h_score);
  for (int k = 0; k < 2; ++k) {
    if (ctx->side[k]) {
      cudaStreamSynchronize(ctx->side[k]);
      cudaStreamDestroy(ctx->side[k]);
    }
    if (ctx->join_ev[k]) cudaEventDestroy(ctx->join_ev[k]);
  }
  if (ctx->fork_ev) cudaEventDestroy(ctx->fork_ev);
  cudaStreamDestroy(ctx->own_stream);
  delete ctx;
  return JPXLG_OK;
}

int jpxlg_ctx_set_stream(jpxlg_ctx* ctx, void* stream) {
  if (!ctx) return JPXLG_ERR_ARGUMENT;
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
  return JPXLG_OK;
}

void* jpxlg_ctx_stream(jpxlg_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int jpxlg_ctx_synchronize(jpxlg_ctx* ctx) {
  if (!ctx) return JPXLG_ERR_ARGUMENT;
  cudaSetDevice(ctx->device);
  return sync_and_check(ctx);
}

const char* jpxlg_last_error(const jpxlg_ctx* ctx) {
  return ctx ? ctx->last_error.c_str() : "null context";
}

uint64_t jpxlg_ctx_launches(const jpxlg_ctx* ctx) { return ctx ? ctx->launches : 0; }

uint32_t jpxlg_ctx_cfl_fallbacks(jpxlg_ctx* ctx) {
  if (!ctx) return 0;
  cudaSetDevice(ctx->device);
  uint32_t v = 0;
  cudaStreamSynchronize(ctx->stream);
  cudaMemcpy(&v, ctx->d_words + 2, sizeof(uint32_t), cudaMemcpyDeviceToHost);
  return v;
}

int jpxlg_stage_timing(jpxlg_ctx* ctx, int enable) {
  if (!ctx) return JPXLG_ERR_ARGUMENT;
  ctx->timing = enable != 0;
  return JPXLG_OK;
}

int jpxlg_stage_times(jpxlg_ctx* ctx, double* ms, uint64_t* launches, int n) {
  if (!ctx) return JPXLG_ERR_ARGUMENT;
  cudaSetDevice(ctx->device);
  CK(cudaStreamSynchronize(ctx->stream));
  for (auto& m : ctx->marks) {
    float t = 0.0f;
    if (cudaEventElapsedTime(&t, m.a, m.b) == cudaSuccess) ctx->stage_ms[m.stage] += t;
    ctx->stage_launches[m.stage] += m.launches;
    ctx->event_pool.push_back(m.a);
    ctx->event_pool.push_back(m.b);
  }
  ctx->marks.clear();
  for (int i = 0; i < JPXLG_STAGE_COUNT && i < n; ++i) {
    if (ms) ms[i] = ctx->stage_ms[i];
    if (launches) launches[i] = ctx->stage_launches[i];
    ctx->stage_ms[i] = 0.0;
    ctx->stage_launches[i] = 0;
  }
  return JPXLG_STAGE_COUNT;
}

int jpxlg_layout_create(jpxlg_ctx* ctx, int width, int height, const uint8_t* block_map,
                        const uint32_t* hf_mul, const uint8_t* sharpness, jpxlg_layout** out) {
  if (!ctx || !out || !block_map || !hf_mul) return fail(ctx, JPXLG_ERR_ARGUMENT, "null argument");
  *out = nullptr;
  if (width <= 0 || height <= 0 || width > 65535 * 8 || height > 65535 * 8)
    return fail(ctx, JPXLG_ERR_ARGUMENT, "frame %dx%d outside 1..524280", width, height);
  cudaSetDevice(ctx->device);
  std::unique_ptr<jpxlg_layout> L(new jpxlg_layout);
  L->ctx = ctx;
  L->device = ctx->device;
  L->geo = make_geo(width, height);
  const Geo& g = L->geo;
  const size_t nb = (size_t)g.bw * g.bh;
  // Validate the cover (every block covered exactly once by varblocks of
  // the carried shapes, inside the frame) and bucket origins.
  std::vector<uint8_t> covered(nb, 0);
  std::vector<uint32_t> bucket[kNumShapes];
  for (int by = 0; by < g.bh; ++by)
    for (int bx = 0; bx < g.bw; ++bx) {
      uint8_t e = block_map[(size_t)by * g.bw + bx];
      if (!(e & 0x80)) continue;
      int sel = e & 0x1f;
      Shape sh;
      if (!shape_of(sel, &sh))
        return fail(ctx, JPXLG_ERR_BLOCK_MAP, "block (%d,%d): DctSelect %d is not carried", bx,
                    by, sel);
      if (bx + sh.bcols > g.bw || by + sh.brows > g.bh)
        return fail(ctx, JPXLG_ERR_BLOCK_MAP, "block (%d,%d): varblock outside the frame", bx,
                    by);
      // jpxl-decode vardct/hf_meta.rs:222: a varblock lies inside one LF
      // group (256 x 256 pixels = 32 x 32 blocks), as every stream carries.
      if (bx / 32 != (bx + sh.bcols - 1) / 32 || by / 32 != (by + sh.brows - 1) / 32)
        return fail(ctx, JPXLG_ERR_BLOCK_MAP,
                    "block (%d,%d): varblock crosses the LF-group boundary", bx, by);
      for (int dy = 0; dy < sh.brows; ++dy)
        for (int dx = 0; dx < sh.bcols; ++dx) {
          size_t i = (size_t)(by + dy) * g.bw + bx + dx;
          if (covered[i] || (block_map[i] & 0x1f) != sel)
            return fail(ctx, JPXLG_ERR_BLOCK_MAP, "block (%d,%d): overlapping varblocks", bx + dx,
                        by + dy);
          covered[i] = 1;
        }
      int cls = 0;
      while (kShapeSel[cls] != sel) ++cls;
      bucket[cls].push_back(((uint32_t)by << 16) | (uint32_t)bx);
      // the encoder's kernels cover naturally aligned DCT8/16/32 only; the
      // format (and the render) place a varblock at any block
      if (sh.brows != sh.bcols || sh.brows > 4 || sel == 2 || bx % sh.bcols || by % sh.brows)
        L->all_square = false;
      if (hf_mul[(size_t)by * g.bw + bx] == 0)
        return fail(ctx, JPXLG_ERR_ARGUMENT, "block (%d,%d): hf_mul must be positive", bx, by);
    }
  for (size_t i = 0; i < nb; ++i)
    if (!covered[i])
      return fail(ctx, JPXLG_ERR_BLOCK_MAP, "block (%zu,%zu) is not covered", i % g.bw, i / g.bw);
  L->base_hf_mul = hf_mul[0];
  size_t total = 0;
  for (auto& b : bucket) total += b.size();
  CK(cudaMalloc(&L->d_map, nb));
  CK(cudaMalloc(&L->d_hf_mul, nb * sizeof(uint32_t)));
  CK(cudaMalloc(&L->d_sharp, nb));
  CK(cudaMalloc(&L->d_lists, std::max<size_t>(total, 1) * sizeof(uint32_t)));
  CK(cudaMemcpy(L->d_map, block_map, nb, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(L->d_hf_mul, hf_mul, nb * sizeof(uint32_t), cudaMemcpyHostToDevice));
  if (sharpness) CK(cudaMemcpy(L->d_sharp, sharpness, nb, cudaMemcpyHostToDevice));
  else CK(cudaMemset(L->d_sharp, 0, nb));
  size_t off = 0;
  for (int c = 0; c < kNumShapes; ++c) {
    L->counts[c] = (int)bucket[c].size();
    L->lists[c] = L->d_lists + off;
    if (!bucket[c].empty())
      CK(cudaMemcpy(L->d_lists + off, bucket[c].data(), bucket[c].size() * sizeof(uint32_t),
                    cudaMemcpyHostToDevice));
    off += bucket[c].size();
  }
  *out = L.release();
  return JPXLG_OK;
}

int jpxlg_layout_destroy(jpxlg_layout* L) {
  if (!L) return JPXLG_ERR_ARGUMENT;
  // The creating context may already be gone; cudaFree waits for the
  // device's queued work itself.
  cudaSetDevice(L->device);
  cudaFree(L->d_map);
  cudaFree(L->d_hf_mul);
  cudaFree(L->d_sharp);
  cudaFree(L->d_lists);
  delete L;
  return JPXLG_OK;
}

int jpxlg_layout_dims(const jpxlg_layout* L, int* bw, int* bh, int* tw, int* th) {
  if (!L) return JPXLG_ERR_ARGUMENT;
  if (bw) *bw = L->geo.bw;
  if (bh) *bh = L->geo.bh;
  if (tw) *tw = L->geo.tw;
  if (th) *th = L->geo.th;
  return JPXLG_OK;
}

int jpxlg_encode_transform(jpxlg_ctx* ctx, const jpxlg_layout* L, const void* rgb, int bits,
                           const jpxlg_params* p, jpxlg_plan* plan, uint32_t mem) {
  if (!ctx || !L || !rgb || !plan) return fail(ctx, JPXLG_ERR_ARGUMENT, "null argument");
  if (L->device != ctx->device) return fail(ctx, JPXLG_ERR_ARGUMENT, "layout on another device");
  if (!(bits == 8 || (bits >= 9 && bits <= 16)))
    return fail(ctx, JPXLG_ERR_ARGUMENT, "bits must be 8 or 9..16");
  int rc = check_params(ctx, p);
  if (rc) return rc;
  cudaSetDevice(ctx->device);
  const Geo& g = L->geo;
  const size_t n = (size_t)g.w * g.h, n8 = (size_t)g.W8 * g.H8, nb = (size_t)g.bw * g.bh;
  const size_t nt = (size_t)g.tw * g.th;
  const size_t rgb_bytes = 3 * n * (bits == 8 ? 1 : 2);
  if (mem == JPXLG_MEM_DEVICE) {
    if (!plan->qcoeff || !plan->lf || !plan->cfl_x || !plan->cfl_b)
      return fail(ctx, JPXLG_ERR_ARGUMENT, "null plan buffer");
    rc = encode_device(ctx, L, rgb, bits, p, plan->qcoeff, plan->lf, plan->cfl_x, plan->cfl_b,
                       plan->lf_factors);
    if (rc) return rc;
    // The two LF factors are plan scalars the caller needs on the host: the
    // call waits for them (8 bytes) and reports device-side errors.
    rc = sync_and_check(ctx);
    if (rc) return rc;
    const int* f = (const int*)(ctx->h_words + 4);
    plan->lf_factors[0] = f[0] + 128;
    plan->lf_factors[1] = f[1] + 128;
    return JPXLG_OK;
  }
  CK(ctx->rgb.ensure(rgb_bytes));
  CK(ctx->qcoeff.ensure(3 * n8 * sizeof(int32_t)));
  CK(ctx->lfq.ensure(3 * nb * sizeof(int32_t)));
  CK(ctx->cflx.ensure(nt));
  CK(ctx->cflb.ensure(nt));
  CK(cudaMemcpyAsync(ctx->rgb.p, rgb, rgb_bytes, cudaMemcpyHostToDevice, ctx->stream));
  rc = encode_device(ctx, L, ctx->rgb.p, bits, p, ctx->qcoeff.as<int32_t>(), ctx->lfq.as<int32_t>(),
                     ctx->cflx.as<int8_t>(), ctx->cflb.as<int8_t>(), plan->lf_factors);
  if (rc) return rc;
  if (plan->qcoeff)
    CK(cudaMemcpyAsync(plan->qcoeff, ctx->qcoeff.p, 3 * n8 * sizeof(int32_t),
                       cudaMemcpyDeviceToHost, ctx->stream));
  if (plan->lf)
    CK(cudaMemcpyAsync(plan->lf, ctx->lfq.p, 3 * nb * sizeof(int32_t), cudaMemcpyDeviceToHost,
                       ctx->stream));
  if (plan->cfl_x) CK(cudaMemcpyAsync(plan->cfl_x, ctx->cflx.p, nt, cudaMemcpyDeviceToHost, ctx->stream));
  if (plan->cfl_b) CK(cudaMemcpyAsync(plan->cfl_b, ctx->cflb.p, nt, cudaMemcpyDeviceToHost, ctx->stream));
  rc = sync_and_check(ctx);
  if (rc) return rc;
  const int* f = (const int*)(ctx->h_words + 4);
  plan->lf_factors[0] = f[0] + 128;
  plan->lf_factors[1] = f[1] + 128;
  return JPXLG_OK;
}

int jpxlg_tune_set(int knob, int value) {
  if (knob != JPXLG_TUNE_TC_CTAS_PER_SM || value < 1 || value > 4) return JPXLG_ERR_ARGUMENT;
  return tc_ctas_per_sm(value);
}

int jpxlg_tune_get(int knob) {
  if (knob != JPXLG_TUNE_TC_CTAS_PER_SM) return JPXLG_ERR_ARGUMENT;
  return tc_ctas_per_sm(0);
}

int jpxlg_diag_special_blocks(jpxlg_ctx* ctx, int kind, const float* coef, int n, float* out,
                              uint32_t mem) {
  if (!ctx || !coef || !out || n <= 0) return fail(ctx, JPXLG_ERR_ARGUMENT, "null argument");
  if (kind < 1 || kind > 9) return fail(ctx, JPXLG_ERR_ARGUMENT, "kind must be 1..9");
  CK(cudaSetDevice(ctx->device));
  const size_t bytes = (size_t)n * 64 * sizeof(float);
  const float* din = coef;
  float* dout = out;
  if (mem != JPXLG_MEM_DEVICE) {
    CK(ctx->coeff.ensure(bytes));
    CK(ctx->out.ensure(bytes));
    CK(cudaMemcpyAsync(ctx->coeff.p, coef, bytes, cudaMemcpyHostToDevice, ctx->stream));
    din = ctx->coeff.as<float>();
    dout = ctx->out.as<float>();
  }
  launch_special_diag(kind, din, n, dout, ctx->stream);
  int rc = after_launch(ctx, 1);
  if (rc) return rc;
  if (mem == JPXLG_MEM_DEVICE) return JPXLG_OK;
  CK(cudaMemcpyAsync(out, dout, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return JPXLG_OK;
}

int jpxlg_encode_stages(jpxlg_ctx* ctx, const jpxlg_layout* L, const void* rgb, int bits,
                        const jpxlg_params* p, float* xyb, float* pre, float* coeff) {
  if (!ctx || !L || !rgb) return fail(ctx, JPXLG_ERR_ARGUMENT, "null argument");
  if (L->device != ctx->device) return fail(ctx, JPXLG_ERR_ARGUMENT, "layout on another device");
  if (!(bits == 8 || (bits >= 9 && bits <= 16)))
    return fail(ctx, JPXLG_ERR_ARGUMENT, "bits must be 8 or 9..16");
  int rc = check_params(ctx, p);
  if (rc) return rc;
  cudaSetDevice(ctx->device);
  const Geo& g = L->geo;
  const size_t n = (size_t)g.w * g.h, n8 = (size_t)g.W8 * g.H8, nb = (size_t)g.bw * g.bh;
  const size_t nt = (size_t)g.tw * g.th;
  const size_t rgb_bytes = 3 * n * (bits == 8 ? 1 : 2);
  CK(ctx->rgb.ensure(rgb_bytes));
  CK(ctx->qcoeff.ensure(3 * n8 * sizeof(int32_t)));
  CK(ctx->lfq.ensure(3 * nb * sizeof(int32_t)));
  CK(ctx->cflx.ensure(nt));
  CK(ctx->cflb.ensure(nt));
  CK(cudaMemcpyAsync(ctx->rgb.p, rgb, rgb_bytes, cudaMemcpyHostToDevice, ctx->stream));
  rc = encode_device(ctx, L, ctx->rgb.p, bits, p, ctx->qcoeff.as<int32_t>(), ctx->lfq.as<int32_t>(),
                     ctx->cflx.as<int8_t>(), ctx->cflb.as<int8_t>(), nullptr);
  if (rc) return rc;
  if (xyb) CK(cudaMemcpyAsync(xyb, ctx->xyb.p, 3 * n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  if (pre)
    CK(cudaMemcpyAsync(pre, p->gaborish ? ctx->pre.p : ctx->xyb.p, 3 * n * sizeof(float),
                       cudaMemcpyDeviceToHost, ctx->stream));
  if (coeff)
    CK(cudaMemcpyAsync(coeff, ctx->coeff.p, 3 * n8 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  return sync_and_check(ctx);
}

int jpxlg_reconstruct(jpxlg_ctx* ctx, const jpxlg_layout* L, const jpxlg_plan* plan,
                      const jpxlg_params* p, int out_kind, int bits, void* out, uint32_t mem) {
  if (!ctx || !L || !plan || !out) return fail(ctx, JPXLG_ERR_ARGUMENT, "null argument");
  if (L->device != ctx->device) return fail(ctx, JPXLG_ERR_ARGUMENT, "layout on another device");
  if (!plan->qcoeff || !plan->lf || !plan->cfl_x || !plan->cfl_b)
    return fail(ctx, JPXLG_ERR_ARGUMENT, "null plan buffer");
  int rc = check_params(ctx, p);
  if (rc) return rc;
  if (out_kind < 0 || out_kind > 4) return fail(ctx, JPXLG_ERR_ARGUMENT, "bad out_kind");
  if (out_kind == JPXLG_OUT_LINEAR_DEPTH && (bits < 1 || bits > 16))
    return fail(ctx, JPXLG_ERR_ARGUMENT, "depth must be 1..16 bits");
  for (int i = 0; i < 2; ++i)
    if (plan->lf_factors[i] < 0 || plan->lf_factors[i] > 255)
      return fail(ctx, JPXLG_ERR_ARGUMENT, "LF factor outside u8");
  cudaSetDevice(ctx->device);
  const Geo& g = L->geo;
  const size_t n = (size_t)g.w * g.h, n8 = (size_t)g.W8 * g.H8, nb = (size_t)g.bw * g.bh;
  const size_t nt = (size_t)g.tw * g.th;
  const size_t out_bytes = out_kind == JPXLG_OUT_SRGB8 ? 3 * n : 3 * n * sizeof(float);
  if (mem == JPXLG_MEM_DEVICE)
    return render_device(ctx, L, plan->qcoeff, plan->lf, plan->cfl_x, plan->cfl_b,
                         plan->lf_factors[0], plan->lf_factors[1], nullptr, p, out_kind, bits, out);
  CK(ctx->qcoeff.ensure(3 * n8 * sizeof(int32_t)));
  CK(ctx->lfq.ensure(3 * nb * sizeof(int32_t)));
  CK(ctx->cflx.ensure(nt));
  CK(ctx->cflb.ensure(nt));
  CK(ctx->out.ensure(out_bytes));
  CK(cudaMemcpyAsync(ctx->qcoeff.p, plan->qcoeff, 3 * n8 * sizeof(int32_t), cudaMemcpyHostToDevice,
                     ctx->stream));
  CK(cudaMemcpyAsync(ctx->lfq.p, plan->lf, 3 * nb * sizeof(int32_t), cudaMemcpyHostToDevice,
                     ctx->stream));
  CK(cudaMemcpyAsync(ctx->cflx.p, plan->cfl_x, nt, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->cflb.p, plan->cfl_b, nt, cudaMemcpyHostToDevice, ctx->stream));
  rc = render_device(ctx, L, ctx->qcoeff.as<int32_t>(), ctx->lfq.as<int32_t>(), ctx->cflx.as<int8_t>(),
                     ctx->cflb.as<int8_t>(), plan->lf_factors[0], plan->lf_factors[1], nullptr, p,
                     out_kind, bits, ctx->out.p);
  if (rc) return rc;
  CK(cudaMemcpyAsync(out, ctx->out.p, out_bytes, cudaMemcpyDeviceToHost, ctx->stream));
  return sync_and_check(ctx);
}

namespace {

// reference.rs:90: the scales (keep halving while the current one is at
// least 8x8) and the floats of a reference's planes (per scale: the RGB
// level, XYB, mu and sigma11, 3 planes each).
int ref_layout(int w, int h, int dims[6][2], size_t* total) {
  int cw = w, ch = h, ns = 0;
  *total = 0;
  for (int s = 0; s < 6; ++s) {
    if (s > 0) {
      if (cw < 8 || ch < 8) break;
      cw = (cw + 1) / 2;
      ch = (ch + 1) / 2;
    }
    dims[s][0] = cw;
    dims[s][1] = ch;
    *total += 9 * (size_t)cw * ch + 3 * (size_t)cw * ch;
    ++ns;
  }
  return ns;
}

int ref_check(jpxlg_ctx* ctx, int w, int h) {
  if (w < 8 || h < 8) return fail(ctx, JPXLG_ERR_TOO_SMALL, "SSIMULACRA2 needs at least 8x8");
  if (w > kBlurMaxWidth)
    return fail(ctx, JPXLG_ERR_ARGUMENT, "SSIMULACRA2 frames are limited to %d columns",
                kBlurMaxWidth);
  return JPXLG_OK;
}

// Fills R (w, h, device set) in `block` (ref_layout's floats): the pyramid,
// positive XYB and the blurred moments of every scale.
int ref_fill(jpxlg_ctx* ctx, jpxlg_ref* R, void* block, const float* rgb, uint32_t mem) {
  int dims[6][2];
  size_t total;
  const int w = R->w, h = R->h;
  const int ns = ref_layout(w, h, dims, &total);
  R->nscales = ns;
  R->block = block;
  float* cursor = (float*)block;
  const size_t n0 = (size_t)w * h;
  CK(ctx->hpl.ensure(9 * n0 * sizeof(float)));
  CK(ctx->bcarry.ensure(blur_carry_floats(w, h) * sizeof(float)));
  CK(ctx->out.ensure(3 * n0 * sizeof(float)));
  const float* src = rgb;
  if (mem == JPXLG_MEM_HOST) {
    CK(cudaMemcpyAsync(ctx->out.p, rgb, 3 * n0 * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    src = ctx->out.as<float>();
  }
  uint64_t k = 0;
  const float* level = src;
  for (int s = 0; s < ns; ++s) {
    SsimScale& sc = R->scales[s];
    sc.w = dims[s][0];
    sc.h = dims[s][1];
    const size_t n = (size_t)sc.w * sc.h;
    float* rgb_s = cursor;
    cursor += 3 * n;
    if (s > 0) {
      launch_downscale3(level, dims[s - 1][0], dims[s - 1][1], rgb_s, nullptr, ctx->stream);
      ++k;
      level = rgb_s;
    }
    sc.xyb = cursor;
    cursor += 3 * n;
    sc.mu = cursor;
    cursor += 3 * n;
    sc.s11 = cursor;
    cursor += 3 * n;
    launch_positive_xyb(level, sc.xyb, n, ctx->num_sms, ctx->stream);
    launch_ref_moments(sc.xyb, sc.mu, sc.s11, ctx->hpl.as<float>(), ctx->bcarry.as<float>(), sc.w,
                       sc.h, ctx->d_words, ctx->stream);
    k += 1 + 2;
  }
  return after_launch(ctx, k);
}

}  // namespace

int jpxlg_ssim2_ref_create(jpxlg_ctx* ctx, const float* rgb, int w, int h, uint32_t mem,
                           jpxlg_ref** out) {
  if (!ctx || !rgb || !out) return fail(ctx, JPXLG_ERR_ARGUMENT, "null argument");
  *out = nullptr;
  int rc = ref_check(ctx, w, h);
  if (rc) return rc;
  cudaSetDevice(ctx->device);
  std::unique_ptr<jpxlg_ref> R(new jpxlg_ref);
  R->ctx = ctx;
  R->device = ctx->device;
  R->w = w;
  R->h = h;
  int dims[6][2];
  size_t total;
  ref_layout(w, h, dims, &total);
  void* block = nullptr;
  CK(cudaMalloc(&block, total * sizeof(float)));
  rc = ref_fill(ctx, R.get(), block, rgb, mem);
  if (rc == JPXLG_OK && mem == JPXLG_MEM_HOST) rc = sync_and_check(ctx);
  if (rc) {
    cudaFree(block);
    return rc;
  }
  *out = R.release();
  return JPXLG_OK;
}

int jpxlg_ssim2_ref_destroy(jpxlg_ref* R) {
  if (!R) return JPXLG_ERR_ARGUMENT;
  cudaSetDevice(R->device);
  cudaFree(R->block);
  delete R;
  return JPXLG_OK;
}

int jpxlg_ssim2_score(jpxlg_ctx* ctx, const jpxlg_ref* R, const float* rgb, uint32_t mem,
                      double* score, double* raw_error, double* terms) {
  if (!ctx || !R || !rgb) return fail(ctx, JPXLG_ERR_ARGUMENT, "null argument");
  if (R->device != ctx->device)
    return fail(ctx, JPXLG_ERR_ARGUMENT, "reference on another device");
  cudaSetDevice(ctx->device);
  const size_t n = (size_t)R->w * R->h;
  CK(ctx->score.ensure(128 * sizeof(double)));
  const float* cand = rgb;
  if (mem == JPXLG_MEM_HOST) {
    CK(ctx->out.ensure(3 * n * sizeof(float)));
    CK(cudaMemcpyAsync(ctx->out.p, rgb, 3 * n * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    cand = ctx->out.as<float>();
  }
  // The finish kernel writes score, raw error and every term into the
  // context's own buffer; callers receive only the outputs they asked for.
  int rc = score_device(ctx, R, cand, nullptr, ctx->score.as<double>());
  if (rc) return rc;
  if (mem == JPXLG_MEM_DEVICE) {
    const double* s = ctx->score.as<double>();
    if (score)
      CK(cudaMemcpyAsync(score, s, sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    if (raw_error)
      CK(cudaMemcpyAsync(raw_error, s + 1, sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    if (terms)
      CK(cudaMemcpyAsync(terms, s + 2, R->nscales * 18 * sizeof(double), cudaMemcpyDeviceToDevice,
                         ctx->stream));
    return JPXLG_OK;
  }
  CK(cudaMemcpyAsync(ctx->h_score, ctx->score.p, (2 + 108) * sizeof(double), cudaMemcpyDeviceToHost,
                     ctx->stream));
  rc = sync_and_check(ctx);
  if (rc) return rc;
  if (score) *score = ctx->h_score[0];
  if (raw_error) *raw_error = ctx->h_score[1];
  if (terms)
    for (int i = 0; i < R->nscales * 18; ++i) terms[i] = ctx->h_score[2 + i];
  return JPXLG_OK;
}

int jpxlg_score_pair(jpxlg_ctx* ctx, const float* ref_rgb, const float* cand_rgb, int w, int h,
                     uint32_t mem, double* score) {
  if (!ctx || !ref_rgb || !cand_rgb || !score)
    return fail(ctx, JPXLG_ERR_ARGUMENT, "null argument");
  int rc = ref_check(ctx, w, h);
  if (rc) return rc;
  cudaSetDevice(ctx->device);
  // The reference side in the context's own buffer, kept for the next call
  // (no allocation or free per pair).
  jpxlg_ref R;
  R.ctx = ctx;
  R.device = ctx->device;
  R.w = w;
  R.h = h;
  int dims[6][2];
  size_t total;
  ref_layout(w, h, dims, &total);
  CK(ctx->pair_ref.ensure(total * sizeof(float)));
  rc = ref_fill(ctx, &R, ctx->pair_ref.p, ref_rgb, mem);
  if (rc) return rc;
  rc = jpxlg_ssim2_score(ctx, &R, cand_rgb, mem, score, nullptr, nullptr);
  if (mem == JPXLG_MEM_DEVICE && rc == JPXLG_OK) rc = sync_and_check(ctx);
  return rc;
}

int jpxlg_probe(jpxlg_ctx* ctx, const jpxlg_layout* L, const jpxlg_ref* R, const void* rgb,
                int bits, const jpxlg_params* p, uint32_t mem, double* score) {
  if (!ctx || !L || !R || !rgb || !score) return fail(ctx, JPXLG_ERR_ARGUMENT, "null argument");
  if (L->device != ctx->device || R->device != ctx->device)
    return fail(ctx, JPXLG_ERR_ARGUMENT, "layout or reference on another device");
  if (R->w != L->geo.w || R->h != L->geo.h)
    return fail(ctx, JPXLG_ERR_MISMATCH, "reference and layout dimensions differ");
  int rc = check_params(ctx, p);
  if (rc) return rc;
  cudaSetDevice(ctx->device);
  const Geo& g = L->geo;
  const size_t n = (size_t)g.w * g.h, n8 = (size_t)g.W8 * g.H8, nb = (size_t)g.bw * g.bh;
  const size_t nt = (size_t)g.tw * g.th;
  CK(ctx->qcoeff.ensure(3 * n8 * sizeof(int32_t)));
  CK(ctx->lfq.ensure(3 * nb * sizeof(int32_t)));
  CK(ctx->cflx.ensure(nt));
  CK(ctx->cflb.ensure(nt));
  CK(ctx->out.ensure(3 * n * sizeof(float)));
  CK(ctx->cxyb.ensure(3 * n * sizeof(float)));
  CK(ctx->score.ensure(128 * sizeof(double)));
  const void* src = rgb;
  if (mem == JPXLG_MEM_HOST) {
    const size_t rgb_bytes = 3 * n * (bits == 8 ? 1 : 2);
    CK(ctx->rgb.ensure(rgb_bytes));
    CK(cudaMemcpyAsync(ctx->rgb.p, rgb, rgb_bytes, cudaMemcpyHostToDevice, ctx->stream));
    src = ctx->rgb.p;
  }
  rc = encode_device(ctx, L, src, bits, p, ctx->qcoeff.as<int32_t>(), ctx->lfq.as<int32_t>(),
                     ctx->cflx.as<int8_t>(), ctx->cflb.as<int8_t>(), nullptr);
  if (rc) return rc;
  rc = render_device(ctx, L, ctx->qcoeff.as<int32_t>(), ctx->lfq.as<int32_t>(),
                     ctx->cflx.as<int8_t>(), ctx->cflb.as<int8_t>(), 128, 128, ctx->d_lf, p,
                     JPXLG_OUT_LINEAR_DEPTH, bits, ctx->out.p, ctx->cxyb.as<float>());
  if (rc) return rc;
  // The finish kernel fills the context's 128-double buffer (score, raw
  // error, terms); the caller's slot receives the score alone.
  rc = score_device(ctx, R, ctx->out.as<float>(), ctx->cxyb.as<float>(), ctx->score.as<double>());
  if (rc) return rc;
  if (mem == JPXLG_MEM_DEVICE) {
    CK(cudaMemcpyAsync(score, ctx->score.p, sizeof(double), cudaMemcpyDeviceToDevice,
                       ctx->stream));
    return JPXLG_OK;
  }
  CK(cudaMemcpyAsync(ctx->h_score, ctx->score.p, sizeof(double), cudaMemcpyDeviceToHost,
                     ctx->stream));
  rc = sync_and_check(ctx);
  if (rc) return rc;
  *score = ctx->h_score[0];
  return JPXLG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Cover selection (policy lib.rs:5260 select_blocks) on the GPU.
extern "C" int jpxlg_select_blocks(jpxlg_ctx* ctx, int width, int height, const void* rgb,
                                   int bits, const jpxlg_params* p, uint8_t* block_map,
                                   uint32_t mem) {
  if (!ctx || !rgb || !block_map) return fail(ctx, JPXLG_ERR_ARGUMENT, "null argument");
  if (width <= 0 || height <= 0) return fail(ctx, JPXLG_ERR_ARGUMENT, "empty frame");
  if (!(bits == 8 || (bits >= 9 && bits <= 16)))
    return fail(ctx, JPXLG_ERR_ARGUMENT, "bits must be 8 or 9..16");
  int rc = check_params(ctx, p);
  if (rc) return rc;
  CK(cudaSetDevice(ctx->device));
  const Geo g = make_geo(width, height);
  const size_t n = (size_t)g.w * g.h, nb = (size_t)g.bw * g.bh;
  const void* src = rgb;
  if (mem == JPXLG_MEM_HOST) {
    const size_t rgb_bytes = 3 * n * (bits == 8 ? 1 : 2);
    CK(ctx->rgb.ensure(rgb_bytes));
    CK(cudaMemcpyAsync(ctx->rgb.p, rgb, rgb_bytes, cudaMemcpyHostToDevice, ctx->stream));
    src = ctx->rgb.p;
  }
  const float* pre = nullptr;
  rc = transform_frame(ctx, g, src, bits, p, &pre);
  if (rc) return rc;
  CK(ctx->cover.ensure(cover_scratch_bytes(g)));
  uint8_t* map = block_map;
  if (mem == JPXLG_MEM_HOST) {
    CK(ctx->cover_map.ensure(nb));
    map = ctx->cover_map.as<uint8_t>();
  }
  CoverArgs a;
  a.geo = g;
  a.pre = pre;
  a.dq = ctx->d_dq;
  // The quantizers of the three square transforms at the baseline HfMul
  // (adaptive quantization off), as HfQuantizer::new_with_matrices forms
  // them, and lib.rs:2094's lambda from the DCT8x8 steps.
  const float mul = host_hf_multiplier(p->global_scale, 1);
  a.scale[0] = mul * host_qm_multiplier(p->x_qm_scale);
  a.scale[1] = mul;
  a.scale[2] = mul * host_qm_multiplier(p->b_qm_scale);
  std::vector<float> dq(3 * kDequantTableFloats);
  build_dequant_tables(dq.data());
  for (int c = 0; c < 3; ++c) {
    double sum = 0.0;
    uint32_t count = 0;
    for (int cell = 1; cell < 64; ++cell) {
      const float step = a.scale[c] * dq[c * kDequantTableFloats + dq_offset(0) + cell];
      const double s8 = 8.0 * (double)step;
      sum += s8 * s8;
      ++count;
    }
    const double mean = sum / (double)std::max(count, 1u);
    a.lambda[c] = mean > 0.0 ? 1.0 * 16.0 / mean : 0.0;
    for (int s = 0; s < 3; ++s) {
      const int side = 8 << s;
      a.w[s][c] = a.lambda[c] * ((double)(side * side) * 1.0);
    }
  }
  cover_bind_scratch(&a, ctx->cover.p);
  a.map = map;
  a.fallbacks = ctx->d_words + 3;
  a.err = ctx->d_words;
  rc = after_launch(ctx, launch_cover(a, ctx->stream));
  if (rc) return rc;
  if (mem == JPXLG_MEM_DEVICE) return JPXLG_OK;
  CK(cudaMemcpyAsync(block_map, map, nb, cudaMemcpyDeviceToHost, ctx->stream));
  return sync_and_check(ctx);
}

extern "C" uint32_t jpxlg_ctx_cover_fallbacks(jpxlg_ctx* ctx) {
  if (!ctx) return 0;
  cudaSetDevice(ctx->device);
  uint32_t v = 0;
  cudaStreamSynchronize(ctx->stream);
  cudaMemcpy(&v, ctx->d_words + 3, sizeof(uint32_t), cudaMemcpyDeviceToHost);
  return v;
}

// ---------------------------------------------------------------------------
// Batched probes as one CUDA graph.  Each lane is a full context (tables,
// workspace, stream) owned by the batch; item i runs on lane i % lanes.  The
// warm-up pass sizes every lane's workspace and builds its lookup tables, so
// the captured pass performs stream work only.
struct jpxlg_batch {
  jpxlg_ctx* owner = nullptr;
  int device = 0;
  std::vector<jpxlg_ctx*> lanes;
  std::vector<jpxlg_batch_item> items;
  double* d_scores = nullptr;
  double* h_scores = nullptr;  // pinned
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> joins;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {

void batch_free(jpxlg_batch* b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->fork) cudaEventDestroy(b->fork);
  for (cudaEvent_t e : b->joins) cudaEventDestroy(e);
  for (jpxlg_ctx* l : b->lanes) jpxlg_ctx_destroy(l);
  cudaFree(b->d_scores);
  cudaFreeHost(b->h_scores);
  delete b;
}

// Queues every item on its lane (device mode, scores into d_scores).
int batch_enqueue(jpxlg_ctx* ctx, jpxlg_batch* b) {
  const int L = (int)b->lanes.size();
  for (size_t i = 0; i < b->items.size(); ++i) {
    const jpxlg_batch_item& it = b->items[i];
    jpxlg_ctx* lane = b->lanes[i % L];
    int rc = jpxlg_probe(lane, it.layout, it.ref, it.rgb, it.bits, &it.params, JPXLG_MEM_DEVICE,
                         b->d_scores + i);
    if (rc) return fail(ctx, rc, "batch item %zu: %s", i, lane->last_error.c_str());
  }
  return JPXLG_OK;
}

// Reads and clears each lane's device error word once the batch is done.
int batch_check(jpxlg_ctx* ctx, jpxlg_batch* b) {
  for (jpxlg_ctx* lane : b->lanes) {
    int rc = sync_and_check(lane);
    if (rc) return fail(ctx, rc, "batch lane: %s", lane->last_error.c_str());
  }
  return JPXLG_OK;
}

}  // namespace

extern "C" int jpxlg_batch_create(jpxlg_ctx* ctx, int n_items, const jpxlg_batch_item* items,
                                  int lanes, jpxlg_batch** out) {
  if (!ctx || !items || !out || n_items <= 0) return fail(ctx, JPXLG_ERR_ARGUMENT, "null argument");
  *out = nullptr;
  for (int i = 0; i < n_items; ++i) {
    const jpxlg_batch_item& it = items[i];
    if (!it.layout || !it.ref || !it.rgb) return fail(ctx, JPXLG_ERR_ARGUMENT, "item %d: null", i);
    if (!(it.bits == 8 || (it.bits >= 9 && it.bits <= 16)))
      return fail(ctx, JPXLG_ERR_ARGUMENT, "item %d: bits must be 8 or 9..16", i);
    int rc = check_params(ctx, &it.params);
    if (rc) return rc;
  }
  if (lanes <= 0) lanes = std::min(n_items, 4);
  lanes = std::min(lanes, n_items);
  CK(cudaSetDevice(ctx->device));
  std::unique_ptr<jpxlg_batch, void (*)(jpxlg_batch*)> b(new jpxlg_batch, batch_free);
  b->owner = ctx;
  b->device = ctx->device;
  b->items.assign(items, items + n_items);
  for (int l = 0; l < lanes; ++l) {
    jpxlg_ctx* lane = nullptr;
    int rc = jpxlg_ctx_create(ctx->device, 0, &lane);
    if (rc) return fail(ctx, rc, "batch lane %d: context creation failed", l);
    b->lanes.push_back(lane);
    cudaEvent_t e = nullptr;
    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    b->joins.push_back(e);
  }
  CK(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
  CK(cudaMalloc(&b->d_scores, n_items * sizeof(double)));
  CK(cudaMallocHost(&b->h_scores, n_items * sizeof(double)));
  // Warm-up: every allocation and table the probes need happens here.
  int rc = batch_enqueue(ctx, b.get());
  if (rc) return rc;
  rc = batch_check(ctx, b.get());
  if (rc) return rc;
  // Capture: fork from ctx's stream, the lanes' probes, join back.
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  cudaEventRecord(b->fork, ctx->stream);
  for (jpxlg_ctx* lane : b->lanes) cudaStreamWaitEvent(lane->stream, b->fork, 0);
  rc = batch_enqueue(ctx, b.get());
  for (size_t l = 0; l < b->lanes.size(); ++l) {
    cudaEventRecord(b->joins[l], b->lanes[l]->stream);
    cudaStreamWaitEvent(ctx->stream, b->joins[l], 0);
  }
  cudaError_t ce = cudaStreamEndCapture(ctx->stream, &b->graph);
  if (rc) return rc;
  if (ce != cudaSuccess)
    return fail(ctx, JPXLG_ERR_CUDA, "batch capture: %s", cudaGetErrorString(ce));
  CK(cudaGraphInstantiate(&b->exec, b->graph, 0));
  *out = b.release();
  return JPXLG_OK;
}

extern "C" int jpxlg_batch_run(jpxlg_ctx* ctx, jpxlg_batch* b, double* scores, uint32_t mem) {
  if (!ctx || !b || !scores) return fail(ctx, JPXLG_ERR_ARGUMENT, "null argument");
  if (b->owner != ctx) return fail(ctx, JPXLG_ERR_ARGUMENT, "batch belongs to another context");
  CK(cudaSetDevice(ctx->device));
  CK(cudaGraphLaunch(b->exec, ctx->stream));
  const size_t bytes = b->items.size() * sizeof(double);
  if (mem == JPXLG_MEM_DEVICE) {
    CK(cudaMemcpyAsync(scores, b->d_scores, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    return JPXLG_OK;
  }
  CK(cudaMemcpyAsync(b->h_scores, b->d_scores, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  int rc = batch_check(ctx, b);
  if (rc) return rc;
  std::memcpy(scores, b->h_scores, bytes);
  return JPXLG_OK;
}

extern "C" int jpxlg_batch_destroy(jpxlg_batch* b) {
  if (!b) return JPXLG_ERR_ARGUMENT;
  // The owning context may already be gone: wait for the device instead of
  // its stream before the graph and the lanes are released.
  cudaSetDevice(b->device);
  cudaDeviceSynchronize();
  batch_free(b);
  return JPXLG_OK;
}

extern "C" int jpxlg_batch_probe(jpxlg_ctx* ctx, int n_items, const jpxlg_batch_item* items,
                                 double* scores) {
  jpxlg_batch* b = nullptr;
  int rc = jpxlg_batch_create(ctx, n_items, items, 0, &b);
  if (rc) return rc;
  rc = jpxlg_batch_run(ctx, b, scores, JPXLG_MEM_HOST);
  jpxlg_batch_destroy(b);
  return rc;
}

// ---------------------------------------------------------------------------
// Allocation-free scoring.  jpxlg_ssim2_score_static runs the same kernels as
// jpxlg_ssim2_score but keeps its workspace in one file-scope device array
// instead of the context's buffers, so no call ever reaches cudaMalloc or
// cudaFree.
//
// Capacity: reference frames up to kStaticMaxSide x kStaticMaxSide.  For a
// 2048 x 2048 frame the workspace holds the linear pyramid of scales 1..5,
// 3 * (1024^2 + 512^2 + 256^2 + 128^2 + 64^2) = 4,190,208 floats; the
// current scale's candidate positive XYB, 3 * 2048^2 = 12,582,912 floats;
// the row pass of one channel (three planes), 12,582,912 floats; the column
// pass's segment responses and entry states of one channel,
// 2 x 64 segments x 18 x 2048 = 4,718,592 floats; and the partial sums, one
// row of 18 double-float sums per 32 x 32 tile of each scale,
// 4096 + 1024 + 256 + 64 + 16 + 4 = 5,460 rows: 137 MB in all.  Every count grows with width and height, so any frame within the
// side limit fits.
// Channels are scored one after another so that the row pass needs one
// channel's planes.
//
// Nothing in the scratch has to start at zero: each call writes every level,
// plane and partial row before reading it.  There is one scratch per device,
// so calls whose work overlaps on a device (two streams, two contexts, or
// two host threads) race on it; callers serialise them.
namespace {

constexpr int kStaticMaxSide = 2048;
constexpr size_t kStaticPyrFloats = 4190208;
constexpr size_t kStaticPlaneFloats = (size_t)kStaticMaxSide * kStaticMaxSide;
constexpr size_t kStaticPartialRows = 5460;
constexpr size_t kStaticCarryFloats = 4718592;
// pyramid, positive XYB, row pass, segment states
constexpr size_t kStaticFloats = kStaticPyrFloats + 6 * kStaticPlaneFloats + kStaticCarryFloats;
constexpr size_t kStaticFloatBytes = kStaticFloats * sizeof(float);  // a multiple of 256
constexpr size_t kStaticScratchBytes = kStaticFloatBytes + kStaticPartialRows * 18 * sizeof(DF);
constexpr int kStaticMaxDevices = 64;

static __device__ __align__(256) unsigned char g_score_scratch[kStaticScratchBytes];

std::mutex g_scratch_mu;
void* g_scratch_ptr[kStaticMaxDevices] = {};

// Resolves the scratch address on the current device, once per device.  The
// first resolution can load the module's device globals, so the first call
// on a device should come before any stream capture that includes it.
int static_scratch(jpxlg_ctx* ctx, unsigned char** out) {
  if (ctx->device < 0 || ctx->device >= kStaticMaxDevices)
    return fail(ctx, JPXLG_ERR_ARGUMENT, "device ordinal %d beyond %d", ctx->device,
                kStaticMaxDevices);
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[ctx->device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_score_scratch);
    if (e != cudaSuccess || !p)
      return fail(ctx, JPXLG_ERR_CUDA, "static scratch address: %s", cudaGetErrorString(e));
    g_scratch_ptr[ctx->device] = p;
  }
  *out = (unsigned char*)g_scratch_ptr[ctx->device];
  return JPXLG_OK;
}

}  // namespace

extern "C" int jpxlg_ssim2_score_static(jpxlg_ctx* ctx, const jpxlg_ref* ref,
                                        const float* linear_rgb_dev, double* out_dev) {
  if (!ctx || !ref || !linear_rgb_dev || !out_dev)
    return fail(ctx, JPXLG_ERR_ARGUMENT, "null argument");
  if (ref->w > kStaticMaxSide || ref->h > kStaticMaxSide)
    return fail(ctx, JPXLG_ERR_ARGUMENT,
                "%dx%d exceeds the static scoring scratch limit of %dx%d; use jpxlg_ssim2_score",
                ref->w, ref->h, kStaticMaxSide, kStaticMaxSide);
  CK(cudaSetDevice(ctx->device));
  unsigned char* scratch = nullptr;
  int rc = static_scratch(ctx, &scratch);
  if (rc) return rc;
  // Every region checked against its capacity at run time, not only through
  // the side limit: the pyramid, the partial-sum rows, and per scale the
  // candidate's positive XYB and one channel's row-pass planes (three planes
  // each) and its column-pass carry (a third of the three channels').
  size_t pyr = 0, rows = 0;
  bool fits = true;
  for (int s = 0; s < ref->nscales; ++s) {
    const SsimScale& rs = ref->scales[s];
    if (s > 0) pyr += 3 * (size_t)rs.w * rs.h;
    rows += (size_t)blur_partial_rows(rs.w, rs.h);
    fits = fits && (size_t)rs.w * rs.h <= kStaticPlaneFloats &&
           blur_carry_floats(rs.w, rs.h) / 3 <= kStaticCarryFloats;
  }
  if (!fits || pyr > kStaticPyrFloats || rows > kStaticPartialRows)
    return fail(ctx, JPXLG_ERR_ARGUMENT, "static scoring scratch too small for %dx%d", ref->w,
                ref->h);
  float* next = (float*)scratch;
  float* xyb = next + kStaticPyrFloats;
  float* hpl = xyb + 3 * kStaticPlaneFloats;
  float* carry = hpl + 3 * kStaticPlaneFloats;
  DF* part0 = (DF*)(scratch + kStaticFloatBytes);
  DF* part = part0;
  const float* cur = linear_rgb_dev;
  int ctas[6], pixels[6];
  uint64_t k = 0;
  for (int s = 0; s < ref->nscales; ++s) {
    const SsimScale& rs = ref->scales[s];
    if (s > 0) {
      launch_downscale3(cur, ref->scales[s - 1].w, ref->scales[s - 1].h, next, xyb, ctx->stream);
      ++k;
      cur = next;
      next += 3 * (size_t)rs.w * rs.h;
    } else {
      launch_positive_xyb(cur, xyb, (size_t)rs.w * rs.h, ctx->num_sms, ctx->stream);
      ++k;
    }
    for (int c = 0; c < 3; ++c) {
      ctas[s] = launch_score_scale(xyb, rs, hpl, carry, c, 1, part, ctx->d_words, ctx->stream);
      k += kScoreScaleKernels;
    }
    pixels[s] = rs.w * rs.h;
    part += (size_t)ctas[s] * 18;
  }
  k += launch_score_finish(part0, ctas, ref->nscales, pixels, out_dev, ctx->stream);
  return after_launch(ctx, k);
}

// ---------------------------------------------------------------------------
// Decoded codestreams: the frame's integer content from the host reader,
// reconstructed by the same kernels as a plan (decode.rs:2700-3061).
// ---------------------------------------------------------------------------

namespace {

// A parsed VarDCT frame staged for the GPU render: its layout and
// parameters, and in one host block (pinned for batches) the coefficient
// image, the LF planes, the CfL tiles and (an LF frame) the LF XYB planes.
struct DecodeStage {
  jpxlg_layout* L = nullptr;
  jpxlg_params p{};
  size_t n = 0, n8 = 0, nb = 0, nt = 0;
  void* host = nullptr;
  bool pinned = false;
  int32_t* q = nullptr;
  int32_t* lfq = nullptr;
  int8_t* cflx = nullptr;
  int8_t* cflb = nullptr;
  float* lf_frame = nullptr;  // 3 * nb, or null
  float m[3] = {0, 0, 0};
  float kx = 0, kb = 1, div = 1;
  bool smooth = false;
  int fx = 128, fb = 128;
  DecodeStage() = default;
  DecodeStage(const DecodeStage&) = delete;
  DecodeStage& operator=(const DecodeStage&) = delete;
  ~DecodeStage() {
    if (L) jpxlg_layout_destroy(L);
    if (pinned) cudaFreeHost(host);
    else std::free(host);
  }
};

// Checks that the renderer carries everything the frame uses, and stages
// it (host work only: the coefficient image from the parsed groups).
int decode_stage(jpxlg_ctx* ctx, const jpxlg_codestream* cs, int out_kind, bool pinned,
                 DecodeStage& st, uint32_t precision = JPXLG_PRECISION_FP32) {
  if (out_kind < 0 || out_kind > 4 || out_kind == JPXLG_OUT_LINEAR_DEPTH)
    return fail(ctx, JPXLG_ERR_ARGUMENT, "bad out_kind");
  const jpxlg::cs::Decoded& d = cs->d;
  const jpxlg::cs::VarDctFrame& v = d.vardct;
  const jpxlg::cs::FrameInfo& f = d.frame;
  if (f.encoding != 0) return fail(ctx, JPXLG_ERR_STREAM, "not a VarDCT frame");
  if (!v.default_matrices)
    return fail(ctx, JPXLG_ERR_STREAM, "custom dequantization matrices are not carried");
  if (v.colour_factor != 84 || v.base_corr_x != 0.0f || v.base_corr_b != 1.0f)
    return fail(ctx, JPXLG_ERR_STREAM, "custom chroma correlation is not carried");
  if (f.gab_custom) return fail(ctx, JPXLG_ERR_STREAM, "custom Gabor weights are not carried");
  static const jpxlg::cs::FrameInfo kDefaults;
  for (int i = 0; i < 8; ++i)
    if (f.epf_sharp_lut[i] != kDefaults.epf_sharp_lut[i])
      return fail(ctx, JPXLG_ERR_STREAM, "a custom EPF sharpness table is not carried");
  for (int c = 0; c < 3; ++c)
    if (f.epf_channel_scale[c] != kDefaults.epf_channel_scale[c])
      return fail(ctx, JPXLG_ERR_STREAM, "custom EPF channel scales are not carried");
  if (f.epf_quant_mul != kDefaults.epf_quant_mul ||
      f.epf_pass0_sigma_scale != kDefaults.epf_pass0_sigma_scale ||
      f.epf_pass2_sigma_scale != kDefaults.epf_pass2_sigma_scale ||
      f.epf_border_sad_mul != kDefaults.epf_border_sad_mul)
    return fail(ctx, JPXLG_ERR_STREAM, "custom EPF sigma parameters are not carried");
  if (!d.image.default_opsin || !d.image.xyb_encoded)
    return fail(ctx, JPXLG_ERR_STREAM, "only XYB frames with the default opsin matrix");
  if (out_kind == JPXLG_OUT_SRGB_FLOAT && d.image.transfer != 13)
    return fail(ctx, JPXLG_ERR_STREAM, "only the sRGB transfer function is carried");
  CK(cudaSetDevice(ctx->device));
  const int W = (int)f.width, H = (int)f.height;
  int rc = jpxlg_layout_create(ctx, W, H, v.block_map.data(), v.hf_mul.data(),
                               v.sharpness.data(), &st.L);
  if (rc) return rc;
  const Geo& g = st.L->geo;
  if ((uint32_t)g.tw != v.tiles_w || (uint32_t)g.th != v.tiles_h)
    return fail(ctx, JPXLG_ERR_ARGUMENT, "CfL tile grid mismatch");
  st.p.global_scale = v.global_scale;
  st.p.quant_lf = v.quant_lf;
  st.p.x_qm_scale = f.x_qm_scale;
  st.p.b_qm_scale = f.b_qm_scale;
  st.p.gaborish = f.gab ? 1u : 0u;
  st.p.epf_iters = f.epf_iters;
  st.p.precision = precision;
  if ((rc = check_params(ctx, &st.p))) return rc;
  st.n = (size_t)g.w * g.h;
  st.n8 = (size_t)g.W8 * g.H8;
  st.nb = (size_t)g.bw * g.bh;
  st.nt = (size_t)g.tw * g.th;
  if (v.lf_from_frame)
    for (int c = 0; c < 3; ++c)
      if (v.lf_frame[c].size() != st.nb) return fail(ctx, JPXLG_ERR_STREAM, "LF frame size");
  const size_t qb = 3 * st.n8 * sizeof(int32_t), lb = 3 * st.nb * sizeof(int32_t);
  const size_t fb = v.lf_from_frame ? 3 * st.nb * sizeof(float) : 0;
  const size_t bytes = qb + lb + fb + 2 * st.nt;
  st.pinned = pinned;
  if (pinned) CK(cudaMallocHost(&st.host, bytes));
  else if (!(st.host = std::malloc(bytes)))
    return fail(ctx, JPXLG_ERR_CUDA, "host staging of %zu bytes", bytes);
  char* h = (char*)st.host;
  st.q = (int32_t*)h;
  st.lfq = (int32_t*)(h + qb);
  st.lf_frame = fb ? (float*)(h + qb + lb) : nullptr;
  st.cflx = (int8_t*)(h + qb + lb + fb);
  st.cflb = st.cflx + st.nt;
  if ((rc = jpxlg_codestream_coefficients(cs, st.q))) return rc;
  for (int c = 0; c < 3; ++c) {
    std::copy(v.lf[c].begin(), v.lf[c].end(), st.lfq + c * st.nb);
    if (st.lf_frame) std::copy(v.lf_frame[c].begin(), v.lf_frame[c].end(), st.lf_frame + c * st.nb);
  }
  std::copy(v.x_from_y.begin(), v.x_from_y.begin() + st.nt, st.cflx);
  std::copy(v.b_from_y.begin(), v.b_from_y.begin() + st.nt, st.cflb);
  // LF multipliers (quantizer.rs:232): 65536 * (m_lf / 128) / (gs * quant_lf) in f64.
  const double denom = (double)v.global_scale * (double)v.quant_lf;
  for (int c = 0; c < 3; ++c) st.m[c] = (float)(65536.0 * (double)(v.m_lf[c] / 128.0f) / denom);
  st.kx = 0.0f + (float)v.x_factor_lf / 84.0f;
  st.kb = 1.0f + (float)v.b_factor_lf / 84.0f;
  st.div = (float)(1u << v.extra_precision);
  st.smooth = (f.flags & 128) == 0;
  st.fx = v.x_factor_lf + 128;
  st.fb = v.b_factor_lf + 128;
  return JPXLG_OK;
}

// Queues a staged frame's render on ctx's stream: the staged planes to the
// device, the LF image (dequantized, CfL'd and smoothed, or the LF frame's
// XYB as it stands), then the render into out_dev.  No allocation once the
// context's buffers have grown to the frame.
int decode_enqueue(jpxlg_ctx* ctx, const DecodeStage& st, int out_kind, void* out_dev) {
  const Geo& g = st.L->geo;
  CK(ctx->qcoeff.ensure(3 * st.n8 * sizeof(int32_t)));
  CK(ctx->lfq.ensure(3 * st.nb * sizeof(int32_t)));
  CK(ctx->cflx.ensure(st.nt));
  CK(ctx->cflb.ensure(st.nt));
  CK(ctx->lfs.ensure(3 * st.nb * sizeof(float)));
  CK(ctx->aux.ensure(3 * std::max(st.n, st.nb) * sizeof(float)));
  CK(cudaMemcpyAsync(ctx->qcoeff.p, st.q, 3 * st.n8 * sizeof(int32_t), cudaMemcpyHostToDevice,
                     ctx->stream));
  CK(cudaMemcpyAsync(ctx->lfq.p, st.lfq, 3 * st.nb * sizeof(int32_t), cudaMemcpyHostToDevice,
                     ctx->stream));
  CK(cudaMemcpyAsync(ctx->cflx.p, st.cflx, st.nt, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->cflb.p, st.cflb, st.nt, cudaMemcpyHostToDevice, ctx->stream));
  int rc;
  if (st.lf_frame) {
    CK(cudaMemcpyAsync(ctx->lfs.p, st.lf_frame, 3 * st.nb * sizeof(float),
                       cudaMemcpyHostToDevice, ctx->stream));
  } else {
    launch_lf_prepare(ctx->lfq.as<int32_t>(), g.bw, g.bh, st.m, st.div, st.kx, st.kb, st.smooth,
                      ctx->aux.as<float>(), ctx->lfs.as<float>(), ctx->num_sms, ctx->stream);
    if ((rc = after_launch(ctx, st.smooth ? 2 : 1))) return rc;
  }
  return render_device(ctx, st.L, ctx->qcoeff.as<int32_t>(), ctx->lfq.as<int32_t>(),
                       ctx->cflx.as<int8_t>(), ctx->cflb.as<int8_t>(), st.fx, st.fb, nullptr,
                       &st.p, out_kind, 8, out_dev, nullptr, ctx->lfs.as<float>());
}

size_t decode_out_bytes(const DecodeStage& st, int out_kind) {
  return out_kind == JPXLG_OUT_SRGB8 ? 3 * st.n : 3 * st.n * sizeof(float);
}

}  // namespace

extern "C" int jpxlg_codestream_render(jpxlg_ctx* ctx, const jpxlg_codestream* cs, int out_kind,
                                       void* out, uint32_t mem) {
  if (!ctx || !cs || !out) return fail(ctx, JPXLG_ERR_ARGUMENT, "null argument");
  DecodeStage st;
  int rc = decode_stage(ctx, cs, out_kind, false, st);
  if (rc) return rc;
  const size_t out_bytes = decode_out_bytes(st, out_kind);
  void* dst = out;
  if (mem != JPXLG_MEM_DEVICE) {
    CK(ctx->out.ensure(out_bytes));
    dst = ctx->out.p;
  }
  if ((rc = decode_enqueue(ctx, st, out_kind, dst))) return rc;
  if (mem != JPXLG_MEM_DEVICE)
    CK(cudaMemcpyAsync(out, ctx->out.p, out_bytes, cudaMemcpyDeviceToHost, ctx->stream));
  return sync_and_check(ctx);
}

// ---------------------------------------------------------------------------
// Batched decode: many parsed streams rendered by one graph launch.
// ---------------------------------------------------------------------------

struct jpxlg_decode_batch {
  jpxlg_ctx* owner = nullptr;
  int device = 0;
  int out_kind = 0;
  std::vector<jpxlg_ctx*> lanes;
  std::vector<std::unique_ptr<DecodeStage>> items;
  std::vector<size_t> out_bytes, out_off;
  uint8_t* d_out = nullptr;  // every item's pixels, back to back
  uint8_t* h_out = nullptr;  // pinned mirror, filled inside the graph
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> joins;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {

void decode_batch_free(jpxlg_decode_batch* b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->fork) cudaEventDestroy(b->fork);
  for (cudaEvent_t e : b->joins) cudaEventDestroy(e);
  b->items.clear();
  for (jpxlg_ctx* l : b->lanes) jpxlg_ctx_destroy(l);
  cudaFree(b->d_out);
  cudaFreeHost(b->h_out);
  delete b;
}

// Item i on lane i % lanes: its render, then its pixels to the pinned mirror.
int decode_batch_enqueue(jpxlg_ctx* ctx, jpxlg_decode_batch* b) {
  const size_t L = b->lanes.size();
  for (size_t i = 0; i < b->items.size(); ++i) {
    jpxlg_ctx* lane = b->lanes[i % L];
    int rc = decode_enqueue(lane, *b->items[i], b->out_kind, b->d_out + b->out_off[i]);
    if (rc) return fail(ctx, rc, "decode batch item %zu: %s", i, lane->last_error.c_str());
    CK(cudaMemcpyAsync(b->h_out + b->out_off[i], b->d_out + b->out_off[i], b->out_bytes[i],
                       cudaMemcpyDeviceToHost, lane->stream));
  }
  return JPXLG_OK;
}

int decode_batch_check(jpxlg_ctx* ctx, jpxlg_decode_batch* b) {
  for (jpxlg_ctx* lane : b->lanes) {
    int rc = sync_and_check(lane);
    if (rc) return fail(ctx, rc, "decode batch lane: %s", lane->last_error.c_str());
  }
  return JPXLG_OK;
}

}  // namespace

extern "C" int jpxlg_decode_batch_create(jpxlg_ctx* ctx, int n, const jpxlg_codestream* const* streams,
                                         int out_kind, uint32_t precision, int lanes,
                                         jpxlg_decode_batch** out) {
  if (!ctx || !streams || !out || n <= 0) return fail(ctx, JPXLG_ERR_ARGUMENT, "null argument");
  *out = nullptr;
  if (out_kind < 0 || out_kind > 4 || out_kind == JPXLG_OUT_LINEAR_DEPTH)
    return fail(ctx, JPXLG_ERR_ARGUMENT, "bad out_kind");
  for (int i = 0; i < n; ++i)
    if (!streams[i]) return fail(ctx, JPXLG_ERR_ARGUMENT, "stream %d: null", i);
  const bool auto_lanes = lanes <= 0;
  CK(cudaSetDevice(ctx->device));
  std::unique_ptr<jpxlg_decode_batch, void (*)(jpxlg_decode_batch*)> b(new jpxlg_decode_batch,
                                                                       decode_batch_free);
  b->owner = ctx;
  b->device = ctx->device;
  b->out_kind = out_kind;
  size_t total = 0;
  for (int i = 0; i < n; ++i) {
    b->items.emplace_back(new DecodeStage);
    int rc = decode_stage(ctx, streams[i], out_kind, true, *b->items.back(), precision);
    if (rc) return fail(ctx, rc, "decode batch stream %d: %s", i, ctx->last_error.c_str());
    const size_t bytes = decode_out_bytes(*b->items.back(), out_kind);
    total = (total + 255) & ~(size_t)255;
    b->out_off.push_back(total);
    b->out_bytes.push_back(bytes);
    total += bytes;
  }
  if (auto_lanes) {
    // Each lane is an internal context (its own streams, and a workspace
    // sized for the largest frame it renders, about 64 bytes per pixel).
    // Small frames are latency-bound chains of small launches, so more
    // lanes overlap more of them (256 small streams: 467 / 1003 / 1407
    // MPix/s at 4 / 16 / 32 lanes); the workspaces are held to 16 GiB.
    size_t max_px = 1;
    for (const auto& it : b->items) max_px = std::max(max_px, it->n);
    const size_t cap = ((size_t)16 << 30) / (64 * max_px);
    lanes = (int)std::max<size_t>(4, std::min<size_t>(32, cap));
  }
  lanes = std::min(lanes, n);
  for (int l = 0; l < lanes; ++l) {
    jpxlg_ctx* lane = nullptr;
    int rc = jpxlg_ctx_create(ctx->device, 0, &lane);
    if (rc) return fail(ctx, rc, "decode batch lane %d: context creation failed", l);
    b->lanes.push_back(lane);
    cudaEvent_t e = nullptr;
    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    b->joins.push_back(e);
  }
  CK(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
  CK(cudaMalloc(&b->d_out, total));
  CK(cudaMallocHost(&b->h_out, total));
  // Warm-up: the lanes' buffers grow to their largest frame here.
  int rc = decode_batch_enqueue(ctx, b.get());
  if (rc) return rc;
  if ((rc = decode_batch_check(ctx, b.get()))) return rc;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  cudaEventRecord(b->fork, ctx->stream);
  for (jpxlg_ctx* lane : b->lanes) cudaStreamWaitEvent(lane->stream, b->fork, 0);
  rc = decode_batch_enqueue(ctx, b.get());
  for (size_t l = 0; l < b->lanes.size(); ++l) {
    cudaEventRecord(b->joins[l], b->lanes[l]->stream);
    cudaStreamWaitEvent(ctx->stream, b->joins[l], 0);
  }
  cudaError_t ce = cudaStreamEndCapture(ctx->stream, &b->graph);
  if (rc) return rc;
  if (ce != cudaSuccess)
    return fail(ctx, JPXLG_ERR_CUDA, "decode batch capture: %s", cudaGetErrorString(ce));
  CK(cudaGraphInstantiate(&b->exec, b->graph, 0));
  *out = b.release();
  return JPXLG_OK;
}

extern "C" int jpxlg_decode_batch_run(jpxlg_ctx* ctx, jpxlg_decode_batch* b, void* const* outs,
                                      uint32_t mem) {
  if (!ctx || !b) return fail(ctx, JPXLG_ERR_ARGUMENT, "null argument");
  if (b->owner != ctx) return fail(ctx, JPXLG_ERR_ARGUMENT, "batch belongs to another context");
  CK(cudaSetDevice(ctx->device));
  CK(cudaGraphLaunch(b->exec, ctx->stream));
  if (mem == JPXLG_MEM_DEVICE) {
    if (outs)
      for (size_t i = 0; i < b->items.size(); ++i)
        if (outs[i])
          CK(cudaMemcpyAsync(outs[i], b->d_out + b->out_off[i], b->out_bytes[i],
                             cudaMemcpyDeviceToDevice, ctx->stream));
    return JPXLG_OK;
  }
  CK(cudaStreamSynchronize(ctx->stream));
  int rc = decode_batch_check(ctx, b);
  if (rc) return rc;
  if (outs)
    for (size_t i = 0; i < b->items.size(); ++i)
      if (outs[i]) std::memcpy(outs[i], b->h_out + b->out_off[i], b->out_bytes[i]);
  return JPXLG_OK;
}

extern "C" int jpxlg_decode_batch_destroy(jpxlg_decode_batch* b) {
  if (!b) return JPXLG_ERR_ARGUMENT;
  cudaSetDevice(b->device);
  cudaDeviceSynchronize();
  decode_batch_free(b);
  return JPXLG_OK;
}
