/*
 * jpxlg.h — C ABI of the GB300 (sm_103a) lossy VarDCT pixel path and
 * SSIMULACRA2 metric of JPXL.
 *
 * The library replaces, behind plain pointers and sizes, the data-parallel
 * stages that the reference (the JPXL Rust workspace) runs on CPU threads:
 *
 *   jpxlg_encode_transform  replaces jpxl-encode-policy's per-frame transform
 *                           and quantization: PreparedFrame::from_srgb8_with /
 *                           from_srgb16_with (crates/jpxl-encode-policy/src/
 *                           source.rs:226, :355), prepare_gaborish_frame
 *                           (lib.rs:2256 -> jpxl-encode vardct/gaborish.rs:218),
 *                           the forward cache (lib.rs:2683), estimate_cfl
 *                           (lib.rs:3437) and quantize_square_varblock
 *                           (lib.rs:3237), for a cover the caller supplies.
 *   jpxlg_select_blocks     replaces select_blocks (jpxl-encode-policy
 *                           lib.rs:5260), the hierarchical cover.
 *   jpxlg_reconstruct       replaces PlanRenderer::render / render_linear_at_
 *                           depth_with (crates/jpxl-plan-render/src/lib.rs:
 *                           680, :749) and the decoder's VarDCT tail
 *                           (crates/jpxl-decode/src/decode.rs:2955-3061,
 *                           vardct/render.rs:427, :563, :880).
 *   jpxlg_ssim2_ref_create  replaces PrecomputedReference::new
 *                           (crates/jpxl-perceptual/src/reference.rs:90).
 *   jpxlg_ssim2_score       replaces Ssimulacra2::score (ssimulacra2.rs:79).
 *   jpxlg_score_pair        replaces jpxl_perceptual::score_pair (lib.rs:195).
 *   jpxlg_probe             replaces one PlanRenderEvaluator::evaluate_with
 *                           (crates/jpxl-perceptual/src/evaluator.rs:243):
 *                           plan, render at depth, score against the source.
 *
 * Conventions.  Every function returns 0 on success and a negative
 * jpxlg_status on failure and never aborts; jpxlg_last_error() describes the
 * last failure of a context.  Buffers are owned by the caller.  With
 * JPXLG_MEM_HOST the pointers are host memory (pinned or pageable) and the
 * call returns after the results are in place; with JPXLG_MEM_DEVICE they
 * are device pointers on the context's device, work is queued on the
 * context's stream and device-side errors are reported by the next
 * jpxlg_ctx_synchronize().  A context serves one host thread at a time.
 * Layouts and references are read-only device data of their device: any
 * context on that device may use them, so several contexts (streams, host
 * threads) can probe the same frame concurrently.  Destroying a layout,
 * reference or batch waits for the device's queued work and does not need
 * the context that created it.
 *
 * Layouts.
 *   planes      float, row-major width x height, three planes back to back
 *               ([X,Y,B] or [R,G,B]).
 *   RGB input   interleaved 8-bit (bits == 8) or 16-bit (bits 9..16) samples.
 *   block map   one byte per 8x8 block of the ceil(w/8) x ceil(h/8) grid:
 *               bits 0..4 the Table I.1 DctSelect (0 DCT8, 4 DCT16,
 *               5 DCT32, 6 DCT16x8, 7 DCT8x16, 8 DCT32x8, 9 DCT8x32,
 *               10 DCT32x16, 11 DCT16x32), bit 7 set on the top-left block of
 *               each varblock.  A varblock may start at any block inside
 *               the frame; encoding needs naturally aligned DCT8/16/32.
 *   coeff image int32, three planes of (8*bh) x (8*bw): a varblock at block
 *               (bx,by) of R x C blocks stores its landscape coefficient
 *               matrix (min(R,C)*8 rows, max(R,C)*8 cols, row-major as the
 *               reference's CoeffMatrix) at row by*8.., column bx*8.. when
 *               R <= C, transposed when R > C.
 *   lf          int32, three planes of bw x bh quantized LF samples.
 *   cfl tiles   int8 per 64x64 tile, ceil(bw/8) x ceil(bh/8), X then B.
 */
#ifndef JPXLG_H
#define JPXLG_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  JPXLG_OK = 0,
  JPXLG_ERR_ARGUMENT = -1,     /* null pointer, bad size or parameter */
  JPXLG_ERR_BLOCK_MAP = -2,    /* block map does not tile the frame */
  JPXLG_ERR_QUANT = -3,        /* quantization out of range (PolicyError::Unsupported) */
  JPXLG_ERR_CUDA = -4,         /* CUDA runtime failure */
  JPXLG_ERR_NO_DEVICE = -5,    /* no usable sm_103 device */
  JPXLG_ERR_TOO_SMALL = -6,    /* SSIMULACRA2 needs 8x8 (MetricError::TooSmall) */
  JPXLG_ERR_MISMATCH = -7,     /* dimensions differ (MetricError::DimensionMismatch) */
  JPXLG_ERR_STREAM = -8        /* malformed or truncated entropy-coded stream (EntropyError) */
} jpxlg_status;

enum { JPXLG_MEM_HOST = 0, JPXLG_MEM_DEVICE = 1 };

/* Output kinds of jpxlg_reconstruct. */
enum {
  JPXLG_OUT_XYB = 0,          /* three float planes after restoration */
  JPXLG_OUT_LINEAR = 1,       /* three float linear-sRGB planes */
  JPXLG_OUT_SRGB8 = 2,        /* interleaved 8-bit sRGB, as the decoder writes it */
  JPXLG_OUT_LINEAR_DEPTH = 3, /* linear planes after a round trip through `bits` */
  JPXLG_OUT_SRGB_FLOAT = 4    /* three float planes through the sRGB curve, unclipped,
                                 as jpxl-decode's float output (decode.rs:3441) */
};

typedef struct jpxlg_ctx jpxlg_ctx;
typedef struct jpxlg_layout jpxlg_layout;
typedef struct jpxlg_ref jpxlg_ref;

/* The request fields of jpxl-encode-policy EncodeRequest (request.rs:855)
 * that the transform path reads. */
typedef struct {
  uint32_t global_scale;  /* I.2.1 global_scale */
  uint32_t quant_lf;      /* I.2.1 quant_lf */
  uint32_t x_qm_scale;    /* I.2.4 x_qm_scale (2 = neutral) */
  uint32_t b_qm_scale;    /* I.2.4 b_qm_scale (2 = neutral) */
  uint32_t gaborish;      /* RestorationDecision::gaborish */
  uint32_t epf_iters;     /* RestorationDecision::epf_iters, 0..3 */
  uint32_t cfl;           /* chroma-from-luma estimation on */
  uint32_t precision;     /* JPXLG_PRECISION_*: how the DCTs are evaluated (no
                           * reference field; 0 = the reference's arithmetic) */
} jpxlg_params;

/* Precision of the DCTs of the encode transform and the render (the other
 * stages are the same in every mode).
 *   FP32    the reference's butterflies in FP32 on the CUDA cores, bit-exact
 *           with jpxl-core dct.rs (quantized coefficients, pixels).
 *   BF16X3  batched dense contractions on the tcgen05 tensor cores, each f32
 *           operand split into two bf16 terms and the three leading products
 *           accumulated in FP32 (about 2^-16 relative error per product).
 *   BF16X6  the same with three bf16 terms and six products (FP32-level
 *           error).
 * The split forms cover the square DCT8/16/32 varblocks (every shape the
 * encoder produces); other shapes render through the FP32 kernels. Their
 * coefficients differ from the reference's in the last bits, so quantized
 * integers can differ where a coefficient sits at a decision boundary. */
enum {
  JPXLG_PRECISION_FP32 = 0,
  JPXLG_PRECISION_BF16X3 = 1,
  JPXLG_PRECISION_BF16X6 = 2
};

/* The quantized half of a plan (jpxl-encode vardct/plan.rs:434 LfQuantPlanes,
 * :519 VarblockCoefficients, :251 CflGrid, LfCorrelationDecision). */
typedef struct {
  int32_t* qcoeff;        /* 3 * (8*bh) * (8*bw) */
  int32_t* lf;            /* 3 * bw * bh */
  int8_t* cfl_x;          /* tw * th */
  int8_t* cfl_b;          /* tw * th */
  int32_t lf_factors[2];  /* x_factor_lf, b_factor_lf, biased by +128 */
} jpxlg_plan;

/* Context: owns device tables, workspace and a stream. device < 0 picks the
 * current device. flags: reserved, pass 0. */
int jpxlg_ctx_create(int device, uint32_t flags, jpxlg_ctx** out);
int jpxlg_ctx_destroy(jpxlg_ctx* ctx);
/* Queue work on an external cudaStream_t (NULL restores the context's own). */
int jpxlg_ctx_set_stream(jpxlg_ctx* ctx, void* cuda_stream);
void* jpxlg_ctx_stream(jpxlg_ctx* ctx);
/* Waits for queued work; returns the first device-side error since the last
 * synchronize (quantization range, block map) or a CUDA error. */
int jpxlg_ctx_synchronize(jpxlg_ctx* ctx);
const char* jpxlg_last_error(const jpxlg_ctx* ctx);
/* Kernel launches the context issued since creation (for accounting). */
uint64_t jpxlg_ctx_launches(const jpxlg_ctx* ctx);
/* CfL decisions (per tile, or the frame's LF pair) that the tree-ordered f64
 * sums could not settle and that were recomputed in the reference's
 * sequential order, since creation (synchronizes). */
uint32_t jpxlg_ctx_cfl_fallbacks(jpxlg_ctx* ctx);

/* Stage timers (the GPU counterpart of plan-render lib.rs:472 RenderTimings
 * and the policy's stage diagnostics): when enabled, CUDA events recorded on
 * the context's stream at stage boundaries accumulate device time per
 * stage.  jpxlg_stage_times() synchronizes, writes up to `n` entries of
 * milliseconds and launch counts in JPXLG_STAGE_* order, returns the number
 * of stages, and resets the accumulators. */
enum {
  JPXLG_STAGE_XYB = 0,          /* K1 RGB -> XYB */
  JPXLG_STAGE_PRECONDITION,     /* K2 inverse Gaborish, 12 steps */
  JPXLG_STAGE_FDCT_LUMA,        /* K3 forward DCT, LF, luma quantization */
  JPXLG_STAGE_CFL,              /* K4 CfL estimation */
  JPXLG_STAGE_QUANT_CHROMA,     /* K5 chroma quantization */
  JPXLG_STAGE_RENDER_VARBLOCKS, /* R1 dequant, CfL, LLF, IDCT */
  JPXLG_STAGE_GABORISH,         /* R2 */
  JPXLG_STAGE_EPF,              /* R3, all steps */
  JPXLG_STAGE_COLOUR,           /* R4 */
  JPXLG_STAGE_SSIM,             /* S1-S5 candidate side, but for the three below */
  JPXLG_STAGE_SSIM_ROWS,        /* S3 blur row pass (every scale) */
  JPXLG_STAGE_SSIM_COL_RIPPLE,  /* S3 the reset of the column scan's flags (the ripple's
                                   segment scan runs inside the column pass) */
  JPXLG_STAGE_SSIM_COL_OUT,     /* S3/S4 blur column pass with the per-pixel terms */
  JPXLG_STAGE_COUNT
};
int jpxlg_stage_timing(jpxlg_ctx* ctx, int enable);
int jpxlg_stage_times(jpxlg_ctx* ctx, double* ms, uint64_t* launches, int n);

/* Frame structure of a plan (jpxl-encode vardct/plan.rs:239 varblocks with
 * hf_mul, :318 SharpnessGrid): validated once, reused by every call on
 * frames of this shape.  hf_mul and sharpness are per 8x8 block (hf_mul read
 * at varblock origins); sharpness may be NULL (all zero). Host memory. */
int jpxlg_layout_create(jpxlg_ctx* ctx, int width, int height, const uint8_t* block_map,
                        const uint32_t* hf_mul, const uint8_t* sharpness, jpxlg_layout** out);
int jpxlg_layout_destroy(jpxlg_layout* layout);
int jpxlg_layout_dims(const jpxlg_layout* layout, int* bw, int* bh, int* tw, int* th);

/* RGB -> quantized plan.  `rgb`, `plan->*` follow `mem`. */
int jpxlg_encode_transform(jpxlg_ctx* ctx, const jpxlg_layout* layout, const void* rgb,
                           int bits, const jpxlg_params* params, jpxlg_plan* plan,
                           uint32_t mem);

/* Diagnostic: the intermediate planes of jpxlg_encode_transform for one
 * frame, in host memory (any may be NULL): the XYB planes
 * (PreparedFrame::xyb, 3*w*h floats), the Gaborish-preconditioned planes
 * (3*w*h) and the forward coefficient image before quantization (3 planes
 * of (8*bh) x (8*bw) floats). */
int jpxlg_encode_stages(jpxlg_ctx* ctx, const jpxlg_layout* layout, const void* rgb, int bits,
                        const jpxlg_params* params, float* xyb, float* pre, float* coeff);

/* Launch tunables (no reference counterpart), process-wide, for the
 * autotuner (jpxl_gb300/tune.py):
 *   JPXLG_TUNE_TC_CTAS_PER_SM  persistent CTAs per SM of the split-precision
 *                              tensor-core kernels, 1..4 (default 4: four
 *                              128-column TMEM allocations fill an SM).
 * jpxlg_tune_set returns the previous value (JPXLG_ERR_ARGUMENT for an
 * unknown knob or a value out of range); launches queued afterwards use the
 * new value (a batch captures it when it is created). */
enum { JPXLG_TUNE_TC_CTAS_PER_SM = 0 };
int jpxlg_tune_set(int knob, int value);
int jpxlg_tune_get(int knob);

/* Diagnostic: the decoder's 8x8 special transforms (jpxl-core varblock.rs:
 * 1218 samples_from_coefficients for DCT2x2, Hornuss, DCT4x4, DCT8x4,
 * DCT4x8 and AFV0-3, I.9.3-I.9.8) on n dequantized coefficient blocks
 * (64 floats each, row-major, the LLF at 0) into n blocks of 64 samples, the
 * kernels jpxlg_codestream_render runs for those transforms.  kind: 1 DCT2x2,
 * 2 Hornuss, 3 DCT4x4, 4 DCT8x4, 5 DCT4x8, 6..9 AFV0..AFV3. */
int jpxlg_diag_special_blocks(jpxlg_ctx* ctx, int kind, const float* coef, int n, float* out,
                              uint32_t mem);

/* Quantized plan -> pixels.  `out` sizes: JPXLG_OUT_SRGB8 w*h*3 bytes, other
 * kinds 3*w*h floats.  `bits` is the depth of JPXLG_OUT_LINEAR_DEPTH. */
int jpxlg_reconstruct(jpxlg_ctx* ctx, const jpxlg_layout* layout, const jpxlg_plan* plan,
                      const jpxlg_params* params, int out_kind, int bits, void* out,
                      uint32_t mem);

/* SSIMULACRA2 reference moments of a linear-sRGB image (planes follow mem).
 * Frames are limited to 8192 columns (the row pass stages a row pair in
 * shared memory); wider ones return JPXLG_ERR_ARGUMENT. */
int jpxlg_ssim2_ref_create(jpxlg_ctx* ctx, const float* linear_rgb, int width, int height,
                           uint32_t mem, jpxlg_ref** out);
int jpxlg_ssim2_ref_destroy(jpxlg_ref* ref);
/* Score a candidate against a reference.  score, raw_error (one double each)
 * and terms (scales x 3 channels x 6 norms, at most 108) are optional; they
 * follow mem like the planes (device pointers with JPXLG_MEM_DEVICE). */
int jpxlg_ssim2_score(jpxlg_ctx* ctx, const jpxlg_ref* ref, const float* linear_rgb,
                      uint32_t mem, double* score, double* raw_error, double* terms);
/* One-shot pair score.  The reference side is built in a device buffer the
 * context keeps for the next call (its pyramid: about 64 bytes per source
 * pixel), freed with the context. */
int jpxlg_score_pair(jpxlg_ctx* ctx, const float* ref_rgb, const float* cand_rgb, int width,
                     int height, uint32_t mem, double* score);

/* One quality-controller probe: encode `rgb` with `params`, render the plan
 * at the source depth `bits` and score it against `ref` (built from the same
 * source).  With JPXLG_MEM_DEVICE, `rgb` is device memory, exactly one double
 * is written at the device pointer `score`, and the call does not
 * synchronize. */
int jpxlg_probe(jpxlg_ctx* ctx, const jpxlg_layout* layout, const jpxlg_ref* ref,
                const void* rgb, int bits, const jpxlg_params* params, uint32_t mem,
                double* score);

/* The encoder's cover: replaces jpxl-encode-policy's select_blocks
 * (crates/jpxl-encode-policy/src/lib.rs:5260, with tile_region_with :5115 and
 * block_cost_bounded :4909) for a fixed quantizer with adaptive quantization
 * off: per aligned 32x32 region, DCT32 or four DCT16 / DCT8 quadrants by the
 * rate-distortion objective (residual bits + lambda * sample-domain squared
 * error, fixed bits 2 / 34), ties keeping the split.  Fills `block_map`
 * (ceil(w/8) x ceil(h/8) bytes in the layout format above; host or device
 * per `mem`, like `rgb`).  params: global_scale, x/b_qm_scale and gaborish
 * are read. */
int jpxlg_select_blocks(jpxlg_ctx* ctx, int width, int height, const void* rgb, int bits,
                        const jpxlg_params* params, uint8_t* block_map, uint32_t mem);
/* Regions whose decisions the GPU's tree-ordered error sums could not settle
 * and that were recomputed in the reference's sequential order, since
 * creation (synchronizes). */
uint32_t jpxlg_ctx_cover_fallbacks(jpxlg_ctx* ctx);

/* Batched probes (the quality controller's candidate sweep: many frames, many
 * quantizers per frame).  Replaces a loop of PlanRenderEvaluator::evaluate
 * calls (evaluator.rs:295) inside search_frame_perceptual (quality.rs:2405)
 * with one graph launch.  An item is one probe of a frame: its layout and
 * reference (created on this context's device), the frame's RGB in device
 * memory (interleaved, `bits` per sample) and the candidate's parameters.
 *
 * jpxlg_batch_create spreads the items over `lanes` internal contexts (each
 * with its own stream and workspace; 0 picks min(items, 4)), runs every
 * probe once to size the workspaces, and captures the whole batch — fork,
 * the lanes' probes, join — as one CUDA graph on `ctx`'s stream.  The items
 * and the RGB buffers they point to must stay valid while the batch lives;
 * the buffers' contents may change between runs.
 * jpxlg_batch_run launches the graph on ctx's stream.  With JPXLG_MEM_HOST,
 * `scores` (n doubles) is filled and the call returns when the batch is done;
 * with JPXLG_MEM_DEVICE, `scores` is a device array written on the stream.
 * jpxlg_batch_probe is create + run + destroy in one call (host scores). */
typedef struct jpxlg_batch jpxlg_batch;
typedef struct {
  const jpxlg_layout* layout;
  const jpxlg_ref* ref;
  const void* rgb;   /* device memory */
  int bits;
  jpxlg_params params;
} jpxlg_batch_item;
int jpxlg_batch_create(jpxlg_ctx* ctx, int n_items, const jpxlg_batch_item* items, int lanes,
                       jpxlg_batch** out);
int jpxlg_batch_run(jpxlg_ctx* ctx, jpxlg_batch* batch, double* scores, uint32_t mem);
int jpxlg_batch_destroy(jpxlg_batch* batch);
int jpxlg_batch_probe(jpxlg_ctx* ctx, int n_items, const jpxlg_batch_item* items,
                      double* scores);

/* Host-side entropy decoding (ISO/IEC 18181-1 Annex C), replacing
 * jpxl-entropy's SymbolDecoder (crates/jpxl-entropy/src/decoder.rs):
 *   jpxlg_symbols_open     SymbolDecoder::open: reads the distribution bundle
 *                          (LZ77 parameters, context map, hybrid-uint
 *                          configurations, prefix codes or ANS
 *                          distributions) starting at bit `bit_offset` of
 *                          data[0..size) (LSB-first, the codestream's bit
 *                          order) and seeds the ANS state; num_dist is the
 *                          number of contexts the referencing clause supplies
 *   jpxlg_symbols_read     SymbolDecoder::read_uint for context `ctx`
 *   jpxlg_symbols_read_many  read_uint for a sequence of contexts
 *   jpxlg_symbols_set_dist_multiplier  set_dist_multiplier (LZ77 row stride)
 *   jpxlg_symbols_finish   SymbolDecoder::finish: JPXLG_OK when an ANS stream
 *                          ends in its final state (C.3.2)
 *   jpxlg_symbols_bits_read  the reader position, in bits from data[0]
 * The stream is copied at open.  Malformed or truncated streams return
 * JPXLG_ERR_STREAM.  Host code only: no device is needed. */
typedef struct jpxlg_symbols jpxlg_symbols;
int jpxlg_symbols_open(const uint8_t* data, size_t size, size_t bit_offset, uint32_t num_dist,
                       jpxlg_symbols** out);
int jpxlg_symbols_read(jpxlg_symbols* s, uint32_t ctx, uint32_t* value);
int jpxlg_symbols_read_many(jpxlg_symbols* s, const uint32_t* ctx, size_t n, uint32_t* values);
int jpxlg_symbols_set_dist_multiplier(jpxlg_symbols* s, uint32_t multiplier);
int jpxlg_symbols_finish(const jpxlg_symbols* s);
size_t jpxlg_symbols_bits_read(const jpxlg_symbols* s);
int jpxlg_symbols_destroy(jpxlg_symbols* s);

/* Host-side codestream reader for the lossy VarDCT path, replacing the front
 * end of jpxl-decode's decode (crates/jpxl-decode/src/decode.rs:400 decode,
 * :2513 decode_vardct_frame, vardct/hf_coeff.rs:689 decode_hf_group): the
 * image headers, frame header and TOC, modular sub-bitstreams (MA trees,
 * H.3/H.5 predictors) and the VarDCT sections, decoded to the frame's integer
 * content.  Bare codestreams or ISO/IEC 18181-2 containers (jxlc, or jxlp
 * fragments) with one regular frame, optionally after a modular LF frame
 * (kUseLfFrame); modular transforms RCT, squeeze and palette; modular
 * frames of several groups (one pass) with extra channels; a VarDCT frame's
 * extra channels, except those with a dim_shift and, in a frame of several
 * passes, those larger than a group (both return JPXLG_ERR_STREAM).  ICC profiles, previews, patches, splines, noise and
 * upsampling are reported as unsupported (JPXLG_ERR_STREAM with a reason in
 * jpxlg_codestream_last_error).  Host code only: no device is needed.
 * Streams may be opened from several host threads at once: the allocation
 * meter and the last error are per thread, and handles share no state.
 *   jpxlg_codestream_open          parse and decode; *out owns the result
 *   jpxlg_codestream_info          sizes, frame parameters, per-DctSelect
 *                                  varblock counts, and how many sections
 *                                  ended in their TOC entry's last byte
 *   jpxlg_codestream_blocks        quantized LF (3 planes X, Y, B of
 *                                  blocks_w x blocks_h), the block map
 *                                  (DctSelect | 0x80 at varblock origins), HF
 *                                  multipliers, EPF sharpness, and the CfL
 *                                  factors of each 64x64 tile; NULL skips one
 *   jpxlg_codestream_coefficients  quantized HF coefficients as the plan's
 *                                  coefficient image, 3 x (8*blocks_h) x
 *                                  (8*blocks_w)
 *   jpxlg_codestream_channel       a modular frame's channel, width x height
 *                                  (its colour channels, then its extra
 *                                  channels) */
typedef struct jpxlg_codestream jpxlg_codestream;
typedef struct {
  uint32_t width, height, bits_per_sample, xyb_encoded, colour_space;
  int32_t transfer;
  uint32_t encoding, num_passes, gaborish, gaborish_custom, epf_iters, x_qm_scale, b_qm_scale;
  uint32_t adaptive_lf_smoothing, global_scale, quant_lf, extra_precision, default_matrices;
  uint32_t default_lf_dequant, default_chroma_correlation;
  int32_t x_factor_lf, b_factor_lf;
  uint32_t blocks_w, blocks_h, num_varblocks, num_channels, sections, sections_exact;
  uint32_t transform_counts[27];
  uint32_t orientation, num_extra; /* Exif orientation 1-8 (not applied); extra channels */
} jpxlg_codestream_info_t;
int jpxlg_codestream_open(const uint8_t* data, size_t size, jpxlg_codestream** out);
/* jpxl-core limits.rs Limits: the largest image (width x height) and the
 * cumulative bytes of channels and planes one stream may make the reader
 * allocate; each allocation is charged before it is made, and a stream past
 * either limit returns JPXLG_ERR_STREAM.  jpxlg_codestream_open uses the
 * reference's defaults (Limits::new, limits.rs:38): 2^30 pixels, 4 GiB. */
typedef struct {
  uint64_t max_pixels;
  uint64_t max_alloc_bytes;
} jpxlg_codestream_limits;
int jpxlg_codestream_open_limits(const uint8_t* data, size_t size,
                                 const jpxlg_codestream_limits* limits, jpxlg_codestream** out);
const char* jpxlg_codestream_last_error(void);
int jpxlg_codestream_info(const jpxlg_codestream* cs, jpxlg_codestream_info_t* info);
int jpxlg_codestream_blocks(const jpxlg_codestream* cs, int32_t* lf, uint8_t* block_map,
                            uint32_t* hf_mul, uint8_t* sharpness, int8_t* x_from_y,
                            int8_t* b_from_y);
int jpxlg_codestream_coefficients(const jpxlg_codestream* cs, int32_t* out);
int jpxlg_codestream_channel(const jpxlg_codestream* cs, uint32_t index, int32_t* out);
/* A VarDCT frame's extra channel (alpha, ...) as sample / (2^bits - 1),
 * width x height (channels no larger than a 256x256 group). */
int jpxlg_codestream_extra(const jpxlg_codestream* cs, uint32_t index, float* out);
int jpxlg_codestream_destroy(jpxlg_codestream* cs);
/* Reconstruction of a decoded VarDCT frame on the GPU (jpxl-decode
 * decode.rs:2700-3061): LF dequantization with the LF CfL and, unless the
 * frame skips it, adaptive LF smoothing (vardct/lf.rs:351), then the
 * varblock render (DCT8..DCT32 and their rectangles, DCT2x2, DCT64x64,
 * DCT64x32, DCT32x64), Gaborish, EPF and the colour transform, into three
 * float planes (JPXLG_OUT_XYB, _LINEAR, _SRGB_FLOAT) or interleaved sRGB8.
 * A grey image's value is the first plane.  Frames that need parameters the
 * kernels do not carry (custom dequantization matrices, chroma correlation,
 * Gabor weights or EPF parameters, a custom opsin matrix, other transforms)
 * return JPXLG_ERR_STREAM. */
int jpxlg_codestream_render(jpxlg_ctx* ctx, const jpxlg_codestream* cs, int out_kind, void* out,
                            uint32_t mem);

/* Batched decode: replaces a loop of jpxl-decode decode() calls
 * (crates/jpxl-decode/src/decode.rs:400, through decode_vardct_frame :2513
 * and quantize_sample :3498 for 8-bit output) over many streams with one
 * graph launch.  jpxlg_decode_batch_create stages every opened stream
 * (the host's entropy decoding is done at open; here the coefficient image,
 * LF planes and CfL tiles go into pinned host memory), spreads the streams
 * over `lanes` internal contexts (0 picks up to 32, fewer when the frames
 * are large: each lane keeps a workspace of about 64 bytes per pixel of its
 * largest frame, held to 16 GiB in all), renders each once to
 * size the workspaces, and captures one CUDA graph on ctx's stream: per
 * stream, the staged planes to the device, LF preparation, the render into
 * `out_kind` (as jpxlg_codestream_render) and the pixels back to a pinned
 * host buffer.  `precision` (JPXLG_PRECISION_*) picks how the square
 * DCT8/16/32 varblocks' IDCTs run; every other transform renders through
 * the FP32 kernels.  The streams must stay open while the batch lives.
 * jpxlg_decode_batch_run launches the graph; with JPXLG_MEM_HOST it waits
 * and copies stream i's pixels to outs[i] (host; NULL entries, or outs
 * NULL, skip the copy); with JPXLG_MEM_DEVICE it queues device-to-device
 * copies to outs[i] and returns without waiting.  Streams the renderer does
 * not carry fail creation with JPXLG_ERR_STREAM, naming the stream. */
typedef struct jpxlg_decode_batch jpxlg_decode_batch;
int jpxlg_decode_batch_create(jpxlg_ctx* ctx, int n, const jpxlg_codestream* const* streams,
                              int out_kind, uint32_t precision, int lanes,
                              jpxlg_decode_batch** out);
int jpxlg_decode_batch_run(jpxlg_ctx* ctx, jpxlg_decode_batch* batch, void* const* outs,
                           uint32_t mem);
int jpxlg_decode_batch_destroy(jpxlg_decode_batch* batch);

/* Allocation-free variant of jpxlg_ssim2_score; it has no counterpart in the
 * reference.  The candidate (device planes) is scored against `ref` using a
 * fixed device scratch inside the library instead of the context's
 * workspace, so the call never allocates or frees device memory: for callers
 * that score between launches of their own and cannot take cudaFree's
 * device-wide synchronisation, or that run beside a caching allocator which
 * already holds the free device memory.  `out_dev` (device, 2 + 18 * scales
 * doubles, at most 110) receives the score, the raw error and the terms.
 * Work is queued on the context's stream and the call does not synchronize.
 * Limits: reference frames up to 2048 x 2048 (larger ones return
 * JPXLG_ERR_ARGUMENT); the first call on a device resolves the scratch
 * address and should come before any stream capture; there is one scratch
 * per device, so calls in flight at the same time on one device race.  The
 * scratch is a 137 MB __device__ array, resident on every device where the
 * library's module loads, whether or not this entry point is called. */
int jpxlg_ssim2_score_static(jpxlg_ctx* ctx, const jpxlg_ref* ref,
                             const float* linear_rgb_dev, double* out_dev);

#ifdef __cplusplus
}
#endif
#endif
