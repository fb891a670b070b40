/*
 * oracle.h — C-ABI of the CPU restatement of JPXL's lossy VarDCT pixel path
 * and of its in-tree SSIMULACRA2.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA path
 * is compared against; it is never linked into, loaded by or called from the
 * product library (jpxl_gb300/csrc).  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg load it.
 *
 * Every function restates the reference's arithmetic in the reference's
 * operation order (no FMA contraction: the file is built with
 * -ffp-contract=off; std::fma exactly where the reference calls mul_add).
 * Each definition in oracle*.cpp cites the reference file:line it follows,
 * relative to the reference project's JPXL/ directory.
 *
 * Layouts (shared with the product library):
 *   planes     : float, row-major, width x height, channel order X,Y,B
 *                (or R,G,B for linear/sRGB planes).
 *   block map  : one byte per 8x8 block of the ceil(w/8) x ceil(h/8) grid:
 *                bits 0..4 = DctSelect (Table I.1 value), bit 7 = the block
 *                is the top-left origin of its varblock.
 *   coeff image: int32 (or float) per channel, (8*bh) rows x (8*bw) cols; a
 *                varblock at block (bx,by) with R x C blocks stores its
 *                landscape coefficient matrix (min(R,C)*8 rows by
 *                max(R,C)*8 cols) at rows by*8.., cols bx*8.. when R <= C and
 *                transposed (coefficient (y,x) at row by*8+x, col bx*8+y)
 *                when R > C.
 *   lf planes  : int32 per channel, bw x bh (one LF sample per 8x8 block).
 *   cfl tiles  : int8 per 64x64 tile, ceil(bw/8) x ceil(bh/8).
 */
#ifndef JPXL_ORACLE_H
#define JPXL_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Encoder request (policy request.rs:855 defaults, with the fields the
 * fixed-quantizer configs set). */
typedef struct {
  uint32_t global_scale;   /* request.rs:857, 32768 default */
  uint32_t quant_lf;       /* request.rs:858, 16 default */
  uint32_t x_qm_scale;     /* 2 = neutral */
  uint32_t b_qm_scale;     /* 2 = neutral */
  uint32_t gaborish;       /* restoration.gaborish: precondition on encode */
  uint32_t cfl;            /* chroma-from-luma estimation on */
} orc_encode_params;

/* Frame-wide CfL bundle produced by the encoder (plan LfCorrelationDecision). */
typedef struct {
  int32_t x_factor_lf;     /* stored biased by +128, i.e. 0..255 */
  int32_t b_factor_lf;
} orc_lf_cfl;

typedef struct {
  uint32_t global_scale;
  uint32_t quant_lf;
  uint32_t x_qm_scale;
  uint32_t b_qm_scale;
  uint32_t gaborish;
  uint32_t epf_iters;      /* 0..3 */
  int32_t x_factor_lf;     /* biased, 0..255 */
  int32_t b_factor_lf;
} orc_render_params;

/* ---- scalar building blocks (exported for known-answer tests) ---- */
float orc_cbrt_core(float v);        /* jpxl-core simd.rs:36 */
float orc_cbrt_perceptual(float v);  /* jpxl-perceptual color.rs:46 */
float orc_srgb_to_linear(float v);   /* jpxl-core color.rs:517 */
float orc_linear_to_srgb(float v);   /* jpxl-core color.rs:490 */
void orc_linear_to_xyb(const float* rgb3, float* xyb3);
void orc_opsin_inverse(const float* xyb3, float* rgb3);
float orc_hf_multiplier(uint32_t gs, uint32_t hf_mul);
float orc_bias_adjust(int32_t q, float bias, float num);
float orc_scale_f(int c, int lf_count);
/* dequant (multiplier) matrix of a transform/channel, rows*cols floats. */
int orc_dequant_matrix(int dct_select, int channel, float* out, int* rows, int* cols);
/* orthonormal DCT-II / DCT-III butterflies (dct.rs:431-463), no 1/sqrt(n) */
void orc_dct_ii_ortho(float* v, int n);
void orc_dct_iii_ortho(float* v, int n);
/* 1-D normative DCT / IDCT (dct.rs:731/749) of length n in place. */
void orc_dct_1d(float* v, int n);
void orc_idct_1d(float* v, int n);
/* DCT_2D / IDCT_2D of I.7.3 (dct.rs:956/982) in place. */
void orc_dct_2d(float* work, int rows, int cols);
void orc_idct_2d(float* work, int rows, int cols);

/* ---- plane stages ---- */
void orc_srgb8_to_xyb(const uint8_t* rgb, int w, int h, float* x, float* y, float* b);
void orc_srgb16_to_xyb(const uint16_t* rgb, int w, int h, int bits, float* x, float* y,
                       float* b);
/* encoder inverse Gaborish, 12 Jacobi iterations (encode gaborish.rs:218) */
void orc_gab_precondition(const float* in, int w, int h, float* out);
/* decoder J.3 with the Table J.1 default kernel (restoration.rs:148) */
void orc_gaborish(const float* in, int w, int h, float* out);
/* J.3 with explicit weight1/weight2 (restoration.rs:111 GaborKernel::new) */
void orc_gaborish_w(const float* in, int w, int h, float w1, float w2, float* out);
/* one J.4 step (0,1,2) over three planes with a per-block sigma field */
void orc_epf_step(int step, const float* const* in, int w, int h, const float* sigma,
                  float* const* out);
/* the depth classifier's thresholds: levels-1 floats (plan-render lib.rs:333) */
void orc_depth_thresholds(int bits, float* out);

/* ---- the pipelines ----
 * Returns 0 on success, a negative error code where the reference returns an
 * Err (degenerate quantizer, out-of-range coefficient, bad shapes).
 * Optional outputs may be NULL. */
int orc_encode(const void* rgb, int w, int h, int bits, const uint8_t* block_map,
               const uint32_t* hf_mul_blocks, const orc_encode_params* p,
               float* xyb_out /* 3*w*h or NULL */, float* pre_out /* 3*w*h or NULL */,
               float* coeff_out /* 3*H8*W8 or NULL */, int32_t* qcoeff_out,
               int32_t* lf_out, int8_t* cfl_x, int8_t* cfl_b, orc_lf_cfl* lf_cfl);

/* The encoder's cover (policy lib.rs:5260 select_blocks) for a fixed
 * quantizer with adaptive quantization off: fills the block map (one byte
 * per 8x8 block, DctSelect | 0x80 on varblock origins). candidates_scored
 * (optional) receives the number of candidate costs evaluated. */
int orc_select_blocks(const void* rgb, int w, int h, int bits, const orc_encode_params* p,
                      uint8_t* block_map, int64_t* candidates_scored);

/* out_kind: 0 = XYB after restoration (3 planes), 1 = linear sRGB planes,
 * 2 = 8-bit sRGB interleaved (u8, w*h*3), 3 = linear at depth `bits`
 * (3 planes), 4 = XYB before restoration (3 planes). */
int orc_reconstruct(int w, int h, const uint8_t* block_map, const uint32_t* hf_mul_blocks,
                    const uint8_t* sharpness, const int32_t* qcoeff, const int32_t* lf,
                    const int8_t* cfl_x, const int8_t* cfl_b, const orc_render_params* p,
                    int out_kind, int bits, void* out);

/* SSIMULACRA2 of two linear-sRGB images (perceptual lib.rs:195 score_pair).
 * terms (optional): 6 scales x 3 channels x 6 norms (ssim0,art0,lost0,ssim1,
 * art1,lost1 in the order weighted_error consumes them). Returns the number of
 * scales, negative on error. */
int orc_ssim2(const float* const* ref, const float* const* cand, int w, int h,
              double* score, double* raw_error, double* terms);

/* ssimulacra2.rs:391 WEIGHTS[i]; the f64 recursive blur of one plane. */
double orc_ssim2_weight(int i);
void orc_blur_plane(const float* in, int w, int h, float* out);
/* The decoder's 8x8 special transforms (varblock.rs:898-1230): a dequantized
 * coefficient block (row-major, LLF at 0) to its 8x8 samples.  kind: 1 DCT2x2,
 * 2 Hornuss, 3 DCT4x4, 4 DCT8x4, 5 DCT4x8, 6..9 AFV0..AFV3; afv_basis is
 * Table I.11 (16 x 16 f64), needed for AFV.  Returns 0, or -1 for a bad kind. */
int orc_special_block(int kind, const float* coef, const double* afv_basis, float* out);
/* entry (u, n) of the orthonormal DCT-IV leaf of size M (dct.rs:148-211) */
float orc_dct_iv_entry(int M, int u, int n);

/* seeded synthetic image of the reference's perceptual tests
 * (tests/common/mod.rs:66 synthetic, :112 add_noise), linear planes. */
void orc_perceptual_synthetic(int w, int h, uint32_t seed, float* r, float* g, float* b);
void orc_perceptual_add_noise(float* r, float* g, float* b, int n, float amp, uint32_t seed);

/* ---- FP64 truth (oracle_fp64.cpp) ----
 * The same algorithm with every operation in f64 and the transforms as exact
 * cosine sums; tables and constants at the values the f32 path holds. */
void orc64_dct_2d(const double* in, int rows, int cols, double* out);
void orc64_idct_2d(const double* coef, int rows, int cols, double* out);
int orc64_encode_transform(const void* rgb, int w, int h, int bits, const uint8_t* block_map,
                           int gaborish, double* xyb_out, double* pre_out, double* coeff_out);
/* out_kind: 0 = XYB after restoration, 1 = linear sRGB, 4 = XYB before
 * restoration; out holds 3*w*h doubles. */
int orc64_reconstruct(int w, int h, const uint8_t* block_map, const uint32_t* hf_mul_blocks,
                      const uint8_t* sharpness, const int32_t* qcoeff, const int32_t* lf,
                      const int8_t* cfl_x, const int8_t* cfl_b, const orc_render_params* p,
                      int out_kind, double* out);
/* Inputs as f32 planes (ref/cand) or f64 planes (ref64/cand64, used when
 * non-NULL). Returns the number of scales. */
int orc64_ssim2(const float* const* ref, const float* const* cand, const double* const* ref64,
                const double* const* cand64, int w, int h, double* score, double* terms);

#ifdef __cplusplus
}
#endif
#endif
