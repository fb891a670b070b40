// jpxlg_kernels.h — argument blocks and launchers of the sm_103a kernels.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "jpxlg_internal.h"

namespace jpxlg {

struct DF;  // double-float partial sums (jpxlg_common.cuh)

// Everything the encoder kernels read and write (device pointers).
struct EncArgs {
  Geo geo;
  QuantScalars qs;
  const float* pre;          // 3 planes w*h: XYB after the optional precondition
  const float* dq;           // [3][kDequantTableFloats] dequant multipliers
  const float* mul_table;    // [kMulTableN] hf multipliers of this call's global_scale
  const uint32_t* hf_mul;    // per 8x8 block (read at varblock origins)
  const uint8_t* block_map;  // per 8x8 block
  float* coeff;              // [3][W8*H8] forward coefficients (f32)
  float* dyhf;               // [W8*H8] reconstructed luma HF
  int32_t* qcoeff;           // [3][W8*H8] quantized coefficients
  float* lfs;                // [3][bw*bh] LF samples
  float* dylf;               // [bw*bh] reconstructed luma LF
  int32_t* lfq;              // [3][bw*bh] quantized LF
  int8_t* cfl_x;             // [tw*th]
  int8_t* cfl_b;             // [tw*th]
  int* lf_factors;           // [2] frame LF factors, unbiased
  const uint32_t* not_gray;  // set by the colour kernel when any pixel is not grey
  uint32_t cfl_enabled;
  float base_mul;            // hf multiplier of the frame's baseline hf_mul
  uint32_t* err;
  uint32_t* cfl_fallbacks;   // count of sequential-order fallbacks taken
};

// Everything the render kernels read and write.
struct RenderArgs {
  Geo geo;
  QuantScalars qs;
  const float* dq;
  const float* mul_table;    // [kMulTableN] hf multipliers of this call's global_scale
  const uint32_t* hf_mul;
  const uint8_t* sharpness;
  const int32_t* qcoeff;     // [3][W8*H8]
  const int32_t* lfq;        // [3][bw*bh]
  const int8_t* cfl_x;
  const int8_t* cfl_b;
  float k_x_lf, k_b_lf;      // frame LF CfL multipliers
  const int* lf_factors_dev; // when non-null, read the LF factors from here
  float* planes;             // [3][w*h] XYB out
  float* sigma;              // [bw*bh]
  const float* lf_float = nullptr;  // [3][bw*bh] final LF (decoded frames); else from lfq
  uint32_t* err = nullptr;   // device error word
};

// LF of a decoded frame: dequantize, LF CfL and (smooth) adaptive smoothing
// into out [3][bw*bh]; tmp holds as much when smoothing.
void launch_lf_prepare(const int32_t* lfq, int bw, int bh, const float m[3], float div, float kx,
                       float kb, bool smooth, float* tmp, float* out, int num_sms,
                       cudaStream_t s);
void upload_dct64(const float* matrix, cudaStream_t s);
void upload_afv(const double* basis, cudaStream_t s);
bool launch_special_diag(int kind, const float* coef, int n, float* out, cudaStream_t s);

// Fills table[h] = hf_multiplier_f64(global_scale, h) for h < kMulTableN.
void launch_mul_table(uint32_t global_scale, float* table, cudaStream_t s);

// Per-device kernel attributes (dynamic shared memory above 48 KB); call once
// per device with it current, before any launch or stream capture.
cudaError_t configure_encode_kernels();
cudaError_t configure_ssim_kernels();

void upload_dct_constants(const float* iv4, const float* iv8, const float* iv16,
                          const float* scale_f, cudaStream_t s);
void launch_srgb_to_xyb(const void* rgb, int bits, size_t n, const float* lut, float* x, float* y,
                        float* b, uint32_t* not_gray, int num_sms, cudaStream_t s);
// One launch (the ring of tiles along the frame's rows and columns of other
// rules, then the tiles inside it); returns 1.
int launch_precondition(const float* in, float* out, int w, int h, cudaStream_t s);
// The per-shape-class launchers take one stream per class (s[i] for class
// i), so that independent classes can run side by side.  Each returns the
// number of kernels it launched.
int launch_fdct_luma(const EncArgs& a, const uint32_t* const* lists, const int* counts,
                     const cudaStream_t* s);
// LF CfL partials: kLfCtas CTAs, each 7 double-float sums and 8 bit counts.
constexpr int kLfCtas = 128;
constexpr size_t kCflScratchBytes = (size_t)kLfCtas * (7 * 8 + 8 * 4);
// Per-tile CfL scratch: 8 double-float sums and 2 seeds per 64x64 tile.
inline size_t cfl_tile_scratch_bytes(int ntiles) { return (size_t)ntiles * (8 * 8 + 2 * 4); }
// The per-tile chain runs on s, the LF factors' chain on lf_s (it reads
// only the LF planes); the caller joins lf_s back before the factors are
// read.
int launch_cfl(const EncArgs& a, int* lf_seeds, void* lf_scratch, void* tile_scratch,
               cudaStream_t s, cudaStream_t lf_s);
int launch_quant_chroma(const EncArgs& a, const uint32_t* const* lists, const int* counts,
                        const cudaStream_t* s);

void launch_render_varblocks(const RenderArgs& a, const uint32_t* const* lists,
                             const int* counts, const cudaStream_t* s);

// Split-precision transforms on the tensor cores (k_tc.cu), square shape
// classes 0..2 (DCT8, DCT16, DCT32); terms = 2 (BF16x3) or 3 (BF16x6).
// Each returns the number of kernels it launched.  The render form needs
// 16-byte aligned coefficient planes.
cudaError_t configure_tc_kernels();
// Sets the tensor-core kernels' persistent CTAs per SM (1..4; other values
// leave it) and returns the previous value.
int tc_ctas_per_sm(int value);
void upload_tc_basis(cudaStream_t s);
int launch_fdct_tc(const EncArgs& a, const uint32_t* const* lists, const int* counts, int terms,
                   int num_sms, const cudaStream_t* s);
int launch_render_tc(const RenderArgs& a, const uint32_t* const* lists, const int* counts,
                     const float* const* llf, int terms, int num_sms, const cudaStream_t* s);
// The LLF rectangles (48 floats per varblock: 3 channels x 16) and the EPF
// sigma of square classes 0..2, for launch_render_tc (k_render.cu).
int launch_llf_sigma(const RenderArgs& a, const uint32_t* const* lists, const int* counts,
                     float* const* llf, const cudaStream_t* s);
// Luma LF and HF quantization of the square varblocks from a coefficient
// image the split-precision forward transform wrote (k_fdct_luma without its
// own transform).
int launch_luma_from_image(const EncArgs& a, const uint32_t* const* lists, const int* counts,
                           const cudaStream_t* s);
void launch_gaborish(const float* in, float* out, int w, int h, cudaStream_t s);
void launch_epf_step(int step, const float* in, float* out, const float* sigma, int w, int h,
                     cudaStream_t s);
// out_kind: 1 linear f32 planes, 2 sRGB8 interleaved, 3 linear at depth
// pxyb (optional, out_kind 3 only): also the SSIMULACRA2 positive XYB planes
// of the output pixels.
// bracket (out_kind 3, more than 256 levels): per level (the threshold
// below, the threshold above, the level's value).
void launch_colour_out(const float* xyb, int w, int h, int out_kind, const float* thresholds,
                       const float* levels, const float4* bracket, int nlevels, void* out,
                       float* pxyb, int num_sms, cudaStream_t s);
void upload_render_constants(const float* opsin_m, const float* opsin_bias,
                             const float* opsin_bias_cbrt, cudaStream_t s);

// Cover selection (k_cover.cu).  Shape s: 0 DCT8, 1 DCT16, 2 DCT32;
// candidates of shape s sit at every (1 << s)-aligned block position that
// fits the grid, indexed row-major over (bw >> s) x (bh >> s).
struct CoverArgs {
  Geo geo;
  const float* pre;        // 3 planes w*h: the transform frame
  const float* dq;         // [3][kDequantTableFloats]
  float scale[3];          // Mul * qm[c] at the baseline HfMul
  double lambda[3];        // lib.rs:2094 per-channel Lagrange multipliers
  double w[3][3];          // [shape][channel] lambda[c] * side^2
  uint32_t* bits[3];       // [shape][candidate] residual bits, three channels
  DF* sse[3];              // [shape][candidate][channel] sum of squared error
  float* coef[3];          // [shape] 3 coefficient planes of W8*H8
  uint8_t* map;            // block map out (bw*bh)
  uint32_t* fallbacks;     // regions replayed in the reference's order
  uint32_t* err;
};
size_t cover_scratch_bytes(const Geo& g);
// Points a's scratch arrays into `scratch` (cover_scratch_bytes(g) bytes).
void cover_bind_scratch(CoverArgs* a, void* scratch);
int launch_cover(const CoverArgs& a, cudaStream_t s);

// SSIMULACRA2
struct SsimScale {
  int w, h;
  float* xyb;   // [3][w*h]  (reference side)
  float* mu;    // [3][w*h]
  float* s11;   // [3][w*h]
};
// The blur's constants (taps, resonators) into constant memory.
void upload_blur_consts(cudaStream_t s);
// Widest frame the row pass stages in shared memory (a line plus its output).
constexpr int kBlurMaxWidth = 8192;
size_t blur_row_smem(int w);
cudaError_t configure_blur_kernels();
// Rows of partial sums one scale writes (one per 32 x 32 tile), and the
// floats of the column pass's segment-state scratch for three channels.
int blur_partial_rows(int w, int h);
size_t blur_carry_floats(int w, int h);
// 2x2 mean of linear RGB planes; xyb (optional) receives the result's
// positive XYB planes.
void launch_downscale3(const float* in, int w, int h, float* out, float* xyb, cudaStream_t s);
void launch_positive_xyb(const float* rgb, float* xyb, size_t n, int num_sms, cudaStream_t s);
// Reference side of one scale: mu = blur(xyb), s11 = blur(xyb * xyb) per
// channel; hpl (6 w*h planes) and carry (blur_carry_floats) are scratch; a
// column-scan wait that runs out raises kDevBlurTimeout in err.  Three
// launches: the row pass, the column flags' reset, the column pass.
void launch_ref_moments(const float* xyb, float* mu, float* s11, float* hpl, float* carry, int w,
                        int h, uint32_t* err, cudaStream_t s);
// Candidate side of one scale for channels c0 .. c0+nch-1: cand_xyb is the
// candidate's positive XYB [3][w*h]; hpl (3 * nch w*h planes) and carry
// (blur_carry_floats) are scratch; partial receives one row of 18
// double-float sums (8 bytes each) per 32 x 32 tile, each channel filling
// its six.  Returns the number of rows (blur_partial_rows).
struct DF;
// Called between a scale's launches when the caller times them: part 0
// before the row pass, 1 after it, 2 before the column pass (its flags'
// reset and its kernel, which runs the ripple's segment scan inside), 3
// after it.  Two kernels per scale (kScoreScaleKernels).
using ScaleHook = void (*)(void* user, int part);
constexpr int kScoreScaleKernels = 2;
int launch_score_scale(const float* cand_xyb, const SsimScale& ref, float* hpl, float* carry,
                       int c0, int nch, DF* partial, uint32_t* err, cudaStream_t s,
                       ScaleHook hook = nullptr, void* user = nullptr);
// Two launches (the per-scale sums, then the score); returns 2.  The sums
// overwrite row 0 of each scale's partial rows.
int launch_score_finish(DF* partials, const int* ctas_per_scale, int nscales,
                        const int* pixels_per_scale, double* out, cudaStream_t s);

}  // namespace jpxlg
