// jpxlg_internal.h — host-side declarations shared by the library's
// translation units: frame geometry, the per-call parameter blocks passed to
// kernels, the host table builders and the kernel launchers.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace jpxlg {

struct Geo {
  int w, h;    // pixels
  int bw, bh;  // 8x8 blocks
  int W8, H8;  // coefficient image = 8*bw x 8*bh
  int tw, th;  // 64x64 CfL tiles
};

inline Geo make_geo(int w, int h) {
  Geo g;
  g.w = w;
  g.h = h;
  g.bw = (w + 7) / 8;
  g.bh = (h + 7) / 8;
  g.W8 = g.bw * 8;
  g.H8 = g.bh * 8;
  g.tw = (g.bw + 7) / 8;
  g.th = (g.bh + 7) / 8;
  return g;
}

// Quantizer scalars shared by encode and render (formed on the host exactly
// as the reference forms them; see tables.cu).
struct QuantScalars {
  uint32_t global_scale;
  float m_dc[3];       // LF multipliers (reconstruct.rs:67 / quantize.rs:150)
  float qm[3];         // {qm_multiplier(x), 1, qm_multiplier(b)}
};

// Shape classes, in this order: the nine plain DCTRxC types up to 32, then
// DCT2x2, DCT64x64, DCT64x32, DCT32x64, Hornuss, DCT4x4, DCT8x4, DCT4x8 and
// AFV0-3.
constexpr int kNumShapes = 21;
constexpr int kShapeSel[kNumShapes] = {0, 4,  5,  6,  7, 8, 9,  10, 11, 2,  18,
                                       19, 20, 1, 3, 13, 12, 14, 15, 16, 17};

// ---- host tables (tables.cu) -------------------------------------------------
void build_dequant_tables(float* out /* 3 * kDequantTableFloats */);
void build_iv_tables(float* iv4, float* iv8, float* iv16);
void build_scale_f(float* out /* [4][8]: lf counts 1,2,4,8 x c<8 */);
void build_dct64_matrix(float* out /* [64][64]: DCT-II rows u, columns x */);
extern const double kAfvBasis[16][16];  // jpxl-core varblock.rs AFV_BASIS (Table I.11)
float host_hf_multiplier(uint32_t gs, uint32_t hf_mul);
float host_qm_multiplier(uint32_t qm_scale);
void host_lf_multipliers(uint32_t gs, uint32_t quant_lf, float out[3]);
float host_srgb_to_linear(float v);
float host_linear_to_srgb(float v);
void build_srgb_lut(int bits, float* out /* 256 or 65536 */);
int build_depth_thresholds(int bits, float* thresholds, float* levels_linear);
void build_opsin_inverse(float* matrix9, float* bias3, float* bias_cbrt3);
float host_cbrt_core(float v);

}  // namespace jpxlg
