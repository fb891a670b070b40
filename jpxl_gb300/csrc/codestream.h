// codestream.h — host-side reader of JPEG XL codestreams (ISO/IEC 18181-1)
// for the lossy VarDCT path: image headers, the frame header and TOC, modular
// sub-bitstreams (MA trees, the predictors of H.3/H.5) and the VarDCT
// sections (LF global, LF groups, HF global, HF passes and groups), as
// jpxl-decode reads them (crates/jpxl-decode/src/decode.rs:2513-2950,
// vardct/hf_coeff.rs:689).  The result is the frame's integer content —
// quantized LF, the varblock map, HF multipliers, CfL factors, EPF sharpness
// and quantized HF coefficients — that the GPU reconstruction consumes.
// Integer arithmetic only; every read is bounds-checked and a malformed
// stream throws Malformed (caught at the C ABI as JPXLG_ERR_STREAM).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace jpxlg {
namespace cs {

struct Malformed {
  std::string what;
};

// One modular channel (H.1): width x height signed samples.
struct Channel {
  uint32_t w = 0, h = 0;
  int hshift = 0, vshift = 0;
  std::vector<int32_t> v;
  int32_t at(uint32_t x, uint32_t y) const { return v[(size_t)y * w + x]; }
  int32_t& at(uint32_t x, uint32_t y) { return v[(size_t)y * w + x]; }
  bool same_shape(const Channel& o) const {
    return w == o.w && h == o.h && hshift == o.hshift && vshift == o.vshift;
  }
};

struct ImageInfo {
  uint32_t width = 0, height = 0;
  uint32_t bits_per_sample = 8, exp_bits = 0;
  bool float_sample = false;
  bool xyb_encoded = true;
  int colour_space = 0;  // 0 RGB, 1 grey, 2 XYB, 3 unknown
  bool want_icc = false;
  int transfer = 13;     // Table E.4 enum (13 sRGB, 8 linear, ...); -1: gamma
  uint32_t gamma = 0;
  uint32_t num_extra = 0;
  uint32_t orientation = 1;
  float intensity_target = 255.0f;
  struct Extra {
    uint32_t type = 0, bits = 8, dim_shift = 0;
  };
  std::vector<Extra> extra;  // extra channels (alpha, depth, ...)
  bool default_opsin = true;
  float opsin_inv[9], opsin_bias[3], quant_bias[4], quant_bias_numerator = 0.145f;
};

struct FrameInfo {
  int encoding = 0;  // 0 VarDCT, 1 modular
  int frame_type = 0;
  uint64_t flags = 0;
  uint32_t upsampling = 1;
  uint32_t group_size_shift = 1;
  uint32_t x_qm_scale = 3, b_qm_scale = 2;
  uint32_t num_passes = 1;
  std::vector<uint32_t> pass_shift;  // per pass, the coefficient shift
  bool is_last = true;
  bool gab = true, gab_custom = false;
  float gab_w1[3] = {0.115169525f, 0.115169525f, 0.115169525f};
  float gab_w2[3] = {0.061248592f, 0.061248592f, 0.061248592f};
  uint32_t epf_iters = 2;
  float epf_sharp_lut[8] = {0.0f,        1.0f / 7.0f, 2.0f / 7.0f, 3.0f / 7.0f,
                            4.0f / 7.0f, 5.0f / 7.0f, 6.0f / 7.0f, 1.0f};
  float epf_channel_scale[3] = {40.0f, 5.0f, 3.5f};
  float epf_quant_mul = 0.46f, epf_pass0_sigma_scale = 0.9f, epf_pass2_sigma_scale = 6.5f;
  float epf_border_sad_mul = 2.0f / 3.0f;
  uint32_t width = 0, height = 0;  // frame samples (image / upsampling)
  uint32_t lf_level = 0;           // LF frames
};

// A varblock of an LF group: its top-left 8x8 block (frame block coordinates),
// DctSelect and HF multiplier.
struct Varblock {
  uint32_t bx, by;
  uint8_t transform;
  uint32_t hf_mul;
  uint32_t coeff_offset;  // into VarDctFrame::coeffs, per channel
};

struct VarDctFrame {
  uint32_t global_scale = 0, quant_lf = 0;
  float m_lf[3] = {1.0f / 32.0f, 1.0f / 4.0f, 1.0f / 2.0f};  // LfChannelDequantization
  uint32_t colour_factor = 84;
  float base_corr_x = 0.0f, base_corr_b = 1.0f;
  int x_factor_lf = 0, b_factor_lf = 0;
  bool default_matrices = true;
  uint32_t bw = 0, bh = 0;  // block grid of the frame
  uint32_t extra_precision = 0;
  std::vector<int32_t> lf[3];          // quantized LF, [c][by * bw + bx] (X, Y, B)
  std::vector<uint8_t> block_map;      // DctSelect | 0x80 at varblock origins, [by * bw + bx]
  std::vector<uint32_t> hf_mul;        // per block (the varblock's value at its blocks)
  std::vector<uint8_t> sharpness;      // per block
  uint32_t tiles_w = 0, tiles_h = 0;   // 64x64 CfL tiles
  std::vector<int8_t> x_from_y, b_from_y;
  std::vector<Varblock> varblocks;
  std::vector<int32_t> coeffs[3];      // per channel, varblocks back to back, raster
  uint32_t histogram_counts[27] = {};  // varblocks per DctSelect
  bool lf_from_frame = false;          // LF taken from an LF frame (kUseLfFrame)
  std::vector<float> lf_frame[3];      // that LF, X, Y, B planes of bw x bh
};

struct Decoded {
  ImageInfo image;
  FrameInfo frame;
  VarDctFrame vardct;
  std::vector<Channel> modular;        // a modular frame's channels
  std::vector<Channel> extra;          // a VarDCT frame's extra channels
  uint64_t sections = 0;
  std::vector<uint64_t> section_bits;  // bits each section's reader consumed
  std::vector<uint64_t> section_sizes; // TOC entries, bytes
};

// Block rows and columns of a DctSelect (Table I.1).
struct TransformShape {
  uint32_t rows, cols;
};
TransformShape transform_shape(uint8_t dct_select);

// Parses the codestream (a bare one, starting 0xFF 0x0A) and decodes the
// integer content of its first frame.  Throws Malformed.
void decode(const uint8_t* data, size_t size, Decoded* out);

}  // namespace cs
}  // namespace jpxlg

// The C ABI's handle (include/jpxlg.h jpxlg_codestream).
struct jpxlg_codestream {
  jpxlg::cs::Decoded d;
};
