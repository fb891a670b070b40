// oracle_internal.h — shared declarations of the CPU restatement (test
// infrastructure only; see oracle.h).
#ifndef JPXL_ORACLE_INTERNAL_H
#define JPXL_ORACLE_INTERNAL_H
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace orc {

inline uint32_t fbits(float v) { uint32_t b; std::memcpy(&b, &v, 4); return b; }
inline float ffrom(uint32_t b) { float v; std::memcpy(&v, &b, 4); return v; }

enum Err { kOk = 0, kErrShape = -1, kErrQuant = -2, kErrParam = -3, kErrBlockMap = -4 };

float cbrt_core(float v);
float cbrt_perceptual(float v);
void linear_to_xyb(const float rgb[3], float out[3]);
void linear_to_positive_xyb(const float rgb[3], float out[3]);
float srgb_to_linear(float v);
float linear_to_srgb(float v);
void opsin_inverse(const float xyb[3], float out[3]);

float dct_iv_entry(int M, int u, int n);
void dct_ii_ortho(float* v, int n);
void dct_iii_ortho(float* v, int n);
void dct_1d(float* v, int n);
void idct_1d(float* v, int n);
void dct_2d(float* work, int rows, int cols);
void idct_2d(float* work, int rows, int cols);

struct TransformInfo {
  int sel;       // DctSelect
  int brows;     // footprint rows in 8x8 blocks
  int bcols;     // footprint cols
  int dq_index;  // Table I.4 parameters index
  int crows;     // landscape coefficient rows = min*8
  int ccols;     // landscape coefficient cols = max*8
};
bool transform_info(int sel, TransformInfo* t);

// A varblock decoded from the block map.
struct Varblock {
  int bx, by;
  TransformInfo t;
};
// Parses the per-block map into varblocks (raster order of their origins);
// kErrBlockMap unless the footprints tile the block grid exactly.
int parse_block_map(const uint8_t* map, int bw, int bh, std::vector<Varblock>* out);
// Coefficient image addressing (see oracle.h): landscape cell (y, x) of a
// varblock at (bx, by).
inline size_t coeff_index(const Varblock& vb, int y, int x, int W8) {
  bool portrait = vb.t.brows > vb.t.bcols;
  int row = vb.by * 8 + (portrait ? x : y);
  int col = vb.bx * 8 + (portrait ? y : x);
  return (size_t)row * W8 + col;
}
float scale_f(int c, int lf_count);
void dequant_matrix(int dq, int channel, float* out, int* rows, int* cols);
const float* dequant_matrix_cached(int dq, int channel);

extern const float kQuantBias[3];
extern const float kQuantBiasNumerator;
float hf_multiplier(uint32_t gs, uint32_t hf_mul);
float qm_multiplier(uint32_t qm_scale);
float bias_adjust(int32_t q, float bias, float num);
bool clamp_round(float v, int32_t* out);
float cfl_multiplier(float base, int32_t factor, uint32_t colour_factor);

struct LfQuant {
  float m_dc[3];
  int ep;
  LfQuant(uint32_t gs, uint32_t quant_lf, int extra_precision);
  float reconstruct(int32_t q, int c) const;
  bool quantize(float target, int c, int32_t* q) const;
};

struct HfQuant {
  float steps[3][1024];
  float thr[3][1024];
  int cells;
  HfQuant(const TransformInfo& t, uint32_t gs, uint32_t hf_mul, uint32_t x_qm, uint32_t b_qm);
  float reconstruct(int32_t q, int c, int cell) const;
  bool choose(float target, int c, int cell, int32_t* out) const;
};

int mirror1d(int64_t c, int size);
std::vector<float> pad_mirror(const float* in, int w, int h, int r);
void gab_precondition(const float* f, int w, int h, float* x);
void gaborish(const float* in, int w, int h, float* out);
void gaborish_w(const float* in, int w, int h, float w1, float w2, float* out);
float epf_inv_sigma(int step, float sigma);
float vardct_sigma(float mul, int sharpness);
void epf_step(int step, const float* const* in, int w, int h, const float* sigma,
              float* const* out);
float full_scale(int bits);
int composed_level(float x, float max);
void depth_thresholds(int bits, float* out);

}  // namespace orc
#endif
