// jpxlg_defs.cuh — device definitions that refer to no device symbol of
// another translation unit (the error word, the transform table, the packed
// dequant table's layout, the hf multiplier), so that a unit built as whole
// program code (without relocatable device code) can include them.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace jpxlg {

// ---- error word (device -> host) -------------------------------------------
// A kernel that meets a condition for which the reference returns an Err
// records it with atomicOr into the context's error word instead of
// trapping; the host reads the word after the stage and returns a status.
enum DevError : uint32_t {
  kDevQuantRange = 1u << 0,   // clamp_round saw a non-finite or |q| > 2^20 target
  kDevBadStep = 1u << 1,      // degenerate quantization step
  kDevBlockMap = 1u << 2,     // a block-map entry the kernel cannot place
  kDevTcTimeout = 1u << 3,    // a bounded wait on a tensor-core MMA ran out
  kDevBlurTimeout = 1u << 4,  // a bounded wait on a previous column segment ran out
};

__device__ __forceinline__ void raise_error(uint32_t* err, uint32_t bit) {
  if (err) atomicOr(err, bit);
}

// ---- transforms -------------------------------------------------------------
// The varblock types the pixel path carries (Table I.1): the nine plain
// DCTRxC types up to 32 (the encoder's) and, for decoded streams, the 8x8
// special transforms (Hornuss, DCT2x2, DCT4x4, DCT4x8/8x4, AFV0-3) and
// DCT64x64 / DCT64x32 / DCT32x64: DctSelect and footprint rows/cols in blocks.
struct Shape {
  int brows, bcols;
};
__host__ __device__ __forceinline__ bool shape_of(int sel, Shape* s) {
  switch (sel) {
    case 0: *s = {1, 1}; return true;
    case 4: *s = {2, 2}; return true;
    case 5: *s = {4, 4}; return true;
    case 6: *s = {2, 1}; return true;
    case 7: *s = {1, 2}; return true;
    case 8: *s = {4, 1}; return true;
    case 9: *s = {1, 4}; return true;
    case 10: *s = {4, 2}; return true;
    case 11: *s = {2, 4}; return true;
    case 1: case 2: case 3: case 12: case 13: case 14: case 15: case 16: case 17:
      *s = {1, 1};
      return true;
    case 18: *s = {8, 8}; return true;
    case 19: *s = {8, 4}; return true;
    case 20: *s = {4, 8}; return true;
    default: return false;
  }
}
// compact dequant slot: 0 DCT8, 1 DCT16x16, 2 DCT32x32, 3 DCT16x8/8x16,
// 4 DCT32x8/8x32, 5 DCT32x16/16x32, 6 DCT2x2, 7 DCT64x64, 8 DCT64x32/32x64,
// 9 Hornuss, 10 DCT4x4, 11 DCT4x8/8x4, 12 AFV0-3 (Table I.4 indices
// 0,4,5,6,7,8,2,11,12,1,3,9,10).
__host__ __device__ __forceinline__ int dq_slot(int sel) {
  switch (sel) {
    case 0: return 0;
    case 4: return 1;
    case 5: return 2;
    case 6: case 7: return 3;
    case 8: case 9: return 4;
    case 2: return 6;
    case 18: return 7;
    case 19: case 20: return 8;
    case 1: return 9;
    case 3: return 10;
    case 12: case 13: return 11;
    case 14: case 15: case 16: case 17: return 12;
    default: return 5;
  }
}
// Offsets of each slot's landscape matrix in the packed dequant table.
__host__ __device__ __forceinline__ int dq_offset(int slot) {
  // sizes: 64, 256, 1024, 128, 256, 512, 64, 4096, 2048, 64, 64, 64, 64
  const int off[13] = {0, 64, 320, 1344, 1472, 1728, 2240, 2304, 6400, 8448, 8512, 8576, 8640};
  return off[slot];
}
constexpr int kDequantTableFloats = 8704;  // per channel

// ---- reconstruct.rs:27 hf_multiplier -----------------------------------------
// Mul = 65536 / (global_scale * hf_mul), formed in f64 and narrowed to f32.
// A context tabulates it for hf_mul < kMulTableN once per call (the same
// expression, so the same bits); larger hf_mul evaluate it in place.
constexpr int kMulTableN = 256;
__device__ __forceinline__ float hf_multiplier_f64(uint32_t global_scale, uint32_t hf_mul) {
  const double denom = (double)global_scale * (double)hf_mul;
  return denom <= 0.0 ? 0.0f : (float)(65536.0 / denom);
}
__device__ __forceinline__ float hf_multiplier(const float* table, uint32_t global_scale,
                                               uint32_t hf_mul) {
  return hf_mul < (uint32_t)kMulTableN ? __ldg(&table[hf_mul])
                                       : hf_multiplier_f64(global_scale, hf_mul);
}

}  // namespace jpxlg
