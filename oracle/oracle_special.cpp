// oracle_special.cpp — test infrastructure: the CPU restatement of the
// decoder's 8x8 special transforms (jpxl-core varblock.rs:898-1230, ISO/IEC
// 18181-1 I.9.3-I.9.8), the checker of the GPU's special_block kernels.
//
// Each function maps a dequantized 8x8 coefficient block (row-major, cell
// (x, y) at y * 8 + x, the block's LLF at (0, 0)) to its 8x8 samples, in the
// reference's expression order.  The AFV basis (Table I.11) is not held here:
// the caller passes the 256 f64 entries, read from the reference source into
// the committed fixture tests/golden/reference_constants.json.
#include <cstring>

#include "oracle.h"
#include "oracle_internal.h"

namespace {

struct B8 {
  float v[64];
  float at(int x, int y) const { return v[y * 8 + x]; }
  void set(int x, int y, float f) { v[y * 8 + x] = f; }
};

// varblock.rs:898 aux_idct_2x2: the top-left s x s window through the
// unnormalized 2x2 butterflies, the rest copied through.
B8 aux_2x2(const B8& in, int s) {
  B8 r = in;
  const int h = s / 2;
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < h; ++x) {
      const float c00 = in.at(x, y), c01 = in.at(h + x, y);
      const float c10 = in.at(x, y + h), c11 = in.at(h + x, y + h);
      r.set(2 * x, 2 * y, c00 + c01 + c10 + c11);
      r.set(2 * x + 1, 2 * y, c00 + c01 - c10 - c11);
      r.set(2 * x, 2 * y + 1, c00 - c01 + c10 - c11);
      r.set(2 * x + 1, 2 * y + 1, c00 - c01 - c10 + c11);
    }
  return r;
}

// dct.rs:1065 idct_2d_raw: landscape coefficients (min x max) to rows x cols.
void idct_raw(const float* coef, int rows, int cols, float* out) {
  std::memcpy(out, coef, sizeof(float) * rows * cols);
  orc::idct_2d(out, rows, cols);
}

// I.9.3 DCT2x2 (varblock.rs:917).
void dct2x2(const B8& c, B8& o) { o = aux_2x2(aux_2x2(aux_2x2(c, 2), 4), 8); }

// I.9.4 DCT4x4 (varblock.rs:926).
void dct4x4(const B8& c, B8& o) {
  const B8 dcs = aux_2x2(c, 2);
  for (int y = 0; y < 2; ++y)
    for (int x = 0; x < 2; ++x) {
      float blk[16] = {}, smp[16];
      for (int iy = 0; iy < 4; ++iy)
        for (int ix = iy == 0 ? 1 : 0; ix < 4; ++ix) blk[iy * 4 + ix] = c.at(x + 2 * ix, y + 2 * iy);
      blk[0] = dcs.at(x, y);
      idct_raw(blk, 4, 4, smp);
      for (int l = 0; l < 4; ++l)
        for (int k = 0; k < 4; ++k) o.set(4 * x + k, 4 * y + l, smp[l * 4 + k]);
    }
}

// I.9.5 Hornuss (varblock.rs:953): the (0, 0) cell is written last, from
// coefficient (x + 2, y + 2).
void hornuss(const B8& c, B8& o) {
  const B8 dcs = aux_2x2(c, 2);
  for (int y = 0; y < 2; ++y)
    for (int x = 0; x < 2; ++x) {
      float rs = 0.0f;
      for (int iy = 0; iy < 4; ++iy)
        for (int ix = iy == 0 ? 1 : 0; ix < 4; ++ix) rs += c.at(x + 2 * ix, y + 2 * iy);
      const float centre = dcs.at(x, y) - rs / 16.0f;
      o.set(4 * x + 1, 4 * y + 1, centre);
      for (int iy = 0; iy < 4; ++iy)
        for (int ix = 0; ix < 4; ++ix)
          if (!(ix == 1 && iy == 1)) o.set(4 * x + ix, 4 * y + iy, c.at(x + 2 * ix, y + 2 * iy) + centre);
      o.set(4 * x, 4 * y, c.at(x + 2, y + 2) + centre);
    }
}

// I.9.6 DCT8x4 (vertical) and I.9.7 DCT4x8 (varblock.rs:1008): rows of one
// parity form each half, the DC pair is (c00 + c10', c00 - c10') of cells
// (0, 0) and (0, 1); half h lands at the low coordinate 4h
// (DCT8X4_HALF_INDEX_IS_LOW_COORDINATE).
void dct8x4_or_4x8(const B8& c, bool vertical, B8& o) {
  const float c0 = c.at(0, 0), c1 = c.at(0, 1);
  const float dcs[2] = {c0 + c1, c0 - c1};
  for (int half = 0; half < 2; ++half) {
    float g[32] = {}, s[32];
    for (int iy = 0; iy < 4; ++iy)
      for (int ix = iy == 0 ? 1 : 0; ix < 8; ++ix) g[iy * 8 + ix] = c.at(ix, half + 2 * iy);
    g[0] = dcs[half];
    if (vertical) {
      idct_raw(g, 8, 4, s);
      for (int iy = 0; iy < 8; ++iy)
        for (int ix = 0; ix < 4; ++ix) o.set(4 * half + ix, iy, s[iy * 4 + ix]);
    } else {
      idct_raw(g, 4, 8, s);
      for (int iy = 0; iy < 4; ++iy)
        for (int ix = 0; ix < 8; ++ix) o.set(ix, 4 * half + iy, s[iy * 8 + ix]);
    }
  }
}

// I.9.8 AFV n (varblock.rs:1150): the AFV quadrant from the basis (f64 dot
// products rounded once to f32), the DCT4x4 quadrant beside it and the DCT4x8
// half below or above, flipped by n's bits.
void afv(const B8& c, int n, const double* basis, B8& o) {
  const int fx = n & 1, fy = n / 2;
  float ca[16] = {}, sa[16];
  ca[0] = (c.at(0, 0) + c.at(0, 1) + c.at(1, 0)) * 4.0f;
  for (int iy = 0; iy < 4; ++iy)
    for (int ix = iy == 0 ? 1 : 0; ix < 4; ++ix) ca[iy * 4 + ix] = c.at(2 * ix, 2 * iy);
  for (int p = 0; p < 16; ++p) {
    double acc = 0.0;
    for (int j = 0; j < 16; ++j) acc += (double)ca[j] * basis[j * 16 + p];
    sa[p] = (float)acc;
  }
  for (int iy = 0; iy < 4; ++iy)
    for (int ix = 0; ix < 4; ++ix) {
      const int sx = fx ? 3 - ix : ix, sy = fy ? 3 - iy : iy;
      o.set(fx * 4 + ix, fy * 4 + iy, sa[sy * 4 + sx]);
    }
  float c44[16] = {}, s44[16];
  for (int iy = 0; iy < 4; ++iy)
    for (int ix = iy == 0 ? 1 : 0; ix < 4; ++ix) c44[iy * 4 + ix] = c.at(2 * ix + 1, 2 * iy);
  c44[0] = c.at(0, 0) - c.at(1, 0) + c.at(0, 1);
  idct_raw(c44, 4, 4, s44);
  for (int iy = 0; iy < 4; ++iy)
    for (int ix = 0; ix < 4; ++ix) o.set((fx ? 0 : 4) + ix, fy * 4 + iy, s44[iy * 4 + ix]);
  float c48[32] = {}, s48[32];
  for (int iy = 0; iy < 4; ++iy)
    for (int ix = iy == 0 ? 1 : 0; ix < 8; ++ix) c48[iy * 8 + ix] = c.at(ix, 1 + 2 * iy);
  c48[0] = c.at(0, 0) - c.at(0, 1);
  idct_raw(c48, 4, 8, s48);
  for (int iy = 0; iy < 4; ++iy)
    for (int ix = 0; ix < 8; ++ix) o.set(ix, (fy ? 0 : 4) + iy, s48[iy * 8 + ix]);
}

}  // namespace

// kind: 1 DCT2x2, 2 Hornuss, 3 DCT4x4, 4 DCT8x4, 5 DCT4x8, 6..9 AFV0..AFV3
// (varblock.rs:1218 samples_from_coefficients).  afv_basis: Table I.11, 16
// rows of 16, needed for kinds 6..9.
extern "C" int orc_special_block(int kind, const float* coef, const double* afv_basis,
                                 float* out) {
  B8 c, o;
  std::memcpy(c.v, coef, sizeof c.v);
  std::memset(o.v, 0, sizeof o.v);
  switch (kind) {
    case 1: dct2x2(c, o); break;
    case 2: hornuss(c, o); break;
    case 3: dct4x4(c, o); break;
    case 4: dct8x4_or_4x8(c, true, o); break;
    case 5: dct8x4_or_4x8(c, false, o); break;
    case 6: case 7: case 8: case 9:
      if (!afv_basis) return -1;
      afv(c, kind - 6, afv_basis, o);
      break;
    default: return -1;
  }
  std::memcpy(out, o.v, sizeof o.v);
  return 0;
}
