// oracle_pipeline.cpp — CPU restatement of the encoder's transform and
// quantization path (XYB, inverse Gaborish, forward DCT, LF, chroma-from-luma
// estimation, quantization) and of the plan renderer (dequantization, CfL,
// LLF, IDCT, Gaborish, EPF, colour, output depth).
//
// TEST INFRASTRUCTURE ONLY (the checker, never the product).
#include <algorithm>
#include <cstdlib>
#include <memory>
#include <thread>

#include "oracle.h"
#include "oracle_internal.h"

namespace orc {

// Parses the per-block map into varblocks (raster order of their origins)
// and checks that the footprints tile the block grid exactly.
int parse_block_map(const uint8_t* map, int bw, int bh, std::vector<Varblock>* out) {
  std::vector<uint8_t> covered((size_t)bw * bh, 0);
  for (int by = 0; by < bh; ++by) {
    for (int bx = 0; bx < bw; ++bx) {
      uint8_t v = map[(size_t)by * bw + bx];
      if (!(v & 0x80)) continue;
      Varblock vb;
      vb.bx = bx;
      vb.by = by;
      if (!transform_info(v & 0x1f, &vb.t)) return kErrBlockMap;
      if (bx % vb.t.bcols || by % vb.t.brows) return kErrBlockMap;
      if (bx + vb.t.bcols > bw || by + vb.t.brows > bh) return kErrBlockMap;
      for (int dy = 0; dy < vb.t.brows; ++dy)
        for (int dx = 0; dx < vb.t.bcols; ++dx) {
          size_t i = (size_t)(by + dy) * bw + bx + dx;
          if (covered[i] || (map[i] & 0x1f) != (v & 0x1f)) return kErrBlockMap;
          covered[i] = 1;
        }
      out->push_back(vb);
    }
  }
  for (uint8_t c : covered)
    if (!c) return kErrBlockMap;
  return kOk;
}


// ---------------------------------------------------------------------------
// Source (jpxl-encode-policy/src/source.rs:226 / :355)
// ---------------------------------------------------------------------------

static bool source_to_xyb(const void* rgb, int w, int h, int bits, float* x, float* y,
                          float* b) {
  size_t n = (size_t)w * h;
  bool gray = true;
  std::vector<float> lut;
  if (bits == 8) {
    lut.resize(256);
    for (int i = 0; i < 256; ++i) lut[i] = srgb_to_linear((float)i / 255.0f);
  } else {
    float max = std::min(65535.0f, (float)((1u << bits) - 1));
    float divisor = max > 0.0f ? max : 1.0f;
    lut.resize(65536);
    for (int i = 0; i < 65536; ++i) lut[i] = srgb_to_linear((float)i / divisor);
  }
  for (size_t i = 0; i < n; ++i) {
    uint32_t cr, cg, cb;
    if (bits == 8) {
      const uint8_t* p = (const uint8_t*)rgb + 3 * i;
      cr = p[0]; cg = p[1]; cb = p[2];
    } else {
      const uint16_t* p = (const uint16_t*)rgb + 3 * i;
      cr = p[0]; cg = p[1]; cb = p[2];
    }
    gray = gray && cr == cg && cg == cb;
    float lin[3] = {lut[cr], lut[cg], lut[cb]}, out[3];
    linear_to_xyb(lin, out);
    x[i] = out[0]; y[i] = out[1]; b[i] = out[2];
  }
  return gray;
}

// ---------------------------------------------------------------------------
// Forward transform of one varblock (policy lib.rs:3008 gather_square with
// edge replication, forward.rs:451 forward_dct_rc) into landscape coeffs.
// ---------------------------------------------------------------------------

static void forward_varblock(const float* plane, int w, int h, const Varblock& vb, float* out) {
  int rows = vb.t.brows * 8, cols = vb.t.bcols * 8;
  int x0 = vb.bx * 8, y0 = vb.by * 8;
  for (int dy = 0; dy < rows; ++dy)
    for (int dx = 0; dx < cols; ++dx) {
      int xx = std::min(x0 + dx, w - 1), yy = std::min(y0 + dy, h - 1);
      out[dy * cols + dx] = plane[(size_t)yy * w + xx];
    }
  dct_2d(out, rows, cols);
}

// forward.rs:779 lf_from_llf_into for a square varblock: n x n LF samples
// from the top-left n x n of a side x side coefficient array.
static void lf_from_llf(const float* coeff, int n, int side, float* lf) {
  float work[16];
  for (int y = 0; y < n; ++y)
    for (int x = 0; x < n; ++x)
      work[y * n + x] = coeff[y * side + x] / (scale_f(y, n) * scale_f(x, n));
  idct_2d(work, n, n);
  for (int i = 0; i < n * n; ++i) lf[i] = work[i];
}

// ---------------------------------------------------------------------------
// Chroma-from-luma estimation (policy lib.rs:3437 estimate_cfl,
// quantize.rs:1620 CflAccumulator, lib.rs:3831/:3966 refinements).
// ---------------------------------------------------------------------------

struct Acc {
  double s_yy = 0, s_yc = 0, s_cc = 0;
  void add(float y, float c) {
    double yd = y, cd = c;
    s_yy += yd * yd;
    s_yc += yd * cd;
    s_cc += cd * cd;
  }
  double energy(double k) const { return s_cc - 2.0 * k * s_yc + k * k * s_yy; }
  int best_factor(float base, uint32_t cf, int lo, int hi) const {
    if (s_yy <= 0.0) return 0;
    double k_ls = s_yc / s_yy;
    double star = (k_ls - (double)base) * (double)cf;
    int64_t centre = (int64_t)std::round(star);
    bool have = false;
    int best = 0;
    double best_e = 0;
    auto consider = [&](int cand) {
      double k = (double)cfl_multiplier(base, cand, cf);
      double e = energy(k);
      if (!have || e < best_e || (e == best_e && std::abs(cand) < std::abs(best))) {
        have = true;
        best = cand;
        best_e = e;
      }
    };
    for (int d = -2; d <= 2; ++d) {
      int64_t c = centre + d;
      c = std::min<int64_t>(std::max<int64_t>(c, lo), hi);
      consider((int)c);
    }
    consider(0);
    return best;
  }
};

struct Sample { float source, recon_y; int cell; };

static uint64_t residual_bits(int32_t q) {
  if (q == 0) return 0;
  uint32_t a = (uint32_t)std::abs((int64_t)q);
  return (uint64_t)(32 - __builtin_clz(a)) + 1;
}
static uint64_t factor_bits(int32_t f) {
  if (f == 0) return 0;
  uint32_t a = (uint32_t)std::abs((int64_t)f);
  return (uint64_t)(32 - __builtin_clz(a)) + 2;
}

static std::vector<int> factor_candidates(int seed, int lo, int hi) {
  std::vector<int> out;
  for (int d = -1; d <= 1; ++d) {
    int c = std::min(std::max(seed + d, lo), hi);
    if (std::find(out.begin(), out.end(), c) == out.end()) out.push_back(c);
  }
  if (std::find(out.begin(), out.end(), 0) == out.end()) out.push_back(0);
  return out;
}

// lib.rs:3898 hf_residual_cost_bounded; returns false on a quantizer error,
// *none = true when the running cost exceeds the cutoff.
static bool hf_cost(const std::vector<Sample>& s, float base, int f, int ch, const HfQuant& q,
                    bool has_cutoff, uint64_t cutoff, uint64_t* bits, bool* none) {
  float k = cfl_multiplier(base, f, 84);
  uint64_t acc = 0;
  *none = false;
  for (const Sample& smp : s) {
    int32_t v;
    if (!q.choose(smp.source - k * smp.recon_y, ch, smp.cell, &v)) return false;
    acc += residual_bits(v);
    if (has_cutoff && acc > cutoff) { *none = true; return true; }
  }
  *bits = acc;
  return true;
}

// lib.rs:3966 refine_hf_factor.
static bool refine_hf(const std::vector<Sample>& s, const Acc& reg, float base, int ch,
                      const HfQuant& q, int* out) {
  *out = 0;
  if (s.empty()) return true;
  int seed = reg.best_factor(base, 84, -128, 127);
  if (seed == 0) return true;
  int best_f = 0;
  uint64_t best_cost;
  bool none;
  if (!hf_cost(s, base, 0, ch, q, false, 0, &best_cost, &none)) return false;
  for (int f : factor_candidates(seed, -128, 127)) {
    if (f == 0) continue;
    uint64_t fb = factor_bits(f);
    uint64_t cutoff = best_cost > fb ? best_cost - fb : 0;
    uint64_t residual;
    if (!hf_cost(s, base, f, ch, q, true, cutoff, &residual, &none)) return false;
    if (none) continue;
    uint64_t cost = residual + fb;
    if (cost < best_cost || (cost == best_cost && std::abs(f) < std::abs(best_f))) {
      best_cost = cost;
      best_f = f;
    }
  }
  *out = best_f;
  return true;
}

// lib.rs:3814 lf_residual_cost.
static bool lf_cost(const std::vector<Sample>& s, float base, int f, int ch, const LfQuant& q,
                    uint64_t* bits) {
  float k = cfl_multiplier(base, f, 84);
  uint64_t acc = 0;
  for (const Sample& smp : s) {
    int32_t v;
    if (!q.quantize(smp.source - k * smp.recon_y, ch, &v)) return false;
    acc += residual_bits(v);
  }
  *bits = acc;
  return true;
}

// lib.rs:3831 refine_lf_factors.
static bool refine_lf(const std::vector<Sample>& xs, const Acc& xr, const std::vector<Sample>& bs,
                      const Acc& br, const LfQuant& q, int* xf, int* bf) {
  const uint64_t kExtra = 50;
  int x_seed = xr.best_factor(0.0f, 84, -128, 127);
  int b_seed = br.best_factor(1.0f, 84, -128, 127);
  std::vector<std::pair<int, uint64_t>> xc, bc;
  for (int f : factor_candidates(x_seed, -128, 127)) {
    uint64_t c;
    if (!lf_cost(xs, 0.0f, f, 0, q, &c)) return false;
    xc.push_back({f, c});
  }
  for (int f : factor_candidates(b_seed, -128, 127)) {
    uint64_t c;
    if (!lf_cost(bs, 1.0f, f, 2, q, &c)) return false;
    bc.push_back({f, c});
  }
  uint64_t nx = 0, nb = 0;
  for (auto& e : xc) if (e.first == 0) { nx = e.second; break; }
  for (auto& e : bc) if (e.first == 0) { nb = e.second; break; }
  int bx = 0, bb = 0;
  uint64_t best = nx + nb;
  for (auto& xe : xc)
    for (auto& be : bc) {
      uint64_t cost = xe.second + be.second;
      if (xe.first != 0 || be.first != 0) cost += kExtra + factor_bits(xe.first) + factor_bits(be.first);
      uint32_t mag = std::abs(xe.first) + std::abs(be.first);
      uint32_t bmag = std::abs(bx) + std::abs(bb);
      if (cost < best || (cost == best && mag < bmag)) {
        bx = xe.first;
        bb = be.first;
        best = cost;
      }
    }
  *xf = bx;
  *bf = bb;
  return true;
}

}  // namespace orc

using namespace orc;

// ---------------------------------------------------------------------------
// Encode: policy lib.rs:555 build_pixel_plan with a host-supplied cover, AQ
// off (one hf_mul for the frame), LF extra precision 0.
// ---------------------------------------------------------------------------

extern "C" int orc_encode(const void* rgb, int w, int h, int bits, const uint8_t* block_map,
                          const uint32_t* hf_mul_blocks, const orc_encode_params* p,
                          float* xyb_out, float* pre_out, float* coeff_out, int32_t* qcoeff_out,
                          int32_t* lf_out, int8_t* cfl_x, int8_t* cfl_b, orc_lf_cfl* lf_cfl) {
  if (w <= 0 || h <= 0 || !(bits == 8 || (bits >= 1 && bits <= 16))) return kErrShape;
  const int bw = (w + 7) / 8, bh = (h + 7) / 8, W8 = bw * 8, H8 = bh * 8;
  const int tw = (bw + 7) / 8, th = (bh + 7) / 8;
  std::vector<Varblock> vbs;
  int rc = parse_block_map(block_map, bw, bh, &vbs);
  if (rc) return rc;
  for (auto& vb : vbs)
    if (vb.t.brows != vb.t.bcols) return kErrBlockMap;  // the encoder covers with squares
  const size_t n = (size_t)w * h;
  std::vector<float> xyb(3 * n);
  bool gray = source_to_xyb(rgb, w, h, bits, &xyb[0], &xyb[n], &xyb[2 * n]);
  if (xyb_out) std::memcpy(xyb_out, xyb.data(), sizeof(float) * 3 * n);
  std::vector<float> pre = xyb;
  if (p->gaborish)
    for (int c = 0; c < 3; ++c) gab_precondition(&xyb[c * n], w, h, &pre[c * n]);
  if (pre_out) std::memcpy(pre_out, pre.data(), sizeof(float) * 3 * n);

  // Forward transforms of every selected varblock (the forward cache).
  const size_t plane8 = (size_t)W8 * H8;
  std::vector<float> coeff(3 * plane8, 0.0f);
  std::vector<float> tmp(1024);
  for (auto& vb : vbs) {
    for (int c = 0; c < 3; ++c) {
      forward_varblock(&pre[c * n], w, h, vb, tmp.data());
      for (int y = 0; y < vb.t.crows; ++y)
        for (int x = 0; x < vb.t.ccols; ++x)
          coeff[c * plane8 + coeff_index(vb, y, x, W8)] = tmp[y * vb.t.ccols + x];
    }
  }
  if (coeff_out) std::memcpy(coeff_out, coeff.data(), sizeof(float) * 3 * plane8);

  const LfQuant lfq(p->global_scale, p->quant_lf, 0);
  auto hf_mul_of = [&](const Varblock& vb) { return hf_mul_blocks[(size_t)vb.by * bw + vb.bx]; };
  auto get_block = [&](int c, const Varblock& vb, float* out) {
    int s = vb.t.ccols;
    for (int y = 0; y < s; ++y)
      for (int x = 0; x < s; ++x) out[y * s + x] = coeff[c * plane8 + coeff_index(vb, y, x, W8)];
  };

  // --- CfL estimation ---
  std::vector<int8_t> tx((size_t)tw * th, 0), tb((size_t)tw * th, 0);
  int x_lf = 0, b_lf = 0;
  if (p->cfl && !gray) {
    std::vector<std::vector<Sample>> hx((size_t)tw * th), hb((size_t)tw * th);
    std::vector<Acc> rx((size_t)tw * th), rb((size_t)tw * th);
    std::vector<Sample> lx, lb;
    Acc lrx, lrb;
    // Index varblocks by origin block for the ordered group/band walk.
    std::vector<int> at_origin((size_t)bw * bh, -1);
    for (size_t i = 0; i < vbs.size(); ++i) at_origin[(size_t)vbs[i].by * bw + vbs[i].bx] = (int)i;
    const int G = 256;  // LF group side in blocks (2048 px)
    int gw = (bw + G - 1) / G, gh = (bh + G - 1) / G;
    std::vector<float> cy(1024), cx(1024), cb(1024), ly(16), lxs(16), lbs(16);
    for (int gy = 0; gy < gh; ++gy)
      for (int gx = 0; gx < gw; ++gx) {
        int by0 = gy * G, bx0 = gx * G;
        int gbh = std::min(G, bh - by0), gbw = std::min(G, bw - bx0);
        for (int trow = 0; trow < (gbh + 7) / 8; ++trow)
          for (int by = by0 + trow * 8; by < std::min(by0 + trow * 8 + 8, by0 + gbh); ++by)
            for (int bx = bx0; bx < bx0 + gbw; ++bx) {
              int vi = at_origin[(size_t)by * bw + bx];
              if (vi < 0) continue;
              const Varblock& vb = vbs[vi];
              int nb = vb.t.brows, side = vb.t.ccols;
              HfQuant hq(vb.t, p->global_scale, hf_mul_of(vb), p->x_qm_scale, p->b_qm_scale);
              get_block(1, vb, cy.data());
              get_block(0, vb, cx.data());
              get_block(2, vb, cb.data());
              lf_from_llf(cy.data(), nb, side, ly.data());
              lf_from_llf(cx.data(), nb, side, lxs.data());
              lf_from_llf(cb.data(), nb, side, lbs.data());
              for (int i = 0; i < nb * nb; ++i) {
                int32_t q;
                if (!lfq.quantize(ly[i], 1, &q)) return kErrQuant;
                float dy = lfq.reconstruct(q, 1);
                lx.push_back({lxs[i], dy, 0});
                lb.push_back({lbs[i], dy, 0});
                lrx.add(ly[i], lxs[i]);
                lrb.add(ly[i], lbs[i]);
              }
              int fold = side / 8;
              size_t tile = (size_t)(by / 8) * tw + (bx / 8);
              for (int row = 0; row < side; ++row) {
                int first = row < nb ? nb : 0;
                for (int col = first; col < side; ++col) {
                  int cell = row * side + col;
                  int32_t qy;
                  if (!hq.choose(cy[cell], 1, cell, &qy)) return kErrQuant;
                  float dy = hq.reconstruct(qy, 1, cell);
                  int cell8 = (row / fold) * 8 + (col / fold);
                  hx[tile].push_back({cx[cell], dy, cell8});
                  rx[tile].add(cy[cell], cx[cell]);
                  hb[tile].push_back({cb[cell], dy, cell8});
                  rb[tile].add(cy[cell], cb[cell]);
                }
              }
            }
      }
    int xf, bf;
    if (!refine_lf(lx, lrx, lb, lrb, lfq, &xf, &bf)) return kErrQuant;
    x_lf = xf;
    b_lf = bf;
    TransformInfo t8;
    transform_info(0, &t8);
    // Baseline DCT8x8 quantizer at the frame's hf_mul (AQ off).
    HfQuant base(t8, p->global_scale, hf_mul_blocks[0], p->x_qm_scale, p->b_qm_scale);
    for (size_t t = 0; t < tx.size(); ++t) {
      int f;
      if (!refine_hf(hx[t], rx[t], 0.0f, 0, base, &f)) return kErrQuant;
      tx[t] = (int8_t)f;
      if (!refine_hf(hb[t], rb[t], 1.0f, 2, base, &f)) return kErrQuant;
      tb[t] = (int8_t)f;
    }
  }
  if (cfl_x) std::memcpy(cfl_x, tx.data(), tx.size());
  if (cfl_b) std::memcpy(cfl_b, tb.data(), tb.size());
  if (lf_cfl) {
    lf_cfl->x_factor_lf = x_lf + 128;
    lf_cfl->b_factor_lf = b_lf + 128;
  }

  // --- quantization: lib.rs:3237 quantize_square_varblock ---
  const float k_x_lf = cfl_multiplier(0.0f, x_lf, 84);
  const float k_b_lf = cfl_multiplier(1.0f, b_lf, 84);
  std::vector<float> cblk[3], lfs(16), dylf(16), dyhf(1024), targets(1024);
  for (auto& v : cblk) v.resize(1024);
  if (qcoeff_out) std::fill(qcoeff_out, qcoeff_out + 3 * plane8, 0);
  if (lf_out) std::fill(lf_out, lf_out + 3 * (size_t)bw * bh, 0);
  for (auto& vb : vbs) {
    int nb = vb.t.brows, side = vb.t.ccols, cells = side * side;
    HfQuant hq(vb.t, p->global_scale, hf_mul_of(vb), p->x_qm_scale, p->b_qm_scale);
    size_t tile = (size_t)(vb.by / 8) * tw + (vb.bx / 8);
    float k_x_hf = cfl_multiplier(0.0f, tx[tile], 84);
    float k_b_hf = cfl_multiplier(1.0f, tb[tile], 84);
    for (int c = 0; c < 3; ++c) get_block(c, vb, cblk[c].data());
    int32_t q;
    // Y
    lf_from_llf(cblk[1].data(), nb, side, lfs.data());
    for (int i = 0; i < nb * nb; ++i) {
      if (!lfq.quantize(lfs[i], 1, &q)) return kErrQuant;
      if (lf_out) lf_out[1 * (size_t)bw * bh + (size_t)(vb.by + i / nb) * bw + vb.bx + i % nb] = q;
      dylf[i] = lfq.reconstruct(q, 1);
    }
    for (int cell = 0; cell < cells; ++cell) {
      int row = cell / side, col = cell % side;
      if (row < nb && col < nb) {
        q = 0;
        dyhf[cell] = hq.reconstruct(0, 1, cell);
      } else {
        if (!hq.choose(cblk[1][cell], 1, cell, &q)) return kErrQuant;
        dyhf[cell] = hq.reconstruct(q, 1, cell);
      }
      if (qcoeff_out) qcoeff_out[1 * plane8 + coeff_index(vb, row, col, W8)] = q;
    }
    // X then B
    for (int c : {0, 2}) {
      float k_lf = c == 0 ? k_x_lf : k_b_lf;
      float k_hf = c == 0 ? k_x_hf : k_b_hf;
      lf_from_llf(cblk[c].data(), nb, side, lfs.data());
      for (int i = 0; i < nb * nb; ++i) {
        float target = lfs[i] - k_lf * dylf[i];
        if (!lfq.quantize(target, c, &q)) return kErrQuant;
        if (lf_out) lf_out[(size_t)c * bw * bh + (size_t)(vb.by + i / nb) * bw + vb.bx + i % nb] = q;
      }
      for (int cell = 0; cell < cells; ++cell) {
        int row = cell / side, col = cell % side;
        if (row < nb && col < nb) {
          q = 0;
        } else {
          float target = cblk[c][cell] - k_hf * dyhf[cell];
          if (!hq.choose(target, c, cell, &q)) return kErrQuant;
        }
        if (qcoeff_out) qcoeff_out[c * plane8 + coeff_index(vb, row, col, W8)] = q;
      }
    }
  }
  return kOk;
}

// ---------------------------------------------------------------------------
// Reconstruct: plan-render lib.rs:749 render_inner (canonical, not decimated).
// ---------------------------------------------------------------------------

extern "C" int orc_reconstruct(int w, int h, const uint8_t* block_map,
                               const uint32_t* hf_mul_blocks, const uint8_t* sharpness,
                               const int32_t* qcoeff, const int32_t* lf, const int8_t* cfl_x,
                               const int8_t* cfl_b, const orc_render_params* p, int out_kind,
                               int bits, void* out) {
  if (w <= 0 || h <= 0 || p->epf_iters > 3) return kErrShape;
  const int bw = (w + 7) / 8, bh = (h + 7) / 8, W8 = bw * 8;
  const int tw = (bw + 7) / 8;
  std::vector<Varblock> vbs;
  int rc = parse_block_map(block_map, bw, bh, &vbs);
  if (rc) return rc;
  const size_t n = (size_t)w * h, nb_blocks = (size_t)bw * bh, plane8 = (size_t)W8 * bh * 8;
  const float qm[3] = {qm_multiplier(p->x_qm_scale), 1.0f, qm_multiplier(p->b_qm_scale)};
  // reconstruct.rs:67 lf_multipliers with G.1.2 default weights / 128.
  float lf_mul[3];
  {
    static const float wts[3] = {1.0f / 32.0f, 1.0f / 4.0f, 1.0f / 2.0f};
    double denom = (double)p->global_scale * (double)p->quant_lf;
    for (int c = 0; c < 3; ++c) {
      float wc = wts[c] / 128.0f;
      lf_mul[c] = denom > 0.0 ? (float)(65536.0 * (double)wc / denom) : 0.0f;
    }
  }
  const float k_x_lf = cfl_multiplier(0.0f, p->x_factor_lf - 128, 84);
  const float k_b_lf = cfl_multiplier(1.0f, p->b_factor_lf - 128, 84);
  // lf_planes (lib.rs:1314): dequantize (reconstruct.rs:84) then LF CfL.
  std::vector<float> lfd(3 * nb_blocks);
  for (size_t i = 0; i < nb_blocks; ++i) {
    float d[3];
    for (int c = 0; c < 3; ++c) d[c] = lf_mul[c] * (float)lf[c * nb_blocks + i] / 1.0f;
    lfd[i] = d[0] + k_x_lf * d[1];
    lfd[nb_blocks + i] = d[1];
    lfd[2 * nb_blocks + i] = d[2] + k_b_lf * d[1];
  }
  std::vector<float> planes(3 * n, 0.0f), sigma(nb_blocks, 0.0f);
  std::vector<float> co[3], samp(1024), rect(16);
  for (auto& v : co) v.resize(1024);
  for (auto& vb : vbs) {
    const int rows = vb.t.crows, cols = vb.t.ccols;
    const uint32_t hf_mul = hf_mul_blocks[(size_t)vb.by * bw + vb.bx];
    const float mul = hf_multiplier(p->global_scale, hf_mul);
    for (int c = 0; c < 3; ++c) {
      const float* m = dequant_matrix_cached(vb.t.dq_index, c);
      float scale = mul * qm[c];
      for (int y = 0; y < rows; ++y)
        for (int x = 0; x < cols; ++x) {
          int32_t q = qcoeff[c * plane8 + coeff_index(vb, y, x, W8)];
          float adjusted = bias_adjust(q, kQuantBias[c], kQuantBiasNumerator);
          co[c][y * cols + x] = adjusted * scale * m[y * cols + x];
        }
    }
    size_t tile = (size_t)(vb.by / 8) * tw + (vb.bx / 8);
    float k_x = cfl_multiplier(0.0f, cfl_x[tile], 84);
    float k_b = cfl_multiplier(1.0f, cfl_b[tile], 84);
    for (int i = 0; i < rows * cols; ++i) {  // lib.rs:1344 apply_hf_cfl
      float dy = co[1][i];
      co[0][i] = co[0][i] + k_x * dy;
      co[2][i] = co[2][i] + k_b * dy;
    }
    // I.8 llf_from_lf (varblock.rs:817): LF rect in image orientation,
    // transposed for a portrait varblock, DCT_2D, times scale_f.
    const int br = vb.t.brows, bc = vb.t.bcols;
    const int cx = std::max(br, bc), cy = std::min(br, bc);
    for (int c = 0; c < 3; ++c) {
      for (int dy = 0; dy < br; ++dy)
        for (int dx = 0; dx < bc; ++dx) {
          float v = lfd[c * nb_blocks + (size_t)(vb.by + dy) * bw + vb.bx + dx];
          if (br > bc) rect[dx * br + dy] = v; else rect[dy * bc + dx] = v;
        }
      dct_2d(rect.data(), cy, cx);
      for (int y = 0; y < cy; ++y)
        for (int x = 0; x < cx; ++x)
          co[c][y * cols + x] = rect[y * cx + x] * scale_f(y, cy) * scale_f(x, cx);
    }
    // I.9: IDCT_2D into samples of the varblock's own orientation, then the
    // in-frame scatter.
    const int srows = br * 8, scols = bc * 8;
    for (int c = 0; c < 3; ++c) {
      std::memcpy(samp.data(), co[c].data(), sizeof(float) * rows * cols);
      idct_2d(samp.data(), srows, scols);
      for (int y = 0; y < srows; ++y) {
        int fy = vb.by * 8 + y;
        if (fy >= h) continue;
        for (int x = 0; x < scols; ++x) {
          int fx = vb.bx * 8 + x;
          if (fx >= w) continue;
          planes[c * n + (size_t)fy * w + fx] = samp[y * scols + x];
        }
      }
    }
    for (int dy = 0; dy < br; ++dy)
      for (int dx = 0; dx < bc; ++dx) {
        size_t bi = (size_t)(vb.by + dy) * bw + vb.bx + dx;
        sigma[bi] = vardct_sigma(mul, std::min<int>(sharpness[bi], 7));
      }
  }
  if (out_kind == 4) {
    std::memcpy(out, planes.data(), sizeof(float) * 3 * n);
    return kOk;
  }
  std::vector<float> aux(3 * n);
  if (p->gaborish) {
    for (int c = 0; c < 3; ++c) gaborish(&planes[c * n], w, h, &aux[c * n]);
    planes.swap(aux);
  }
  static const int steps_for[4][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 2, -1}, {0, 1, 2}};
  for (int s = 0; s < 3; ++s) {
    int step = steps_for[p->epf_iters][s];
    if (step < 0) break;
    const float* in[3] = {&planes[0], &planes[n], &planes[2 * n]};
    float* o[3] = {&aux[0], &aux[n], &aux[2 * n]};
    epf_step(step, in, w, h, sigma.data(), o);
    planes.swap(aux);
  }
  if (out_kind == 0) {
    std::memcpy(out, planes.data(), sizeof(float) * 3 * n);
    return kOk;
  }
  // colour (lib.rs:1268): opsin inverse, then the output encoding.
  for (size_t i = 0; i < n; ++i) {
    float xyb[3] = {planes[i], planes[n + i], planes[2 * n + i]}, rgb[3];
    opsin_inverse(xyb, rgb);
    planes[i] = rgb[0];
    planes[n + i] = rgb[1];
    planes[2 * n + i] = rgb[2];
  }
  if (out_kind == 1) {
    std::memcpy(out, planes.data(), sizeof(float) * 3 * n);
    return kOk;
  }
  if (out_kind == 2) {
    uint8_t* o8 = (uint8_t*)out;
    for (size_t i = 0; i < n; ++i)
      for (int c = 0; c < 3; ++c) o8[3 * i + c] = (uint8_t)composed_level(planes[c * n + i], 255.0f);
    return kOk;
  }
  if (out_kind == 3) {
    float max = full_scale(bits);
    int levels = bits >= 32 ? 65536 : (1 << std::min(std::max(bits, 1), 16));
    std::vector<float> lut(levels);
    for (int q = 0; q < levels; ++q) lut[q] = srgb_to_linear((float)q / max);
    float* of = (float*)out;
    for (size_t i = 0; i < 3 * n; ++i) {
      int lvl = composed_level(planes[i], max);
      of[i] = lut[lvl];
    }
    return kOk;
  }
  return kErrParam;
}

// ---------------------------------------------------------------------------
// Cover selection (jpxl-encode-policy lib.rs:5260 select_blocks, :5115
// tile_region_with, :4909 block_cost_bounded, :4685 score_channel_lanes) for
// the fixed-quantizer request: adaptive quantization off (every HfMul is the
// baseline, its signal bits 0), the Legacy rate model (residual-bit scale 1,
// fixed bits 2 for DCT8x8 and 34 otherwise, request.rs:614), neutral size
// penalty, flat frequency weights and lambda scale 1.
// ---------------------------------------------------------------------------

namespace orc {

struct CoverCtx {
  const float* pre;  // 3 planes, w x h (the transform frame)
  int w, h;
  const HfQuant* quant[3];  // DCT8, DCT16, DCT32 at the baseline HfMul
  TransformInfo info[3];
  double lambda[3];
  std::vector<float> d_y;  // 32 x 32 luma reconstruction of the current candidate
  int64_t candidates = 0, pruned = 0;
};

// One channel of a candidate in the reference's order: rows, then the
// non-LLF columns; bits and the weighted error accumulate cell by cell and
// the cutoff is tested at the end of each row (lib.rs:4724-4800).
static bool score_channel(CoverCtx& cc, int ti, int c, const float* plane, float k,
                          bool luma_sink, double cutoff, bool has_cutoff, uint64_t* bits,
                          double* sse) {
  const TransformInfo& t = cc.info[ti];
  const int side = t.ccols, n = t.brows;
  const double flat_weight = cc.lambda[c] * ((double)(side * side) * 1.0);
  for (int row = 0; row < side; ++row) {
    for (int col = row < n ? n : 0; col < side; ++col) {
      const int cell = row * side + col;
      float target = luma_sink ? plane[cell] : plane[cell] - k * cc.d_y[cell];
      int32_t q;
      if (!cc.quant[ti]->choose(target, c, cell, &q)) return false;
      float recon = cc.quant[ti]->reconstruct(q, c, cell);
      if (luma_sink) cc.d_y[cell] = recon;
      *bits += residual_bits(q);
      double d = (double)(recon - target);
      *sse += flat_weight * (d * d);
    }
    if (has_cutoff && (double)*bits * 1.0 + *sse >= cutoff) return false;
  }
  return true;
}

// Returns false when pruned (or a cell fails, which the reference reports as
// an error; the encoder's covers never reach it).
static bool block_cost(CoverCtx& cc, int ti, int px, int py, double cutoff, bool has_cutoff,
                       double* cost) {
  const TransformInfo& t = cc.info[ti];
  const int side = t.ccols;
  Varblock vb{px / 8, py / 8, t};
  const size_t n = (size_t)cc.w * cc.h;
  std::vector<float> cf[3];
  for (int c = 0; c < 3; ++c) {
    cf[c].resize((size_t)side * side);
    forward_varblock(cc.pre + c * n, cc.w, cc.h, vb, cf[c].data());
  }
  ++cc.candidates;
  uint64_t bits = 0;
  double sse = 0.0;
  if (!score_channel(cc, ti, 1, cf[1].data(), 0.0f, true, cutoff, has_cutoff, &bits, &sse)) {
    ++cc.pruned;
    return false;
  }
  if (!score_channel(cc, ti, 0, cf[0].data(), 0.0f, false, cutoff, has_cutoff, &bits, &sse) ||
      !score_channel(cc, ti, 2, cf[2].data(), 1.0f, false, cutoff, has_cutoff, &bits, &sse)) {
    ++cc.pruned;
    return false;
  }
  *cost = (double)bits * 1.0 + sse;
  return true;
}

struct CoverBlock { int bx, by, ti; };

static double tile_region(CoverCtx& cc, int gbw, int gbh, int bx, int by, int size, int x0,
                          int y0, std::vector<CoverBlock>* out) {
  if (bx >= gbw || by >= gbh) return 0.0;
  if (size == 1) {
    double rd = 0.0;
    block_cost(cc, 0, x0 + bx * 8, y0 + by * 8, 0.0, false, &rd);
    out->push_back({bx, by, 0});
    return rd + 2.0 + 0.0;
  }
  const int half = size / 2;
  double split = 0.0;
  std::vector<CoverBlock> split_blocks;
  const int qx[4] = {bx, bx + half, bx, bx + half}, qy[4] = {by, by, by + half, by + half};
  for (int i = 0; i < 4; ++i) split += tile_region(cc, gbw, gbh, qx[i], qy[i], half, x0, y0,
                                                   &split_blocks);
  const bool fits = bx + size <= gbw && by + size <= gbh;
  if (fits) {
    const int ti = size == 2 ? 1 : 2;
    const double fixed = 34.0 + 0.0;
    if (!(fixed >= split)) {
      const double cutoff = split - fixed;
      double rd;
      if (block_cost(cc, ti, x0 + bx * 8, y0 + by * 8, cutoff, true, &rd)) {
        const double single = rd + fixed;
        if (single < split) {
          out->push_back({bx, by, ti});
          return single;
        }
      }
    }
  }
  out->insert(out->end(), split_blocks.begin(), split_blocks.end());
  return split;
}

}  // namespace orc

extern "C" int orc_select_blocks(const void* rgb, int w, int h, int bits,
                                 const orc_encode_params* p, uint8_t* block_map,
                                 int64_t* candidates_scored) {
  using namespace orc;
  if (w <= 0 || h <= 0 || !(bits == 8 || (bits >= 1 && bits <= 16))) return kErrShape;
  const int bw = (w + 7) / 8, bh = (h + 7) / 8;
  const size_t n = (size_t)w * h;
  std::vector<float> xyb(3 * n);
  source_to_xyb(rgb, w, h, bits, &xyb[0], &xyb[n], &xyb[2 * n]);
  std::vector<float> pre = xyb;
  if (p->gaborish)
    for (int c = 0; c < 3; ++c) gab_precondition(&xyb[c * n], w, h, &pre[c * n]);
  CoverCtx cc;
  cc.pre = pre.data();
  cc.w = w;
  cc.h = h;
  const int sels[3] = {0, 4, 5};
  std::vector<std::unique_ptr<HfQuant>> quants;
  for (int i = 0; i < 3; ++i) {
    transform_info(sels[i], &cc.info[i]);
    quants.emplace_back(new HfQuant(cc.info[i], p->global_scale, 1, p->x_qm_scale, p->b_qm_scale));
    cc.quant[i] = quants.back().get();
  }
  // lib.rs:2094: lambda = 16 / mean((8 * step)^2) over the DCT8x8 cells but
  // the DC, per channel.
  for (int c = 0; c < 3; ++c) {
    double sum = 0.0;
    uint32_t count = 0;
    for (int cell = 1; cell < 64; ++cell) {
      double step = 8.0 * (double)cc.quant[0]->steps[c][cell];
      sum += step * step;
      ++count;
    }
    double mean = sum / (double)std::max(count, 1u);
    cc.lambda[c] = mean > 0.0 ? 1.0 * 16.0 / mean : 0.0;
  }
  cc.d_y.assign(1024, 0.0f);
  std::memset(block_map, 0, (size_t)bw * bh);
  const int G = 256;  // LF group side in blocks
  for (int gy = 0; gy < (bh + G - 1) / G; ++gy)
    for (int gx = 0; gx < (bw + G - 1) / G; ++gx) {
      const int gbw = std::min(G, bw - gx * G), gbh = std::min(G, bh - gy * G);
      const int x0 = gx * G * 8, y0 = gy * G * 8;
      for (int sby = 0; sby < gbh; sby += 4)
        for (int sbx = 0; sbx < gbw; sbx += 4) {
          std::vector<CoverBlock> blocks;
          tile_region(cc, gbw, gbh, sbx, sby, 4, x0, y0, &blocks);
          for (const CoverBlock& b : blocks) {
            const TransformInfo& t = cc.info[b.ti];
            const int obx = gx * G + b.bx, oby = gy * G + b.by;
            for (int dy = 0; dy < t.brows; ++dy)
              for (int dx = 0; dx < t.bcols; ++dx)
                block_map[(size_t)(oby + dy) * bw + obx + dx] =
                    (uint8_t)(t.sel | ((dx == 0 && dy == 0) ? 0x80 : 0));
          }
        }
    }
  if (candidates_scored) *candidates_scored = cc.candidates;
  return kOk;
}
