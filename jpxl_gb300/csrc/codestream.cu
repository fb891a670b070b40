// codestream.cu — the host-side codestream reader declared in codestream.h.
// Follows ISO/IEC 18181-1 as jpxl-decode reads it; each part cites the
// reference file it restates (paths under JPXL/crates/jpxl-decode/src unless
// noted).  Supported: bare codestreams and containers, image headers without ICC profiles or
// previews, one frame; VarDCT frames without patches, splines or noise and
// modular sub-bitstreams without transforms (what cjxl writes for the VarDCT
// fixtures); modular frames whose channels all fit the global section.
// Anything else is reported as unsupported, never decoded wrongly.
#include "codestream.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>

#include "entropy.h"
#include "jpxlg.h"

namespace jpxlg {
namespace cs {
namespace {

using entropy::Bits;
using entropy::Stream;
using entropy::U32Dist;

[[noreturn]] void fail(const char* what) { throw Malformed{what}; }
void need(bool c, const char* what) {
  if (!c) fail(what);
}

// jpxl-core limits.rs max_alloc_bytes: every channel and plane the reader
// allocates for one stream is charged to a running total (as
// modular/channel.rs:106 charges each channel to the reference's meter), and
// the stream is rejected as malformed once the total would pass 4 GiB,
// before the allocation is made.  A header of a few bytes can otherwise
// declare planes whose zero-fill alone exhausts the host.
// The limits default to the reference's Limits::new() (limits.rs:38):
// 2^30 pixels, 4 GiB; jpxlg_codestream_open_limits sets them per stream.
thread_local uint64_t t_alloc_bytes = 0;
thread_local uint64_t t_max_alloc_bytes = 4ull << 30;
thread_local uint64_t t_max_pixels = 1ull << 30;
void charge(uint64_t count, uint64_t elem_bytes) {
  const uint64_t bytes = count * elem_bytes;
  need(count == 0 || bytes / count == elem_bytes, "allocation size");
  t_alloc_bytes += bytes;
  need(t_alloc_bytes >= bytes && t_alloc_bytes <= t_max_alloc_bytes,
       "the stream's planes exceed the allocation limit");
}

int32_t unpack_signed(uint32_t u) {
  return (u & 1) ? (int32_t)(-(int64_t)(u >> 1) - 1) : (int32_t)(u >> 1);
}
uint32_t ceil_log2(uint64_t n) {
  uint32_t b = 0;
  while (b < 64 && ((uint64_t)1 << b) < n) ++b;
  return b;
}

// ---- field readers (18181-1 4.2-4.4; jpxl-bitstream) ------------------------

struct Reader {
  Bits b;
  uint32_t bits(uint32_t n) {
    uint32_t v;
    need(b.read(n, &v), "truncated stream");
    return v;
  }
  bool flag() { return bits(1) != 0; }
  uint32_t u32(const U32Dist (&d)[4]) {
    uint32_t v;
    need(entropy::read_u32(b, d, &v), "truncated stream");
    return v;
  }
  uint64_t u64() {
    const uint32_t sel = bits(2);
    if (sel == 0) return 0;
    if (sel == 1) return 1 + bits(4);
    if (sel == 2) return 17 + bits(8);
    uint64_t v = bits(12);
    uint32_t shift = 12;
    while (flag()) {
      if (shift == 60) {
        v |= (uint64_t)bits(4) << 60;
        break;
      }
      v |= (uint64_t)bits(8) << shift;
      shift += 8;
    }
    return v;
  }
  float f16() {
    const uint32_t h = bits(16);
    const uint32_t e = (h >> 10) & 31, m = h & 1023;
    need(e != 31, "F16 infinity or NaN");
    const float v = e == 0 ? std::ldexp((float)m, -24) : std::ldexp((float)(m + 1024), (int)e - 25);
    return (h >> 15) ? -v : v;
  }
  uint32_t enumv() {
    static const U32Dist d[4] = {{0, 0}, {0, 1}, {4, 2}, {6, 18}};
    return u32(d);
  }
  void pad_to_byte() {
    const uint32_t r = (uint32_t)(b.pos & 7);
    if (r) need(bits(8 - r) == 0, "non-zero padding");
  }
  void skip(uint64_t n) {
    need(n <= b.size_bits - b.pos, "truncated stream");
    b.pos += (size_t)n;
  }
};

// D.2 SizeHeader (headers/size.rs:156).
void size_header(Reader& r, uint32_t* w, uint32_t* h) {
  static const U32Dist kDim[4] = {{9, 1}, {13, 1}, {18, 1}, {30, 1}};
  const bool div8 = r.flag();
  const uint32_t hh = div8 ? (r.bits(5) + 1) * 8 : r.u32(kDim);
  const uint32_t ratio = r.bits(3);
  uint64_t ww;
  if (ratio == 0) {
    ww = div8 ? (r.bits(5) + 1) * 8 : r.u32(kDim);
  } else {
    static const uint32_t num[8] = {0, 1, 12, 4, 3, 16, 5, 2}, den[8] = {1, 1, 10, 3, 2, 9, 4, 1};
    ww = (uint64_t)hh * num[ratio] / den[ratio];
  }
  need(ww >= 1 && ww <= 0x3fffffff && hh >= 1, "image dimensions");
  *w = (uint32_t)ww;
  *h = hh;
}

void preview_header(Reader& r) {
  static const U32Dist k8[4] = {{0, 16}, {0, 32}, {5, 1}, {9, 33}};
  static const U32Dist kd[4] = {{6, 1}, {8, 65}, {10, 321}, {12, 1345}};
  const bool div8 = r.flag();
  if (div8) r.u32(k8);
  else r.u32(kd);
  if (r.bits(3) == 0) {
    if (div8) r.u32(k8);
    else r.u32(kd);
  }
}

// headers/bit_depth.rs:112.
void bit_depth(Reader& r, uint32_t* bits, uint32_t* exp_bits, bool* fl) {
  *fl = r.flag();
  if (!*fl) {
    static const U32Dist d[4] = {{0, 8}, {0, 10}, {0, 12}, {6, 1}};
    *bits = r.u32(d);
    *exp_bits = 0;
  } else {
    static const U32Dist d[4] = {{0, 32}, {0, 16}, {0, 24}, {6, 1}};
    *bits = r.u32(d);
    *exp_bits = r.bits(4) + 1;
  }
}

void extensions(Reader& r) {
  const uint64_t ext = r.u64();
  uint64_t total = 0;
  for (int i = 0; i < 64; ++i)
    if ((ext >> i) & 1) {
      const uint64_t n = r.u64();
      need(total + n >= total, "extension size");
      total += n;
    }
  r.skip(total);
}

// headers/extra_channels.rs:154.
void extra_channel(Reader& r, ImageInfo::Extra* ec) {
  *ec = ImageInfo::Extra{};
  if (r.flag()) return;  // all_default: 8-bit alpha
  const uint32_t type = r.enumv();
  uint32_t b, e;
  bool f;
  bit_depth(r, &b, &e, &f);
  need(!f, "floating-point extra channels are not supported");
  static const U32Dist kShift[4] = {{0, 0}, {0, 3}, {0, 4}, {3, 1}};
  static const U32Dist kName[4] = {{0, 0}, {4, 0}, {5, 16}, {10, 48}};
  ec->type = type;
  ec->bits = b;
  ec->dim_shift = r.u32(kShift);
  r.skip(8ull * r.u32(kName));
  if (type == 0) r.flag();  // alpha_associated
  if (type == 2)
    for (int i = 0; i < 4; ++i) r.f16();  // spot colour
  if (type == 5) {
    static const U32Dist kCfa[4] = {{0, 1}, {2, 0}, {4, 3}, {8, 19}};
    r.u32(kCfa);
  }
}

// headers/colour.rs:203.
void colour_encoding(Reader& r, ImageInfo* m) {
  if (r.flag()) return;  // sRGB
  m->want_icc = r.flag();
  m->colour_space = (int)r.enumv();
  const bool use_desc = !m->want_icc, not_xyb = m->colour_space != 2;
  static const U32Dist kXy[4] = {{19, 0}, {19, 524288}, {20, 1048576}, {21, 2097152}};
  if (use_desc && not_xyb) {
    if (r.enumv() == 2) {
      r.u32(kXy);
      r.u32(kXy);
    }
  }
  if (use_desc && not_xyb && m->colour_space != 1) {
    if (r.enumv() == 2)
      for (int i = 0; i < 6; ++i) r.u32(kXy);
  }
  if (use_desc) {
    if (r.flag()) {
      m->transfer = -1;
      m->gamma = r.bits(24);
    } else {
      m->transfer = (int)r.enumv();
    }
    r.enumv();  // rendering intent
  }
}

// headers/metadata.rs:286 (with the CustomTransformData tail, opsin.rs:85).
void image_metadata(Reader& r, ImageInfo* m, bool* preview, bool* animation, bool* timecodes) {
  for (int i = 0; i < 9; ++i) m->opsin_inv[i] = 0.0f;
  const bool all_default = r.flag();
  if (!all_default) {
    const bool extra_fields = r.flag();
    if (extra_fields) {
      m->orientation = r.bits(3) + 1;
      if (r.flag()) {
        uint32_t a, b;
        size_header(r, &a, &b);
      }
      if ((*preview = r.flag())) preview_header(r);
      if ((*animation = r.flag())) {
        static const U32Dist kNum[4] = {{0, 100}, {0, 1000}, {10, 1}, {30, 1}};
        static const U32Dist kDen[4] = {{0, 1}, {0, 1001}, {8, 1}, {10, 1}};
        static const U32Dist kLoops[4] = {{0, 0}, {3, 0}, {16, 0}, {32, 0}};
        r.u32(kNum);
        r.u32(kDen);
        r.u32(kLoops);
        *timecodes = r.flag();
      }
    }
    bit_depth(r, &m->bits_per_sample, &m->exp_bits, &m->float_sample);
    r.flag();  // modular_16bit_buffers
    static const U32Dist kExtra[4] = {{0, 0}, {0, 1}, {4, 2}, {12, 1}};
    m->num_extra = r.u32(kExtra);
    need(m->num_extra <= 256, "extra channel count");
    m->extra.resize(m->num_extra);
    for (uint32_t i = 0; i < m->num_extra; ++i) extra_channel(r, &m->extra[i]);
    m->xyb_encoded = r.flag();
    colour_encoding(r, m);
    if (extra_fields && !r.flag()) {  // tone mapping
      m->intensity_target = r.f16();
      r.f16();
      r.flag();
      r.f16();
    }
    extensions(r);
  }
  if (!r.flag()) {  // default_m
    if (m->xyb_encoded && !r.flag()) {
      m->default_opsin = false;
      for (int i = 0; i < 9; ++i) m->opsin_inv[i] = r.f16();
      for (int i = 0; i < 3; ++i) m->opsin_bias[i] = r.f16();
      for (int i = 0; i < 4; ++i) m->quant_bias[i] = r.f16();
    }
    const uint32_t cw = r.bits(3);
    if (cw & 1) r.skip(16ull * 15);
    if (cw & 2) r.skip(16ull * 55);
    if (cw & 4) r.skip(16ull * 210);
  }
}

// frame/restoration.rs:196 (the extensions bundle is skipped).
void restoration_filter(Reader& r, FrameInfo* f) {
  const bool all_default = r.flag();
  f->gab = all_default ? true : r.flag();
  f->gab_custom = (f->gab && !all_default) ? r.flag() : false;
  if (f->gab_custom)
    for (int c = 0; c < 3; ++c) {
      f->gab_w1[c] = r.f16();
      f->gab_w2[c] = r.f16();
    }
  if (all_default) return;
  f->epf_iters = r.bits(2);
  if (f->epf_iters) {
    if (f->encoding == 0 && r.flag())
      for (int i = 0; i < 8; ++i) f->epf_sharp_lut[i] = r.f16();
    if (r.flag()) {
      for (int c = 0; c < 3; ++c) f->epf_channel_scale[c] = r.f16();
      r.bits(32);
    }
    if (r.flag()) {
      if (f->encoding == 0) f->epf_quant_mul = r.f16();
      f->epf_pass0_sigma_scale = r.f16();
      f->epf_pass2_sigma_scale = r.f16();
      f->epf_border_sad_mul = r.f16();
    }
    if (f->encoding == 1) r.f16();  // sigma for modular
  }
  extensions(r);
}

// frame/header.rs:451 with passes.rs:124 and blending.rs:124.
void frame_header(Reader& r, const ImageInfo& m, bool animation, bool timecodes, FrameInfo* f) {
  f->width = m.width;
  f->height = m.height;
  f->pass_shift.assign(1, 0);
  const bool all_default = r.flag();
  if (all_default) {
    f->x_qm_scale = m.xyb_encoded ? 3 : 2;
    return;
  }
  f->frame_type = (int)r.bits(2);
  f->encoding = (int)r.bits(1);
  f->flags = r.u64();
  bool ycbcr = false;
  if (!m.xyb_encoded) ycbcr = r.flag();
  const bool use_lf_frame = (f->flags & 32) != 0;
  if (ycbcr && !use_lf_frame)
    for (int i = 0; i < 3; ++i) r.bits(2);
  need(!ycbcr, "YCbCr frames are not supported");
  static const U32Dist kUp[4] = {{0, 1}, {0, 2}, {0, 4}, {0, 8}};
  if (!use_lf_frame) {
    f->upsampling = r.u32(kUp);
    for (uint32_t i = 0; i < m.num_extra; ++i) r.u32(kUp);
  }
  if (f->encoding == 1) f->group_size_shift = r.bits(2);
  f->x_qm_scale = (m.xyb_encoded && f->encoding == 0) ? 3 : 2;
  if (m.xyb_encoded && f->encoding == 0) {
    f->x_qm_scale = r.bits(3);
    f->b_qm_scale = r.bits(3);
  }
  if (f->frame_type != 2) {
    static const U32Dist kPasses[4] = {{0, 1}, {0, 2}, {0, 3}, {3, 4}};
    static const U32Dist kDs[4] = {{0, 0}, {0, 1}, {0, 2}, {1, 3}};
    static const U32Dist kDown[4] = {{0, 1}, {0, 2}, {0, 4}, {0, 8}};
    static const U32Dist kLast[4] = {{0, 0}, {0, 1}, {0, 2}, {3, 0}};
    f->num_passes = r.u32(kPasses);
    if (f->num_passes > 1) {
      const uint32_t num_ds = r.u32(kDs);
      need(num_ds < f->num_passes, "num_ds");
      f->pass_shift.assign(f->num_passes, 0);
      for (uint32_t i = 0; i + 1 < f->num_passes; ++i) f->pass_shift[i] = r.bits(2);
      for (uint32_t i = 0; i < num_ds; ++i) r.u32(kDown);
      for (uint32_t i = 0; i < num_ds; ++i) r.u32(kLast);
    }
  }
  if (f->frame_type == 1) f->lf_level = r.bits(2) + 1;
  bool have_crop = false;
  if (f->frame_type != 1) have_crop = r.flag();
  int64_t x0 = 0, y0 = 0;
  uint32_t cw = f->width, ch = f->height;
  if (have_crop) {
    static const U32Dist kCrop[4] = {{8, 0}, {11, 256}, {14, 2304}, {30, 18688}};
    if (f->frame_type != 2) {
      x0 = unpack_signed(r.u32(kCrop));
      y0 = unpack_signed(r.u32(kCrop));
    }
    cw = r.u32(kCrop);
    ch = r.u32(kCrop);
  }
  need(!have_crop || (x0 == 0 && y0 == 0 && cw == f->width && ch == f->height),
       "cropped frames are not supported");
  const bool normal = f->frame_type == 0 || f->frame_type == 3;
  const bool full = true;
  static const U32Dist kMode[4] = {{0, 0}, {0, 1}, {0, 2}, {2, 3}};
  static const U32Dist kAlpha[4] = {{0, 0}, {0, 1}, {0, 2}, {3, 3}};
  uint32_t mode = 0;
  uint32_t duration = 0, save_as_reference = 0;
  if (normal) {
    const bool extra = m.num_extra >= 1;
    for (uint32_t i = 0; i <= m.num_extra; ++i) {
      const uint32_t md = r.u32(kMode);
      if (i == 0) mode = md;
      if (extra && (md == 2 || md == 3)) r.u32(kAlpha);
      if (extra && (md == 2 || md == 3 || md == 4)) r.flag();
      const bool resets = full && mode == 0;  // shared across the bundles
      if (!resets) r.bits(2);                 // source
    }
    static const U32Dist kDuration[4] = {{0, 0}, {0, 1}, {8, 0}, {32, 0}};
    if (animation) duration = r.u32(kDuration);
    if (timecodes) r.bits(32);
    f->is_last = r.flag();
  } else {
    f->is_last = f->frame_type == 0;
  }
  if (f->frame_type != 1 && !f->is_last) save_as_reference = r.bits(2);
  const bool resets_canvas = full && mode == 0;
  const bool can_reference =
      !f->is_last && (duration == 0 || save_as_reference != 0) && f->frame_type != 1;
  if (f->frame_type == 2 || (resets_canvas && can_reference)) r.flag();  // save_before_ct
  static const U32Dist kNameLen[4] = {{0, 0}, {4, 0}, {5, 16}, {10, 48}};
  r.skip(8ull * r.u32(kNameLen));
  restoration_filter(r, f);
  extensions(r);
}

// frame/toc.rs:213, used by the TOC and the coefficient orders.
int perm_context(uint32_t x) { return (int)std::min<uint32_t>(7, ceil_log2((uint64_t)x + 1)); }

std::vector<uint32_t> read_permutation(Reader& r, Stream& s, uint32_t size, uint32_t skip) {
  need(skip <= size, "permutation skip");
  uint32_t end;
  need(s.read(r.b, (size_t)perm_context(size), &end), "permutation");
  need(end <= size - skip, "permutation end");
  std::vector<uint32_t> lehmer(size, 0);
  uint32_t prev = 0;
  for (uint32_t i = skip; i < skip + end; ++i) {
    uint32_t v;
    need(s.read(r.b, (size_t)perm_context(i > skip ? prev : 0), &v), "permutation");
    need(v < size - i, "Lehmer code");
    lehmer[i] = v;
    prev = v;
  }
  std::vector<uint32_t> temp(size), perm;
  for (uint32_t i = 0; i < size; ++i) temp[i] = i;
  perm.reserve(size);
  for (uint32_t code : lehmer) {
    perm.push_back(temp[code]);
    temp.erase(temp.begin() + code);
  }
  return perm;
}

// ---- modular sub-bitstreams (modular/mod.rs, tree.rs, predictor.rs,
// jpxl-core modular_weighted.rs) --------------------------------------------

struct TreeNode {
  bool leaf;
  uint32_t property;
  int32_t value;
  uint32_t left, right;
  uint32_t ctx;
  uint32_t predictor;
  int32_t offset;
  int64_t mul;
};

struct Tree {
  std::vector<TreeNode> nodes;
  uint32_t num_leaves = 0;
  const TreeNode& lookup(const int32_t* props, size_t nprops) const {
    size_t i = 0;
    for (size_t guard = 0; guard <= nodes.size(); ++guard) {
      const TreeNode& n = nodes[i];
      if (n.leaf) return n;
      const int32_t p = n.property < nprops ? props[n.property] : 0;
      i = p > n.value ? n.left : n.right;
    }
    fail("MA tree traversal");
  }
};

// H.4.2 (tree.rs:265): nodes in queue order, children after every pending node.
Tree read_tree(Reader& r) {
  Stream s;
  need(s.open(r.b, 6, 0, false), "MA tree histograms");
  Tree t;
  size_t pending = 1;
  while (pending > 0) {
    --pending;
    need(t.nodes.size() < (1u << 22), "MA tree size");
    uint32_t p;
    need(s.read(r.b, 1, &p), "MA tree");
    TreeNode n{};
    if (p > 0) {
      uint32_t v;
      need(s.read(r.b, 0, &v), "MA tree");
      n.leaf = false;
      n.property = p - 1;
      n.value = unpack_signed(v);
      n.left = (uint32_t)(t.nodes.size() + pending + 1);
      n.right = n.left + 1;
      pending += 2;
    } else {
      uint32_t pred, off, mul_log, mul_bits;
      need(s.read(r.b, 2, &pred) && s.read(r.b, 3, &off) && s.read(r.b, 4, &mul_log) &&
               s.read(r.b, 5, &mul_bits),
           "MA tree");
      need(pred <= 13, "predictor");
      need(mul_log <= 30, "mul_log");
      need(mul_bits <= (1u << (31 - mul_log)) - 2, "mul_bits");
      n.leaf = true;
      n.predictor = pred;
      n.offset = unpack_signed(off);
      n.mul = (int64_t)(mul_bits + 1) << mul_log;
      n.ctx = t.num_leaves++;
    }
    t.nodes.push_back(n);
  }
  need(s.final_state(), "MA tree final state");
  for (const TreeNode& n : t.nodes)
    if (!n.leaf) need(n.right < t.nodes.size(), "MA tree child");
  return t;
}

struct WpHeader {
  int64_t p1 = 16, p2 = 10, p3[5] = {7, 7, 7, 0, 0}, w[4] = {13, 12, 12, 12};
};

WpHeader read_wp(Reader& r) {
  WpHeader h;
  if (r.flag()) return h;
  h.p1 = r.bits(5);
  h.p2 = r.bits(5);
  for (auto& v : h.p3) v = r.bits(5);
  for (auto& v : h.w) v = r.bits(4);
  return h;
}

struct Neighbours {
  int64_t w, n, nw, ne, nn, nee, ww;
};

// predictor.rs:172.
Neighbours gather(const Channel& c, uint32_t x, uint32_t y) {
  auto at = [&](uint32_t cx, uint32_t cy) { return (int64_t)c.at(cx, cy); };
  Neighbours nb;
  nb.w = x > 0 ? at(x - 1, y) : (y > 0 ? at(x, y - 1) : 0);
  nb.n = y > 0 ? at(x, y - 1) : nb.w;
  nb.nw = (x > 0 && y > 0) ? at(x - 1, y - 1) : nb.w;
  nb.ne = (x + 1 < c.w && y > 0) ? at(x + 1, y - 1) : nb.n;
  nb.nn = y > 1 ? at(x, y - 2) : nb.n;
  nb.nee = (x + 2 < c.w && y > 0) ? at(x + 2, y - 1) : nb.ne;
  nb.ww = x > 1 ? at(x - 2, y) : nb.w;
  return nb;
}

int64_t gradient(int64_t w, int64_t n, int64_t nw) {
  return std::min(std::max(w + n - nw, std::min(w, n)), std::max(w, n));
}

int64_t predict(const Neighbours& nb, uint32_t p, int64_t weighted) {
  switch (p) {
    case 0: return 0;
    case 1: return nb.w;
    case 2: return nb.n;
    case 3: return (nb.w + nb.n) / 2;
    case 4: return std::llabs(nb.n - nb.nw) < std::llabs(nb.w - nb.nw) ? nb.w : nb.n;
    case 5: return gradient(nb.w, nb.n, nb.nw);
    case 6: return (weighted + 3) >> 3;
    case 7: return nb.ne;
    case 8: return nb.nw;
    case 9: return nb.ww;
    case 10: return (nb.w + nb.nw) / 2;
    case 11: return (nb.n + nb.nw) / 2;
    case 12: return (nb.n + nb.ne) / 2;
    default: return (6 * nb.n - 2 * nb.nn + 7 * nb.w + nb.ww + nb.nee + 3 * nb.ne + 8) / 16;
  }
}

uint32_t floor_log2(uint64_t v) { return 63u - (uint32_t)__builtin_clzll(v); }

int64_t error2weight(uint32_t err_sum, int64_t maxweight) {
  const uint32_t l = floor_log2((uint64_t)err_sum + 1);
  const uint32_t shift = l > 5 ? l - 5 : 0;
  const int64_t denom = (int64_t)(err_sum >> shift) + 1;
  return 4 + ((maxweight * ((1ll << 24) / denom)) >> shift);
}

// H.5 self-correcting predictor, one channel row pair at a time
// (modular_weighted.rs: the reference's readings of H.5.2 are kept: the true
// error uses the clamped prediction, max_error takes the larger magnitude,
// and the last column adds the west error twice).
struct Weighted {
  struct Entry {
    int32_t true_err = 0;
    uint64_t err[4] = {0, 0, 0, 0};
  };
  uint32_t width;
  std::vector<Entry> prev, curr;
  bool has_prev = false;
  int64_t sub[4];
  int64_t prediction = 0;
  int32_t max_error = 0;
  explicit Weighted(uint32_t w) : width(w), prev(w), curr(w) {}

  void run(const WpHeader& h, const Neighbours& nb, uint32_t x) {
    const int64_t n3 = nb.n * 8, nw3 = nb.nw * 8, ne3 = nb.ne * 8, w3 = nb.w * 8, nn3 = nb.nn * 8;
    const int64_t te_w = x > 0 ? curr[x - 1].true_err : 0;
    const int64_t te_n = has_prev ? prev[x].true_err : 0;
    const int64_t te_nw = (x > 0 && has_prev) ? prev[x - 1].true_err : te_n;
    const int64_t te_ne = (x + 1 < width && has_prev) ? prev[x + 1].true_err : te_n;
    sub[0] = w3 + ne3 - n3;
    sub[1] = n3 - (((te_w + te_n + te_ne) * h.p1) >> 5);
    sub[2] = w3 - (((te_w + te_n + te_nw) * h.p2) >> 5);
    sub[3] = n3 - ((te_nw * h.p3[0] + te_n * h.p3[1] + te_ne * h.p3[2] + (nn3 - n3) * h.p3[3] +
                    (nw3 - w3) * h.p3[4]) >>
                   5);
    int64_t weight[4];
    for (int i = 0; i < 4; ++i) {
      const uint64_t en = has_prev ? prev[x].err[i] : 0;
      const uint64_t ew = x > 0 ? curr[x - 1].err[i] : 0;
      const uint64_t enw = (x > 0 && has_prev) ? prev[x - 1].err[i] : en;
      const uint64_t eww = x > 1 ? curr[x - 2].err[i] : 0;
      const uint64_t ene = (x + 1 < width && has_prev) ? prev[x + 1].err[i] : en;
      uint64_t sum = en + ew + enw + eww + ene;
      if (x + 1 == width) sum += ew;
      weight[i] = error2weight((uint32_t)sum, h.w[i]);
    }
    int64_t sw = weight[0] + weight[1] + weight[2] + weight[3];
    const uint32_t lw = floor_log2((uint64_t)std::max<int64_t>(sw, 1)) + 1;
    const uint32_t shift = lw > 5 ? lw - 5 : 0;
    for (auto& v : weight) v >>= shift;
    sw = weight[0] + weight[1] + weight[2] + weight[3];
    const int64_t divisor = std::max<int64_t>(sw, 1);
    int64_t s = (sw >> 1) - 1;
    for (int i = 0; i < 4; ++i) s += sub[i] * weight[i];
    const __int128 wide = ((__int128)s * (__int128)((1ll << 24) / divisor)) >> 24;
    prediction = (int64_t)wide;
    if (((te_n ^ te_w) | (te_n ^ te_nw)) <= 0)
      prediction = std::min(std::max(prediction, std::min(w3, std::min(n3, ne3))),
                            std::max(w3, std::max(n3, ne3)));
    int64_t me = te_w;
    for (int64_t c : {te_n, te_nw, te_ne})
      if (std::llabs(c) > std::llabs(me)) me = c;
    max_error = (int32_t)me;
  }
  void update(uint32_t x, int32_t value) {
    const int64_t shifted = (int64_t)value * 8;
    Entry& e = curr[x];
    e.true_err = (int32_t)(prediction - shifted);
    for (int i = 0; i < 4; ++i) e.err[i] = (uint64_t)((std::llabs(sub[i] - shifted) + 3) >> 3);
  }
  void next_row() {
    std::swap(prev, curr);
    std::fill(curr.begin(), curr.end(), Entry{});
    has_prev = true;
  }
};

struct GlobalTree {
  bool present = false;
  Tree tree;
  Stream dists;
};

// H.6 transforms (modular/transform.rs, squeeze.rs, rct.rs, palette.rs).
struct SqueezeStep {
  bool horizontal, in_place;
  uint32_t begin_c, num_c;
};
struct ModTransform {
  int kind = 0;  // 0 RCT, 1 palette, 2 squeeze
  uint32_t begin_c = 0, rct_type = 0;
  uint32_t num_c = 0, nb_colours = 0, nb_deltas = 0, d_pred = 0;  // palette
  std::vector<SqueezeStep> steps;
};

// Table H.10, the delta palette (standard data, as jpxl-decode
// modular/palette.rs prints it).
const int16_t kDeltaPalette[72][3] = {
    {0, 0, 0}, {4, 4, 4}, {11, 0, 0}, {0, 0, -13}, {0, -12, 0}, {-10, -10, -10},
    {-18, -18, -18}, {-27, -27, -27}, {-18, -18, 0}, {0, 0, -32}, {-32, 0, 0}, {-37, -37, -37},
    {0, -32, -32}, {24, 24, 45}, {50, 50, 50}, {-45, -24, -24}, {-24, -45, -45}, {0, -24, -24},
    {-34, -34, 0}, {-24, 0, -24}, {-45, -45, -24}, {64, 64, 64}, {-32, 0, -32}, {0, -32, 0},
    {-32, 0, 32}, {-24, -45, -24}, {45, 24, 45}, {24, -24, -45}, {-45, -24, 24}, {80, 80, 80},
    {64, 0, 0}, {0, 0, -64}, {0, -64, -64}, {-24, -24, 45}, {96, 96, 96}, {64, 64, 0},
    {45, -24, -24}, {34, -34, 0}, {112, 112, 112}, {24, -45, -45}, {45, 45, -24}, {0, -32, 32},
    {24, -24, 45}, {0, 96, 96}, {45, -24, 24}, {24, -45, -24}, {-24, -45, 24}, {0, -64, 0},
    {96, 0, 0}, {128, 128, 128}, {64, 0, 64}, {144, 144, 144}, {96, 96, 0}, {-36, -36, 36},
    {45, -24, -45}, {45, -45, -24}, {0, 0, -96}, {0, 128, 128}, {0, 96, 0}, {45, 24, -45},
    {-128, 0, 0}, {24, -45, 24}, {-45, 24, -45}, {64, 0, -64}, {64, -64, -64}, {96, 0, 96},
    {45, -45, 24}, {24, 45, -45}, {64, 64, -64}, {128, 128, 0}, {0, 0, -128}, {-24, 45, -45},
};


// squeeze.rs default_params: a channel pair split first, then halvings
// until both dimensions are at most 8.
std::vector<SqueezeStep> default_squeeze(const std::vector<Channel>& ch, size_t nb_meta) {
  need(ch.size() > nb_meta, "default squeeze without channels");
  std::vector<SqueezeStep> sp;
  const uint32_t first = (uint32_t)nb_meta;
  uint32_t w = ch[first].w, h = ch[first].h;
  const uint32_t count = (uint32_t)(ch.size() - nb_meta);
  if (count > 2 && ch[first + 1].w == w && ch[first + 1].h == h) {
    sp.push_back({true, false, first + 1, 2});
    sp.push_back({false, false, first + 1, 2});
  }
  if (h >= w && h > 8) {
    sp.push_back({false, true, first, count});
    h = (h + 1) / 2;
  }
  while (w > 8 || h > 8) {
    if (w > 8) {
      sp.push_back({true, true, first, count});
      w = (w + 1) / 2;
    }
    if (h > 8) {
      sp.push_back({false, true, first, count});
      h = (h + 1) / 2;
    }
  }
  return sp;
}

ModTransform read_transform(Reader& r) {
  static const U32Dist kBeginC[4] = {{3, 0}, {6, 8}, {10, 72}, {13, 1096}};
  ModTransform t;
  const uint32_t tr = r.bits(2);
  if (tr == 2) {
    static const U32Dist kNumSq[4] = {{0, 0}, {4, 1}, {6, 9}, {8, 41}};
    static const U32Dist kNumC[4] = {{0, 1}, {0, 2}, {0, 3}, {4, 4}};
    t.kind = 2;
    const uint32_t n = r.u32(kNumSq);
    for (uint32_t i = 0; i < n; ++i) {
      SqueezeStep st;
      st.horizontal = r.flag();
      st.in_place = r.flag();
      st.begin_c = r.u32(kBeginC);
      st.num_c = r.u32(kNumC);
      t.steps.push_back(st);
    }
    return t;
  }
  need(tr <= 1, "transform id");
  t.begin_c = r.u32(kBeginC);
  if (tr == 1) {
    static const U32Dist kNumC[4] = {{0, 1}, {0, 3}, {0, 4}, {13, 1}};
    static const U32Dist kColours[4] = {{8, 0}, {10, 256}, {12, 1280}, {16, 5376}};
    static const U32Dist kDeltas[4] = {{0, 0}, {8, 1}, {10, 257}, {16, 1281}};
    t.kind = 1;
    t.num_c = r.u32(kNumC);
    t.nb_colours = r.u32(kColours);
    t.nb_deltas = r.u32(kDeltas);
    t.d_pred = r.bits(4);
    need(t.d_pred <= 13, "palette predictor");
    return t;
  }
  static const U32Dist kRct[4] = {{0, 6}, {2, 0}, {4, 2}, {6, 10}};
  t.kind = 0;
  t.rct_type = r.u32(kRct);
  need(t.rct_type < 42, "rct_type");
  return t;
}

// transform.rs:291 forward_palette on the channel shapes: the index channel
// stays, the others go, and the palette (nb_colours x num_c) becomes the
// first (meta) channel.
void forward_palette(std::vector<Channel>& ch, const ModTransform& t, size_t* nb_meta) {
  need(t.num_c >= 1 && (size_t)t.begin_c + t.num_c <= ch.size(), "palette channel range");
  const size_t begin = t.begin_c, end = begin + t.num_c;
  for (size_t c = begin + 1; c < end; ++c) need(ch[c].same_shape(ch[begin]), "palette shapes");
  if (begin < *nb_meta) {
    need(end <= *nb_meta && (int64_t)*nb_meta + 2 - (int64_t)t.num_c >= 0, "palette meta range");
    *nb_meta = *nb_meta + 2 - t.num_c;
  } else {
    *nb_meta += 1;
  }
  ch.erase(ch.begin() + (ptrdiff_t)begin + 1, ch.begin() + (ptrdiff_t)end);
  Channel meta;
  meta.w = t.nb_colours;
  meta.h = t.num_c;
  meta.hshift = meta.vshift = -1;
  ch.insert(ch.begin(), meta);
}

// palette.rs:130 lookup: an explicit colour, an implicit one past
// nb_colours, or (negative index) a delta-palette entry.
int64_t palette_lookup(const Channel& pal, const ModTransform& t, uint32_t bits, uint32_t c,
                       int32_t index32) {
  need(bits >= 1 && bits <= 32, "palette bit depth");
  const int64_t bitdepth = bits, full = ((int64_t)1 << bitdepth) - 1;
  const int64_t index = index32, nbc = t.nb_colours;
  if (index >= 0 && index < nbc) return pal.at((uint32_t)index, c);
  if (index >= nbc) {
    int64_t i = index - nbc;
    if (i < 64) {
      const uint32_t shift = 2 * c;
      const int64_t bucket = shift >= 63 ? 0 : (i >> shift) & 3;
      const int64_t bias = (int64_t)1 << std::max<int64_t>(bitdepth - 3, 0);
      return bucket * full / 4 + bias;
    }
    i -= 64;
    for (uint32_t k = 0; k < c; ++k) {
      if (i == 0) break;
      i /= 5;
    }
    return (i % 5) * full / 4;
  }
  if (c >= 3) return 0;
  const int64_t folded = ((-index - 1) % 143 + 143) % 143;
  int64_t value = kDeltaPalette[(folded + 1) >> 1][c];
  if ((folded & 1) == 0) value = -value;
  if (bitdepth > 8) value <<= std::min<int64_t>(bitdepth, 24) - 8;
  return value;
}

// transform.rs:350 forward_squeeze on the channel shapes.
void forward_squeeze(std::vector<Channel>& ch, const std::vector<SqueezeStep>& steps,
                     size_t* nb_meta) {
  for (const SqueezeStep& st : steps) {
    need(st.num_c >= 1, "squeeze num_c");
    const size_t begin = st.begin_c, end = (size_t)st.begin_c + st.num_c - 1;
    need(end < ch.size(), "squeeze channel range");
    const size_t r = st.in_place ? end + 1 : ch.size();
    if (begin < *nb_meta) {
      need(st.in_place && end < *nb_meta, "squeeze inside the meta channels");
      *nb_meta += st.num_c;
    }
    for (size_t c = begin; c <= end; ++c) {
      Channel& sc = ch[c];
      need(sc.w && sc.h, "squeeze of an empty channel");
      Channel res;
      if (st.horizontal) {
        res.w = sc.w / 2;
        res.h = sc.h;
        sc.w = (sc.w + 1) / 2;
        if (sc.hshift >= 0) ++sc.hshift;
      } else {
        res.h = sc.h / 2;
        res.w = sc.w;
        sc.h = (sc.h + 1) / 2;
        if (sc.vshift >= 0) ++sc.vshift;
      }
      res.hshift = sc.hshift;
      res.vshift = sc.vshift;
      const size_t at = r + (c - begin);
      need(at <= ch.size(), "squeeze residual index");
      ch.insert(ch.begin() + (ptrdiff_t)at, res);
    }
    need(ch.size() <= (1u << 16), "channel count");
  }
}

// squeeze.rs:157 tendency.
int64_t tendency(int64_t a, int64_t b, int64_t c) {
  if (a >= b && b >= c) {
    int64_t x = (4 * a - 3 * c - b + 6) / 12;
    if (x - (x & 1) > 2 * (a - b)) x = 2 * (a - b) + 1;
    if (x + (x & 1) > 2 * (b - c)) x = 2 * (b - c);
    return x;
  }
  if (a <= b && b <= c) {
    int64_t x = (4 * a - 3 * c - b - 6) / 12;
    if (x + (x & 1) < 2 * (a - b)) x = 2 * (a - b) - 1;
    if (x - (x & 1) < 2 * (b - c)) x = 2 * (b - c);
    return x;
  }
  return 0;
}

// squeeze.rs:183/:238 horiz_isqueeze / vert_isqueeze.
Channel unsqueeze(const Channel& lo, const Channel& res, bool horizontal) {
  Channel out;
  out.hshift = lo.hshift;
  out.vshift = lo.vshift;
  if (horizontal) {
    need(res.h == lo.h && (lo.w == res.w || lo.w == res.w + 1), "horizontal unsqueeze shapes");
    out.w = lo.w + res.w;
    out.h = lo.h;
    if (out.hshift > 0) --out.hshift;
    charge((uint64_t)out.w * out.h, sizeof(int32_t));
    out.v.assign((size_t)out.w * out.h, 0);
    for (uint32_t y = 0; y < lo.h; ++y) {
      for (uint32_t x = 0; x < res.w; ++x) {
        const int64_t avg = lo.at(x, y), residu = res.at(x, y);
        const int64_t next = x + 1 < lo.w ? (int64_t)lo.at(x + 1, y) : avg;
        const int64_t left = x > 0 ? (int64_t)out.at(2 * x - 1, y) : avg;
        const int64_t diff = residu + tendency(left, avg, next);
        const int64_t first = avg + diff / 2;
        out.at(2 * x, y) = (int32_t)first;
        out.at(2 * x + 1, y) = (int32_t)(first - diff);
      }
      if (lo.w > res.w) out.at(2 * res.w, y) = lo.at(res.w, y);
    }
  } else {
    need(res.w == lo.w && (lo.h == res.h || lo.h == res.h + 1), "vertical unsqueeze shapes");
    out.w = lo.w;
    out.h = lo.h + res.h;
    if (out.vshift > 0) --out.vshift;
    charge((uint64_t)out.w * out.h, sizeof(int32_t));
    out.v.assign((size_t)out.w * out.h, 0);
    for (uint32_t y = 0; y < res.h; ++y)
      for (uint32_t x = 0; x < lo.w; ++x) {
        const int64_t avg = lo.at(x, y), residu = res.at(x, y);
        const int64_t next = y + 1 < lo.h ? (int64_t)lo.at(x, y + 1) : avg;
        const int64_t top = y > 0 ? (int64_t)out.at(x, 2 * y - 1) : avg;
        const int64_t diff = residu + tendency(top, avg, next);
        const int64_t first = avg + diff / 2;
        out.at(x, 2 * y) = (int32_t)first;
        out.at(x, 2 * y + 1) = (int32_t)(first - diff);
      }
    if (lo.h > res.h)
      for (uint32_t x = 0; x < lo.w; ++x) out.at(x, 2 * res.h) = lo.at(x, res.h);
  }
  return out;
}

// rct.rs:59 inverse_pixel over channels begin_c..begin_c+3.
void inverse_rct(std::vector<Channel>& ch, uint32_t begin, uint32_t type) {
  need((size_t)begin + 3 <= ch.size(), "RCT channel range");
  Channel& c0 = ch[begin];
  Channel& c1 = ch[begin + 1];
  Channel& c2 = ch[begin + 2];
  need(c0.same_shape(c1) && c0.same_shape(c2), "RCT channel shapes");
  const uint32_t perm = type / 7, kind = type % 7;
  for (size_t i = 0; i < c0.v.size(); ++i) {
    const int64_t a = c0.v[i];
    int64_t b = c1.v[i], c = c2.v[i], d, e, f;
    if (kind == 6) {
      const int64_t tmp = a - (c >> 1);
      e = c + tmp;
      f = tmp - (b >> 1);
      d = f + b;
    } else {
      if (kind & 1) c += a;
      if ((kind >> 1) == 1) b += a;
      if ((kind >> 1) == 2) b += (a + c) >> 1;
      d = a;
      e = b;
      f = c;
    }
    int64_t v[3];
    const uint32_t half = perm / 3;
    v[perm % 3] = d;
    v[(perm + 1 + half) % 3] = e;
    v[(perm + 2 - half) % 3] = f;
    c0.v[i] = (int32_t)v[0];
    c1.v[i] = (int32_t)v[1];
    c2.v[i] = (int32_t)v[2];
  }
}

// palette.rs:238 apply_inverse.
void inverse_palette(std::vector<Channel>& ch, const ModTransform& t, uint32_t bits,
                     const WpHeader& wp) {
  need(!ch.empty(), "palette without its meta channel");
  const Channel pal = ch[0];
  ch.erase(ch.begin());
  need(pal.h >= t.num_c, "palette height");
  const size_t first = t.begin_c;
  need(first < ch.size(), "palette index channel");
  const Channel idx = ch[first];
  for (uint32_t k = 1; k < t.num_c; ++k) {
    need(first + k <= ch.size(), "palette channel insert");
    ch.insert(ch.begin() + (ptrdiff_t)(first + k), idx);
  }
  for (uint32_t c = 0; c < t.num_c; ++c) {
    Channel& tg = ch[first + c];
    Weighted wpred(tg.w);
    const bool weighted = t.d_pred == 6;
    for (uint32_t y = 0; y < tg.h; ++y) {
      for (uint32_t x = 0; x < tg.w; ++x) {
        const int32_t index = tg.at(x, y);
        int64_t value = palette_lookup(pal, t, bits, c, index);
        const Neighbours nb = gather(tg, x, y);
        if (weighted) wpred.run(wp, nb, x);
        if ((int64_t)index < (int64_t)t.nb_deltas)
          value += predict(nb, t.d_pred, weighted ? wpred.prediction : 0);
        tg.at(x, y) = (int32_t)value;
        if (weighted) wpred.update(x, (int32_t)value);
      }
      if (weighted) wpred.next_row();
    }
  }
}

void inverse_transforms(std::vector<Channel>& ch, const std::vector<ModTransform>& tf,
                        uint32_t bits, const WpHeader& wp) {
  for (size_t k = tf.size(); k-- > 0;) {
    const ModTransform& t = tf[k];
    if (t.kind == 0) {
      inverse_rct(ch, t.begin_c, t.rct_type);
      continue;
    }
    if (t.kind == 1) {
      inverse_palette(ch, t, bits, wp);
      continue;
    }
    for (size_t s = t.steps.size(); s-- > 0;) {
      const SqueezeStep& st = t.steps[s];
      const size_t begin = st.begin_c, end = (size_t)st.begin_c + st.num_c - 1;
      need(end < ch.size(), "inverse squeeze range");
      const size_t r = st.in_place ? end + 1 : ch.size() + begin - (end + 1);
      for (size_t c = begin; c <= end; ++c) {
        need(r < ch.size() && r != c, "inverse squeeze residual");
        ch[c] = unsqueeze(ch[c], ch[r], st.horizontal);
        ch.erase(ch.begin() + (ptrdiff_t)r);
      }
    }
  }
}

// What a GlobalModular stream that stopped at a channel larger than a group
// leaves for the group sections: its transforms (undone once every group is
// in), the weighted-predictor header they use, and the channel indices.
struct Deferred {
  std::vector<ModTransform> transforms;
  WpHeader wp;
  size_t nb_meta = 0, first_undecoded = 0;
};

// H.2-H.4: one modular sub-bitstream over `ch` (shapes set by the caller),
// transforms undone at the end.  With `defer`, decoding stops at the first
// non-meta channel wider or taller than group_dim (G.1.3; modular/mod.rs:649)
// and the transforms are handed back instead of undone.
void modular_stream(Reader& r, std::vector<Channel>& ch, uint32_t stream_index,
                    const GlobalTree& gt, uint32_t bits = 8, uint32_t group_dim = 0,
                    Deferred* defer = nullptr) {
  if (ch.empty()) {
    if (defer) *defer = Deferred{};
    return;
  }
  const bool use_global = r.flag();
  const WpHeader wp = read_wp(r);
  static const U32Dist kNbTransforms[4] = {{0, 0}, {0, 1}, {4, 2}, {8, 18}};
  const uint32_t nbt = r.u32(kNbTransforms);
  need(nbt <= 512, "transform count");
  std::vector<ModTransform> transforms;
  size_t nb_meta = 0;
  for (uint32_t i = 0; i < nbt; ++i) {
    transforms.push_back(read_transform(r));
    ModTransform& t = transforms.back();
    if (t.kind == 2) {
      if (t.steps.empty()) t.steps = default_squeeze(ch, nb_meta);
      forward_squeeze(ch, t.steps, &nb_meta);
    } else if (t.kind == 1) {
      forward_palette(ch, t, &nb_meta);
    } else {
      need((size_t)t.begin_c + 3 <= ch.size(), "RCT channel range");
    }
  }
  for (Channel& c : ch) {
    charge((uint64_t)c.w * c.h, sizeof(int32_t));
    c.v.assign((size_t)c.w * c.h, 0);
  }
  size_t end = ch.size();
  if (defer) {
    end = std::min(nb_meta, ch.size());
    while (end < ch.size() && ch[end].w <= group_dim && ch[end].h <= group_dim) ++end;
  }
  Tree local;
  std::unique_ptr<Stream> owned(new Stream);
  const Tree* tree;
  if (use_global) {
    need(gt.present, "use_global_tree without a global tree");
    *owned = gt.dists;
    need(owned->restart(r.b), "truncated stream");
    tree = &gt.tree;
  } else {
    local = read_tree(r);
    need(owned->open(r.b, local.num_leaves, 0, false), "modular histograms");
    tree = &local;
  }
  Stream& s = *owned;
  uint32_t dist_mult = 0;
  for (size_t i = 0; i < end; ++i)
    if (ch[i].w && ch[i].h) dist_mult = std::max(dist_mult, ch[i].w);
  s.dist_multiplier = dist_mult;
  for (size_t i = 0; i < end; ++i) {
    Channel& cur = ch[i];
    if (!cur.w || !cur.h) continue;
    std::vector<size_t> prev;
    for (size_t j = i; j-- > 0;)
      if (ch[j].same_shape(cur)) prev.push_back(j);
    std::vector<int32_t> props(16 + 4 * prev.size(), 0);
    Weighted wpred(cur.w);
    for (uint32_t y = 0; y < cur.h; ++y) {
      for (uint32_t x = 0; x < cur.w; ++x) {
        const Neighbours nb = gather(cur, x, y);
        wpred.run(wp, nb, x);
        int64_t wge = nb.w;
        if (x > 0) {
          const Neighbours l = gather(cur, x - 1, y);
          wge = nb.w - (l.w + l.n - l.nw);
        }
        const int64_t st[16] = {(int64_t)i,
                                (int64_t)stream_index,
                                (int64_t)y,
                                (int64_t)x,
                                std::llabs(nb.n),
                                std::llabs(nb.w),
                                nb.n,
                                nb.w,
                                wge,
                                nb.w + nb.n - nb.nw,
                                nb.w - nb.nw,
                                nb.nw - nb.n,
                                nb.n - nb.ne,
                                nb.n - nb.nn,
                                nb.w - nb.ww,
                                (int64_t)wpred.max_error};
        for (int k = 0; k < 16; ++k) props[k] = (int32_t)st[k];
        size_t k = 16;
        for (size_t j : prev) {
          const Channel& o = ch[j];
          const int64_t rc = o.at(x, y);
          const int64_t rw = x > 0 ? o.at(x - 1, y) : 0;
          const int64_t rn = y > 0 ? o.at(x, y - 1) : rw;
          const int64_t rnw = (x > 0 && y > 0) ? o.at(x - 1, y - 1) : rw;
          const int64_t rg = gradient(rw, rn, rnw);
          props[k++] = (int32_t)std::llabs(rc);
          props[k++] = (int32_t)rc;
          props[k++] = (int32_t)std::llabs(rc - rg);
          props[k++] = (int32_t)(rc - rg);
        }
        const TreeNode& leaf = tree->lookup(props.data(), props.size());
        uint32_t raw;
        need(s.read(r.b, leaf.ctx, &raw), "modular residual");
        const __int128 diff = (__int128)unpack_signed(raw) * leaf.mul + leaf.offset;
        need(diff >= INT64_MIN && diff <= INT64_MAX, "modular residual overflow");
        const int64_t value = (int64_t)diff + predict(nb, leaf.predictor, wpred.prediction);
        cur.at(x, y) = (int32_t)value;
        wpred.update(x, (int32_t)value);
      }
      wpred.next_row();
    }
  }
  need(s.final_state(), "modular stream final state");
  if (defer) {
    defer->transforms = std::move(transforms);
    defer->wp = wp;
    defer->nb_meta = nb_meta;
    defer->first_undecoded = end;
    return;
  }
  inverse_transforms(ch, transforms, bits, wp);
}

Channel make_channel(uint32_t w, uint32_t h) {
  Channel c;
  c.w = w;
  c.h = h;
  need((uint64_t)w * h <= t_max_pixels, "channel size");
  charge((uint64_t)w * h, sizeof(int32_t));
  c.v.assign((size_t)w * h, 0);
  return c;
}

GlobalTree read_global_tree(Reader& r) {
  GlobalTree gt;
  gt.present = r.flag();
  if (gt.present) {
    gt.tree = read_tree(r);
    need(gt.dists.open(r.b, gt.tree.num_leaves, 0, false, true), "global histograms");
  }
  return gt;
}

// ---- VarDCT (vardct/*.rs) ------------------------------------------------

// Table I.1 as jpxl-core varblock.rs:183 lists it: block rows, block columns,
// coefficient order id.
struct TransformInfo {
  uint8_t rows, cols, order_id;
};
const TransformInfo kTransforms[27] = {
    {1, 1, 0},  {1, 1, 1},  {1, 1, 1},   {1, 1, 1},   {2, 2, 2},  {4, 4, 3},   {2, 1, 4},
    {1, 2, 4},  {4, 1, 5},  {1, 4, 5},   {4, 2, 6},   {2, 4, 6},  {1, 1, 1},   {1, 1, 1},
    {1, 1, 1},  {1, 1, 1},  {1, 1, 1},   {1, 1, 1},   {8, 8, 7},  {8, 4, 8},   {4, 8, 8},
    {16, 16, 9}, {16, 8, 10}, {8, 16, 10}, {32, 32, 11}, {32, 16, 12}, {16, 32, 12}};
// Coefficient columns x rows (landscape) of each order id.
const uint16_t kOrderDims[13][2] = {{8, 8},   {8, 8},   {16, 16},  {32, 32},   {16, 8},
                                    {32, 8},  {32, 16}, {64, 64},  {64, 32},   {128, 128},
                                    {128, 64}, {256, 256}, {256, 128}};

// jpxl-core varblock.rs:709: LLF cells first in raster order, then the rest
// by (x + y) diagonal, alternating direction, on the scaled square grid.
std::vector<uint32_t> natural_order(uint32_t bwidth, uint32_t bheight) {
  const int64_t cx = bwidth / 8, cy = bheight / 8, scale = std::max(cx, cy);
  struct Key {
    int64_t k1, k2;
    uint32_t lin;
  };
  std::vector<std::pair<int64_t, uint32_t>> llf;
  std::vector<Key> hf;
  for (uint32_t y = 0; y < bheight; ++y)
    for (uint32_t x = 0; x < bwidth; ++x) {
      const uint32_t lin = y * bwidth + x;
      if (x < cx && y < cy) {
        llf.push_back({(int64_t)y * cx + x, lin});
        continue;
      }
      const int64_t sx = (int64_t)x * scale / cx, sy = (int64_t)y * scale / cy;
      const int64_t k1 = sx + sy;
      int64_t k2 = sx - sy;
      if (k1 % 2 == 1) k2 = -k2;
      hf.push_back({k1, k2, lin});
    }
  std::stable_sort(llf.begin(), llf.end(),
                   [](const auto& a, const auto& b) { return a.first < b.first; });
  std::stable_sort(hf.begin(), hf.end(), [](const Key& a, const Key& b) {
    return a.k1 != b.k1 ? a.k1 < b.k1 : a.k2 < b.k2;
  });
  std::vector<uint32_t> out;
  out.reserve((size_t)bwidth * bheight);
  for (auto& e : llf) out.push_back(e.second);
  for (auto& e : hf) out.push_back(e.lin);
  return out;
}

// Natural orders are the same for every frame: built once per process.
const std::vector<uint32_t>& cached_natural_order(int order_id) {
  static std::vector<uint32_t> cache[13];
  static std::once_flag once[13];
  std::call_once(once[order_id], [order_id] {
    cache[order_id] = natural_order(kOrderDims[order_id][0], kOrderDims[order_id][1]);
  });
  return cache[order_id];
}

// I.2.2 (block_ctx.rs:212).
struct BlockCtx {
  std::vector<int32_t> lf_thr[3];
  std::vector<uint32_t> qf_thr;
  std::vector<uint8_t> map;
  uint32_t num = 15;
};

BlockCtx read_block_ctx(Reader& r) {
  BlockCtx m;
  if (r.flag()) {
    m.map = {0, 1, 2, 2, 3, 3, 4, 5, 6, 6, 6, 6, 6, 7, 8, 9, 9, 10, 11, 12, 13, 14,
             14, 14, 14, 14, 7, 8, 9, 9, 10, 11, 12, 13, 14, 14, 14, 14, 14};
    return m;
  }
  static const U32Dist kThr[4] = {{4, 0}, {8, 16}, {16, 272}, {32, 65808}};
  static const U32Dist kQf[4] = {{2, 0}, {3, 4}, {5, 12}, {8, 44}};
  for (int i = 0; i < 3; ++i) {
    const uint32_t n = r.bits(4);
    for (uint32_t j = 0; j < n; ++j) m.lf_thr[i].push_back(unpack_signed(r.u32(kThr)));
  }
  const uint32_t nq = r.bits(4);
  for (uint32_t j = 0; j < nq; ++j) m.qf_thr.push_back(r.u32(kQf) + 1);
  const size_t bsize = 39 * (nq + 1) * (m.lf_thr[0].size() + 1) * (m.lf_thr[1].size() + 1) *
                       (m.lf_thr[2].size() + 1);
  need(bsize <= 39 * 64, "block context map size");
  Stream s;
  need(s.read_clusters(r.b, bsize, 0), "block context map");
  need(s.num_clusters <= 16, "block context clusters");
  m.map.assign(s.clusters.begin(), s.clusters.end());
  m.num = (uint32_t)s.num_clusters;
  return m;
}

uint32_t block_context(const BlockCtx& m, int c, uint32_t order_id, uint32_t qf,
                       const int32_t qdc[3], bool lf_idx_is_zero) {
  const int cls = c < 2 ? (c ^ 1) : 2;
  size_t idx = (size_t)cls * 13 + order_id;
  idx *= m.qf_thr.size() + 1;
  for (uint32_t t : m.qf_thr)
    if (qf > t) ++idx;
  for (int i = 0; i < 3; ++i) idx *= m.lf_thr[i].size() + 1;
  size_t lf = 0;
  if (!lf_idx_is_zero) {
    for (int32_t t : m.lf_thr[0])
      if (qdc[0] > t) ++lf;
    lf *= m.lf_thr[2].size() + 1;
    for (int32_t t : m.lf_thr[2])
      if (qdc[2] > t) ++lf;
    lf *= m.lf_thr[1].size() + 1;
    for (int32_t t : m.lf_thr[1])
      if (qdc[1] > t) ++lf;
  }
  need(idx + lf < m.map.size(), "block context index");
  return m.map[idx + lf];
}

// I.2.4 (dequant_matrix.rs:212): the parameters are read to stay in step;
// only the library defaults are carried by the reconstruction.
void read_dequant_params(Reader& r) {
  auto matrix = [&](int n) {
    for (int i = 0; i < 3 * n; ++i) r.f16();
  };
  auto dct_params = [&]() { matrix((int)r.bits(4) + 1); };
  for (int index = 0; index < 17; ++index) {
    const uint32_t mode = r.bits(3);
    switch (mode) {
      case 0: break;
      case 1: matrix(3); break;
      case 2: matrix(6); break;
      case 3: matrix(2); dct_params(); break;
      case 4: matrix(1); dct_params(); break;
      case 5: matrix(9); dct_params(); dct_params(); break;
      case 6: dct_params(); break;
      default: fail("RAW dequantization matrices are not supported");
    }
  }
}

const uint8_t kCoeffFreqCtx[64] = {0,  0,  1,  2,  3,  4,  5,  6,  7,  8,  9,  10, 11,
                                   12, 13, 14, 15, 15, 16, 16, 17, 17, 18, 18, 19, 19,
                                   20, 20, 21, 21, 22, 22, 23, 23, 23, 23, 24, 24, 24,
                                   24, 25, 25, 25, 25, 26, 26, 26, 26, 27, 27, 27, 27,
                                   28, 28, 28, 28, 29, 29, 29, 29, 30, 30, 30, 30};
const uint8_t kCoeffNzCtx[64] = {0,   0,   31,  62,  62,  93,  93,  93,  93,  123, 123, 123, 123,
                                 152, 152, 152, 152, 152, 152, 152, 152, 180, 180, 180, 180, 180,
                                 180, 180, 180, 180, 180, 180, 180, 206, 206, 206, 206, 206, 206,
                                 206, 206, 206, 206, 206, 206, 206, 206, 206, 206, 206, 206, 206,
                                 206, 206, 206, 206, 206, 206, 206, 206, 206, 206, 206, 206};
constexpr uint32_t kNonZeroCtx = 37, kCoeffCtx = 458, kCtxPerBlock = kNonZeroCtx + kCoeffCtx;

// The channel pieces of one LF group (G.2.3) or pass group (G.4.2), rect in
// frame samples: one sub-bitstream over the selected channels' pieces, the
// origin shifted exactly and the extent rounded up (decode.rs:2159), then
// copied back into the frame's channels.
void decode_group_channels(Reader& r, std::vector<Channel>& ch, const std::vector<size_t>& sel,
                           uint32_t x0, uint32_t y0, uint32_t w, uint32_t h,
                           uint32_t stream_index, const GlobalTree& gt) {
  if (sel.empty()) return;
  std::vector<Channel> piece;
  std::vector<std::pair<uint32_t, uint32_t>> origin;
  for (size_t i : sel) {
    const Channel& c = ch[i];
    const uint32_t hs = (uint32_t)std::max(c.hshift, 0), vs = (uint32_t)std::max(c.vshift, 0);
    const uint32_t px = x0 >> hs, py = y0 >> vs;
    const uint32_t ex = (uint32_t)(((uint64_t)x0 + w + (1ull << hs) - 1) >> hs);
    const uint32_t ey = (uint32_t)(((uint64_t)y0 + h + (1ull << vs) - 1) >> vs);
    Channel p;
    p.w = std::min(ex > px ? ex - px : 0u, c.w > px ? c.w - px : 0u);
    p.h = std::min(ey > py ? ey - py : 0u, c.h > py ? c.h - py : 0u);
    p.hshift = c.hshift;
    p.vshift = c.vshift;
    piece.push_back(std::move(p));
    origin.emplace_back(px, py);
  }
  modular_stream(r, piece, stream_index, gt);
  for (size_t k = 0; k < sel.size(); ++k) {
    Channel& dst = ch[sel[k]];
    const Channel& src = piece[k];
    need(src.w == 0 || (origin[k].first + src.w <= dst.w && origin[k].second + src.h <= dst.h),
         "group piece outside its channel");
    for (uint32_t y = 0; y < src.h; ++y)
      for (uint32_t x = 0; x < src.w; ++x)
        dst.at(origin[k].first + x, origin[k].second + y) = src.at(x, y);
  }
}

// G.2.3 and G.4.2 for the channels GlobalModular left undecoded: the
// selections once, then each LF group's and pass group's pieces as their
// sections reach the modular data, then the deferred transforms.  One pass.
struct ModularGroups {
  std::vector<Channel>& ch;
  Deferred& d;
  const GlobalTree& gt;
  uint32_t W, H, gdim, lfdim, gx, lgx;
  uint64_t num_lf;
  std::vector<size_t> lf_sel, pass_sel;

  ModularGroups(std::vector<Channel>& ch_, Deferred& d_, const GlobalTree& gt_, uint32_t W_,
                uint32_t H_, uint32_t gdim_)
      : ch(ch_), d(d_), gt(gt_), W(W_), H(H_), gdim(gdim_), lfdim(8 * gdim_) {
    gx = (W + gdim - 1) / gdim;
    lgx = (W + lfdim - 1) / lfdim;
    num_lf = (uint64_t)lgx * ((H + lfdim - 1) / lfdim);
    for (size_t i = d.first_undecoded; i < ch.size(); ++i) {
      const Channel& c = ch[i];
      if (c.hshift >= 3 && c.vshift >= 3) {
        lf_sel.push_back(i);
        continue;
      }
      if (i < d.nb_meta) continue;
      const uint32_t hs = (uint32_t)std::min(std::max(c.hshift, 0), 31);
      const uint32_t vs = (uint32_t)std::min(std::max(c.vshift, 0), 31);
      if (c.w <= (gdim >> hs) && c.h <= (gdim >> vs)) continue;  // decode.rs:352
      if (std::min(c.hshift, c.vshift) < 3) pass_sel.push_back(i);
    }
  }
  bool any() const { return !lf_sel.empty() || !pass_sel.empty(); }
  void lf_group(uint64_t lg, Reader& r) {
    const uint32_t x0 = (uint32_t)(lg % lgx) * lfdim, y0 = (uint32_t)(lg / lgx) * lfdim;
    decode_group_channels(r, ch, lf_sel, x0, y0, std::min(lfdim, W - x0),
                          std::min(lfdim, H - y0), (uint32_t)(1 + num_lf + lg), gt);
  }
  void pass_group(uint64_t g, Reader& r) {
    const uint32_t x0 = (uint32_t)(g % gx) * gdim, y0 = (uint32_t)(g / gx) * gdim;
    decode_group_channels(r, ch, pass_sel, x0, y0, std::min(gdim, W - x0),
                          std::min(gdim, H - y0), (uint32_t)(1 + 3 * num_lf + 17 + g), gt);
  }
  void finish(uint32_t bits) { inverse_transforms(ch, d.transforms, bits, d.wp); }
};

struct Section {
  Reader r;
  uint64_t start_bits, size_bytes;
};

// ---- the frame --------------------------------------------------------------

void decode_frame_vardct(std::vector<Section>& sec, bool single, Decoded* out) {
  const ImageInfo& img = out->image;
  const FrameInfo& fr = out->frame;
  VarDctFrame& vd = out->vardct;
  auto section = [&](uint64_t i) -> Reader& { return single ? sec[0].r : sec[i].r; };
  need((fr.flags & (1 | 2 | 16)) == 0, "noise, patches and splines are not supported");
  vd.lf_from_frame = (fr.flags & 32) != 0;
  need(!vd.lf_from_frame || !vd.lf_frame[0].empty(), "kUseLfFrame without an LF frame");
  const uint32_t W = fr.width, H = fr.height;
  const uint32_t gdim = 256, lfdim = 2048;
  const uint32_t gx = (W + gdim - 1) / gdim, gy = (H + gdim - 1) / gdim;
  const uint32_t lgx = (W + lfdim - 1) / lfdim, lgy = (H + lfdim - 1) / lfdim;
  const uint64_t num_groups = (uint64_t)gx * gy, num_lf = (uint64_t)lgx * lgy;
  vd.bw = (W + 7) / 8;
  vd.bh = (H + 7) / 8;
  const size_t nblocks = (size_t)vd.bw * vd.bh;
  charge(nblocks, 3 * sizeof(int32_t) + 3 + sizeof(uint32_t));
  for (auto& p : vd.lf) p.assign(nblocks, 0);
  vd.block_map.assign(nblocks, 0);
  vd.hf_mul.assign(nblocks, 0);
  vd.sharpness.assign(nblocks, 0);
  vd.tiles_w = (W + 63) / 64;
  vd.tiles_h = (H + 63) / 64;
  vd.x_from_y.assign((size_t)vd.tiles_w * vd.tiles_h, 0);
  vd.b_from_y.assign((size_t)vd.tiles_w * vd.tiles_h, 0);

  // LfGlobal (G.1; decode.rs:2565-2605).
  Reader& g = section(0);
  if (!g.flag()) {
    for (int c = 0; c < 3; ++c) vd.m_lf[c] = g.f16();
  }
  static const U32Dist kGs[4] = {{11, 1}, {11, 2049}, {12, 4097}, {16, 8193}};
  static const U32Dist kQlf[4] = {{0, 16}, {5, 1}, {8, 1}, {16, 1}};
  vd.global_scale = g.u32(kGs);
  vd.quant_lf = g.u32(kQlf);
  const BlockCtx bctx = read_block_ctx(g);
  if (!g.flag()) {
    static const U32Dist kCf[4] = {{0, 84}, {0, 256}, {8, 2}, {16, 258}};
    vd.colour_factor = g.u32(kCf);
    vd.base_corr_x = g.f16();
    vd.base_corr_b = g.f16();
    vd.x_factor_lf = (int)g.bits(8) - 128;
    vd.b_factor_lf = (int)g.bits(8) - 128;
  }
  const GlobalTree gt = read_global_tree(g);
  // GlobalModular (G.1.3): a VarDCT frame's channels are its extra channels;
  // those no larger than a group are decoded here (decode.rs:2589).
  out->extra.clear();
  for (const ImageInfo::Extra& e : img.extra) {
    need(e.dim_shift == 0, "extra channels with a dim_shift are not supported");
    out->extra.push_back(make_channel(W, H));
  }
  // Channels larger than a group continue in the LF groups (after the LF
  // coefficients) and the pass groups (after the HF coefficients).
  Deferred ed;
  modular_stream(g, out->extra, 0, gt, img.bits_per_sample, gdim, &ed);
  ModularGroups mg(out->extra, ed, gt, W, H, gdim);
  need(!mg.any() || fr.num_passes == 1,
       "extra channels larger than a group in several passes are not supported");

  // LF groups (G.2; decode.rs:2625-2700).
  std::vector<std::vector<Varblock>> placements(num_lf);
  for (uint64_t lg = 0; lg < num_lf; ++lg) {
    Reader& r = section(1 + lg);
    const uint32_t x0 = (uint32_t)(lg % lgx) * lfdim, y0 = (uint32_t)(lg / lgx) * lfdim;
    const uint32_t gw = std::min(lfdim, W - x0), gh = std::min(lfdim, H - y0);
    const uint32_t bw = (gw + 7) / 8, bh = (gh + 7) / 8;
    const uint32_t bx0 = x0 / 8, by0 = y0 / 8;
    if (!vd.lf_from_frame) {
      vd.extra_precision = r.bits(2);
      std::vector<Channel> lfch = {make_channel(bw, bh), make_channel(bw, bh),
                                   make_channel(bw, bh)};
      modular_stream(r, lfch, (uint32_t)(1 + lg), gt);
      // stream order Y, X, B (lf.rs:80)
      const int plane_of[3] = {1, 0, 2};
      for (int k = 0; k < 3; ++k)
        for (uint32_t y = 0; y < bh; ++y)
          for (uint32_t x = 0; x < bw; ++x)
            vd.lf[plane_of[k]][(size_t)(by0 + y) * vd.bw + bx0 + x] = lfch[k].at(x, y);
    }
    mg.lf_group(lg, r);  // ModularLfGroup (G.2.3)
    // HF metadata (G.2.4; hf_meta.rs:111).
    const uint32_t nb = 1 + r.bits(ceil_log2((uint64_t)bw * bh));
    const uint32_t cw = (gw + 63) / 64, chh = (gh + 63) / 64;
    std::vector<Channel> meta = {make_channel(cw, chh), make_channel(cw, chh),
                                 make_channel(nb, 2), make_channel(bw, bh)};
    modular_stream(r, meta, (uint32_t)(1 + 2 * num_lf + lg), gt);
    for (uint32_t y = 0; y < chh; ++y)
      for (uint32_t x = 0; x < cw; ++x) {
        const int32_t xf = meta[0].at(x, y), bf = meta[1].at(x, y);
        need(xf >= -128 && xf <= 127 && bf >= -128 && bf <= 127, "CfL factor range");
        const size_t t = (size_t)(y0 / 64 + y) * vd.tiles_w + x0 / 64 + x;
        vd.x_from_y[t] = (int8_t)xf;
        vd.b_from_y[t] = (int8_t)bf;
      }
    for (uint32_t y = 0; y < bh; ++y)
      for (uint32_t x = 0; x < bw; ++x) {
        const int32_t s = meta[3].at(x, y);
        need(s >= 0 && s <= 7, "EPF sharpness range");
        vd.sharpness[(size_t)(by0 + y) * vd.bw + bx0 + x] = (uint8_t)s;
      }
    // Varblock placement (hf_meta.rs:178): each entry takes the first block
    // not yet covered, in raster order.
    std::vector<uint8_t> covered((size_t)bw * bh, 0);
    size_t cursor = 0;
    for (uint32_t i = 0; i < nb; ++i) {
      while (cursor < covered.size() && covered[cursor]) ++cursor;
      need(cursor < covered.size(), "BlockInfo past a covered LF group");
      const uint32_t bx = (uint32_t)(cursor % bw), by = (uint32_t)(cursor / bw);
      const int32_t sel = meta[2].at(i, 0), mul = meta[2].at(i, 1);
      need(sel >= 0 && sel < 27, "DctSelect range");
      need(mul >= 0 && mul < 0x7fffffff, "HfMul range");
      const TransformInfo& ti = kTransforms[sel];
      need(bx + ti.cols <= bw && by + ti.rows <= bh, "varblock crosses the LF group");
      for (uint32_t dy = 0; dy < ti.rows; ++dy)
        for (uint32_t dx = 0; dx < ti.cols; ++dx) {
          uint8_t& cv = covered[(size_t)(by + dy) * bw + bx + dx];
          need(!cv, "overlapping varblocks");
          cv = 1;
          const size_t blk = (size_t)(by0 + by + dy) * vd.bw + bx0 + bx + dx;
          vd.block_map[blk] = (uint8_t)sel;
          vd.hf_mul[blk] = (uint32_t)mul + 1;
        }
      vd.block_map[(size_t)(by0 + by) * vd.bw + bx0 + bx] |= 0x80;
      placements[lg].push_back(Varblock{bx0 + bx, by0 + by, (uint8_t)sel, (uint32_t)mul + 1, 0});
      vd.histogram_counts[sel]++;
    }
  }

  // HfGlobal (G.3; dequant_matrix.rs:417, hf_coeff.rs:435, order.rs:253).
  Reader& hg = section(1 + num_lf);
  vd.default_matrices = hg.flag();
  if (!vd.default_matrices) read_dequant_params(hg);
  const uint32_t num_presets = hg.bits(ceil_log2(num_groups)) + 1;
  const std::vector<uint32_t>* natural[13];
  for (int o = 0; o < 13; ++o) natural[o] = &cached_natural_order(o);
  struct Pass {
    std::vector<std::vector<uint32_t>> orders;  // permuted orders, [order_id * 3 + c]
    const std::vector<uint32_t>* ordering[39];  // the order in force: natural or permuted
    std::unique_ptr<Stream> hist;
  };
  std::vector<Pass> passes(fr.num_passes);
  const size_t num_dist = (size_t)kCtxPerBlock * bctx.num * num_presets;
  for (auto& p : passes) {
    static const U32Dist kUsed[4] = {{0, 0x5F}, {0, 0x13}, {0, 0}, {13, 0}};
    const uint32_t used = hg.u32(kUsed);
    p.orders.resize(39);
    for (int o = 0; o < 39; ++o) p.ordering[o] = natural[o / 3];
    if (used) {
      Stream s;
      need(s.open(hg.b, 8, 0, false), "coefficient order histograms");
      for (int o = 0; o < 13; ++o) {
        if (!((used >> o) & 1)) continue;
        const std::vector<uint32_t>& nat = *natural[o];
        const uint32_t size = (uint32_t)nat.size();
        for (int c = 0; c < 3; ++c) {
          const std::vector<uint32_t> perm = read_permutation(hg, s, size, size / 64);
          std::vector<uint32_t>& dst = p.orders[o * 3 + c];
          dst.resize(size);
          for (uint32_t k = 0; k < size; ++k) dst[k] = nat[perm[k]];
          p.ordering[o * 3 + c] = &dst;
        }
      }
      need(s.final_state(), "coefficient order final state");
    }
    p.hist.reset(new Stream);
    need(p.hist->open(hg.b, num_dist, 0, false, true), "HF histograms");
  }

  // Coefficient storage: varblocks of every LF group back to back.
  uint32_t offset = 0;
  for (auto& lgp : placements)
    for (Varblock& v : lgp) {
      v.coeff_offset = offset;
      const TransformInfo& ti = kTransforms[v.transform];
      offset += 64u * ti.rows * ti.cols;
    }
  charge(offset, 3 * sizeof(int32_t));
  for (auto& c : vd.coeffs) c.assign(offset, 0);

  // Pass groups (G.4; hf_coeff.rs:689).
  for (uint32_t pass = 0; pass < fr.num_passes; ++pass) {
    Pass& P = passes[pass];
    for (uint64_t grp = 0; grp < num_groups; ++grp) {
      Reader& r = section(2 + num_lf + num_groups * pass + grp);
      const uint32_t x0 = (uint32_t)(grp % gx) * gdim, y0 = (uint32_t)(grp / gx) * gdim;
      const uint32_t gw = std::min(gdim, W - x0), gh = std::min(gdim, H - y0);
      const uint32_t gbx = x0 / 8, gby = y0 / 8, gbw = (gw + 7) / 8, gbh = (gh + 7) / 8;
      const uint64_t lg = (uint64_t)(y0 / lfdim) * lgx + x0 / lfdim;
      const uint32_t hfp = r.bits(ceil_log2(num_presets));
      need(hfp < num_presets, "HF preset");
      const size_t ctx_off = (size_t)kCtxPerBlock * bctx.num * hfp;
      Stream& s = *P.hist;
      need(s.restart(r.b), "truncated stream");
      std::vector<uint32_t> nz[3];
      for (auto& v : nz) v.assign((size_t)gbw * gbh, 0);
      auto nz_at = [&](int c, uint32_t x, uint32_t y) -> uint32_t {
        return (x < gbw && y < gbh) ? nz[c][(size_t)y * gbw + x] : 0;
      };
      for (const Varblock& vb : placements[lg]) {
        if (vb.bx < gbx || vb.by < gby || vb.bx >= gbx + gbw || vb.by >= gby + gbh) continue;
        const uint32_t lx = vb.bx - gbx, ly = vb.by - gby;
        const TransformInfo& ti = kTransforms[vb.transform];
        need(lx + ti.cols <= gbw && ly + ti.rows <= gbh, "varblock outside its group");
        const uint32_t nblk = (uint32_t)ti.rows * ti.cols, size = 64 * nblk;
        const size_t lfi = (size_t)vb.by * vd.bw + vb.bx;
        const int32_t qdc[3] = {vd.lf[0][lfi], vd.lf[1][lfi], vd.lf[2][lfi]};
        for (int c : {1, 0, 2}) {
          const uint32_t bc =
              block_context(bctx, c, ti.order_id, vb.hf_mul, qdc, vd.lf_from_frame);
          uint32_t pred;
          if (lx == 0 && ly == 0) pred = 32;
          else if (lx == 0) pred = nz_at(c, lx, ly - 1);
          else if (ly == 0) pred = nz_at(c, lx - 1, ly);
          else pred = (nz_at(c, lx, ly - 1) + nz_at(c, lx - 1, ly) + 1) >> 1;
          pred = std::min<uint32_t>(pred, 64);
          const uint32_t m = pred < 8 ? pred : 4 + pred / 2;
          uint32_t non_zeros;
          need(s.read(r.b, bc + (size_t)bctx.num * m + ctx_off, &non_zeros), "non-zero count");
          need(non_zeros <= size - nblk, "non-zero count range");
          const uint32_t per = (non_zeros + nblk - 1) / nblk;
          for (uint32_t j = 0; j < ti.rows; ++j)
            for (uint32_t i = 0; i < ti.cols; ++i) nz[c][(size_t)(ly + j) * gbw + lx + i] = per;
          if (non_zeros == 0) continue;
          const std::vector<uint32_t>& order = *P.ordering[ti.order_id * 3 + c];
          need(order.size() == size, "coefficient order size");
          int32_t* blk = vd.coeffs[c].data() + vb.coeff_offset;
          uint32_t remaining = non_zeros;
          bool prev_nz = non_zeros <= size / 16;
          for (uint32_t k = nblk; k < size; ++k) {
            const uint32_t nzc = (remaining + nblk - 1) / nblk, kk = k / nblk;
            need(nzc < 64 && kk < 64, "coefficient context");
            const size_t ctx = ((size_t)(kCoeffNzCtx[nzc] + kCoeffFreqCtx[kk]) * 2 + prev_nz) +
                               (size_t)bc * kCoeffCtx + (size_t)kNonZeroCtx * bctx.num + ctx_off;
            uint32_t u;
            need(s.read(r.b, ctx, &u), "coefficient");
            if (u != 0) {
              const int64_t v = (int64_t)unpack_signed(u) * ((int64_t)1 << fr.pass_shift[pass]);
              need(v >= INT32_MIN && v <= INT32_MAX, "coefficient range");
              blk[order[k]] += (int32_t)v;
              if (--remaining == 0) break;
            }
            prev_nz = u != 0;
          }
          need(remaining == 0, "undelivered non-zero coefficients");
        }
      }
      need(s.final_state(), "HF final state");
      mg.pass_group(grp, r);  // ModularGroup (G.4.2)
    }
  }
  mg.finish(img.bits_per_sample);
  // Varblocks in raster order of their origins.
  for (auto& lgp : placements)
    for (const Varblock& v : lgp) vd.varblocks.push_back(v);
  std::sort(vd.varblocks.begin(), vd.varblocks.end(), [](const Varblock& a, const Varblock& b) {
    return a.by != b.by ? a.by < b.by : a.bx < b.bx;
  });
}

void decode_frame_modular(std::vector<Section>& sec, Decoded* out, float m_lf[3] = nullptr) {
  const ImageInfo& img = out->image;
  const FrameInfo& fr = out->frame;
  need((fr.flags & (2 | 16 | 32)) == 0, "patches, splines and LF frames are not supported");
  Reader& g = sec[0].r;
  if (!g.flag()) {
    for (int c = 0; c < 3; ++c) {
      const float v = g.f16();
      if (m_lf) m_lf[c] = v;
    }
  }
  const GlobalTree gt = read_global_tree(g);
  const uint32_t n = (img.xyb_encoded || img.colour_space != 1) ? 3 : 1;
  const uint32_t gdim = 128u << fr.group_size_shift;
  need(fr.num_passes == 1 || (fr.width <= gdim && fr.height <= gdim),
       "modular frames of several passes and groups are not supported");
  out->modular.clear();
  for (uint32_t c = 0; c < n; ++c) out->modular.push_back(make_channel(fr.width, fr.height));
  // The extra channels follow the colour channels in the one channel list
  // of GlobalModular (G.1.3; decode.rs:1226 initial_channels); they are handed out apart.
  for (const ImageInfo::Extra& e : img.extra) {
    const uint32_t sh = e.dim_shift;
    need(sh == 0, "extra channels with a dim_shift are not supported");
    out->modular.push_back(make_channel(fr.width, fr.height));
  }
  Deferred d;
  modular_stream(g, out->modular, 0, gt, img.bits_per_sample, gdim, &d);
  const bool single = sec.size() == 1;
  ModularGroups mg(out->modular, d, gt, fr.width, fr.height, gdim);
  if (mg.any()) {
    const uint64_t num_groups = (uint64_t)mg.gx * ((fr.height + gdim - 1) / gdim);
    for (uint64_t lg = 0; lg < mg.num_lf; ++lg) mg.lf_group(lg, single ? sec[0].r : sec[1 + lg].r);
    for (uint64_t gi = 0; gi < num_groups; ++gi)
      mg.pass_group(gi, single ? sec[0].r : sec[2 + mg.num_lf + gi].r);
  }
  mg.finish(img.bits_per_sample);
  out->extra.assign(out->modular.begin() + n, out->modular.end());
  out->modular.resize(n);
}

// F.3 TOC (toc.rs:127) of frame f, read at r: the frame's sections, and the
// byte after the last one.
void read_toc(Reader& r, const uint8_t* data, size_t size, const FrameInfo& f,
              std::vector<Section>* sections, uint64_t* end_byte) {
  const uint32_t gdim = f.encoding == 0 ? 256 : (128u << f.group_size_shift);
  const uint64_t groups = (uint64_t)((f.width + gdim - 1) / gdim) * ((f.height + gdim - 1) / gdim);
  const uint64_t lf_groups =
      (uint64_t)((f.width + 8 * gdim - 1) / (8 * gdim)) * ((f.height + 8 * gdim - 1) / (8 * gdim));
  const uint64_t nsec = (groups == 1 && f.num_passes == 1) ? 1 : 1 + lf_groups + 1 + f.num_passes * groups;
  need(nsec <= (1u << 20), "section count");
  const bool permuted = r.flag();
  std::vector<uint32_t> perm;
  if (permuted) {
    Stream s;
    need(s.open(r.b, 8, 0, false), "TOC permutation");
    perm = read_permutation(r, s, (uint32_t)nsec, 0);
    need(s.final_state(), "TOC permutation final state");
  }
  r.pad_to_byte();
  static const U32Dist kEntry[4] = {{10, 0}, {14, 1024}, {22, 17408}, {30, 4211712}};
  std::vector<uint64_t> sizes(nsec), offsets(nsec);
  for (auto& s : sizes) s = r.u32(kEntry);
  r.pad_to_byte();
  uint64_t running = 0;
  for (uint64_t i = 0; i < nsec; ++i) {
    offsets[i] = running;
    running += sizes[i];
  }
  if (permuted) {
    std::vector<uint64_t> po(nsec), ps(nsec);
    for (uint64_t i = 0; i < nsec; ++i) {
      po[i] = offsets[perm[i]];
      ps[i] = sizes[perm[i]];
    }
    offsets = po;
    sizes = ps;
  }
  const uint64_t base = r.b.pos / 8;
  need(base + running <= size, "sections past the end of the codestream");
  std::vector<Section>& sec = *sections;
  sec.assign(nsec, Section{});
  for (uint64_t i = 0; i < nsec; ++i) {
    sec[i].r.b.data = data;
    sec[i].r.b.pos = (size_t)(base + offsets[i]) * 8;
    sec[i].r.b.size_bits = (size_t)(base + offsets[i] + sizes[i]) * 8;
    sec[i].start_bits = sec[i].r.b.pos;
    sec[i].size_bytes = sizes[i];
  }
  *end_byte = base + running;
}

}  // namespace

TransformShape transform_shape(uint8_t dct_select) {
  const TransformInfo& t = kTransforms[dct_select < 27 ? dct_select : 0];
  return TransformShape{t.rows, t.cols};
}

// ISO/IEC 18181-2 container (jpxl-decode container.rs): the codestream of a
// boxed file, from its one jxlc box or its jxlp fragments in index order.
bool unbox(const uint8_t* data, size_t size, std::vector<uint8_t>* cs) {
  static const uint8_t kSig[12] = {0, 0, 0, 0x0C, 'J', 'X', 'L', ' ', 0x0D, 0x0A, 0x87, 0x0A};
  if (size < 12 || std::memcmp(data, kSig, 12) != 0) return false;
  size_t pos = 0;
  bool jxlc = false, last_seen = false;
  uint32_t next_index = 0;
  while (pos < size) {
    need(size - pos >= 8, "truncated container box");
    uint64_t len = ((uint64_t)data[pos] << 24) | ((uint64_t)data[pos + 1] << 16) |
                   ((uint64_t)data[pos + 2] << 8) | data[pos + 3];
    const uint8_t* type = data + pos + 4;
    size_t header = 8;
    if (len == 1) {
      need(size - pos >= 16, "truncated container box");
      len = 0;
      for (int i = 0; i < 8; ++i) len = (len << 8) | data[pos + 8 + i];
      header = 16;
    } else if (len == 0) {
      len = size - pos;
    }
    need(len >= header && len <= size - pos, "container box size");
    const uint8_t* body = data + pos + header;
    const size_t body_len = (size_t)len - header;
    if (std::memcmp(type, "jxlc", 4) == 0) {
      need(!jxlc && next_index == 0, "jxlc with another codestream box");
      jxlc = true;
      cs->assign(body, body + body_len);
    } else if (std::memcmp(type, "jxlp", 4) == 0) {
      need(!jxlc && !last_seen && body_len >= 4, "jxlp box");
      const uint32_t idx = ((uint32_t)body[0] << 24) | ((uint32_t)body[1] << 16) |
                           ((uint32_t)body[2] << 8) | body[3];
      need((idx & 0x7fffffffu) == next_index, "jxlp fragments out of order");
      ++next_index;
      last_seen = (idx >> 31) != 0;
      cs->insert(cs->end(), body + 4, body + body_len);
    } else {
      need(std::memcmp(type, "brob", 4) != 0 || body_len < 4 ||
               (std::memcmp(body, "jxlc", 4) != 0 && std::memcmp(body, "jxlp", 4) != 0),
           "a Brotli-compressed codestream box is not supported");
    }
    pos += (size_t)len;
  }
  need(jxlc || last_seen, "container without a complete codestream");
  return true;
}

void decode(const uint8_t* data, size_t size, Decoded* out) {
  std::vector<uint8_t> boxed;
  if (data && unbox(data, size, &boxed)) {
    decode(boxed.data(), boxed.size(), out);
    return;
  }
  need(data && size >= 2 && data[0] == 0xFF && data[1] == 0x0A, "not a JPEG XL codestream");
  Reader r;
  r.b.data = data;
  r.b.size_bits = size * 8;
  r.b.pos = 16;
  ImageInfo& m = out->image;
  size_header(r, &m.width, &m.height);
  // The reference's default pixel budget (jpxl-core limits.rs:42, 2^30),
  // which bounds every allocation a hostile header can ask for.
  need((uint64_t)m.width * m.height <= t_max_pixels, "image larger than the pixel limit");
  bool preview = false, animation = false, timecodes = false;
  image_metadata(r, &m, &preview, &animation, &timecodes);
  need(!m.want_icc, "ICC profiles are not supported");
  r.pad_to_byte();
  need(!preview, "preview frames are not supported");
  FrameInfo& f = out->frame;
  for (;;) {
  f = FrameInfo{};
  frame_header(r, m, animation, timecodes, &f);
  if (f.frame_type == 1) {
    // An LF frame (F.1): modular, 1/8^lf_level of the image; its XYB is the
    // next VarDCT frame's LF (decode.rs:1686 decode_lf_frame, :1747).
    need(f.encoding == 1 && f.lf_level == 1 && m.xyb_encoded,
         "only modular LF frames at level 1 of XYB images are supported");
    f.width = (f.width + 7) / 8;
    f.height = (f.height + 7) / 8;
    std::vector<Section> sec;
    uint64_t end_byte = 0;
    read_toc(r, data, size, f, &sec, &end_byte);
    float m_lf[3] = {1.0f / 32.0f, 1.0f / 4.0f, 1.0f / 2.0f};
    decode_frame_modular(sec, out, m_lf);
    need(out->modular.size() == 3, "LF frame channels");
    const size_t cells = (size_t)f.width * f.height;
    VarDctFrame& vd = out->vardct;
    charge(cells, 3 * sizeof(float));
    for (auto& pl : vd.lf_frame) pl.assign(cells, 0.0f);
    const float mx = m_lf[0] / 128.0f, my = m_lf[1] / 128.0f, mb = m_lf[2] / 128.0f;
    for (size_t i = 0; i < cells; ++i) {
      const float yp = (float)out->modular[0].v[i], xp = (float)out->modular[1].v[i];
      const float bp = (float)out->modular[2].v[i];
      vd.lf_frame[0][i] = xp * mx;
      vd.lf_frame[1][i] = yp * my;
      vd.lf_frame[2][i] = (bp + yp) * mb;
    }
    out->modular.clear();
    r.b.pos = (size_t)end_byte * 8;
    continue;
  }
  break;
  }
  if (f.frame_type != 0) {
    static const char* kTypes[4] = {"regular", "LF", "reference-only", "skip-progressive"};
    throw Malformed{std::string("only regular frames are supported (first frame: ") +
                    kTypes[f.frame_type & 3] + ", " + (f.encoding ? "modular" : "VarDCT") +
                    ", flags " + std::to_string(f.flags) + ")"};
  }
  need(f.upsampling == 1, "upsampled frames are not supported");
  std::vector<Section> sec;
  uint64_t end_byte = 0;
  read_toc(r, data, size, f, &sec, &end_byte);
  const uint64_t nsec = sec.size();
  out->sections = nsec;
  out->section_sizes.resize(nsec);
  for (uint64_t i = 0; i < nsec; ++i) out->section_sizes[i] = sec[i].size_bytes;
  if (f.encoding == 0) decode_frame_vardct(sec, nsec == 1, out);
  else decode_frame_modular(sec, out);
  out->section_bits.resize(nsec);
  for (uint64_t i = 0; i < nsec; ++i) out->section_bits[i] = sec[i].r.b.pos - sec[i].start_bits;
}


}  // namespace cs
}  // namespace jpxlg

// ---- C ABI --------------------------------------------------------------------

namespace {
thread_local std::string g_codestream_error;
}

extern "C" const char* jpxlg_codestream_last_error(void) { return g_codestream_error.c_str(); }

extern "C" int jpxlg_codestream_open(const uint8_t* data, size_t size, jpxlg_codestream** out) {
  return jpxlg_codestream_open_limits(data, size, nullptr, out);
}

extern "C" int jpxlg_codestream_open_limits(const uint8_t* data, size_t size,
                                            const jpxlg_codestream_limits* limits,
                                            jpxlg_codestream** out) {
  if (!out || (!data && size)) return JPXLG_ERR_ARGUMENT;
  if (limits && (limits->max_pixels == 0 || limits->max_alloc_bytes == 0))
    return JPXLG_ERR_ARGUMENT;
  jpxlg::cs::t_max_pixels = limits ? limits->max_pixels : (1ull << 30);
  jpxlg::cs::t_max_alloc_bytes = limits ? limits->max_alloc_bytes : (4ull << 30);
  *out = nullptr;
  std::unique_ptr<jpxlg_codestream> cs(new (std::nothrow) jpxlg_codestream);
  if (!cs) return JPXLG_ERR_ARGUMENT;
  try {
    jpxlg::cs::t_alloc_bytes = 0;
    jpxlg::cs::decode(data, size, &cs->d);
  } catch (const jpxlg::cs::Malformed& e) {
    g_codestream_error = e.what;
    return JPXLG_ERR_STREAM;
  } catch (const std::bad_alloc&) {
    g_codestream_error = "out of host memory";
    return JPXLG_ERR_STREAM;
  }
  g_codestream_error.clear();
  *out = cs.release();
  return JPXLG_OK;
}

extern "C" int jpxlg_codestream_info(const jpxlg_codestream* cs, jpxlg_codestream_info_t* info) {
  if (!cs || !info) return JPXLG_ERR_ARGUMENT;
  const jpxlg::cs::Decoded& d = cs->d;
  std::memset(info, 0, sizeof(*info));
  info->width = d.image.width;
  info->height = d.image.height;
  info->bits_per_sample = d.image.bits_per_sample;
  info->xyb_encoded = d.image.xyb_encoded;
  info->colour_space = (uint32_t)d.image.colour_space;
  info->transfer = d.image.transfer;
  info->encoding = (uint32_t)d.frame.encoding;
  info->num_passes = d.frame.num_passes;
  info->gaborish = d.frame.gab;
  info->gaborish_custom = d.frame.gab_custom;
  info->epf_iters = d.frame.epf_iters;
  info->x_qm_scale = d.frame.x_qm_scale;
  info->b_qm_scale = d.frame.b_qm_scale;
  info->adaptive_lf_smoothing = (d.frame.flags & 128) ? 0 : 1;
  info->global_scale = d.vardct.global_scale;
  info->quant_lf = d.vardct.quant_lf;
  info->extra_precision = d.vardct.extra_precision;
  info->default_matrices = d.vardct.default_matrices;
  info->default_lf_dequant = d.vardct.m_lf[0] == 1.0f / 32.0f && d.vardct.m_lf[1] == 0.25f &&
                             d.vardct.m_lf[2] == 0.5f;
  info->default_chroma_correlation = d.vardct.colour_factor == 84 &&
                                     d.vardct.base_corr_x == 0.0f && d.vardct.base_corr_b == 1.0f;
  info->x_factor_lf = d.vardct.x_factor_lf;
  info->b_factor_lf = d.vardct.b_factor_lf;
  info->blocks_w = d.vardct.bw;
  info->blocks_h = d.vardct.bh;
  info->num_varblocks = (uint32_t)d.vardct.varblocks.size();
  info->num_channels = (uint32_t)(d.modular.size() + d.extra.size());
  info->sections = (uint32_t)d.sections;
  uint32_t exact = 0;
  for (uint64_t i = 0; i < d.sections && i < d.section_bits.size(); ++i)
    if ((d.section_bits[i] + 7) / 8 == d.section_sizes[i]) ++exact;
  info->sections_exact = exact;
  for (int i = 0; i < 27; ++i) info->transform_counts[i] = d.vardct.histogram_counts[i];
  info->orientation = d.image.orientation;
  info->num_extra = (uint32_t)d.image.extra.size();
  return JPXLG_OK;
}

extern "C" int jpxlg_codestream_blocks(const jpxlg_codestream* cs, int32_t* lf, uint8_t* block_map,
                                       uint32_t* hf_mul, uint8_t* sharpness, int8_t* x_from_y,
                                       int8_t* b_from_y) {
  if (!cs) return JPXLG_ERR_ARGUMENT;
  const jpxlg::cs::VarDctFrame& v = cs->d.vardct;
  const size_t n = (size_t)v.bw * v.bh, t = (size_t)v.tiles_w * v.tiles_h;
  if (lf)
    for (int c = 0; c < 3; ++c) std::memcpy(lf + c * n, v.lf[c].data(), n * sizeof(int32_t));
  if (block_map) std::memcpy(block_map, v.block_map.data(), n);
  if (hf_mul) std::memcpy(hf_mul, v.hf_mul.data(), n * sizeof(uint32_t));
  if (sharpness) std::memcpy(sharpness, v.sharpness.data(), n);
  if (x_from_y) std::memcpy(x_from_y, v.x_from_y.data(), t);
  if (b_from_y) std::memcpy(b_from_y, v.b_from_y.data(), t);
  return JPXLG_OK;
}

// The quantized coefficients as the plan's coefficient image: 3 planes of
// (8*bh) x (8*bw); a varblock's landscape matrix sits at its position, and a
// portrait varblock's matrix transposed.
extern "C" int jpxlg_codestream_coefficients(const jpxlg_codestream* cs, int32_t* out) {
  if (!cs || !out) return JPXLG_ERR_ARGUMENT;
  const jpxlg::cs::VarDctFrame& v = cs->d.vardct;
  const size_t W8 = (size_t)v.bw * 8, H8 = (size_t)v.bh * 8, plane = W8 * H8;
  std::memset(out, 0, 3 * plane * sizeof(int32_t));
  for (const jpxlg::cs::Varblock& vb : v.varblocks) {
    const jpxlg::cs::TransformShape s = jpxlg::cs::transform_shape(vb.transform);
    const uint32_t cr = std::min(s.rows, s.cols) * 8, cc = std::max(s.rows, s.cols) * 8;
    const bool portrait = s.rows > s.cols;
    for (int c = 0; c < 3; ++c)
      for (uint32_t y = 0; y < cr; ++y)
        for (uint32_t x = 0; x < cc; ++x) {
          const size_t pos = portrait ? (size_t)(vb.by * 8 + x) * W8 + vb.bx * 8 + y
                                      : (size_t)(vb.by * 8 + y) * W8 + vb.bx * 8 + x;
          out[c * plane + pos] = v.coeffs[c][vb.coeff_offset + y * cc + x];
        }
  }
  return JPXLG_OK;
}

extern "C" int jpxlg_codestream_channel(const jpxlg_codestream* cs, uint32_t index, int32_t* out) {
  const size_t nm = cs ? cs->d.modular.size() : 0;
  if (!cs || !out || index >= nm + (cs->d.frame.encoding == 1 ? cs->d.extra.size() : 0))
    return JPXLG_ERR_ARGUMENT;
  const jpxlg::cs::Channel& c = index < nm ? cs->d.modular[index] : cs->d.extra[index - nm];
  std::memcpy(out, c.v.data(), c.v.size() * sizeof(int32_t));
  return JPXLG_OK;
}

// A frame's extra channel as floats (sample / (2^bits - 1)), its width x
// height.
extern "C" int jpxlg_codestream_extra(const jpxlg_codestream* cs, uint32_t index, float* out) {
  if (!cs || !out || index >= cs->d.extra.size() || index >= cs->d.image.extra.size())
    return JPXLG_ERR_ARGUMENT;
  const jpxlg::cs::Channel& c = cs->d.extra[index];
  const uint32_t bits = cs->d.image.extra[index].bits;
  const float maxv = bits >= 32 ? 4294967295.0f : (float)((1ull << bits) - 1);
  for (size_t i = 0; i < c.v.size(); ++i) out[i] = (float)c.v[i] / maxv;
  return JPXLG_OK;
}

extern "C" int jpxlg_codestream_destroy(jpxlg_codestream* cs) {
  delete cs;
  return JPXLG_OK;
}
