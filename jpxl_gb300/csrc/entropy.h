// entropy.h — host-side entropy decoding of JPEG XL entropy-coded streams
// (ISO/IEC 18181-1 Annex C), as jpxl-entropy's SymbolDecoder reads them
// (crates/jpxl-entropy/src/decoder.rs): the distribution bundle (LZ77
// parameters, context-to-cluster map, hybrid-uint configurations, then
// prefix codes or 12-bit ANS distributions) and the symbol stream (rANS or
// canonical prefix decoding, hybrid-uint extra bits, LZ77 copies).
//
// Integer arithmetic only, so the result is exact by construction.  Every
// read is bounds-checked: a stream that ends early or breaks a rule of the
// standard makes the call return false, never a crash.  Where Annex C admits
// two readings the reference's choice is followed: a nested (context-map)
// decoder of a two-context stream must not enable LZ77, and the nesting
// depth is bounded at four.  Shared by the symbol-decoder C ABI (entropy.cu)
// and the codestream reader (codestream.cu).  Code only; no GPU is involved.
#pragma once
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

namespace jpxlg {
namespace entropy {

// LSB-first bit reader over a byte buffer (the codestream's bit order).
struct Bits {
  const uint8_t* data = nullptr;
  size_t size_bits = 0;
  size_t pos = 0;
  bool read(uint32_t n, uint32_t* out) {
    if (n > 32 || pos + n > size_bits) return false;
    uint64_t v = 0;
    for (uint32_t i = 0; i < n;) {
      const size_t byte = (pos + i) >> 3, shift = (pos + i) & 7;
      const uint32_t take = std::min<uint32_t>(n - i, 8 - (uint32_t)shift);
      const uint64_t chunk = (data[byte] >> shift) & ((1u << take) - 1);
      v |= chunk << i;
      i += take;
    }
    pos += n;
    *out = (uint32_t)v;
    return true;
  }
  bool bit(bool* b) {
    uint32_t v;
    if (!read(1, &v)) return false;
    *b = v != 0;
    return true;
  }
};

#define JPXLG_REQ(cond) \
  do {                  \
    if (!(cond)) return false; \
  } while (0)

// U8() of the standard: Bool() ? u(3) = n, (1 << n) + u(n) : 0.
static bool read_u8(Bits& b, uint32_t* out) {
  bool nz;
  JPXLG_REQ(b.bit(&nz));
  if (!nz) {
    *out = 0;
    return true;
  }
  uint32_t n, v;
  JPXLG_REQ(b.read(3, &n) && b.read(n, &v));
  *out = (1u << n) + v;
  return true;
}

// U32(d0, d1, d2, d3): a 2-bit selector, then the chosen distribution,
// either a constant or u(bits) + offset.
struct U32Dist {
  uint32_t bits, value;  // bits == 0: the constant `value`
};
static bool read_u32(Bits& b, const U32Dist d[4], uint32_t* out) {
  uint32_t sel, v = 0;
  JPXLG_REQ(b.read(2, &sel));
  if (d[sel].bits) JPXLG_REQ(b.read(d[sel].bits, &v));
  *out = v + d[sel].value;
  return true;
}

static uint32_t bit_width(uint32_t n) { return n ? 32u - (uint32_t)__builtin_clz(n) : 0u; }

// C.2.3 hybrid unsigned integer configuration and C.3.3 value reconstruction.
struct Hybrid {
  uint32_t split_exp = 0, msb = 0, lsb = 0;
  bool read_config(Bits& b, uint32_t log_alpha) {
    JPXLG_REQ(log_alpha <= 15);
    JPXLG_REQ(b.read(bit_width(log_alpha), &split_exp));
    msb = lsb = 0;
    if (split_exp == log_alpha) return true;
    JPXLG_REQ(b.read(bit_width(split_exp), &msb));
    JPXLG_REQ(msb <= split_exp);
    JPXLG_REQ(b.read(bit_width(split_exp - msb), &lsb));
    JPXLG_REQ(lsb <= split_exp - msb);
    return true;
  }
  bool value(Bits& b, uint32_t token, uint32_t* out) const {
    const uint32_t split = 1u << split_exp;
    if (token < split) {
      *out = token;
      return true;
    }
    const uint32_t in_token = msb + lsb;
    const uint64_t n = (uint64_t)(split_exp - in_token) + ((token - split) >> in_token);
    JPXLG_REQ(n < 32);
    const uint32_t low = token & ((1u << lsb) - 1);
    const uint32_t mid = ((token >> lsb) & ((1u << msb) - 1)) | (1u << msb);
    uint32_t extra;
    JPXLG_REQ(b.read((uint32_t)n, &extra));
    const uint64_t v = ((((uint64_t)mid << n) | extra) << lsb) | low;
    JPXLG_REQ(v <= 0xffffffffull);
    *out = (uint32_t)v;
    return true;
  }
};

// ---- C.2.5 / C.2.6 / C.3.2: 12-bit ANS ------------------------------------

constexpr uint32_t kAnsTotal = 1u << 12;
constexpr uint32_t kAnsFinal = 0x130000u;

// The standard's prefix code for log counts (C.2.5): (length, code bits read
// most-significant first) of symbols 0..13.
static const uint8_t kLogCountLen[14] = {5, 4, 4, 4, 4, 4, 3, 3, 3, 3, 3, 6, 7, 7};
static const uint8_t kLogCountCode[14] = {0x11, 0xd, 0xf, 0xc, 0x9, 0xe, 0x1,
                                          0x2,  0x5, 0x3, 0x0, 0x21, 0x40, 0x41};

static bool read_logcount(Bits& b, uint32_t* out) {
  uint32_t code = 0;
  for (uint32_t len = 1; len <= 7; ++len) {
    uint32_t bit;
    JPXLG_REQ(b.read(1, &bit));
    code = (code << 1) | bit;
    for (uint32_t s = 0; s < 14; ++s)
      if (kLogCountLen[s] == len && kLogCountCode[s] == code) {
        *out = s;
        return true;
      }
  }
  return false;
}

struct Ans {
  uint32_t log_bucket = 0, bucket = 0;
  std::vector<uint32_t> prob, sym, off, cut;

  // C.2.5 ReadDistribution: a one- or two-symbol form, a flat form, or log
  // counts with run-length repeats and refinement bits; the largest log
  // count's position takes the remainder of the 4096 total.
  bool read(Bits& b, uint32_t log_alpha) {
    JPXLG_REQ(log_alpha <= 12);
    const uint32_t table = 1u << log_alpha;
    std::vector<uint32_t> d(table, 0);
    size_t alphabet = 0;
    bool f;
    JPXLG_REQ(b.bit(&f));
    if (f) {
      JPXLG_REQ(b.bit(&f));
      if (f) {
        uint32_t v1, v2, p;
        JPXLG_REQ(read_u8(b, &v1) && read_u8(b, &v2));
        JPXLG_REQ(v1 < table && v2 < table && v1 != v2);
        JPXLG_REQ(b.read(12, &p));
        d[v1] = p;
        d[v2] = kAnsTotal - p;
        alphabet = 1 + std::max(v1, v2);
      } else {
        uint32_t x;
        JPXLG_REQ(read_u8(b, &x) && x < table);
        d[x] = kAnsTotal;
        alphabet = 1 + x;
      }
      return build(std::move(d), alphabet, log_alpha);
    }
    JPXLG_REQ(b.bit(&f));
    if (f) {
      uint32_t a;
      JPXLG_REQ(read_u8(b, &a));
      alphabet = (size_t)a + 1;
      JPXLG_REQ(alphabet <= table);
      const uint32_t share = kAnsTotal / (uint32_t)alphabet, rem = kAnsTotal % (uint32_t)alphabet;
      for (size_t i = 0; i < alphabet; ++i) d[i] = share + (i < rem ? 1u : 0u);
      return build(std::move(d), alphabet, log_alpha);
    }
    uint32_t len = 0;
    while (len < 3) {
      JPXLG_REQ(b.bit(&f));
      if (!f) break;
      ++len;
    }
    uint32_t sh;
    JPXLG_REQ(b.read(len, &sh));
    const int shift = (int)(sh + (1u << len) - 1);
    JPXLG_REQ(shift <= 13);
    uint32_t a;
    JPXLG_REQ(read_u8(b, &a));
    alphabet = (size_t)a + 3;
    JPXLG_REQ(alphabet <= table);
    std::vector<uint32_t> logc(alphabet, 0), same(alphabet, 0);
    int omit_log = -1, omit_pos = -1;
    for (size_t i = 0; i < alphabet;) {
      uint32_t lc;
      JPXLG_REQ(read_logcount(b, &lc));
      logc[i] = lc;
      if (lc == 13) {
        uint32_t rle;
        JPXLG_REQ(read_u8(b, &rle));
        same[i] = rle + 5;
        i += (size_t)rle + 4;
        continue;
      }
      if ((int)lc > omit_log) {
        omit_log = (int)lc;
        omit_pos = (int)i;
      }
      ++i;
    }
    JPXLG_REQ(omit_pos >= 0);
    uint32_t total = 0, numsame = 0, prev = 0;
    for (size_t i = 0; i < alphabet; ++i) {
      if (same[i]) {
        numsame = same[i] - 1;
        prev = i > 0 ? d[i - 1] : 0;
      }
      if (numsame > 0) {
        d[i] = prev;
        --numsame;
      } else {
        const uint32_t code = logc[i];
        if ((int)i == omit_pos || code == 0) continue;
        if (code == 1) {
          d[i] = 1;
        } else {
          const int bc = std::min(std::max(shift - ((12 - (int)code + 1) >> 1), 0), (int)code - 1);
          uint32_t extra;
          JPXLG_REQ(b.read((uint32_t)bc, &extra));
          d[i] = (1u << (code - 1)) + (extra << (code - 1 - (uint32_t)bc));
        }
      }
      total += d[i];
      JPXLG_REQ(total <= kAnsTotal);
    }
    d[omit_pos] = kAnsTotal - total;
    return build(std::move(d), alphabet, log_alpha);
  }

  // C.2.6 alias mapping: every bucket of 2^(12 - log_alpha) slots holds its
  // own symbol below `cut` and one overfull symbol's slots above it.
  bool build(std::vector<uint32_t> d, size_t alphabet, uint32_t log_alpha) {
    const size_t table = (size_t)1 << log_alpha;
    JPXLG_REQ(d.size() == table && alphabet <= table);
    uint64_t sum = 0;
    for (uint32_t p : d) sum += p;
    JPXLG_REQ(sum == kAnsTotal);
    log_bucket = 12 - log_alpha;
    bucket = 1u << log_bucket;
    prob = std::move(d);
    sym.assign(table, 0);
    off.assign(table, 0);
    cut.assign(table, 0);
    size_t nonzero = 0, last = 0;
    for (size_t i = 0; i < table; ++i)
      if (prob[i]) {
        ++nonzero;
        last = i;
      }
    if (nonzero == 1) {
      for (size_t i = 0; i < table; ++i) {
        sym[i] = (uint32_t)last;
        off[i] = bucket * (uint32_t)i;
        cut[i] = 0;
      }
      return true;
    }
    std::vector<int64_t> c(table, 0), o(table, 0);
    std::vector<size_t> over, under;
    const int64_t bk = bucket;
    for (size_t i = 0; i < alphabet; ++i) {
      c[i] = prob[i];
      sym[i] = (uint32_t)i;
      if (c[i] > bk) over.push_back(i);
      else if (c[i] < bk) under.push_back(i);
    }
    for (size_t i = alphabet; i < table; ++i) {
      c[i] = 0;
      under.push_back(i);
    }
    while (!over.empty()) {
      const size_t ov = over.back();
      over.pop_back();
      JPXLG_REQ(!under.empty());
      const size_t un = under.back();
      under.pop_back();
      const int64_t by = bk - c[un];
      c[ov] -= by;
      sym[un] = (uint32_t)ov;
      o[un] = c[ov];
      if (c[ov] < bk) under.push_back(ov);
      else if (c[ov] > bk) over.push_back(ov);
    }
    JPXLG_REQ(under.empty());
    for (size_t i = 0; i < table; ++i) {
      if (c[i] == bk) {
        sym[i] = (uint32_t)i;
        o[i] = 0;
        c[i] = 0;
      } else {
        o[i] -= c[i];
      }
      JPXLG_REQ(c[i] >= 0 && o[i] >= 0 && o[i] <= 0xffffffffll);
      cut[i] = (uint32_t)c[i];
      off[i] = (uint32_t)o[i];
    }
    return true;
  }

  // C.3.2: one symbol from the 32-bit state, refilling 16 bits below 2^16.
  bool decode(Bits& b, uint32_t* state, uint32_t* out) const {
    const uint32_t x = *state & 0xfff;
    const uint32_t i = x >> log_bucket, pos = x & (bucket - 1);
    uint32_t s, offset;
    if (pos >= cut[i]) {
      s = sym[i];
      offset = off[i] + pos;
    } else {
      s = i;
      offset = pos;
    }
    const uint64_t next = (uint64_t)prob[s] * (*state >> 12) + offset;
    JPXLG_REQ(next <= 0xffffffffull);
    uint32_t st = (uint32_t)next;
    if (st < (1u << 16)) {
      uint32_t more;
      JPXLG_REQ(b.read(16, &more));
      st = (st << 16) | more;
    }
    *state = st;
    *out = s;
    return true;
  }
};

// ---- C.2.4: prefix codes (RFC 7932 sections 3.2, 3.4, 3.5) ----------------

constexpr int kMaxCodeLen = 15;

struct Prefix {
  uint32_t counts[kMaxCodeLen + 1] = {};
  std::vector<uint32_t> sorted;  // symbols by code length, then symbol
  int64_t single = -1;

  bool from_lengths(const uint8_t* len, size_t n) {
    std::fill(counts, counts + kMaxCodeLen + 1, 0u);
    sorted.clear();
    size_t present = 0, last = 0;
    for (size_t s = 0; s < n; ++s) {
      if (!len[s]) continue;
      JPXLG_REQ(len[s] <= kMaxCodeLen);
      ++counts[len[s]];
      ++present;
      last = s;
    }
    JPXLG_REQ(present > 0);
    if (present == 1) {
      single = (int64_t)last;
      return true;
    }
    single = -1;
    uint64_t used = 0;
    for (int l = 1; l <= kMaxCodeLen; ++l) used += (uint64_t)counts[l] << (kMaxCodeLen - l);
    JPXLG_REQ(used == (1ull << kMaxCodeLen));  // complete: neither short nor over-subscribed
    for (int l = 1; l <= kMaxCodeLen; ++l)
      for (size_t s = 0; s < n; ++s)
        if (len[s] == l) sorted.push_back((uint32_t)s);
    return true;
  }

  // Canonical decoding one bit at a time, the code's most significant bit
  // first (RFC 7932 3.1).
  bool decode(Bits& b, uint32_t* out) const {
    if (single >= 0) {
      *out = (uint32_t)single;
      return true;
    }
    uint32_t code = 0, first = 0, index = 0;
    for (int l = 1; l <= kMaxCodeLen; ++l) {
      uint32_t bit;
      JPXLG_REQ(b.read(1, &bit));
      code |= bit;
      if (code < first + counts[l]) {
        const uint32_t p = index + (code - first);
        JPXLG_REQ(p < sorted.size());
        *out = sorted[p];
        return true;
      }
      index += counts[l];
      first = (first + counts[l]) << 1;
      code <<= 1;
    }
    return false;
  }

  bool read(Bits& b, size_t alphabet) {
    JPXLG_REQ(alphabet >= 1);
    if (alphabet == 1) {
      single = 0;
      return true;
    }
    uint32_t hskip;
    JPXLG_REQ(b.read(2, &hskip));
    return hskip == 1 ? read_simple(b, alphabet) : read_complex(b, alphabet, hskip);
  }

  bool read_simple(Bits& b, size_t alphabet) {
    const uint32_t abits = bit_width((uint32_t)(alphabet - 1));
    uint32_t nsym;
    JPXLG_REQ(b.read(2, &nsym));
    ++nsym;
    uint32_t syms[4];
    for (uint32_t i = 0; i < nsym; ++i) {
      JPXLG_REQ(b.read(abits, &syms[i]));
      JPXLG_REQ(syms[i] < alphabet);
      for (uint32_t k = 0; k < i; ++k) JPXLG_REQ(syms[k] != syms[i]);
    }
    if (nsym == 1) {
      single = syms[0];
      return true;
    }
    static const uint8_t k2[2] = {1, 1}, k3[3] = {1, 2, 2}, k4a[4] = {1, 2, 3, 3},
                         k4b[4] = {2, 2, 2, 2};
    const uint8_t* lens = nsym == 2 ? k2 : (nsym == 3 ? k3 : nullptr);
    if (nsym == 4) {
      bool tree;
      JPXLG_REQ(b.bit(&tree));
      lens = tree ? k4a : k4b;
    }
    std::vector<uint8_t> l(alphabet, 0);
    for (uint32_t i = 0; i < nsym; ++i) l[syms[i]] = lens[i];
    return from_lengths(l.data(), alphabet);
  }

  bool read_complex(Bits& b, size_t alphabet, uint32_t hskip) {
    // The code-length code: lengths of the 18 code-length symbols in the
    // RFC's order, each read with the fixed code of lengths {2,4,3,2,2,4}.
    static const uint8_t kOrder[18] = {1, 2, 3, 4, 0, 5, 17, 6, 16, 7, 8, 9, 10, 11, 12, 13, 14, 15};
    static const uint8_t kFixed[6] = {2, 4, 3, 2, 2, 4};
    Prefix fixed;
    JPXLG_REQ(fixed.from_lengths(kFixed, 6));
    uint8_t clc[18] = {};
    int space = 32, nonzero = 0;
    for (int k = (int)hskip; k < 18; ++k) {
      uint32_t v;
      JPXLG_REQ(fixed.decode(b, &v));
      clc[kOrder[k]] = (uint8_t)v;
      if (v) {
        ++nonzero;
        space -= 32 >> v;
        if (space <= 0) break;
      }
    }
    JPXLG_REQ(nonzero == 1 || space == 0);
    Prefix lc;
    JPXLG_REQ(lc.from_lengths(clc, 18));
    std::vector<uint8_t> l(alphabet, 0);
    int64_t room = 32768;
    size_t i = 0;
    uint8_t prev_nz = 8, rep_len = 0;
    uint32_t repeat = 0;
    while (i < alphabet && room > 0) {
      uint32_t s;
      JPXLG_REQ(lc.decode(b, &s));
      if (s < 16) {
        repeat = 0;
        l[i++] = (uint8_t)s;
        if (s) {
          prev_nz = (uint8_t)s;
          room -= 32768 >> s;
        }
        continue;
      }
      JPXLG_REQ(s == 16 || s == 17);
      const uint32_t extra_bits = s == 16 ? 2 : 3;
      const uint8_t new_len = s == 16 ? prev_nz : 0;
      if (rep_len != new_len) {
        repeat = 0;
        rep_len = new_len;
      }
      const uint32_t before = repeat;
      if (repeat > 0) {
        JPXLG_REQ(repeat >= 2);
        const uint64_t r = (uint64_t)(repeat - 2) << extra_bits;
        JPXLG_REQ(r <= 0xffffffffull);
        repeat = (uint32_t)r;
      }
      uint32_t e;
      JPXLG_REQ(b.read(extra_bits, &e));
      const uint64_t r = (uint64_t)repeat + 3 + e;
      JPXLG_REQ(r <= 0xffffffffull);
      repeat = (uint32_t)r;
      const uint32_t count = repeat - before;
      JPXLG_REQ((uint64_t)i + count <= alphabet);
      std::fill(l.begin() + i, l.begin() + i + count, new_len);
      i += count;
      if (new_len) room -= (int64_t)count * (32768 >> new_len);
    }
    JPXLG_REQ(room == 0);
    return from_lengths(l.data(), alphabet);
  }
};

// ---- C.3.3 LZ77 -------------------------------------------------------------

constexpr uint32_t kLogWindow = 20;
constexpr uint64_t kWindow = 1ull << kLogWindow;

// Table C.2 (the standard's data): (dx, dy) of the 120 special distances.
static const int8_t kSpecial[120][2] = {
    {0, 1},  {1, 0},  {1, 1},  {-1, 1}, {0, 2},  {2, 0},  {1, 2},  {-1, 2}, {2, 1},  {-2, 1},
    {2, 2},  {-2, 2}, {0, 3},  {3, 0},  {1, 3},  {-1, 3}, {3, 1},  {-3, 1}, {2, 3},  {-2, 3},
    {3, 2},  {-3, 2}, {0, 4},  {4, 0},  {1, 4},  {-1, 4}, {4, 1},  {-4, 1}, {3, 3},  {-3, 3},
    {2, 4},  {-2, 4}, {4, 2},  {-4, 2}, {0, 5},  {3, 4},  {-3, 4}, {4, 3},  {-4, 3}, {5, 0},
    {1, 5},  {-1, 5}, {5, 1},  {-5, 1}, {2, 5},  {-2, 5}, {5, 2},  {-5, 2}, {4, 4},  {-4, 4},
    {3, 5},  {-3, 5}, {5, 3},  {-5, 3}, {0, 6},  {6, 0},  {1, 6},  {-1, 6}, {6, 1},  {-6, 1},
    {2, 6},  {-2, 6}, {6, 2},  {-6, 2}, {4, 5},  {-4, 5}, {5, 4},  {-5, 4}, {3, 6},  {-3, 6},
    {6, 3},  {-6, 3}, {0, 7},  {7, 0},  {1, 7},  {-1, 7}, {5, 5},  {-5, 5}, {7, 1},  {-7, 1},
    {4, 6},  {-4, 6}, {6, 4},  {-6, 4}, {2, 7},  {-2, 7}, {7, 2},  {-7, 2}, {3, 7},  {-3, 7},
    {7, 3},  {-7, 3}, {5, 6},  {-5, 6}, {6, 5},  {-6, 5}, {8, 0},  {4, 7},  {-4, 7}, {7, 4},
    {-7, 4}, {8, 1},  {8, 2},  {6, 6},  {-6, 6}, {8, 3},  {5, 7},  {-5, 7}, {7, 5},  {-7, 5},
    {8, 4},  {6, 7},  {-6, 7}, {7, 6},  {-7, 6}, {8, 5},  {7, 7},  {-7, 7}, {8, 6},  {8, 7}};

static uint64_t lz77_distance(uint32_t raw, uint32_t dist_multiplier) {
  if (dist_multiplier == 0) return (uint64_t)raw + 1;
  if (raw < 120) {
    const int64_t d = (int64_t)kSpecial[raw][0] + (int64_t)dist_multiplier * kSpecial[raw][1];
    return (uint64_t)std::max<int64_t>(d, 1);
  }
  return (uint64_t)raw - 119;
}

// ---- C.2.1 the distribution bundle and C.3 the symbol stream ---------------

constexpr size_t kMaxClusters = 256;
constexpr int kMaxDepth = 4;

struct Stream {
  bool lz_enabled = false;
  uint32_t lz_min_symbol = 0, lz_min_length = 0;
  size_t lz_dist_ctx = 0;
  Hybrid lz_len;
  std::vector<uint8_t> clusters;
  size_t num_clusters = 0;
  std::vector<Hybrid> configs;
  bool use_prefix = false;
  std::vector<Prefix> prefix;
  std::vector<Ans> ans;
  uint32_t state = 0;
  std::vector<uint32_t> window;
  uint64_t num_decoded = 0, copy_pos = 0;
  uint32_t num_to_copy = 0;
  uint32_t dist_multiplier = 0;

  // C.2.1: the bundle for num_dist contexts.  With defer_state the ANS state
  // is not read here but by restart(), for a bundle whose distributions are
  // shared by several later streams (a global MA tree's).
  bool open(Bits& b, size_t num_dist, int depth, bool forbid_lz77, bool defer_state = false) {
    JPXLG_REQ(depth <= kMaxDepth && num_dist >= 1);
    JPXLG_REQ(b.bit(&lz_enabled));
    if (lz_enabled) {
      JPXLG_REQ(!forbid_lz77);
      static const U32Dist kMinSymbol[4] = {{0, 224}, {0, 512}, {0, 4096}, {15, 8}};
      static const U32Dist kMinLength[4] = {{0, 3}, {0, 4}, {2, 5}, {8, 9}};
      JPXLG_REQ(read_u32(b, kMinSymbol, &lz_min_symbol));
      JPXLG_REQ(read_u32(b, kMinLength, &lz_min_length));
      lz_dist_ctx = num_dist;
      ++num_dist;
      JPXLG_REQ(lz_len.read_config(b, 8));
    }
    JPXLG_REQ(read_clusters(b, num_dist, depth));
    JPXLG_REQ(b.bit(&use_prefix));
    uint32_t log_alpha = 15;
    if (!use_prefix) {
      uint32_t v;
      JPXLG_REQ(b.read(2, &v));
      log_alpha = 5 + v;
    }
    configs.resize(num_clusters);
    for (auto& c : configs) JPXLG_REQ(c.read_config(b, log_alpha));
    if (use_prefix) {
      std::vector<size_t> counts(num_clusters, 1);
      for (auto& n : counts) {
        bool big;
        JPXLG_REQ(b.bit(&big));
        if (big) {
          uint32_t e, v;
          JPXLG_REQ(b.read(4, &e) && b.read(e, &v));
          n = 1 + ((size_t)1 << e) + v;
          JPXLG_REQ(n <= ((size_t)1 << 15));
        }
      }
      prefix.resize(num_clusters);
      for (size_t i = 0; i < num_clusters; ++i) JPXLG_REQ(prefix[i].read(b, counts[i]));
    } else {
      ans.resize(num_clusters);
      for (auto& a : ans) JPXLG_REQ(a.read(b, log_alpha));
      if (!defer_state) JPXLG_REQ(b.read(32, &state));
    }
    window.clear();
    return true;
  }

  // A new stream over the same distributions: a fresh ANS state and an empty
  // LZ77 window (jpxl-entropy decoder.rs:255 restart).
  bool restart(Bits& b) {
    if (!use_prefix) JPXLG_REQ(b.read(32, &state));
    window.clear();
    num_decoded = copy_pos = 0;
    num_to_copy = 0;
    return true;
  }

  // C.2.2: one cluster per context, read as fixed-width fields or as an
  // entropy-coded sequence (a nested single-context stream, optionally
  // move-to-front coded); the clusters must be dense.
  bool read_clusters(Bits& b, size_t num_dist, int depth) {
    clusters.assign(num_dist, 0);
    if (num_dist == 1) {
      num_clusters = 1;
      return true;
    }
    bool simple;
    JPXLG_REQ(b.bit(&simple));
    if (simple) {
      uint32_t nbits;
      JPXLG_REQ(b.read(2, &nbits));
      for (auto& c : clusters) {
        uint32_t v;
        JPXLG_REQ(b.read(nbits, &v));
        c = (uint8_t)v;
      }
    } else {
      bool mtf;
      JPXLG_REQ(b.bit(&mtf));
      JPXLG_REQ(depth < kMaxDepth);
      std::unique_ptr<Stream> nested(new Stream);
      JPXLG_REQ(nested->open(b, 1, depth + 1, num_dist == 2));
      for (auto& c : clusters) {
        uint32_t v;
        JPXLG_REQ(nested->read(b, 0, &v));
        JPXLG_REQ(v < 256);
        c = (uint8_t)v;
      }
      JPXLG_REQ(nested->final_state());
      if (mtf) {
        uint8_t order[256];
        for (int i = 0; i < 256; ++i) order[i] = (uint8_t)i;
        for (auto& c : clusters) {
          const uint8_t idx = c, v = order[idx];
          c = v;
          if (idx) {
            std::memmove(order + 1, order, idx);
            order[0] = v;
          }
        }
      }
    }
    num_clusters = 0;
    for (uint8_t c : clusters) num_clusters = std::max<size_t>(num_clusters, (size_t)c + 1);
    JPXLG_REQ(num_clusters <= kMaxClusters);
    std::vector<bool> seen(num_clusters, false);
    for (uint8_t c : clusters) seen[c] = true;
    for (bool s : seen) JPXLG_REQ(s);
    return true;
  }

  bool token(Bits& b, size_t cluster, uint32_t* out) {
    if (use_prefix) return prefix[cluster].decode(b, out);
    return ans[cluster].decode(b, &state, out);
  }

  // The window grows with the symbols decoded (up to 2^20 entries, then
  // wraps); slots not yet written read as zero, as in a zero-filled window.
  void push(uint32_t v) {
    if (window.size() < kWindow) window.push_back(v);
    else window[num_decoded & (kWindow - 1)] = v;
    ++num_decoded;
  }

  bool copied(uint32_t* out) {
    const uint64_t slot = copy_pos & (kWindow - 1);
    const uint32_t v = slot < window.size() ? window[slot] : 0u;
    ++copy_pos;
    --num_to_copy;
    push(v);
    *out = v;
    return true;
  }

  // C.3.3 DecodeHybridVarLenUint.
  bool read(Bits& b, size_t ctx, uint32_t* out) {
    if (lz_enabled && num_to_copy > 0) return copied(out);
    JPXLG_REQ(ctx < clusters.size());
    const size_t cl = clusters[ctx];
    uint32_t tok;
    JPXLG_REQ(token(b, cl, &tok));
    if (lz_enabled && tok >= lz_min_symbol) {
      uint32_t len;
      JPXLG_REQ(lz_len.value(b, tok - lz_min_symbol, &len));
      const uint64_t length = (uint64_t)len + lz_min_length;
      JPXLG_REQ(length <= 0xffffffffull);
      const size_t dcl = clusters[lz_dist_ctx];
      uint32_t dtok, raw;
      JPXLG_REQ(token(b, dcl, &dtok));
      JPXLG_REQ(configs[dcl].value(b, dtok, &raw));
      uint64_t dist = lz77_distance(raw, dist_multiplier);
      dist = std::min<uint64_t>(std::min<uint64_t>(dist, num_decoded), kWindow);
      num_to_copy = (uint32_t)length;
      copy_pos = num_decoded - dist;
      return copied(out);
    }
    uint32_t v;
    JPXLG_REQ(configs[cl].value(b, tok, &v));
    if (lz_enabled) push(v);
    *out = v;
    return true;
  }

  bool final_state() const { return use_prefix || state == kAnsFinal; }
};


}  // namespace entropy
}  // namespace jpxlg

