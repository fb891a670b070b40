// entropy.cu — the symbol-decoder C ABI (jpxlg_symbols_*) over entropy.h.
#include "entropy.h"

#include "jpxlg.h"

struct jpxlg_symbols {
  std::vector<uint8_t> data;
  jpxlg::entropy::Bits bits;
  jpxlg::entropy::Stream stream;
};

extern "C" int jpxlg_symbols_open(const uint8_t* data, size_t size, size_t bit_offset,
                                  uint32_t num_dist, jpxlg_symbols** out) {
  if (!out || (!data && size) || num_dist == 0 || bit_offset > size * 8) return JPXLG_ERR_ARGUMENT;
  *out = nullptr;
  jpxlg_symbols* s = new (std::nothrow) jpxlg_symbols;
  if (!s) return JPXLG_ERR_ARGUMENT;
  s->data.assign(data, data + size);
  s->bits.data = s->data.data();
  s->bits.size_bits = size * 8;
  s->bits.pos = bit_offset;
  if (!s->stream.open(s->bits, num_dist, 0, false)) {
    delete s;
    return JPXLG_ERR_STREAM;
  }
  *out = s;
  return JPXLG_OK;
}

extern "C" int jpxlg_symbols_read(jpxlg_symbols* s, uint32_t ctx, uint32_t* value) {
  if (!s || !value) return JPXLG_ERR_ARGUMENT;
  return s->stream.read(s->bits, ctx, value) ? JPXLG_OK : JPXLG_ERR_STREAM;
}

extern "C" int jpxlg_symbols_read_many(jpxlg_symbols* s, const uint32_t* ctx, size_t n,
                                       uint32_t* values) {
  if (!s || (n && (!ctx || !values))) return JPXLG_ERR_ARGUMENT;
  for (size_t i = 0; i < n; ++i)
    if (!s->stream.read(s->bits, ctx[i], values + i)) return JPXLG_ERR_STREAM;
  return JPXLG_OK;
}

extern "C" int jpxlg_symbols_set_dist_multiplier(jpxlg_symbols* s, uint32_t multiplier) {
  if (!s) return JPXLG_ERR_ARGUMENT;
  s->stream.dist_multiplier = multiplier;
  return JPXLG_OK;
}

extern "C" int jpxlg_symbols_finish(const jpxlg_symbols* s) {
  if (!s) return JPXLG_ERR_ARGUMENT;
  return s->stream.final_state() ? JPXLG_OK : JPXLG_ERR_STREAM;
}

extern "C" size_t jpxlg_symbols_bits_read(const jpxlg_symbols* s) { return s ? s->bits.pos : 0; }

extern "C" int jpxlg_symbols_destroy(jpxlg_symbols* s) {
  delete s;
  return JPXLG_OK;
}
