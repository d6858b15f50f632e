// codecs.cpp -- decoders for the compressed ExtendedOctree brick formats
// (IO/UVF/ExtendedOctree/ExtendedOctree.cpp:337-350): CT_ZLIB, CT_LZMA and
// CT_BZLIB, written from the public format descriptions:
//   * zlib / DEFLATE: RFC 1950 (stream wrapper, Adler-32) and RFC 1951
//     (stored, fixed-Huffman and dynamic-Huffman blocks);
//   * LZMA: the LZMA specification of the LZMA SDK (range decoder, literal /
//     match / repeated-match model), raw stream with properties lc, lp, pb and
//     no end marker, as LzmaCompression.cpp writes it;
//   * bzip2: the bzip2 stream format (Huffman + move-to-front + zero-run coding
//     of the Burrows-Wheeler transform of run-length-encoded data, CRC-32 per
//     block and per stream).
// Host code.  Every read is bounds-checked: corrupt input fails with
// TVK_ERR_INVALID_ARG instead of reading or writing out of range.
#include <cstring>
#include <string>
#include <vector>

#include "tvk_internal.h"

namespace tvk {
namespace {

[[noreturn]] void corrupt(const char* what) {
  fail(TVK_ERR_INVALID_ARG, std::string("ExtendedOctree: corrupt brick (") + what + ")");
}

// ------------------------------------------------------------------ DEFLATE

// LSB-first bit reader over a byte buffer (RFC 1951 section 3.1.1).
struct LsbBits {
  const uint8_t* p;
  size_t n, pos = 0;
  uint64_t acc = 0;
  int cnt = 0;
  LsbBits(const uint8_t* d, size_t len) : p(d), n(len) {}
  void refill(int need) {
    while (cnt < need) {
      if (pos >= n) corrupt("deflate stream ends early");
      acc |= uint64_t(p[pos++]) << cnt;
      cnt += 8;
    }
  }
  uint32_t bits(int k) {
    if (k == 0) return 0;
    refill(k);
    const uint32_t v = uint32_t(acc & ((uint64_t(1) << k) - 1));
    acc >>= k;
    cnt -= k;
    return v;
  }
  void align_byte() {
    const int drop = cnt & 7;
    acc >>= drop;
    cnt -= drop;
  }
};

// Canonical Huffman decoding table (RFC 1951 section 3.2.2): counts per code
// length and the symbols sorted by code.
struct Huffman {
  uint16_t count[16] = {0};
  std::vector<uint16_t> symbol;
  void build(const uint8_t* lengths, int n) {
    std::memset(count, 0, sizeof count);
    for (int i = 0; i < n; ++i) count[lengths[i]]++;
    count[0] = 0;
    int left = 1;
    for (int len = 1; len < 16; ++len) {
      left <<= 1;
      left -= count[len];
      if (left < 0) corrupt("over-subscribed Huffman code");
    }
    uint16_t offs[16];
    offs[1] = 0;
    for (int len = 1; len < 15; ++len) offs[len + 1] = uint16_t(offs[len] + count[len]);
    symbol.assign(size_t(n), 0);
    for (int i = 0; i < n; ++i)
      if (lengths[i]) symbol[offs[lengths[i]]++] = uint16_t(i);
  }
  int decode(LsbBits& br) const {
    int code = 0, first = 0, index = 0;
    for (int len = 1; len < 16; ++len) {
      code |= int(br.bits(1));
      const int c = count[len];
      if (code - c < first) return symbol[size_t(index + (code - first))];
      index += c;
      first += c;
      first <<= 1;
      code <<= 1;
    }
    corrupt("invalid Huffman code");
  }
};

const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2,
                               2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,    2,    3,    4,    5,    7,     9,     13,    17,  25,
                                33,   49,   65,   97,   129,  193,   257,   385,   513, 769,
                                1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2,  3,  3,  4,  4,  5,  5,  6,
                                6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

void inflate_block(LsbBits& br, const Huffman& lit, const Huffman& dist, uint8_t* out,
                   size_t out_n, size_t& o) {
  for (;;) {
    const int sym = lit.decode(br);
    if (sym < 256) {
      if (o >= out_n) corrupt("deflate output overruns the brick");
      out[o++] = uint8_t(sym);
    } else if (sym == 256) {
      return;
    } else {
      const int li = sym - 257;
      if (li >= 29) corrupt("bad length symbol");
      const size_t len = kLenBase[li] + br.bits(kLenExtra[li]);
      const int di = dist.decode(br);
      if (di >= 30) corrupt("bad distance symbol");
      const size_t d = kDistBase[di] + br.bits(kDistExtra[di]);
      if (d > o) corrupt("distance before the start of the brick");
      if (len > out_n - o) corrupt("deflate output overruns the brick");
      for (size_t k = 0; k < len; ++k, ++o) out[o] = out[o - d];
    }
  }
}

}  // namespace

// RFC 1950 wrapper around RFC 1951 blocks, then the Adler-32 of the output.
void zlib_decode(const uint8_t* in, size_t n, uint8_t* out, size_t out_n) {
  if (n < 6) corrupt("zlib stream too short");
  const uint32_t cmf = in[0], flg = in[1];
  if ((cmf & 15) != 8 || (cmf >> 4) > 7 || ((cmf << 8) | flg) % 31 != 0)
    corrupt("bad zlib header");
  if (flg & 0x20) corrupt("zlib preset dictionary");
  LsbBits br(in + 2, n - 2);
  size_t o = 0;
  int last = 0;
  while (!last) {
    last = int(br.bits(1));
    const uint32_t type = br.bits(2);
    if (type == 0) {  // stored
      br.align_byte();
      const uint32_t len = br.bits(16), nlen = br.bits(16);
      if ((len ^ 0xffffu) != nlen) corrupt("stored block length");
      for (uint32_t k = 0; k < len; ++k) {
        if (o >= out_n) corrupt("deflate output overruns the brick");
        out[o++] = uint8_t(br.bits(8));
      }
    } else if (type == 1) {  // fixed Huffman codes (RFC 1951 section 3.2.6)
      static const Huffman lit = [] {
        uint8_t l[288];
        for (int i = 0; i < 144; ++i) l[i] = 8;
        for (int i = 144; i < 256; ++i) l[i] = 9;
        for (int i = 256; i < 280; ++i) l[i] = 7;
        for (int i = 280; i < 288; ++i) l[i] = 8;
        Huffman h;
        h.build(l, 288);
        return h;
      }();
      static const Huffman dist = [] {
        uint8_t d[30];
        for (int i = 0; i < 30; ++i) d[i] = 5;
        Huffman h;
        h.build(d, 30);
        return h;
      }();
      inflate_block(br, lit, dist, out, out_n, o);
    } else if (type == 2) {  // dynamic Huffman codes (RFC 1951 section 3.2.7)
      const int hlit = int(br.bits(5)) + 257, hdist = int(br.bits(5)) + 1,
                hclen = int(br.bits(4)) + 4;
      if (hlit > 286 || hdist > 30) corrupt("too many length or distance codes");
      static const uint8_t order[19] = {16, 17, 18, 0, 8,  7, 9,  6, 10, 5,
                                        11, 4,  12, 3, 13, 2, 14, 1, 15};
      uint8_t cl[19] = {0};
      for (int i = 0; i < hclen; ++i) cl[order[i]] = uint8_t(br.bits(3));
      Huffman clh;
      clh.build(cl, 19);
      uint8_t lens[320] = {0};
      int i = 0;
      while (i < hlit + hdist) {
        const int sym = clh.decode(br);
        if (sym < 16) {
          lens[i++] = uint8_t(sym);
        } else {
          int rep = 0;
          uint8_t val = 0;
          if (sym == 16) {
            if (i == 0) corrupt("repeat with no previous length");
            val = lens[i - 1];
            rep = 3 + int(br.bits(2));
          } else if (sym == 17) {
            rep = 3 + int(br.bits(3));
          } else {
            rep = 11 + int(br.bits(7));
          }
          if (i + rep > hlit + hdist) corrupt("code lengths overrun");
          while (rep--) lens[i++] = val;
        }
      }
      if (lens[256] == 0) corrupt("no end-of-block code");
      Huffman lit, dist;
      lit.build(lens, hlit);
      dist.build(lens + hlit, hdist);
      inflate_block(br, lit, dist, out, out_n, o);
    } else {
      corrupt("reserved deflate block type");
    }
  }
  if (o != out_n) corrupt("deflate output shorter than the brick");
  // Adler-32 (RFC 1950 section 8.2), big-endian after the last block
  br.align_byte();
  uint32_t want = 0;
  for (int k = 0; k < 4; ++k) want = (want << 8) | br.bits(8);
  uint32_t a = 1, b = 0;
  for (size_t k = 0; k < out_n; ++k) {
    a = (a + out[k]) % 65521u;
    b = (b + a) % 65521u;
  }
  if (((b << 16) | a) != want) corrupt("zlib checksum");
}

// ------------------------------------------------------------------ LZMA

namespace {

// Range decoder of the LZMA specification: 11-bit probabilities adapted by
// 1/32 of the distance to 0 or 1, normalised one byte at a time.
struct RangeDec {
  const uint8_t* p;
  size_t n, pos = 0;
  uint32_t range = 0xffffffffu, code = 0;
  RangeDec(const uint8_t* d, size_t len) : p(d), n(len) {
    if (n < 5 || p[0] != 0) corrupt("LZMA range coder start");
    for (int i = 1; i < 5; ++i) code = (code << 8) | p[i];
    pos = 5;
    if (code == range) corrupt("LZMA range coder start");
  }
  void normalize() {
    if (range < (1u << 24)) {
      if (pos >= n) corrupt("LZMA stream ends early");
      range <<= 8;
      code = (code << 8) | p[pos++];
    }
  }
  uint32_t bit(uint16_t& prob) {
    const uint32_t bound = (range >> 11) * prob;
    uint32_t b;
    if (code < bound) {
      range = bound;
      prob = uint16_t(prob + ((2048u - prob) >> 5));
      b = 0;
    } else {
      range -= bound;
      code -= bound;
      prob = uint16_t(prob - (prob >> 5));
      b = 1;
    }
    normalize();
    return b;
  }
  uint32_t direct(int nbits) {
    uint32_t res = 0;
    for (int i = 0; i < nbits; ++i) {
      range >>= 1;
      uint32_t b = 0;
      if (code >= range) {
        code -= range;
        b = 1;
      }
      res = (res << 1) | b;
      normalize();
    }
    return res;
  }
  uint32_t tree(uint16_t* probs, int nbits) {  // most significant bit first
    uint32_t m = 1;
    for (int i = 0; i < nbits; ++i) m = (m << 1) | bit(probs[m]);
    return m - (1u << nbits);
  }
  uint32_t tree_reverse(uint16_t* probs, int nbits) {  // least significant bit first
    uint32_t m = 1, sym = 0;
    for (int i = 0; i < nbits; ++i) {
      const uint32_t b = bit(probs[m]);
      m = (m << 1) | b;
      sym |= b << i;
    }
    return sym;
  }
};

struct LenDec {
  uint16_t choice = 1024, choice2 = 1024;
  uint16_t low[16][8], mid[16][8], high[256];
  LenDec() {
    for (auto& r : low) for (auto& v : r) v = 1024;
    for (auto& r : mid) for (auto& v : r) v = 1024;
    for (auto& v : high) v = 1024;
  }
  uint32_t decode(RangeDec& rc, uint32_t ps) {
    if (!rc.bit(choice)) return rc.tree(low[ps], 3);
    if (!rc.bit(choice2)) return 8 + rc.tree(mid[ps], 3);
    return 16 + rc.tree(high, 8);
  }
};

}  // namespace

// Raw LZMA stream without end marker, exactly out_n bytes of output.
void lzma_decode(const uint8_t* in, size_t n, uint8_t* out, size_t out_n, uint32_t lc,
                 uint32_t lp, uint32_t pb) {
  if (lc > 8 || lp > 4 || pb > 4) corrupt("LZMA properties");
  RangeDec rc(in, n);
  std::vector<uint16_t> lit(size_t(0x300) << (lc + lp), 1024);
  uint16_t is_match[12 * 16], is_rep[12], is_rep_g0[12], is_rep_g1[12], is_rep_g2[12],
      is_rep0_long[12 * 16];
  uint16_t pos_slot[4][64], pos_dec[115], align[16];
  for (auto& v : is_match) v = 1024;
  for (auto* a : {is_rep, is_rep_g0, is_rep_g1, is_rep_g2})
    for (int i = 0; i < 12; ++i) a[i] = 1024;
  for (auto& v : is_rep0_long) v = 1024;
  for (auto& r : pos_slot) for (auto& v : r) v = 1024;
  for (auto& v : pos_dec) v = 1024;
  for (auto& v : align) v = 1024;
  LenDec len_dec, rep_len_dec;
  uint32_t state = 0, rep0 = 0, rep1 = 0, rep2 = 0, rep3 = 0;
  size_t o = 0;
  const uint32_t pb_mask = (1u << pb) - 1, lp_mask = (1u << lp) - 1;
  while (o < out_n) {
    const uint32_t ps = uint32_t(o) & pb_mask;
    if (!rc.bit(is_match[(state << 4) + ps])) {
      // literal, with the byte at rep0 as context after a match
      const uint32_t prev = o ? out[o - 1] : 0;
      uint16_t* probs =
          &lit[size_t(0x300) * (((uint32_t(o) & lp_mask) << lc) + (prev >> (8 - lc)))];
      uint32_t sym = 1;
      if (state >= 7) {
        if (rep0 >= o) corrupt("LZMA match byte before the start");
        uint32_t mb = out[o - rep0 - 1];
        do {
          const uint32_t mbit = (mb >> 7) & 1;
          mb <<= 1;
          const uint32_t b = rc.bit(probs[((1 + mbit) << 8) + sym]);
          sym = (sym << 1) | b;
          if (mbit != b) break;
        } while (sym < 0x100);
      }
      while (sym < 0x100) sym = (sym << 1) | rc.bit(probs[sym]);
      out[o++] = uint8_t(sym - 0x100);
      state = state < 4 ? 0 : (state < 10 ? state - 3 : state - 6);
      continue;
    }
    uint32_t len;
    if (rc.bit(is_rep[state])) {
      if (o == 0) corrupt("LZMA repeated match at the start");
      if (!rc.bit(is_rep_g0[state])) {
        if (!rc.bit(is_rep0_long[(state << 4) + ps])) {  // one byte at rep0
          state = state < 7 ? 9 : 11;
          if (rep0 >= o) corrupt("LZMA distance before the start");
          out[o] = out[o - rep0 - 1];
          ++o;
          continue;
        }
      } else {
        uint32_t dist;
        if (!rc.bit(is_rep_g1[state])) {
          dist = rep1;
        } else {
          if (!rc.bit(is_rep_g2[state])) {
            dist = rep2;
          } else {
            dist = rep3;
            rep3 = rep2;
          }
          rep2 = rep1;
        }
        rep1 = rep0;
        rep0 = dist;
      }
      len = rep_len_dec.decode(rc, ps);
      state = state < 7 ? 8 : 11;
    } else {
      rep3 = rep2;
      rep2 = rep1;
      rep1 = rep0;
      len = len_dec.decode(rc, ps);
      state = state < 7 ? 7 : 10;
      // distance: 6-bit slot per length class, then direct / modelled bits
      const uint32_t ls = len < 3 ? len : 3;
      const uint32_t slot = rc.tree(pos_slot[ls], 6);
      if (slot < 4) {
        rep0 = slot;
      } else {
        const int nd = int(slot >> 1) - 1;
        uint32_t dist = (2 | (slot & 1)) << nd;
        if (slot < 14) {
          dist += rc.tree_reverse(pos_dec + dist - slot, nd);
        } else {
          dist += rc.direct(nd - 4) << 4;
          dist += rc.tree_reverse(align, 4);
        }
        rep0 = dist;
      }
      if (rep0 == 0xffffffffu) corrupt("LZMA end marker before the end of the brick");
    }
    len += 2;
    if (rep0 >= o) corrupt("LZMA distance before the start");
    if (len > out_n - o) corrupt("LZMA output overruns the brick");
    for (uint32_t k = 0; k < len; ++k, ++o) out[o] = out[o - rep0 - 1];
  }
}

// ------------------------------------------------------------------ bzip2

namespace {

// MSB-first bit reader (bzip2 packs its fields most significant bit first).
struct MsbBits {
  const uint8_t* p;
  size_t n, pos = 0;
  uint64_t acc = 0;
  int cnt = 0;
  MsbBits(const uint8_t* d, size_t len) : p(d), n(len) {}
  uint32_t bits(int k) {
    while (cnt < k) {
      if (pos >= n) corrupt("bzip2 stream ends early");
      acc = (acc << 8) | p[pos++];
      cnt += 8;
    }
    cnt -= k;
    return uint32_t((acc >> cnt) & ((uint64_t(1) << k) - 1));
  }
};

// CRC-32 with the polynomial 0x04c11db7, most significant bit first (the
// checksum bzip2 keeps per block and per stream).
uint32_t crc32_msb_update(uint32_t crc, uint8_t b) {
  static const auto table = [] {
    std::vector<uint32_t> t(256);
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t c = i << 24;
      for (int k = 0; k < 8; ++k) c = (c & 0x80000000u) ? (c << 1) ^ 0x04c11db7u : (c << 1);
      t[i] = c;
    }
    return t;
  }();
  return (crc << 8) ^ table[((crc >> 24) ^ b) & 0xffu];
}

// Canonical Huffman code of one bzip2 coding group (lengths 1..20).
struct BzHuff {
  int count[21] = {0};
  int first[22] = {0}, offs[22] = {0};
  std::vector<uint16_t> sym;
  void build(const uint8_t* len, int n) {
    for (int i = 0; i < n; ++i) count[len[i]]++;
    int code = 0, k = 0;
    for (int l = 1; l <= 20; ++l) {
      first[l] = code;
      offs[l] = k;
      code = (code + count[l]) << 1;
      k += count[l];
    }
    sym.assign(size_t(n), 0);
    std::vector<int> next(offs, offs + 21);
    for (int i = 0; i < n; ++i) sym[size_t(next[len[i]]++)] = uint16_t(i);
  }
  int decode(MsbBits& br) const {
    int code = 0;
    for (int l = 1; l <= 20; ++l) {
      code = (code << 1) | int(br.bits(1));
      if (code - first[l] < count[l]) return sym[size_t(offs[l] + code - first[l])];
    }
    corrupt("invalid bzip2 Huffman code");
  }
};

}  // namespace

// A bzip2 stream ("BZh1".."BZh9", blocks, end-of-stream record), exactly
// out_n bytes of output.
void bzip2_decode(const uint8_t* in, size_t n, uint8_t* out, size_t out_n) {
  if (n < 14 || in[0] != 'B' || in[1] != 'Z' || in[2] != 'h' || in[3] < '1' || in[3] > '9')
    corrupt("bzip2 header");
  const uint32_t max_block = uint32_t(in[3] - '0') * 100000u;
  MsbBits br(in + 4, n - 4);
  size_t o = 0;
  uint32_t combined = 0;
  std::vector<uint32_t> tt(max_block);
  std::vector<uint8_t> ll(max_block);
  for (;;) {
    const uint64_t magic = (uint64_t(br.bits(24)) << 24) | br.bits(24);
    if (magic == 0x177245385090ull) {  // end of stream
      const uint32_t want = br.bits(32);
      if (want != combined) corrupt("bzip2 stream checksum");
      break;
    }
    if (magic != 0x314159265359ull) corrupt("bzip2 block magic");
    const uint32_t block_crc = br.bits(32);
    if (br.bits(1)) corrupt("randomised bzip2 block");
    const uint32_t orig_ptr = br.bits(24);
    // byte values in use (16 groups of 16)
    uint8_t seq_to_unseq[256];
    int n_in_use = 0;
    const uint32_t groups = br.bits(16);
    for (int g = 0; g < 16; ++g)
      if (groups & (0x8000u >> g)) {
        const uint32_t m = br.bits(16);
        for (int j = 0; j < 16; ++j)
          if (m & (0x8000u >> j)) seq_to_unseq[n_in_use++] = uint8_t(16 * g + j);
      }
    if (n_in_use == 0) corrupt("bzip2 block without symbols");
    const int alpha = n_in_use + 2;
    const int n_groups = int(br.bits(3));
    if (n_groups < 2 || n_groups > 6) corrupt("bzip2 coding group count");
    const int n_sel = int(br.bits(15));
    if (n_sel < 1) corrupt("bzip2 selector count");
    std::vector<uint8_t> sel(static_cast<size_t>(n_sel));
    uint8_t mtf_g[6] = {0, 1, 2, 3, 4, 5};
    for (int i = 0; i < n_sel; ++i) {
      int j = 0;
      while (br.bits(1)) {
        if (++j >= n_groups) corrupt("bzip2 selector");
      }
      const uint8_t v = mtf_g[j];
      for (; j > 0; --j) mtf_g[j] = mtf_g[j - 1];
      mtf_g[0] = v;
      sel[size_t(i)] = v;
    }
    BzHuff codes[6];
    for (int g = 0; g < n_groups; ++g) {
      uint8_t len[258];
      int cur = int(br.bits(5));
      for (int i = 0; i < alpha; ++i) {
        for (;;) {
          if (cur < 1 || cur > 20) corrupt("bzip2 code length");
          if (!br.bits(1)) break;
          cur += br.bits(1) ? -1 : 1;
        }
        len[i] = uint8_t(cur);
      }
      codes[g].build(len, alpha);
    }
    // symbols: zero runs (RUNA, RUNB), move-to-front indices, end of block
    uint8_t mtf[256];
    for (int i = 0; i < 256; ++i) mtf[i] = uint8_t(i);
    uint32_t counts[256] = {0};
    uint32_t nblock = 0;
    int group_left = 0, sel_i = -1;
    uint32_t run = 0, run_bit = 1;
    const BzHuff* cur_code = nullptr;
    auto flush_run = [&] {
      if (!run) return;
      const uint8_t b = seq_to_unseq[mtf[0]];
      if (run > max_block - nblock) corrupt("bzip2 block overruns its size");
      for (uint32_t k = 0; k < run; ++k) ll[nblock++] = b;
      counts[b] += run;
      run = 0;
      run_bit = 1;
    };
    for (;;) {
      if (group_left == 0) {
        if (++sel_i >= n_sel) corrupt("bzip2 selectors exhausted");
        cur_code = &codes[sel[size_t(sel_i)]];
        group_left = 50;
      }
      --group_left;
      const int s = cur_code->decode(br);
      if (s <= 1) {  // RUNA / RUNB: bijective base-2 digits of the run length
        if (run_bit > max_block) corrupt("bzip2 run too long");
        run += (s == 0 ? 1u : 2u) * run_bit;
        run_bit <<= 1;
        continue;
      }
      flush_run();
      if (s == alpha - 1) break;  // end of block
      const int idx = s - 1;
      const uint8_t v = mtf[idx];
      for (int j = idx; j > 0; --j) mtf[j] = mtf[j - 1];
      mtf[0] = v;
      if (nblock >= max_block) corrupt("bzip2 block overruns its size");
      const uint8_t b = seq_to_unseq[v];
      ll[nblock++] = b;
      counts[b]++;
    }
    if (orig_ptr >= nblock) corrupt("bzip2 origin pointer");
    // inverse Burrows-Wheeler transform
    uint32_t cum[256];
    uint32_t sum = 0;
    for (int c = 0; c < 256; ++c) {
      cum[c] = sum;
      sum += counts[c];
    }
    for (uint32_t i = 0; i < nblock; ++i) tt[cum[ll[i]]++] = i;
    // undo the initial run-length coding (4 equal bytes, then a repeat count)
    uint32_t crc = 0xffffffffu;
    uint32_t p = tt[orig_ptr];
    int last = -1, same = 0;
    for (uint32_t k = 0; k < nblock; ++k) {
      const uint8_t b = ll[p];
      p = tt[p];
      if (same == 4) {
        if (b > out_n - o) corrupt("bzip2 output overruns the brick");
        for (uint32_t r = 0; r < b; ++r) {
          out[o++] = uint8_t(last);
          crc = crc32_msb_update(crc, uint8_t(last));
        }
        same = 0;
        last = -1;
        continue;
      }
      if (o >= out_n) corrupt("bzip2 output overruns the brick");
      out[o++] = b;
      crc = crc32_msb_update(crc, b);
      same = (int(b) == last) ? same + 1 : 1;
      last = b;
    }
    if (~crc != block_crc) corrupt("bzip2 block checksum");
    combined = ((combined << 1) | (combined >> 31)) ^ block_crc;
  }
  if (o != out_n) corrupt("bzip2 output shorter than the brick");
}

}  // namespace tvk
