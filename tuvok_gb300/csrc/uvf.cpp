// UVF container walk (host only): the global header (IO/UVF/GlobalHeader.cpp:
// 37-46 GetHeaderFromFile, :59-65 GetSize/GetMinSize), the optional MD5 check
// (IO/UVF/UVF.cpp:160-266 ComputeChecksum / VerifyChecksum) and the chain of
// data-block headers (UVF.cpp:269-291 ParseDataBlocks, DataBlock.cpp:51-75).
// The ExtendedOctree inside a TOC block is opened by eo.cpp at the block's
// payload, as TOCBlock::GetHeaderFromFile does (TOCBlock.cpp:48-65).
//
// Every read is bounds-checked against the file size: a truncated file or a
// block chain that leaves the file is an error, never a read past the end.

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>

#include "tvk_internal.h"

namespace tvk {

namespace {

struct File {
  std::FILE* f = nullptr;
  explicit File(const char* path) : f(std::fopen(path, "rb")) {}
  ~File() {
    if (f) std::fclose(f);
  }
};

void read_at(std::FILE* f, uint64_t pos, void* dst, size_t n) {
  if (fseeko(f, off_t(pos), SEEK_SET) != 0 || std::fread(dst, 1, n, f) != n)
    fail(TVK_ERR_INVALID_ARG, "UVF: read failed");
}

// LargeRAWFile::ReadData (Basics/LargeRAWFile.h:78-82): the value in the
// writer's order.  Its byte swap for a file flagged big-endian calls
// EndianConvert::Swap (Basics/EndianConvert.h:92-111), which returns the
// swapped value and leaves its argument unchanged, so the reference writes and
// reads every header in the host's order whatever the flag says.  Files come
// from little-endian hosts, and are read as such on any host.
uint64_t get_u64(const uint8_t* p) {
  uint64_t v = 0;
  for (int i = 0; i < 8; ++i) v |= uint64_t(p[i]) << (8 * i);
  return v;
}

// MD5 (RFC 1321 section 3): 64-byte blocks, four rounds of sixteen steps,
// additive constants floor(|sin(i + 1)| * 2^32).
class Md5 {
 public:
  void update(const uint8_t* p, size_t n) {
    total_ += n;
    while (n > 0) {
      const size_t take = fill_ + n < 64 ? n : 64 - fill_;
      std::memcpy(buf_ + fill_, p, take);
      fill_ += take;
      p += take;
      n -= take;
      if (fill_ == 64) {
        block(buf_);
        fill_ = 0;
      }
    }
  }
  void finish(uint8_t out[16]) {
    const uint64_t bits = total_ * 8;
    const uint8_t one = 0x80, zero = 0;
    update(&one, 1);
    while (fill_ != 56) update(&zero, 1);
    uint8_t len[8];
    for (int i = 0; i < 8; ++i) len[i] = uint8_t(bits >> (8 * i));
    update(len, 8);
    for (int i = 0; i < 16; ++i) out[i] = uint8_t(h_[i / 4] >> (8 * (i % 4)));
  }

 private:
  static uint32_t rotl(uint32_t x, int s) { return (x << s) | (x >> (32 - s)); }
  void block(const uint8_t* p) {
    static const uint32_t K[64] = {
        0xd76aa478, 0xe8c7b756, 0x242070db, 0xc1bdceee, 0xf57c0faf, 0x4787c62a, 0xa8304613,
        0xfd469501, 0x698098d8, 0x8b44f7af, 0xffff5bb1, 0x895cd7be, 0x6b901122, 0xfd987193,
        0xa679438e, 0x49b40821, 0xf61e2562, 0xc040b340, 0x265e5a51, 0xe9b6c7aa, 0xd62f105d,
        0x02441453, 0xd8a1e681, 0xe7d3fbc8, 0x21e1cde6, 0xc33707d6, 0xf4d50d87, 0x455a14ed,
        0xa9e3e905, 0xfcefa3f8, 0x676f02d9, 0x8d2a4c8a, 0xfffa3942, 0x8771f681, 0x6d9d6122,
        0xfde5380c, 0xa4beea44, 0x4bdecfa9, 0xf6bb4b60, 0xbebfbc70, 0x289b7ec6, 0xeaa127fa,
        0xd4ef3085, 0x04881d05, 0xd9d4d039, 0xe6db99e5, 0x1fa27cf8, 0xc4ac5665, 0xf4292244,
        0x432aff97, 0xab9423a7, 0xfc93a039, 0x655b59c3, 0x8f0ccc92, 0xffeff47d, 0x85845dd1,
        0x6fa87e4f, 0xfe2ce6e0, 0xa3014314, 0x4e0811a1, 0xf7537e82, 0xbd3af235, 0x2ad7d2bb,
        0xeb86d391};
    static const int S[4][4] = {{7, 12, 17, 22}, {5, 9, 14, 20}, {4, 11, 16, 23}, {6, 10, 15, 21}};
    uint32_t w[16];
    for (int i = 0; i < 16; ++i)
      w[i] = uint32_t(p[4 * i]) | uint32_t(p[4 * i + 1]) << 8 | uint32_t(p[4 * i + 2]) << 16 |
             uint32_t(p[4 * i + 3]) << 24;
    uint32_t a = h_[0], b = h_[1], c = h_[2], d = h_[3];
    for (int i = 0; i < 64; ++i) {
      const int r = i / 16;
      uint32_t f;
      int g;
      if (r == 0) {
        f = (b & c) | (~b & d);
        g = i;
      } else if (r == 1) {
        f = (d & b) | (~d & c);
        g = (5 * i + 1) % 16;
      } else if (r == 2) {
        f = b ^ c ^ d;
        g = (3 * i + 5) % 16;
      } else {
        f = c ^ (b | ~d);
        g = (7 * i) % 16;
      }
      const uint32_t t = d;
      d = c;
      c = b;
      b = b + rotl(a + f + K[i] + w[g], S[r][i % 4]);
      a = t;
    }
    h_[0] += a;
    h_[1] += b;
    h_[2] += c;
    h_[3] += d;
  }
  uint32_t h_[4] = {0x67452301u, 0xefcdab89u, 0x98badcfeu, 0x10325476u};
  uint8_t buf_[64];
  size_t fill_ = 0;
  uint64_t total_ = 0;
};

constexpr uint64_t kMagicBytes = 8;
constexpr uint64_t kGlobalMinBytes = 33;   // GlobalHeader::GetMinSize: bool + 4 x uint64
constexpr uint64_t kBlockFixedBytes = 32;  // id length, semantics, compression, next offset
constexpr uint64_t kBlockRaster = 1;       // BS_REG_NDIM_GRID

}  // namespace

void uvf_open(const char* path, bool verify_checksum, UvfFile& u) {
  File fh(path);
  if (!fh.f) fail(TVK_ERR_INVALID_ARG, std::string("cannot open ") + path);
  std::FILE* f = fh.f;
  if (fseeko(f, 0, SEEK_END) != 0) fail(TVK_ERR_INVALID_ARG, "UVF: seek failed");
  const off_t end = ftello(f);
  if (end < 0) fail(TVK_ERR_INVALID_ARG, "UVF: cannot size the file");
  const uint64_t size = uint64_t(end);
  u = UvfFile();
  u.file_bytes = size;
  // UVF::ParseGlobalHeader: size, magic, then the header fields
  if (size < kMagicBytes + kGlobalMinBytes) fail(TVK_ERR_INVALID_ARG, "UVF: file too small");
  uint8_t head[kMagicBytes + kGlobalMinBytes - 8];  // magic .. checksum length
  read_at(f, 0, head, sizeof(head));
  if (std::memcmp(head, "UVF-DATA", 8) != 0) fail(TVK_ERR_INVALID_ARG, "UVF: file magic not found");
  u.big_endian = head[8] != 0;  // recorded only, see get_u64
  u.version = get_u64(head + 9);
  u.checksum_semantics = get_u64(head + 17);
  u.checksum_bytes = get_u64(head + 25);
  if (u.checksum_bytes > size - (kMagicBytes + kGlobalMinBytes))
    fail(TVK_ERR_INVALID_ARG, "UVF: checksum runs past the end of the file");
  const uint64_t cs_pos = kMagicBytes + kGlobalMinBytes - 8;  // 33
  std::vector<uint8_t> stored(size_t(u.checksum_bytes));
  if (!stored.empty()) read_at(f, cs_pos, stored.data(), stored.size());
  uint8_t b8[8];
  read_at(f, cs_pos + u.checksum_bytes, b8, 8);
  const uint64_t first = get_u64(b8);
  const uint64_t hdr = kMagicBytes + kGlobalMinBytes + u.checksum_bytes;
  if (first > size - hdr) fail(TVK_ERR_INVALID_ARG, "UVF: first data block beyond the end");
  u.data_offset = hdr + first;  // GlobalHeader::GetDataPos

  if (verify_checksum && u.checksum_semantics != TVK_UVF_CS_NONE) {
    if (u.checksum_semantics == TVK_UVF_CS_CRC32)
      fail(TVK_ERR_UNSUPPORTED,
           "UVF: CRC32 checksums are not verified (the writer's CRC32 pass reads past the end "
           "of the file)");
    if (u.checksum_semantics != TVK_UVF_CS_MD5)
      fail(TVK_ERR_INVALID_ARG, "UVF: unknown checksum semantics");
    // ComputeChecksum: MD5 of everything after the 16 checksum bytes
    const uint64_t from = cs_pos + 16;
    if (u.checksum_bytes != 16 || from > size)
      fail(TVK_ERR_INVALID_ARG, "UVF: checksum mismatch (length)");
    Md5 md5;
    std::vector<uint8_t> chunk(size_t(1) << 22);
    for (uint64_t pos = from; pos < size;) {
      const size_t n = size_t(std::min<uint64_t>(chunk.size(), size - pos));
      read_at(f, pos, chunk.data(), n);
      md5.update(chunk.data(), n);
      pos += n;
    }
    uint8_t digest[16];
    md5.finish(digest);
    if (std::memcmp(digest, stored.data(), 16) != 0)
      fail(TVK_ERR_INVALID_ARG, "UVF: checksum mismatch");
    u.checksum_verified = true;
  }

  // UVF::ParseDataBlocks: block headers until the one whose next offset is 0.
  // Each step advances by at least one header, so the walk ends.
  for (uint64_t pos = u.data_offset;;) {
    if (pos > size || size - pos < kBlockFixedBytes)
      fail(TVK_ERR_INVALID_ARG, "UVF: data block header beyond the end of the file");
    read_at(f, pos, b8, 8);
    const uint64_t id_len = get_u64(b8);
    if (id_len > size - pos - kBlockFixedBytes)
      fail(TVK_ERR_INVALID_ARG, "UVF: block id runs past the end of the file");
    tvk_uvf_block b{};
    b.offset = pos;
    b.header_bytes = kBlockFixedBytes + id_len;
    const size_t keep = size_t(std::min<uint64_t>(id_len, sizeof(b.id) - 1));
    if (keep) read_at(f, pos + 8, b.id, keep);
    uint8_t tail[24];
    read_at(f, pos + 8 + id_len, tail, 24);
    b.semantics = get_u64(tail);
    b.compression = get_u64(tail + 8);
    b.offset_to_next = get_u64(tail + 16);
    if (b.semantics == kBlockRaster) u.has_raster = true;
    if (b.semantics == TVK_UVF_BS_TOC_BLOCK) {
      // UVFDataset::VerifyTOCBlock: scalar or colour volumes; the octree
      // header opens with its component type (uint32) and count (uint64)
      const uint64_t eo = pos + b.header_bytes;
      if (eo > size || size - eo < 12)
        fail(TVK_ERR_INVALID_ARG, "UVF: TOC block too short for its octree header");
      uint8_t eh[12];
      read_at(f, eo, eh, 12);
      const uint64_t components = get_u64(eh + 4);
      if (components == 1 || components == 4) u.timesteps.push_back(uint32_t(u.blocks.size()));
    }
    u.blocks.push_back(b);
    if (b.offset_to_next == 0) break;
    if (b.offset_to_next < b.header_bytes)
      fail(TVK_ERR_INVALID_ARG, "UVF: data block shorter than its header");
    if (b.offset_to_next > size - pos)
      fail(TVK_ERR_INVALID_ARG, "UVF: next data block beyond the end of the file");
    pos += b.offset_to_next;
  }
}

}  // namespace tvk
