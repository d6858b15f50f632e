// ExtendedOctree files: the brick container Tuvok's converter writes and its
// UVF TOC block holds (IO/UVF/ExtendedOctree/ExtendedOctree.cpp:67-172 Open,
// :313-361 GetBrickData).  Host code: the header and brick table of contents
// are parsed, bricks are read at their TOC offsets and expanded when they are
// stored compressed (codecs.cpp; LZ4 here); the ABI entry in api.cpp rebuilds the volume from the LOD-0
// bricks and checks every stored brick against the rebuild.

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

void seek(std::FILE* f, uint64_t pos) {
  if (fseeko(f, off_t(pos), SEEK_SET) != 0) fail(TVK_ERR_INVALID_ARG, "ExtendedOctree: seek failed");
}

template <class T>
T read_value(std::FILE* f) {
  T v;
  if (std::fread(&v, sizeof(T), 1, f) != 1)
    fail(TVK_ERR_INVALID_ARG, "ExtendedOctree: file ends inside the header");
  return v;
}

}  // namespace

// LZ4 block format (the public format LZ4_compress / LZ4_compressHC2 write and
// LZ4_decompress_fast reads, Lz4Compression.cpp:13-69): sequences of a token
// (literal count in the high nibble, match length - 4 in the low nibble, 15
// meaning "more length bytes follow, each 255 continuing"), the literals, and
// a 2-byte little-endian back offset; the last sequence ends with literals.
// Every read and write is bounds-checked; returns the input bytes consumed.
size_t lz4_decode_block(const uint8_t* src, size_t src_len, uint8_t* dst, size_t dst_len) {
  size_t i = 0, o = 0;
  auto bad = [] { fail(TVK_ERR_INVALID_ARG, "ExtendedOctree: corrupt LZ4 brick"); };
  auto more = [&](size_t n) {
    for (;;) {
      if (i >= src_len) bad();
      const uint8_t b = src[i++];
      n += b;
      if (b != 255) return n;
    }
  };
  for (;;) {
    if (i >= src_len) bad();
    const uint8_t token = src[i++];
    size_t lit = token >> 4;
    if (lit == 15) lit = more(lit);
    if (lit > src_len - i || lit > dst_len - o) bad();
    std::memcpy(dst + o, src + i, lit);
    i += lit;
    o += lit;
    if (o == dst_len) return i;
    if (src_len - i < 2) bad();
    const size_t off = size_t(src[i]) | (size_t(src[i + 1]) << 8);
    i += 2;
    if (off == 0 || off > o) bad();
    size_t ml = token & 15u;
    if (ml == 15) ml = more(ml);
    ml += 4;
    if (ml > dst_len - o) bad();
    for (size_t k = 0; k < ml; ++k, ++o) dst[o] = dst[o - off];  // may overlap
    if (o == dst_len) return i;
  }
}

void eo_open(const char* path, uint64_t offset, uint32_t uvf_version, EoFile& e) {
  File fh(path);
  if (!fh.f) fail(TVK_ERR_INVALID_ARG, std::string("cannot open ") + path);
  std::FILE* f = fh.f;
  e.path = path;
  e.base = offset;
  if (fseeko(f, 0, SEEK_END) != 0) fail(TVK_ERR_INVALID_ARG, "ExtendedOctree: seek failed");
  const off_t end = ftello(f);
  if (end < 0) fail(TVK_ERR_INVALID_ARG, "ExtendedOctree: cannot size the file");
  const uint64_t file_size = uint64_t(end);
  if (offset > file_size) fail(TVK_ERR_INVALID_ARG, "ExtendedOctree: offset beyond the file");
  seek(f, offset);
  // ExtendedOctree.cpp:91-118: the global header, in the writer's byte order
  // (both are little-endian here)
  e.component_type = read_value<uint32_t>(f);
  e.components = read_value<uint64_t>(f);
  e.normals = read_value<uint8_t>(f) != 0;
  for (int a = 0; a < 3; ++a) e.dims[a] = read_value<uint64_t>(f);
  for (int a = 0; a < 3; ++a) e.aspect[a] = read_value<double>(f);
  for (int a = 0; a < 3; ++a) e.brick_size[a] = read_value<uint64_t>(f);
  e.overlap = read_value<uint32_t>(f);
  // UVF files up to version 4 hold an older header (no version field, 32-bit
  // brick sizes by ExtendedOctree::ComputeHeaderSize) that Open itself does
  // not parse consistently; those are refused
  if (uvf_version <= 4)
    fail(TVK_ERR_UNSUPPORTED, "ExtendedOctree: headers of UVF versions <= 4 are not read");
  e.version = read_value<uint32_t>(f);
  if (e.version == 0) fail(TVK_ERR_INVALID_ARG, "ExtendedOctree: version 0");
  e.size = read_value<uint64_t>(f);
  e.compression_level = e.version > 1 ? read_value<uint32_t>(f) : 0;
  const double asp = e.aspect[0] * e.aspect[1] * e.aspect[2];
  if (e.components == 0 || e.dims[0] == 0 || e.dims[1] == 0 || e.dims[2] == 0 || asp == 0 ||
      e.brick_size[0] == 0 || e.brick_size[1] == 0 || e.brick_size[2] == 0)
    fail(TVK_ERR_INVALID_ARG, "ExtendedOctree: empty volume, aspect or brick size");
  // the voxel count must fit 64 bits (a corrupt header could claim more)
  if (e.dims[1] > UINT64_MAX / e.dims[0] || e.dims[2] > UINT64_MAX / (e.dims[0] * e.dims[1]))
    fail(TVK_ERR_INVALID_ARG, "ExtendedOctree: volume dimensions overflow 64 bits");
  // ExtendedOctree.cpp:131-133: precomputed normals need four components
  if (e.normals && e.components != 4)
    fail(TVK_ERR_INVALID_ARG, "ExtendedOctree: precomputed normals need four components");
  for (int a = 0; a < 3; ++a)
    if (e.brick_size[a] <= 2ull * e.overlap || e.brick_size[a] > 4096)
      fail(TVK_ERR_INVALID_ARG, "ExtendedOctree: brick size out of range");
  // ExtendedOctree.cpp:127-160: the table of contents, one entry per brick of
  // every LOD in TOC order
  uint32_t bs32[3] = {uint32_t(e.brick_size[0]), uint32_t(e.brick_size[1]),
                      uint32_t(e.brick_size[2])};
  const std::vector<LodInfo> lods = lod_table(e.dims, bs32, e.overlap);
  uint64_t n = 0;
  for (const LodInfo& l : lods) n += l.bricks[0] * l.bricks[1] * l.bricks[2];
  // the table must fit in what is left of the file (36 bytes per entry)
  const off_t here = ftello(f);
  if (here < 0 || n > (file_size - uint64_t(here)) / 36)
    fail(TVK_ERR_INVALID_ARG, "ExtendedOctree: the brick table runs past the end of the file");
  e.toc.resize(n);
  for (uint64_t k = 0; k < n; ++k) {
    EoFile::Entry& t = e.toc[k];
    t.offset = read_value<uint64_t>(f);
    t.length = read_value<uint64_t>(f);
    t.compression = read_value<uint32_t>(f);
    t.valid_length = read_value<uint64_t>(f);
    t.atlas[0] = read_value<uint32_t>(f);
    t.atlas[1] = read_value<uint32_t>(f);
    if (t.offset > file_size - offset || t.length > file_size - offset - t.offset)
      fail(TVK_ERR_INVALID_ARG, "ExtendedOctree: a brick lies past the end of the file");
  }
}

// GetBrickData (ExtendedOctree.cpp:313-361): `bytes` is the brick's size
// expanded (voxels incl. overlap x components x component size).
void eo_read_brick(const EoFile& e, uint64_t index, size_t bytes, std::vector<uint8_t>& out) {
  if (index >= e.toc.size()) fail(TVK_ERR_INVALID_ARG, "ExtendedOctree: brick index");
  const EoFile::Entry& t = e.toc[index];
  File fh(e.path.c_str());
  if (!fh.f) fail(TVK_ERR_INVALID_ARG, "cannot reopen " + e.path);
  seek(fh.f, e.base + t.offset);
  out.resize(bytes);
  if (t.compression == 0) {  // CT_NONE
    if (t.length != bytes) fail(TVK_ERR_INVALID_ARG, "ExtendedOctree: brick length mismatch");
    if (std::fread(out.data(), 1, bytes, fh.f) != bytes)
      fail(TVK_ERR_INVALID_ARG, "ExtendedOctree: file ends inside a brick");
    return;
  }
  // COMPRESSION_TYPE (ExtendedOctree.h): CT_ZLIB 1, CT_LZMA 2, CT_LZ4 3, CT_BZLIB 4;
  // CT_LZHAM (5) is refused by the reference as well
  if (t.compression < 1 || t.compression > 4)
    fail(TVK_ERR_UNSUPPORTED, "ExtendedOctree: unknown or unsupported brick compression " +
                                  std::to_string(t.compression));
  std::vector<uint8_t> buf(size_t(t.length));
  if (std::fread(buf.data(), 1, buf.size(), fh.f) != buf.size())
    fail(TVK_ERR_INVALID_ARG, "ExtendedOctree: file ends inside a brick");
  switch (t.compression) {
    case 1:
      zlib_decode(buf.data(), buf.size(), out.data(), bytes);
      break;
    case 2:
      // LzmaCompression.cpp: LzmaEncProps defaults (lc 3, lp 0, pb 2) at every
      // level, raw stream without end marker; the dictionary size does not
      // matter when the whole brick is the window
      lzma_decode(buf.data(), buf.size(), out.data(), bytes, 3, 0, 2);
      break;
    case 3:
      lz4_decode_block(buf.data(), buf.size(), out.data(), bytes);
      break;
    default:
      bzip2_decode(buf.data(), buf.size(), out.data(), bytes);
  }
}

}  // namespace tvk
