// ref_uvf.cpp -- C entry points around the reference's own UVF container code
// (IO/UVF/UVF.cpp, GlobalHeader.cpp, DataBlock.cpp and the block classes).
//
// ref_write_uvf assembles a UVF file the way RAWConverter::ConvertRAWDataset
// does (IO/RAWConverter.cpp:541-689): per timestep a TOCBlock built by
// FlatDataToBrickedLOD, its 1D and 2D histogram blocks (scalar volumes only)
// and its MaxMinDataBlock, then one KeyValuePairDataBlock of metadata; the
// global header's byte order and checksum are parameters.  ref_read_uvf opens
// a file with UVF::Open (UVF.cpp:74-95) and lists what the reference's parser
// found: every block's file offset, semantics, compression, next-block
// distance and id length, and for TOC blocks the octree's offset and shape.
//
// TEST INFRASTRUCTURE ONLY (oracle/_ref).
#include <cstdint>
#include <cstdio>
#include <memory>
#include <string>
#include <vector>

#include "Histogram1DDataBlock.h"
#include "Histogram2DDataBlock.h"
#include "KeyValuePairDataBlock.h"
#include "MaxMinDataBlock.h"
#include "TOCBlock.h"
#include "UVF.h"

namespace {

// The parser keeps a block's position and chain link in protected members;
// member pointers named through a derived class read them without changing
// the classes.
struct PeekBlock : DataBlock {
  static uint64_t offset(const DataBlock& d) { return d.*(&PeekBlock::m_iOffset); }
  static uint64_t next(const DataBlock& d) { return d.*(&PeekBlock::ulOffsetToNextDataBlock); }
};
struct PeekToc : TOCBlock {
  static uint64_t octree(const TOCBlock& t) { return t.*(&PeekToc::m_iOffsetToOctree); }
};

std::wstring wide(const char* s) {
  const std::string n(s);
  return std::wstring(n.begin(), n.end());
}

}  // namespace

extern "C" {

// raw: `timesteps` volumes back to back, each dims[0]*dims[1]*dims[2] voxels
// of `components` x (dtype 0 = uint8, 1 = uint16).  checksum: 0 none, 1 CRC32,
// 2 MD5.
// kv_first puts the metadata block before the first TOC block.  histograms:
// 0 none, 1 the 1D block, 2 both (RAWConverter writes both; the 2D block of a
// 16-bit volume holds up to 4096 x 256 counts).  Returns 1 on success.
int ref_write_uvf(const char* out_path, const char* scratch_dir, const void* raw,
                  uint32_t timesteps, int dtype, uint64_t components, const uint64_t dims[3],
                  const uint32_t brick_size[3], uint32_t overlap, int clamp_to_edge,
                  int compression, uint32_t level, int layout, int checksum, int big_endian,
                  int kv_first, int histograms) {
  const size_t bytes = (dtype == 0 ? 1 : 2) * components;
  const uint64_t n = dims[0] * dims[1] * dims[2];
  tuvok::QuietOut quiet;
  UVF uvf(wide(out_path));
  GlobalHeader gh;
  gh.bIsBigEndian = big_endian != 0;
  gh.ulChecksumSemanticsEntry = checksum == 2   ? UVFTables::CS_MD5
                                : checksum == 1 ? UVFTables::CS_CRC32
                                                : UVFTables::CS_NONE;
  uvf.SetGlobalHeader(gh);

  std::shared_ptr<KeyValuePairDataBlock> meta(new KeyValuePairDataBlock());
  meta->AddPair("Source Endianness", "little");
  meta->AddPair("Source Type", "integer");
  meta->AddPair("Source Bitwidth", dtype == 0 ? "8" : "16");
  if (kv_first && !uvf.AddDataBlock(meta)) return 0;

  std::vector<std::shared_ptr<DataBlock>> keep;
  for (uint32_t ts = 0; ts < timesteps; ++ts) {
    const std::string in_path =
        std::string(scratch_dir) + "/tvk_ref_uvf_in" + std::to_string(ts) + ".raw";
    const std::string tmp_path =
        std::string(scratch_dir) + "/tvk_ref_uvf_toc" + std::to_string(ts) + ".tmp";
    {
      FILE* f = std::fopen(in_path.c_str(), "wb");
      if (!f) return 0;
      std::fwrite(static_cast<const uint8_t*>(raw) + size_t(ts) * n * bytes, bytes, n, f);
      std::fclose(f);
    }
    std::shared_ptr<MaxMinDataBlock> mm(new MaxMinDataBlock(size_t(components)));
    std::shared_ptr<TOCBlock> toc(new TOCBlock(UVF::ms_ulReaderVersion));
    toc->strBlockID = "Volume converted by the tuvok_gb300 fixture writer, timestep " +
                      std::to_string(ts);
    const bool ok = toc->FlatDataToBrickedLOD(
        in_path, tmp_path, dtype == 0 ? ExtendedOctree::CT_UINT8 : ExtendedOctree::CT_UINT16,
        components, UINT64VECTOR3(dims[0], dims[1], dims[2]), DOUBLEVECTOR3(1, 1, 1),
        UINT64VECTOR3(brick_size[0], brick_size[1], brick_size[2]), overlap, false,
        clamp_to_edge != 0, 256ull << 20, mm, &quiet, COMPRESSION_TYPE(compression), level,
        LAYOUT_TYPE(layout));
    std::remove(in_path.c_str());
    if (!ok || !uvf.AddDataBlock(toc)) return 0;
    keep.push_back(toc);
    if (components == 1 && histograms > 0) {
      std::shared_ptr<Histogram1DDataBlock> h1(new Histogram1DDataBlock());
      if (!h1->Compute(toc.get(), 0) || !uvf.AddDataBlock(h1)) return 0;
      keep.push_back(h1);
      if (histograms > 1) {
        std::shared_ptr<Histogram2DDataBlock> h2(new Histogram2DDataBlock());
        if (!h2->Compute(toc.get(), 0, h1->GetHistogram().size(),
                         mm->GetGlobalValue().maxScalar) ||
            !uvf.AddDataBlock(h2))
          return 0;
        keep.push_back(h2);
      }
    }
    if (!uvf.AddDataBlock(mm)) return 0;
    keep.push_back(mm);
  }
  if (!kv_first && !uvf.AddDataBlock(meta)) return 0;
  if (!uvf.Create()) return 0;
  uvf.Close();  // rewrites the block headers and the checksum
  return 1;
}

// Opens `path` with UVF::Open(bMustBeSameVersion = false, bVerify = verify).
// rows (capacity cap rows of 8): offset, semantics, compression, offset to
// next, id length, octree offset (TOC blocks, else 0), component count (TOC),
// LOD count (TOC).  Returns the block count, or -1 when Open fails (problem
// receives the reason, up to problem_cap bytes).
int64_t ref_read_uvf(const char* path, int verify, uint64_t* version, int* big_endian,
                     uint64_t* rows, size_t cap, char* problem, size_t problem_cap) {
  tuvok::QuietOut quiet;
  UVF uvf(wide(path));
  std::string why;
  if (!uvf.Open(false, verify != 0, false, &why)) {
    if (problem && problem_cap) std::snprintf(problem, problem_cap, "%s", why.c_str());
    return -1;
  }
  *version = uvf.GetGlobalHeader().ulFileVersion;
  *big_endian = uvf.GetGlobalHeader().bIsBigEndian ? 1 : 0;
  const uint64_t count = uvf.GetDataBlockCount();
  for (uint64_t i = 0; i < count && i < cap; ++i) {
    const std::shared_ptr<DataBlock> b = uvf.GetDataBlock(i);
    uint64_t* r = rows + 8 * i;
    r[0] = PeekBlock::offset(*b);
    r[1] = uint64_t(b->GetBlockSemantic());
    r[2] = uint64_t(b->ulCompressionScheme);
    r[3] = PeekBlock::next(*b);
    r[4] = b->strBlockID.size();
    r[5] = r[6] = r[7] = 0;
    if (b->GetBlockSemantic() == UVFTables::BS_TOC_BLOCK) {
      const TOCBlock& t = static_cast<const TOCBlock&>(*b);
      r[5] = PeekToc::octree(t);
      r[6] = t.GetComponentCount();
      r[7] = t.GetLoDCount();
    }
  }
  uvf.Close();
  return int64_t(count);
}

}  // extern "C"
