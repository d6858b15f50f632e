// ref_wrapper.cpp -- C entry points around the reference's own
// ExtendedOctreeConverter (IO/UVF/ExtendedOctree/ExtendedOctreeConverter.cpp:128-280),
// compiled from the reference sources by oracle/ref/Makefile into
// oracle/_ref/libtuvok_ref.so.
//
// TEST INFRASTRUCTURE ONLY: it pins the CPU restatement in oracle/ and the GPU
// bricking path against the reference's real code on the same input.  The raw
// volume is written to a scratch file, converted (no compression, scanline
// layout), reopened with ExtendedOctree::Open and read back brick by brick.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "Controller/Controller.h"
#include "IO/UVF/ExtendedOctree/ExtendedOctree.h"
#include "IO/UVF/ExtendedOctree/ExtendedOctreeConverter.h"

namespace {

struct RefTree {
  ExtendedOctree tree;
  BrickStatVec stats;
  std::vector<UINT64VECTOR4> coords;  // TOC index -> (x, y, z, lod)
  std::string out_path;
};

}  // namespace

extern "C" {

// dtype 0 = uint8, 1 = uint16.  brick_size includes the overlap.  Returns a
// handle or nullptr on failure.
void* ref_convert(const void* raw, int dtype, const uint64_t dims[3], const uint32_t brick_size[3],
                  uint32_t overlap, int clamp_to_edge, int median, const char* scratch_dir) {
  const size_t bytes = dtype == 0 ? 1 : 2;
  const uint64_t n = dims[0] * dims[1] * dims[2];
  const std::string in_path = std::string(scratch_dir) + "/tvk_ref_in.raw";
  auto* t = new RefTree();
  t->out_path = std::string(scratch_dir) + "/tvk_ref_out.eo";
  {
    FILE* f = std::fopen(in_path.c_str(), "wb");
    if (!f) { delete t; return nullptr; }
    std::fwrite(raw, bytes, n, f);
    std::fclose(f);
  }
  tuvok::QuietOut quiet;
  ExtendedOctreeConverter conv(UINT64VECTOR3(brick_size[0], brick_size[1], brick_size[2]),
                               overlap, 256ull << 20, quiet);
  const bool ok = conv.Convert(in_path, 0,
                               dtype == 0 ? ExtendedOctree::CT_UINT8 : ExtendedOctree::CT_UINT16,
                               1, UINT64VECTOR3(dims[0], dims[1], dims[2]),
                               DOUBLEVECTOR3(1, 1, 1), t->out_path, 0, &t->stats, CT_NONE, 0,
                               median != 0, clamp_to_edge != 0, LT_SCANLINE);
  std::remove(in_path.c_str());
  if (!ok || !t->tree.Open(t->out_path, 0, 5)) {
    delete t;
    return nullptr;
  }
  for (uint64_t l = 0; l < t->tree.GetLODCount(); ++l) {
    const UINT64VECTOR3 bc = t->tree.GetBrickCount(l);
    for (uint64_t z = 0; z < bc.z; ++z)
      for (uint64_t y = 0; y < bc.y; ++y)
        for (uint64_t x = 0; x < bc.x; ++x) t->coords.push_back(UINT64VECTOR4(x, y, z, l));
  }
  return t;
}

// Writes the converter's ExtendedOctree file for a flat volume: dtype 0 =
// uint8, 1 = uint16; `components` per voxel; compression 0 = none, 3 = LZ4
// (level 1 = LZ4_compress, > 1 = LZ4 HC); layout 0..3 = scanline, Morton,
// Hilbert, random.  Returns 1 on success.
int ref_write_eo(const void* raw, int dtype, uint64_t components, const uint64_t dims[3],
                 const uint32_t brick_size[3], uint32_t overlap, int clamp_to_edge, int median,
                 int compression, uint32_t level, int layout, const char* out_path,
                 const char* scratch_dir) {
  const size_t bytes = (dtype == 0 ? 1 : 2) * components;
  const uint64_t n = dims[0] * dims[1] * dims[2];
  const std::string in_path = std::string(scratch_dir) + "/tvk_ref_eo_in.raw";
  {
    FILE* f = std::fopen(in_path.c_str(), "wb");
    if (!f) return 0;
    std::fwrite(raw, bytes, n, f);
    std::fclose(f);
  }
  tuvok::QuietOut quiet;
  BrickStatVec stats;  // Convert requires somewhere to put them
  ExtendedOctreeConverter conv(UINT64VECTOR3(brick_size[0], brick_size[1], brick_size[2]),
                               overlap, 256ull << 20, quiet);
  const bool ok = conv.Convert(in_path, 0,
                               dtype == 0 ? ExtendedOctree::CT_UINT8 : ExtendedOctree::CT_UINT16,
                               components, UINT64VECTOR3(dims[0], dims[1], dims[2]),
                               DOUBLEVECTOR3(1, 1, 1), out_path, 0, &stats,
                               COMPRESSION_TYPE(compression), level, median != 0,
                               clamp_to_edge != 0, LAYOUT_TYPE(layout));
  std::remove(in_path.c_str());
  return ok ? 1 : 0;
}

uint64_t ref_brick_count(void* h) { return static_cast<RefTree*>(h)->coords.size(); }

uint64_t ref_lod_count(void* h) { return static_cast<RefTree*>(h)->tree.GetLODCount(); }

// coords: x, y, z, lod; size: voxels incl. overlap; stats from Convert.
void ref_brick_info(void* h, uint64_t index, uint64_t coords[4], uint64_t size[3], double* mn,
                    double* mx) {
  RefTree* t = static_cast<RefTree*>(h);
  const UINT64VECTOR4 c = t->coords[index];
  const UINT64VECTOR3 s = t->tree.ComputeBrickSize(c);
  for (int a = 0; a < 4; ++a) coords[a] = c[a];
  for (int a = 0; a < 3; ++a) size[a] = s[a];
  *mn = t->stats[index].minScalar;
  *mx = t->stats[index].maxScalar;
}

void ref_brick_data(void* h, uint64_t index, void* out) {
  RefTree* t = static_cast<RefTree*>(h);
  t->tree.GetBrickData(static_cast<uint8_t*>(out), t->coords[index]);
}

void ref_free(void* h) {
  RefTree* t = static_cast<RefTree*>(h);
  t->tree.Close();
  std::remove(t->out_path.c_str());
  delete t;
}

}  // extern "C"
