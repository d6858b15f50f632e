// ref_histograms.cpp -- C entry point around the reference's own UVF histogram
// blocks: TOCBlock::FlatDataToBrickedLOD (IO/UVF/TOCBlock.cpp:106-183) bricks
// the raw volume, then Histogram1DDataBlock::Compute (Histogram1DDataBlock.cpp:60-118)
// and Histogram2DDataBlock::Compute (Histogram2DDataBlock.cpp:69-126) run on it
// with the arguments RAWConverter::ConvertRAWDataset passes
// (IO/RAWConverter.cpp:644-662): the 1D histogram's length as the value-bin
// count and the global maximum as the largest non-zero value.
//
// TEST INFRASTRUCTURE ONLY (oracle/_ref).
#include <cstdint>
#include <cstdio>
#include <memory>
#include <string>

#include "Histogram1DDataBlock.h"
#include "Histogram2DDataBlock.h"
#include "MaxMinDataBlock.h"
#include "TOCBlock.h"

extern "C" {

// dtype 0 = uint8, 1 = uint16.  hist1d receives up to cap1 bins (*len1 = the
// block's length); hist2d receives [value][gradient] rows of 256 bins, up to
// cap2 entries (*value_bins = the number of rows).  bins_override != 0 replaces
// the value-bin count RAWConverter would pass.  Returns 0 on success.
int ref_histograms(const void* raw, int dtype, const uint64_t dims[3], const uint32_t brick_size[3],
                   uint32_t overlap, int clamp_to_edge, const char* scratch_dir,
                   uint64_t bins_override, uint64_t* hist1d,
                   size_t cap1, size_t* len1, uint64_t* hist2d, size_t cap2, size_t* value_bins,
                   float* max_gradient) {
  const size_t bytes = dtype == 0 ? 1 : 2;
  const uint64_t n = dims[0] * dims[1] * dims[2];
  const std::string in_path = std::string(scratch_dir) + "/tvk_ref_hist_in.raw";
  const std::string tmp_path = std::string(scratch_dir) + "/tvk_ref_hist.eo";
  {
    FILE* f = std::fopen(in_path.c_str(), "wb");
    if (!f) return 1;
    std::fwrite(raw, bytes, n, f);
    std::fclose(f);
  }
  int rc = 0;
  {
    tuvok::QuietOut quiet;
    std::shared_ptr<MaxMinDataBlock> mm(new MaxMinDataBlock(1));
    TOCBlock toc(5);
    if (!toc.FlatDataToBrickedLOD(in_path, tmp_path,
                                  dtype == 0 ? ExtendedOctree::CT_UINT8 : ExtendedOctree::CT_UINT16,
                                  1, UINT64VECTOR3(dims[0], dims[1], dims[2]),
                                  DOUBLEVECTOR3(1, 1, 1),
                                  UINT64VECTOR3(brick_size[0], brick_size[1], brick_size[2]),
                                  overlap, false, clamp_to_edge != 0, 256ull << 20, mm, &quiet,
                                  CT_NONE, 0, LT_SCANLINE)) {
      rc = 2;
    } else {
      Histogram1DDataBlock h1;
      Histogram2DDataBlock h2;
      if (!h1.Compute(&toc, 0)) {
        rc = 3;
      } else if (!h2.Compute(&toc, 0, bins_override ? bins_override : h1.GetHistogram().size(),
                             mm->GetGlobalValue().maxScalar)) {
        rc = 4;
      } else {
        const auto& a = h1.GetHistogram();
        *len1 = a.size();
        for (size_t i = 0; i < a.size() && i < cap1; ++i) hist1d[i] = a[i];
        const auto& b = h2.GetHistogram();
        *value_bins = b.size();
        size_t k = 0;
        for (size_t v = 0; v < b.size(); ++v)
          for (size_t g = 0; g < b[v].size(); ++g, ++k)
            if (k < cap2) hist2d[k] = b[v][g];
        *max_gradient = h2.GetMaxGradMagnitude();
      }
    }
  }
  std::remove(in_path.c_str());
  return rc;
}

}  // extern "C"
