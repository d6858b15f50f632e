// ref_raster_stub.cpp -- stand-ins for the RasterDataBlock members that the
// reference's Histogram{1,2}DDataBlock objects reference from their
// RasterDataBlock overloads.  The real RasterDataBlock.cpp needs boost; the
// wrapper only ever computes histograms from a TOCBlock, so none of these is
// called.  Each aborts if it ever is.
//
// TEST INFRASTRUCTURE ONLY (oracle/_ref).
#include <cstdlib>
#include <vector>

#include "RasterDataBlock.h"

bool RasterDataBlock::GetData(std::vector<uint8_t>&, const std::vector<uint64_t>&,
                              const std::vector<uint64_t>&) const {
  std::abort();
}

const std::vector<uint64_t>& RasterDataBlock::GetBrickCount(const std::vector<uint64_t>&) const {
  std::abort();
}

const std::vector<uint64_t> RasterDataBlock::LargestSingleBrickLODBrickIndex() const {
  std::abort();
}

const std::vector<uint64_t>& RasterDataBlock::LargestSingleBrickLODBrickSize() const {
  std::abort();
}

const std::vector<uint64_t> RasterDataBlock::GetSmallestBrickIndex() const { std::abort(); }
