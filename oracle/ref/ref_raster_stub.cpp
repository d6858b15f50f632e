// ref_raster_stub.cpp -- stand-ins for the RasterDataBlock members that the
// reference's Histogram{1,2}DDataBlock objects reference from their
// RasterDataBlock overloads, and the constructor the UVF block factory names.
// The real RasterDataBlock.cpp needs boost; the
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

// UVFTables::CreateBlockFromSemanticEntry constructs a RasterDataBlock for a
// BS_REG_NDIM_GRID block.  The UVF files the wrapper writes and reads hold no
// such block; one that does aborts in the constructor.  The virtual members
// below only give the class its vtable.
RasterDataBlock::RasterDataBlock(LargeRAWFile_ptr, uint64_t, bool) { std::abort(); }
RasterDataBlock& RasterDataBlock::operator=(const RasterDataBlock&) { std::abort(); }
RasterDataBlock::~RasterDataBlock() {}
bool RasterDataBlock::Verify(uint64_t, std::string*) const { std::abort(); }
bool RasterDataBlock::Verify(std::string*) const { std::abort(); }
uint64_t RasterDataBlock::ComputeDataSize(std::string*) const { std::abort(); }
uint64_t RasterDataBlock::ComputeHeaderSize() const { std::abort(); }
bool RasterDataBlock::SetBlockSemantic(UVFTables::BlockSemanticTable) { std::abort(); }
void RasterDataBlock::CopyHeaderToFile(LargeRAWFile_ptr, uint64_t, bool, bool) { std::abort(); }
uint64_t RasterDataBlock::GetHeaderFromFile(LargeRAWFile_ptr, uint64_t, bool) { std::abort(); }
uint64_t RasterDataBlock::CopyToFile(LargeRAWFile_ptr, uint64_t, bool, bool) { std::abort(); }
DataBlock* RasterDataBlock::Clone() const { std::abort(); }
uint64_t RasterDataBlock::GetOffsetToNextBlock() const { std::abort(); }
uint64_t RasterDataBlock::GetLODSize(std::vector<uint64_t>&) const { std::abort(); }
uint64_t RasterDataBlock::ComputeLODLevelSize(const std::vector<uint64_t>&) const { std::abort(); }
std::vector<std::vector<uint64_t>> RasterDataBlock::ComputeBricks(
    const std::vector<uint64_t>&) const { std::abort(); }
std::vector<std::vector<uint64_t>> RasterDataBlock::GenerateCartesianProduct(
    const std::vector<std::vector<uint64_t>>&, uint64_t) const { std::abort(); }
