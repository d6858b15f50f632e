// uvf_list.cpp -- a C++ host over include/tvk_renderer.hpp that lists a UVF
// file's data blocks (tvk::ReadUVFBlocks, host code only, no GPU).  Prints the
// global header and one line per block; exits 1 with the library's message on
// an error.
#include <cstdio>
#include <exception>

#include "tvk_renderer.hpp"

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: uvf_list file.uvf [verify]\n");
    return 2;
  }
  try {
    tvk_uvf_info info;
    const auto blocks =
        tvk::ReadUVFBlocks(argv[1], argc > 2 ? TVK_UVF_VERIFY_CHECKSUM : 0u, &info);
    std::printf("version=%llu blocks=%u timesteps=%u verified=%u data=%llu\n",
                (unsigned long long)info.file_version, info.block_count, info.timestep_count,
                info.checksum_verified, (unsigned long long)info.data_offset);
    for (const tvk_uvf_block& b : blocks)
      std::printf("block offset=%llu header=%llu next=%llu semantics=%llu\n",
                  (unsigned long long)b.offset, (unsigned long long)b.header_bytes,
                  (unsigned long long)b.offset_to_next, (unsigned long long)b.semantics);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
