// A C++ host of the C ABI through include/tvk_renderer.hpp: bricks a small
// procedural volume, paints it with the brick-by-brick ray caster and with a
// GridLeaper pool, and prints FNV-1a hashes of the two images so that a test
// can compare them with the same frames painted through the Python binding.
#include <cstdio>
#include <cstring>
#include <vector>

#include "tvk_renderer.hpp"

namespace {

uint64_t fnv1a(const std::vector<float>& img) {
  uint64_t h = 1469598103934665603ull;
  const unsigned char* b = reinterpret_cast<const unsigned char*>(img.data());
  for (size_t i = 0; i < img.size() * sizeof(float); ++i) {
    h ^= b[i];
    h *= 1099511628211ull;
  }
  return h;
}

}  // namespace

int main() {
  const uint64_t nx = 64, ny = 48, nz = 40;
  std::vector<uint8_t> vox(nx * ny * nz);
  for (uint64_t z = 0; z < nz; ++z)
    for (uint64_t y = 0; y < ny; ++y)
      for (uint64_t x = 0; x < nx; ++x) {
        const int64_t dx = int64_t(x) - 30, dy = int64_t(y) - 22, dz = int64_t(z) - 19;
        const int64_t v = 255 - (dx * dx + dy * dy + dz * dz) / 3;
        vox[x + nx * (y + ny * z)] = uint8_t(v < 0 ? 0 : v);
      }
  std::vector<float> tf(256 * 4);
  for (int i = 0; i < 256; ++i) {
    const float t = float(i) / 255.0f;
    tf[4 * i + 0] = t;
    tf[4 * i + 1] = 0.8f * t;
    tf[4 * i + 2] = 1.0f - t;
    tf[4 * i + 3] = i < 40 ? 0.0f : 0.6f * float(i - 40) / 215.0f;
  }
  try {
    auto vol = tvk::BrickedVolume::Create(vox.data(), TVK_U8, {nx, ny, nz}, {18, 18, 18}, 1, 0);
    tvk::Renderer r;
    r.RegisterDataset(*vol);
    r.Set1DTransFloat(tf);
    r.SetUseLighting(true);
    const float eye[3] = {0.4f, 0.5f, 1.4f}, at[3] = {0.0f, 0.0f, 0.0f}, up[3] = {0, 1, 0};
    r.SetViewParameters(50.0f, 0.01f, 1000.0f, eye, at, up);
    r.Resize(96, 64);
    r.Paint();
    const uint64_t plain = fnv1a(r.ReadBackPixels());
    const uint64_t samples = r.Stats().samples;
    tvk::VolumePool pool(*vol, uint64_t(1) << 30, false);
    const tvk_leaper_info li = pool.Paint(r, 64);
    const uint64_t leaper = fnv1a(r.ReadBackPixels());
    std::printf("plain_fnv=%016llx samples=%llu leaper_fnv=%016llx passes=%u converged=%d "
                "paged=%u lods=%llu\n",
                (unsigned long long)plain, (unsigned long long)samples,
                (unsigned long long)leaper, li.passes, li.converged, li.paged,
                (unsigned long long)vol->GetLODLevelCount());
  } catch (const tvk::Exception& e) {
    std::fprintf(stderr, "tvk error: %s\n", e.what());
    return 1;
  }
  return 0;
}
