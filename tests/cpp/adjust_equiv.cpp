// Every byte triple, through the brightness/contrast table of several tile
// adjustments, into adjust_unit and adjust_word (mg_math.h: the composite's
// arithmetic; adjust_word where adjust_word_applies) and adjust_from_bc (the
// definition the oracle restates): prints the number of (setting, colour)
// pairs whose output differs.
#include <cstdio>

#include "../../mosaic-art-rust_gb300/csrc/mg_math.h"

int main() {
  using namespace mg;
  // (brightness, contrast, hue shift, saturation), through adjustment_new's clamps
  const float settings[][4] = {{0.0f, 1.0f, 37.5f, 1.0f},   {0.1f, 1.0f, -64.0f, 0.8f}, {-0.2f, 1.0f, 12.25f, 1.35f},
                               {0.0f, 1.0f, 0.0f, 0.4f},    {0.05f, 1.3f, -90.0f, 1.6f}, {0.0f, 1.0f, 179.0f, 1.0f},
                               {-1.0f, 1.0f, 5.0f, 2.0f},   {1.0f, 0.5f, -180.0f, 0.0f}, {-0.3f, 2.0f, 90.0f, 1.0f},
                               {0.25f, 1.0f, 0.0f, 1.0f},   {-0.5f, 0.0f, -37.0f, 1.7f}, {0.0f, 1.0f, -0.001f, 1.0f},
                               {0.0f, 1.0f, 1e-38f, 1.0f},  {0.1f, 0.9f, 180.0f, 2.0f},  {-0.1f, 1.1f, -180.0f, 0.0f},
                               {0.0f, 1.0f, 0.0f, 0.5f}};
  uint32_t perm[8];
  for (uint32_t i = 0; i < 8; ++i) perm[i] = sector_perm(i);
  long bad = 0, n = 0;
  for (const auto& st : settings) {
    const Adjust a = adjustment_new(st[0], st[1], st[2], st[3]);
    const bool word = adjust_word_applies(a);
    float bc[256];
    for (int v = 0; v < 256; ++v) bc[v] = brightness_contrast(u8_unit((uint32_t)v), a.brightness, a.contrast);
    for (int r = 0; r < 256; ++r)
      for (int g = 0; g < 256; ++g)
        for (int b = 0; b < 256; ++b) {
          uint8_t w0, w1, w2, f0, f1, f2;
          adjust_from_bc(a, bc[r], bc[g], bc[b], w0, w1, w2);
          adjust_unit(a, bc[r], bc[g], bc[b], f0, f1, f2);
          if (word) {
            const uint32_t q = adjust_word(a, bc[r], bc[g], bc[b], perm);
            if ((q & 0xFFFFFFu) != (uint32_t)(f0 | f1 << 8 | f2 << 16)) f0 = (uint8_t)(w0 + 1);
          }
          if (w0 != f0 || w1 != f1 || w2 != f2) {
            if (bad < 5) std::printf("setting %.3f %.3f %.3f %.3f colour %d %d %d: %d %d %d vs %d %d %d\n", st[0], st[1],
                                     st[2], st[3], r, g, b, w0, w1, w2, f0, f1, f2);
            ++bad;
          }
          ++n;
        }
  }
  std::printf("pairs %ld differing %ld\n", n, bad);
  return bad ? 1 : 0;
}
