// png_fuzz.cpp -- mutation fuzzing of the PNG decoder (csrc/io_png.cpp),
// built with AddressSanitizer and UndefinedBehaviorSanitizer by
// tests/test_png.py.  Each seed file is mutated (bit flips, byte writes,
// truncation, 32-bit overwrites); every other mutant gets its chunk CRCs
// recomputed so the damage reaches inflate, the unfilter and the conversion
// (on large seeds, the two-thread pipeline).  Every result must be a status
// code; the sanitizers turn any out-of-bounds access or undefined operation
// into a failed run.
//
//   png_fuzz ITERATIONS SEED.png...
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <random>
#include <string>
#include <vector>

#include "mosaic_gpu.h"

namespace mg {
void set_error(const std::string&) {}
}

static void fix_crcs(std::vector<uint8_t>& d) {
  size_t pos = 8;
  while (pos + 12 <= d.size()) {
    const uint32_t len = (uint32_t)d[pos] << 24 | (uint32_t)d[pos + 1] << 16 | (uint32_t)d[pos + 2] << 8 | d[pos + 3];
    if (len > d.size() - pos - 12) break;
    uint32_t c = 0xFFFFFFFFu;
    for (size_t i = pos + 4; i < pos + 8 + len; ++i) {
      c ^= d[i];
      for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
    }
    c ^= 0xFFFFFFFFu;
    for (int k = 0; k < 4; ++k) d[pos + 8 + len + k] = (uint8_t)(c >> (24 - 8 * k));
    pos += 12 + len;
  }
}

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  const long iters = std::atol(argv[1]);
  std::mt19937_64 rng(12345);
  long decoded = 0, rejected = 0;
  for (int a = 2; a < argc; ++a) {
    std::ifstream f(argv[a], std::ios::binary);
    const std::vector<uint8_t> seed((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    for (long it = 0; it < iters; ++it) {
      std::vector<uint8_t> d = seed;
      const int muts = it % 10 == 0 ? 0 : 1 + (int)(rng() % 6);
      for (int m = 0; m < muts && !d.empty(); ++m) {
        const size_t p = rng() % d.size();
        switch (rng() % 4) {
          case 0: d[p] ^= (uint8_t)(1u << (rng() % 8)); break;
          case 1: d[p] = (uint8_t)rng(); break;
          case 2: d.resize(p); break;
          default:
            if (p + 4 <= d.size()) {
              const uint32_t v = (uint32_t)rng();
              std::memcpy(&d[p], &v, 4);
            }
        }
      }
      if (it % 2) fix_crcs(d);
      int w = 0, h = 0;
      if (mg_png_info(d.data(), d.size(), &w, &h) != MG_OK || (size_t)w * h > (1u << 22)) {
        ++rejected;
        continue;
      }
      std::vector<uint8_t> out((size_t)w * h * 3);
      const int rc = mg_png_decode(d.data(), d.size(), out.data(), 3ll * w);
      if (rc == MG_OK)
        ++decoded;
      else if (rc == MG_ERR_ARG)
        ++rejected;
      else
        return 1;
      if (muts == 0 && rc != MG_OK) return 1;  // an unmutated seed must decode
    }
  }
  std::printf("decoded %ld rejected %ld\n", decoded, rejected);
  return 0;
}
