// jpeg_fuzz.cpp -- mutation fuzzing of the JPEG decoder (csrc/io_jpeg.cpp,
// reached through mg_image_info / mg_image_decode), built with
// AddressSanitizer and UndefinedBehaviorSanitizer by tests/test_jpeg.py.
// Each seed file is mutated (bit flips, byte writes, truncation, 32-bit
// overwrites); every other mutant aims its damage at the headers (the bytes
// before the first scan: frame, tables, restart interval) so that broken
// tables and sampling factors reach the entropy decoder.  Every result must
// be a status code; the sanitizers turn any out-of-bounds access or undefined
// operation into a failed run.  Then the encoder writes random images of
// random small sizes and qualities, each decoded back.
//
//   jpeg_fuzz ITERATIONS SEED.jpg...
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
extern "C" const char* mg_last_error(void) { return ""; }

// Offset of the first start-of-scan marker (the headers end there), or the size.
static size_t header_end(const std::vector<uint8_t>& d) {
  for (size_t i = 2; i + 1 < d.size(); ++i)
    if (d[i] == 0xFF && d[i + 1] == 0xDA) return i + 2;
  return d.size();
}

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  const long iters = std::atol(argv[1]);
  std::mt19937_64 rng(6789);
  long decoded = 0, rejected = 0;
  for (int a = 2; a < argc; ++a) {
    std::ifstream f(argv[a], std::ios::binary);
    const std::vector<uint8_t> seed((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    const size_t head = header_end(seed);
    for (long it = 0; it < iters; ++it) {
      std::vector<uint8_t> d = seed;
      const int muts = it % 10 == 0 ? 0 : 1 + (int)(rng() % 6);
      for (int m = 0; m < muts && !d.empty(); ++m) {
        const size_t span = (it % 2 && head < d.size()) ? head : d.size();
        const size_t p = rng() % span;
        switch (rng() % 4) {
          case 0: d[p] ^= (uint8_t)(1u << (rng() % 8)); break;
          case 1: d[p] = (uint8_t)rng(); break;
          case 2:
            if (rng() % 4 == 0) d.resize(p);  // truncation: rarer, it ends the file
            else d[p] = (uint8_t)(d[p] + 1);
            break;
          default:
            if (p + 4 <= d.size()) {
              const uint32_t v = (uint32_t)rng();
              std::memcpy(&d[p], &v, 4);
            }
        }
      }
      int w = 0, h = 0;
      if (mg_image_info(d.data(), d.size(), &w, &h) != MG_OK || (size_t)w * h > (1u << 22)) {
        ++rejected;
        continue;
      }
      std::vector<uint8_t> out((size_t)w * h * 3);
      const int rc = mg_image_decode(d.data(), d.size(), out.data(), 3ll * w);
      if (rc == MG_OK)
        ++decoded;
      else if (rc == MG_ERR_ARG)
        ++rejected;
      else
        return 1;
      if (muts == 0 && rc != MG_OK) return 1;  // an unmutated seed must decode
    }
  }
  // the encoder on random images of every small size (edges, partial MCUs),
  // each file decoded back
  long encoded = 0;
  for (int it = 0; it < 300; ++it) {
    const int w = 1 + (int)(rng() % 70), h = 1 + (int)(rng() % 70), q = 1 + (int)(rng() % 100);
    std::vector<uint8_t> img((size_t)w * h * 3);
    for (auto& v : img) v = (uint8_t)rng();
    std::vector<uint8_t> file(mg_jpeg_encode_bound(w, h));
    size_t len = 0;
    if (mg_jpeg_encode(img.data(), w, h, 3ll * w, q, 1 + (int)(rng() % 4), file.data(), file.size(), &len) != MG_OK)
      return 1;
    std::vector<uint8_t> back((size_t)w * h * 3);
    if (mg_image_decode(file.data(), len, back.data(), 3ll * w) != MG_OK) return 1;
    ++encoded;
  }
  std::printf("decoded %ld rejected %ld encoded %ld\n", decoded, rejected, encoded);
  return 0;
}
