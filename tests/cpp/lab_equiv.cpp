// Every sRGB8 colour through lab_pixel_q (mg_math.h: the arithmetic the
// reduction kernels evaluate, two pixels at a time in packed FP32x2) against
// the oracle's defined per-pixel Lab, clamped and quantised as the oracle
// sums it.  Prints the number of colours whose L, a or b summand differs.
#include <cstdio>
#include <vector>

#include "../../mosaic-art-rust_gb300/csrc/mg_math.h"
#include "../../oracle/oracle.h"

int main() {
  float lut[256], ms[9], k[3];
  orc_lab_consts(lut, ms, k);
  const long n = 1l << 24;
  std::vector<uint8_t> rgb(3 * (size_t)n);
  for (long i = 0; i < n; ++i) {
    rgb[3 * i] = (uint8_t)(i >> 16);
    rgb[3 * i + 1] = (uint8_t)(i >> 8);
    rgb[3 * i + 2] = (uint8_t)i;
  }
  std::vector<int32_t> q(3 * (size_t)n);
  orc_lab_pixels_q(rgb.data(), n, q.data());
  long bad = 0;
  for (long i = 0; i < n; ++i) {
    int qL, qA, qB;
    mg::lab_pixel_q(lut, ms, k[0], k[1], k[2], rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2], qL, qA, qB);
    if (qL != q[3 * i] || qA != q[3 * i + 1] || qB != q[3 * i + 2]) {
      if (bad < 5)
        std::printf("colour %ld: %d %d %d vs oracle %d %d %d\n", i, qL, qA, qB, q[3 * i], q[3 * i + 1], q[3 * i + 2]);
      ++bad;
    }
  }
  std::printf("colours %ld differing %ld\n", n, bad);
  return bad ? 1 : 0;
}
