// Checks la_f64_to_f32 / la_f32_to_f64 (rust-la_gb300/csrc/f64conv.h) against
// the compiler's conversions bit for bit: every exponent of both formats with
// random mantissas, rounding ties, the ends of the FP32 range, zeros,
// subnormals, infinities and NaNs. Prints "ok <cases>" or the first mismatch.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>

#include "f64conv.h"

static uint64_t state = 0x9e3779b97f4a7c15ull;
static uint64_t next() {  // splitmix64
  uint64_t z = (state += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

static long cases = 0;
static bool check64(uint64_t b) {
  const double d = la_f64_from_bits(b);
  const float want = (float)d, got = la_f64_to_f32(d);
  cases++;
  if (std::isnan(want) && std::isnan(got)) return true;
  if (la_bits_f32(want) != la_bits_f32(got)) {
    printf("f64->f32 mismatch: %016llx want %08x got %08x\n", (unsigned long long)b,
           la_bits_f32(want), la_bits_f32(got));
    return false;
  }
  return true;
}
static bool check32(uint32_t b) {
  const float f = la_f32_from_bits(b);
  const double want = (double)f, got = la_f32_to_f64(f);
  cases++;
  if (std::isnan(want) && std::isnan(got)) return true;
  if (la_bits_f64(want) != la_bits_f64(got)) {
    printf("f32->f64 mismatch: %08x\n", b);
    return false;
  }
  return true;
}

int main() {
  for (uint64_t e = 0; e < 2048; e++)
    for (int s = 0; s < 2; s++)
      for (int t = 0; t < 400; t++) {
        uint64_t mant = next() & 0x000fffffffffffffull;
        if (t == 0) mant = 0;
        if (t == 1) mant = 0x000fffffffffffffull;
        if (t >= 2 && t < 10) mant = (mant & ~0x1fffffffull) | 0x10000000ull;  // exact ties
        if (t >= 10 && t < 14) mant = (mant & ~0x1fffffffull) | (0x10000000ull + (t & 1 ? 1 : -1));
        if (!check64(((uint64_t)s << 63) | (e << 52) | mant)) return 1;
      }
  // the largest finite float and its neighbourhood, rounding up to infinity
  const double fmax = (double)std::numeric_limits<float>::max();
  for (int k = -64; k <= 64; k++) {
    uint64_t b = la_bits_f64(fmax) + (int64_t)k * (1ll << 20);
    if (!check64(b) || !check64(b | 0x8000000000000000ull)) return 1;
  }
  for (uint64_t e = 0; e < 256; e++)
    for (int s = 0; s < 2; s++)
      for (int t = 0; t < 400; t++) {
        uint32_t mant = (uint32_t)next() & 0x007fffffu;
        if (t == 0) mant = 0;
        if (!check32(((uint32_t)s << 31) | ((uint32_t)e << 23) | mant)) return 1;
      }
  for (int i = 0; i < 2000000; i++)
    if (!check64(next())) return 1;
  printf("ok %ld\n", cases);
  return 0;
}
