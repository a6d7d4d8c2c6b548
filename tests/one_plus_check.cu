// Host check of nsm::one_plus_bits (the element kernel's integer 1 + h) against
// the FP64 add, bit for bit: random normal h of either sign with |h| < 1/2,
// values with low significand bits at and next to rounding ties, and edges.
#include <cstdio>
#include <cstring>
#include <random>
#include "hex_math.cuh"
using namespace nsm;
static unsigned long long bits(double x) { unsigned long long b; memcpy(&b, &x, 8); return b; }
static double dbl(unsigned long long b) { double x; memcpy(&x, &b, 8); return x; }
static bool check(double h) {
  unsigned long long hb = bits(h);
  int be = (int)((hb >> 52) & 0x7ff);
  if (be == 0 || be > 1021) return true;
  volatile double one = 1.0;
  double ref = one + h;
  double got = dbl(one_plus_bits(hb));
  if (bits(ref) != bits(got)) { printf("MISMATCH h=%a ref=%a got=%a\n", h, ref, got); return false; }
  return true;
}
int main() {
  std::mt19937_64 g(1);
  long bad = 0, n = 0;
  for (long i = 0; i < 2000000; i++) {
    unsigned long long r = g();
    // random exponents in [1, 1021], random significand and sign
    unsigned long long be = 1 + (r % 1021);
    unsigned long long hb = ((g() & 1ull) << 63) | (be << 52) | (g() & ((1ull << 52) - 1));
    bad += !check(dbl(hb)); n++;
    // values near the rounding boundaries: exponent -53..-1, low bits near ties
    unsigned long long be2 = 1023 - 1 - (r % 56);
    unsigned long long mant = g() & ((1ull << 52) - 1);
    int k = (int)(r >> 40) % 60;
    if (k < 52) mant = (mant & ~((1ull << k) - 1)) | ((g() & 1) ? (1ull << k) >> 1 : 0);
    unsigned long long hb2 = ((g() & 1ull) << 63) | (be2 << 52) | mant;
    bad += !check(dbl(hb2)); n++;
    if (bad > 5) break;
  }
  // exact ties and extremes
  double special[] = {0.25, -0.25, 0.4999999999999999, -0.4999999999999999, 0x1p-53, -0x1p-53, 0x1p-54, -0x1p-54, 0x1.8p-53, -0x1.8p-53, 0x1p-52, -0x1p-52, 0x1.0000000000001p-53, -0x1.0000000000001p-54, 0x1p-1021, 0x1.fffffffffffffp-2, -0x1.fffffffffffffp-2, 0x1.8p-54, -0x1.8p-54};
  for (double h : special) { bad += !check(h); n++; }
  printf("%ld checked, %ld mismatches\n", n, bad);
  return bad != 0;
}
