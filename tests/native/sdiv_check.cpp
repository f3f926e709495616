// Host check of vf::sd_recip / vf::sd_div against IEEE double division (test
// infrastructure). Every divisor is shared by several numerators, as in the
// kernels. Usage: sdiv_check <n> <seed>; prints "mismatches fast_path_count".
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include "vf_sdiv.cuh"

static uint64_t sm(uint64_t& s) {  // splitmix64
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static double make(uint64_t& s, int mode) {
  uint64_t frac = sm(s) & ((1ull << 52) - 1);
  const uint64_t sign = (sm(s) & 1) << 63;
  int e;
  switch (mode % 7) {
    case 0: e = 1023 + (int)(sm(s) % 61) - 30; break;                                         // moderate range
    case 1: e = 1 + (int)(sm(s) % 2046); break;                                               // full normal range
    case 2: frac = (1ull << 52) - 1 - (sm(s) % 4); e = 1023 + (int)(sm(s) % 9) - 4; break;     // all-ones significands
    case 3: frac = sm(s) % 8; e = 1023 + (int)(sm(s) % 9) - 4; break;                          // near powers of two
    case 4: e = 1023 + (int)(sm(s) % 5) - 2; break;
    case 5: frac &= ~((1ull << 30) - 1); e = 1023 + (int)(sm(s) % 21) - 10; break;             // short significands (exact ties)
    default: e = (sm(s) % 50 == 0) ? 0 : 1023 + (int)(sm(s) % 41) - 20; break;                 // zeros and subnormals
  }
  const uint64_t u = sign | ((uint64_t)e << 52) | frac;
  double x;
  std::memcpy(&x, &u, 8);
  return x;
}

int main(int argc, char** argv) {
  const long long n = argc > 1 ? atoll(argv[1]) : 1000000;
  uint64_t s = argc > 2 ? strtoull(argv[2], 0, 10) : 1;
  long long bad = 0, fast = 0;
  for (long long i = 0; i < n; ++i) {
    const int mode = (int)(i % 7);
    const double b = make(s, (mode + 1) % 7);
    const vf::SharedRecip R = vf::sd_recip(b);
    for (int k = 0; k < 4; ++k) {
      double a = make(s, mode + k);
      if (k == 3) a = b * (1.0 + (double)(sm(s) % 5) * 1e-16);  // quotients near 1
      double q;
      if (vf::sd_div_fast(R, a, &q)) ++fast;
      q = vf::sd_div(R, a);
      const double want = a / b;
      uint64_t uq, uw;
      std::memcpy(&uq, &q, 8);
      std::memcpy(&uw, &want, 8);
      if (uq != uw && !(want != want && q != q)) {
        if (bad < 10) std::printf("MISMATCH a=%a b=%a got=%a want=%a\n", a, b, q, want);
        ++bad;
      }
    }
  }
  std::printf("%lld %lld\n", bad, fast);
  return bad != 0;
}
