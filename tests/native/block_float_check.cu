// Host build of the sweeps' block-float helpers (boss_sweep.cuh): prints seeded
// random cases and their results for tests/test_block_float_host.py, which checks
// them against exact integer arithmetic.
#include <cstdio>
#include <cstdlib>
#include <random>

#include "../../theboss_gb300/csrc/boss_sweep.cuh"

using namespace boss;

int main(int argc, char** argv) {
  std::mt19937_64 g(argc > 1 ? std::strtoull(argv[1], nullptr, 10) : 1);
  const int n = argc > 2 ? std::atoi(argv[2]) : 1000;
  for (int t = 0; t < n; ++t) {
    // magnitudes: full 61-bit, random widths, tiny, ~58-bit; some exact zeros
    const int mode = t % 4;
    long long v[8];
    for (int k = 0; k < 8; ++k) {
      const int bits = mode == 0 ? 61 : mode == 1 ? 1 + (int)(g() % 61) : mode == 2 ? 1 + (int)(g() % 8) : 58;
      long long x = (long long)(g() >> (64 - bits));
      if (g() & 1) x = -x;
      if (mode == 3 && k == 3 && (t & 8)) x = 0;
      v[k] = x;  // |x| < 2^61, the fixed-point factors' bound
    }
    const BFloat a = bf_pair(v[0], v[1], v[2], v[3], -100);
    const BFloat b = bf_pair(v[4], v[5], v[6], v[7], -100);
    const BFloat c = bf_norm(v[0], v[1], -50);
    const BFloat m = bf_mul(a, b);
    const BFloat m2 = bf_mul(m, c);
    std::printf("%lld %lld %lld %lld %lld %lld %lld %lld|%lld %lld %d|%lld %lld %d|%lld %lld %d|%lld %lld %d|"
                "%lld %lld %d|%a %a\n",
                v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], a.re, a.im, a.e, b.re, b.im, b.e, c.re, c.im, c.e,
                m.re, m.im, m.e, m2.re, m2.im, m2.e, bf_to_double(m2.re, m2.e), bf_to_double(m2.im, m2.e));
  }
  // conversions at the edges of FP64's range go through the exact slow path
  const long long x = 3ll << 60;
  std::printf("edge %a %a %a %a\n", bf_to_double(x, -1200), bf_to_double(x, 900), bf_to_double(-x, -1150),
              bf_to_double(0, 5));
  return 0;
}
