// Checks born::couple::couple_exact (the float evaluation of the reference's
// double Born coupling, sc17-born_gb300/csrc/born_couple.h) bit for bit
// against the double expression of cpuProp::imageAdd (base/cpu_prop.cc:
// 216-223) on seeded inputs:
//   field   - wavefield-like magnitudes (s, r over 40 decades, m ~ 0.05)
//   wide    - every finite float exponent for r, s and m
//   neartie - r + V within about 2^-49 |r| of a float rounding boundary
//   tiny    - products and levels around the underflow thresholds
//   edge    - results around the smallest normal floats
// Prints one line per class: cases, mismatches, double fallbacks.
// Build: g++ -O2 -std=c++17 -ffp-contract=off -fno-fast-math
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <initializer_list>

#include "born_couple.h"

namespace {

uint64_t g_state = 0x9E3779B97F4A7C15ull;
uint64_t next_u64() {  // SplitMix64
  uint64_t z = (g_state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double uniform() { return (next_u64() >> 11) * 0x1p-53; }
float from_bits(uint32_t u) {
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}
uint32_t to_bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}
// random finite float with a uniformly drawn biased exponent in [lo, hi]
float rand_float(int lo, int hi) {
  const uint32_t e = (uint32_t)(lo + (int)(next_u64() % (uint64_t)(hi - lo + 1)));
  const uint32_t mant = (uint32_t)(next_u64() & 0x7fffffu);
  const uint32_t sign = (uint32_t)(next_u64() & 1u) << 31;
  return from_bits(sign | (e << 23) | mant);
}
float signed_log_uniform(double lo10, double hi10) {
  const double v = std::pow(10.0, lo10 + (hi10 - lo10) * uniform());
  return (float)((next_u64() & 1) ? v : -v);
}

struct Tally {
  long long n = 0, bad = 0, fallback = 0;
};

void check(Tally &t, float r, float s, float m) {
  bool fb = false;
  const float got = born::couple::couple_exact(r, s, m, &fb);
  const float want = (float)((double)r + 1e-6 * (double)s * (double)m);
  ++t.n;
  if (fb) ++t.fallback;
  if (to_bits(got) != to_bits(want)) {
    if (t.bad < 5)
      std::fprintf(stderr, "mismatch r=%a s=%a m=%a got %a want %a\n", r, s,
                   m, got, want);
    ++t.bad;
  }
}

}  // namespace

int main(int argc, char **argv) {
  const long long n = argc > 1 ? std::atoll(argv[1]) : 2000000;
  int fails = 0;
  auto report = [&](const char *name, const Tally &t) {
    std::printf("%s %lld %lld %lld\n", name, t.n, t.bad, t.fallback);
    fails += t.bad != 0;
  };
  {
    Tally t;
    for (long long i = 0; i < n; ++i) {
      const float s = signed_log_uniform(-40, 2);
      const float m = signed_log_uniform(-4, -1);
      const float r = (i % 4 == 0) ? 0.f : signed_log_uniform(-48, 0);
      check(t, r, s, m);
    }
    report("field", t);
  }
  {
    Tally t;
    for (long long i = 0; i < n; ++i)
      check(t, rand_float(0, 254), rand_float(0, 254), rand_float(0, 254));
    report("wide", t);
  }
  {
    // r + V close to r + half an ulp of r: pick r and s, then m so that
    // 1e-6 s m is half an ulp of r times (1 + tiny)
    Tally t;
    for (long long i = 0; i < n; ++i) {
      const float r = rand_float(60, 200);
      const float s = signed_log_uniform(-20, 2);
      const int er = (int)((to_bits(r) >> 23) & 0xffu) - 127;
      const double half = std::ldexp(1.0, er - 24) *
                          (1.0 + std::ldexp(uniform() - 0.5, -(int)(next_u64() % 40)));
      const double sign = (next_u64() & 1) ? 1.0 : -1.0;
      const float m = (float)(sign * half / (1e-6 * (double)s));
      if (!std::isfinite(m) || m == 0.f) continue;
      check(t, r, s, m);
    }
    report("neartie", t);
  }
  {
    Tally t;
    for (long long i = 0; i < n; ++i) {
      const float r = (i % 3 == 0) ? 0.f : rand_float(0, 70);
      check(t, r, rand_float(0, 60), rand_float(90, 140));
    }
    report("tiny", t);
  }
  {
    // results around the smallest normal floats, where the scaled
    // evaluation of small fields hands over to the double expression
    Tally t;
    for (long long i = 0; i < n; ++i)
      check(t, rand_float(0, 6), rand_float(20, 100), rand_float(100, 140));
    report("edge", t);
  }
  {
    // the sign of zero: r = -0/+0 with zero and nonzero products
    Tally t;
    const float zs[] = {0.f, -0.f};
    for (float r : zs)
      for (float s : zs)
        for (float m : {0.f, -0.f, 1e-3f, -1e-3f}) check(t, r, s, m);
    for (float r : zs)
      for (float s : {1e-30f, -1e-30f, 1e-45f})
        for (float m : {1e-20f, -1e-20f}) check(t, r, s, m);
    report("zeros", t);
  }
  return fails ? 1 : 0;
}
