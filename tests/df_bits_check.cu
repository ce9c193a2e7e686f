// Host-only check of the bit-level double <-> double-float conversions of
// mini_mdft_gb300/csrc/common.cuh (the same functions the kernels call),
// against the host's own conversions and exact long-double sums.
// Prints "ok <counts>" and exits 0, or prints the first failures and exits 1.
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "common.cuh"

using mdft::DF;

static unsigned long long rng_state = 0x9e3779b97f4a7c15ull;
static unsigned long long next_u64() {  // splitmix64
  unsigned long long z = (rng_state += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

static int failures = 0;
static void fail(const char* what, double x, double got, double want) {
  if (failures++ < 10)
    std::printf("FAIL %s: x=%a got=%a want=%a\n", what, x, got, want);
}

static bool same_bits(double a, double b) { return mdft::bits_of(a) == mdft::bits_of(b); }

static void check_f2d(float f) {
  const double got = mdft::f2d_bits(f), want = (double)f;
  if (std::isnan(want) ? !std::isnan(got) : !same_bits(got, want)) fail("f2d_bits", f, got, want);
}

static void check_from_double(double x) {
  const DF d = mdft::df_from_double_bits(x);
  const double ax = std::fabs(x);
  if (std::isnan(x)) {
    if (!std::isnan(d.hi) || d.lo != 0.f) fail("from_double nan", x, d.hi, x);
    return;
  }
  if (ax >= std::ldexp(1.0, 128)) {
    if (!std::isinf(d.hi) || std::signbit(d.hi) != std::signbit(x) || d.lo != 0.f)
      fail("from_double huge", x, d.hi, x);
    return;
  }
  if (ax < std::ldexp(1.0, -73)) {
    // hi = x truncated to float, lo = 0
    const float h = d.hi;
    const double ah = std::fabs((double)h);
    const float up = std::nextafter(std::fabs(h), INFINITY);
    if (d.lo != 0.f || ah > ax || (double)up <= ax ||
        (h != 0.f && std::signbit(h) != std::signbit(x)))
      fail("from_double tiny", x, h, x);
    return;
  }
  const long double s = (long double)d.hi + (long double)d.lo;
  const long double err = std::fabs(s - (long double)x);
  // rounded split below 2^127, truncated split in [2^127, 2^128)
  const int bound = ax < std::ldexp(1.0, 127) ? -48 : -47;
  if (err > std::ldexp((long double)ax, bound)) fail("from_double error", x, (double)s, x);
  if (d.hi + d.lo != d.hi) fail("from_double not normalised", x, d.lo, 0.0);
}

// the rounded split carries no bias: the mean signed relative error over many
// values stays far below the 2^-49 a truncating split would show
static void check_from_double_unbiased() {
  long double sum = 0;
  const int n = 2000000;
  for (int k = 0; k < n; ++k) {
    const double x = mdft::double_of((next_u64() & 0x000fffffffffffffull) | (1023ull << 52));  // [1, 2)
    const DF d = mdft::df_from_double_bits(x);
    sum += ((long double)d.hi + (long double)d.lo - (long double)x) / (long double)x;
  }
  const long double mean = sum / n;
  if (std::fabs(mean) > std::ldexp(1.0L, -56)) fail("from_double biased", (double)mean, 0, 0);
}

static void check_to_double(DF a, bool exact_ref) {
  const double got = mdft::df_to_double(a);
  const long double s = (long double)a.hi + (long double)a.lo;
  const double want = (double)s;
  if (std::isnan(want)) {
    if (!std::isnan(got)) fail("to_double nan", a.hi, got, want);
    return;
  }
  if (same_bits(got, want)) return;
  if (want == 0.0 && got == 0.0) return;
  if (exact_ref) {
    // correctly rounded: as close to the exact sum as the host's rounding
    if (std::fabs((long double)got - s) > std::fabs((long double)want - s))
      fail("to_double rounding", a.hi, got, want);
  } else {
    // the long-double reference is rounded itself: one ulp
    const double ulp = std::nextafter(std::fabs(want), INFINITY) - std::fabs(want);
    if (std::fabs(got - want) > ulp) fail("to_double", a.hi, got, want);
  }
}

int main() {
  long n_f2d = 0, n_from = 0, n_to = 0;
  // f2d_bits: every class, then a stride through all 2^32 patterns
  const float specials[] = {0.f, -0.f, 1.f, -1.f, INFINITY, -INFINITY, NAN, 1e-45f, -1e-45f,
                            1.1754942e-38f, 1.17549435e-38f, 3.4028235e38f};
  for (float f : specials) check_f2d(f), ++n_f2d;
  for (unsigned long long u = 0; u < (1ull << 32); u += 251) {
    check_f2d(mdft::float_of((unsigned)u));
    ++n_f2d;
  }
  // df_from_double_bits: every double exponent, random fractions and signs
  const double dspecials[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, 1.0, -1.0, 0.1,
                              std::ldexp(1.0, -73), std::ldexp(1.0, 128), std::ldexp(1.0, -149),
                              std::ldexp(1.0, -150), 3.4028234663852886e38, 5e-324};
  for (double x : dspecials) check_from_double(x), ++n_from;
  for (unsigned e = 0; e < 2048; ++e)
    for (int k = 0; k < 2000; ++k) {
      const unsigned long long b = (next_u64() & 0x800fffffffffffffull) | ((unsigned long long)e << 52);
      check_from_double(mdft::double_of(b));
      ++n_from;
    }
  check_from_double_unbiased();
  // df_to_double: normalised pairs over the float exponent range and
  // every gap between hi and lo, zero/subnormal/inf parts, unnormalised pairs
  for (int k = 0; k < 4000000; ++k) {
    const unsigned long long r = next_u64();
    const unsigned eh = 1 + (unsigned)(r % 254);
    const float hi = mdft::float_of(((unsigned)(r >> 32) & 0x807fffffu) | (eh << 23));
    const int gap = 24 + (int)((r >> 8) % 40);
    const float lo = (float)std::ldexp(((double)(next_u64() >> 11) / 9007199254740992.0 - 0.5),
                                       std::ilogb(hi) - gap + 1);
    const DF a(hi, lo);
    // the long-double reference is exact while the pair spans <= 64 bits
    const bool exact = lo == 0.f || std::ilogb(hi) - std::ilogb(lo) + 24 <= 64;
    check_to_double(a, exact);
    ++n_to;
  }
  const DF pairs[] = {DF(0.f, 0.f), DF(-0.f, 0.f), DF(1.f, 0.f), DF(0.f, 1e-30f), DF(1e-45f, 0.f),
                      DF(1e-40f, -1e-45f), DF(INFINITY, 0.f), DF(-INFINITY, 0.f), DF(NAN, 0.f),
                      DF(1.f, 1.f), DF(1e-8f, 1.f), DF(-2.f, 1.f), DF(3.4028235e38f, 1e30f)};
  for (const DF& a : pairs) check_to_double(a, true), ++n_to;
  // round trip double -> DF -> double within 2^-47 in the full range
  for (int k = 0; k < 1000000; ++k) {
    const unsigned e = 950 + (unsigned)(next_u64() % 201);
    const double x = mdft::double_of((next_u64() & 0x800fffffffffffffull) | ((unsigned long long)e << 52));
    const double y = mdft::df_to_double(mdft::df_from_double_bits(x));
    if (std::fabs(y - x) > std::ldexp(std::fabs(x), -47)) fail("round trip", x, y, x);
  }
  if (failures) {
    std::printf("%d failures\n", failures);
    return 1;
  }
  std::printf("ok f2d %ld from_double %ld to_double %ld\n", n_f2d, n_from, n_to);
  return 0;
}
