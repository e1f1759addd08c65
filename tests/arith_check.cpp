// Host check of the integer-pipe division (and its reciprocal-candidate form), multiplication, square root, doubling, negation, absolute value and 0 + x
// (meshcfd_gb300/csrc/mcfd_arith.cuh compiled as plain C++) against the
// host's IEEE binary64 division and square root, bit for bit.
//
// usage: arith_check N SEED  -> prints "cases=<n> mismatches=<m>" and the
// first mismatch, exits 0 when there is none.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>

#include "../meshcfd_gb300/csrc/mcfd_arith.cuh"

typedef unsigned long long u64;

static u64 g_state;
static u64 next_u64() {
  u64 z = (g_state += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

static u64 bits_of(double x) {
  u64 b;
  memcpy(&b, &x, 8);
  return b;
}
static double of_bits(u64 b) {
  double x;
  memcpy(&x, &b, 8);
  return x;
}

// random double: random sign, biased exponent 1023 +- span, random significand
// with some runs of zeros / ones (rounding ties and carries)
static double random_double(int span) {
  const u64 r = next_u64();
  u64 mant = next_u64() & 0x000fffffffffffffull;
  switch (r & 7) {
    case 0: mant &= 0xffff000000000ull; break;
    case 1: mant |= 0x0000ffffffffffull; break;
    case 2: mant = 0; break;
    default: break;
  }
  int e = 1023 + (int)((r >> 8) % (u64)(2 * span + 1)) - span;
  e = e < 0 ? 0 : (e > 2047 ? 2047 : e);  // zero / subnormal and inf / NaN exponents at the ends
  return of_bits(((r >> 63) << 63) | ((u64)e << 52) | mant);
}

static long g_cases = 0, g_bad = 0;

static bool same(double x, double y) {
  return bits_of(x) == bits_of(y) || (std::isnan(x) && std::isnan(y));
}

static void check(double a, double b) {
  ++g_cases;
  const double q = mcfd::div_rn(a, b), qr = a / b;
  if (!same(q, qr)) {
    if (!g_bad) printf("div %a / %a: got %a expected %a\n", a, b, q, qr);
    ++g_bad;
  }
  const unsigned long long X = mcfd::recip_fixed(b);
  const double qf = mcfd::div_rn_fma(a, b, mcfd::div_rn_recip(1.0, b, X), X);
  if (!same(qf, qr)) {
    if (!g_bad) printf("div (reciprocal candidate) %a / %a: got %a expected %a\n", a, b, qf, qr);
    ++g_bad;
  }
  const double p = mcfd::mul_rn(a, b), pr = a * b;
  if (!same(p, pr)) {
    if (!g_bad) printf("mul %a * %a: got %a expected %a\n", a, b, p, pr);
    ++g_bad;
  }
  const double s = mcfd::sqrt_rn(a), sr = std::sqrt(a);
  if (!same(s, sr)) {
    if (!g_bad) printf("sqrt %a: got %a expected %a\n", a, s, sr);
    ++g_bad;
  }
  if (!same(mcfd::twice(a), 2.0 * a) || !same(mcfd::negate(a), -a) || !same(mcfd::plus_zero(a), 0.0 + a) ||
      !same(mcfd::abs_of(a), std::fabs(a))) {
    if (!g_bad) printf("twice / negate %a\n", a);
    ++g_bad;
  }
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 1000000;
  g_state = argc > 2 ? strtoull(argv[2], nullptr, 10) : 1;
  const double inf = std::numeric_limits<double>::infinity();
  const double nan = std::numeric_limits<double>::quiet_NaN();
  const double specials[] = {0.0, -0.0, 1.0, -1.0, 2.0, 0.5, 3.0, 1e-300, 1e300, 1.7976931348623157e308,
                             2.2250738585072014e-308, 4.9e-324, 2.225073858507201e-308, -2.2250738585072014e-308,
                             inf, -inf, nan, of_bits(0x3fefffffffffffffull), of_bits(0x3ff0000000000001ull),
                             of_bits(0x433fffffffffffffull), 1e-10, 1e10, 0.1, 1.4, 0.4};
  for (double a : specials)
    for (double b : specials) check(a, b);
  const int spans[] = {1, 30, 200, 700, 1100};
  for (long i = 0; i < n; ++i) {
    const int span = spans[i % 5];
    const double a = random_double(span);
    double b = random_double(span);
    switch (i & 15) {
      case 3: b = -a; break;                                         // quotient -1
      case 5: b = of_bits(bits_of(a) ^ 1ull); break;                 // nearly equal
      case 7: b = of_bits(0x3ff0000000000000ull | (next_u64() & 3)); break;  // divisor near 1
      case 9: b = a * random_double(2); break;                       // exact-ish quotients
      default: break;
    }
    check(a, b);
    check(std::fabs(a), b);
    // exact quotients and perfect squares
    const double k = (double)((next_u64() >> 38) | 1ull), d = (double)((next_u64() >> 44) | 1ull);
    check(k * d, d);
    check(k * k, d);
  }
  printf("cases=%ld mismatches=%ld\n", g_cases, g_bad);
  return g_bad ? 1 : 0;
}
