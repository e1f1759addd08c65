// IEEE-754 binary64 division, square root and multiplication, round to
// nearest even, evaluated on the integer pipe (plus exact negation, absolute value,
// doubling and 0 + x).
//
// On GB300 one FP64 division or square root costs ~8.6 FP64 issue slots
// (~58 G/s per GPU) while the integer pipe runs ~38x the FP64 rate, so the
// residual path's 8-12 divisions per face or cell dominate its FP64 budget.
// These routines return exactly the IEEE result (the same bits as the FP64
// unit's `a / b` and `sqrt(x)`) for every input:
//
// * normal operands with a normal result take the integer path: the
//   reciprocal (division) or reciprocal square root (square root) of the
//   53-bit significand is seeded from the fp32 approximation instructions
//   (rcp.approx / rsqrt.approx, relative error < 2^-21 after truncating the
//   significand to 24 bits) and refined by two Newton-Raphson steps in 64-bit
//   fixed point (x' = x + x (1 - b x), y' = y + y (1 - m y^2) / 2; error
//   ~2^-44, then ~2^-61).  The truncated quotient (root) with two bits below
//   the last place is then corrected with its exact integer remainder
//   (A 2^54 - Q B, resp. M 2^56 - S^2, both within a few units of the
//   divisor and so exact in 64-bit two's complement) until 0 <= remainder <
//   divisor — the classical exact-rounding test of a Newton quotient (e.g.
//   Brent & Zimmermann, Modern Computer Arithmetic, 2010, secs. 3.4-3.5) —
//   and rounded to nearest even from the guard bit and the sticky bit
//   (remainder != 0);
// * a zero dividend over a normal divisor gives the signed zero directly;
//   other zeros, subnormals, infinities, NaN, negative square-root arguments
//   and quotients that overflow or underflow fall back to the FP64 unit, and
//   so does a remainder still out of range after the correction (it cannot
//   be for the error bounds above; the test keeps the result exact
//   regardless).
//
// The header also compiles as plain C++ (the host seeds are the correctly
// rounded fp32 reciprocal and reciprocal root), so the integer algorithm can
// be checked on the host against its IEEE division and square root.
#pragma once

#include <stdint.h>
#include <string.h>
#include <math.h>

#if defined(__CUDACC__)
#include <cuda_runtime.h>
#define MCFD_IA_FN __host__ __device__ __forceinline__
#define MCFD_IA_SLOW static __host__ __device__ __noinline__
#else
#define MCFD_IA_FN static inline
#define MCFD_IA_SLOW static
#endif

namespace mcfd {
namespace ia {

typedef unsigned long long u64;

MCFD_IA_FN u64 mulhi(u64 a, u64 b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return (u64)(((unsigned __int128)a * b) >> 64);
#endif
}
// The bit pattern of x.  On the device the move is an inline mov.b64, which
// the compiler cannot see through: integer tests on the bits (zero tests,
// exponent classes, sign masks) would otherwise be recognised as the
// equivalent floating-point compares and issued to the FP64 pipe.
MCFD_IA_FN u64 bits(double x) {
#if defined(__CUDA_ARCH__)
  u64 r;
  asm("mov.b64 %0, %1;" : "=l"(r) : "d"(x));
  return r;
#else
  u64 r;
  memcpy(&r, &x, 8);
  return r;
#endif
}
MCFD_IA_FN double from_bits(u64 b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double r;
  memcpy(&r, &b, 8);
  return r;
#endif
}
// fp32 approximations of 1/t and 1/sqrt(t), t a positive normal float
MCFD_IA_FN float rcp_seed(float t) {
#if defined(__CUDA_ARCH__)
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(t));
  return y;
#else
  return 1.0f / t;
#endif
}
MCFD_IA_FN float rsqrt_seed(float t) {
#if defined(__CUDA_ARCH__)
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(t));
  return y;
#else
  return 1.0f / sqrtf(t);
#endif
}
// (hi:lo) >> s, low 32 bits, for 0 <= s < 32 (a funnel shift)
MCFD_IA_FN unsigned shr_funnel(unsigned lo, unsigned hi, unsigned s) {
#if defined(__CUDA_ARCH__)
  return __funnelshift_r(lo, hi, s);
#else
  return (unsigned)((((unsigned long long)hi << 32) | lo) >> s);
#endif
}
// truncating float -> uint32 conversion, saturating at 2^32 - 1 (v > 0)
MCFD_IA_FN unsigned to_u32(float v) {
#if defined(__CUDA_ARCH__)
  return __float2uint_rz(v);
#else
  return v >= 4294967296.0f ? 0xffffffffu : (unsigned)v;
#endif
}

// The FP64 unit's results for the operands the integer path leaves out.  Out
// of line, so that the rare fallback is a branch around a call rather than
// instructions predicated into every evaluation (predicated-off FP64
// instructions still take FP64 issue slots).
MCFD_IA_SLOW double div_fp64(double a, double b) { return a / b; }
MCFD_IA_SLOW double mul_fp64(double a, double b) { return a * b; }
MCFD_IA_SLOW double sqrt_fp64(double x) { return sqrt(x); }

static constexpr u64 kMant = 0x000fffffffffffffull;
static constexpr u64 kImpl = 0x0010000000000000ull;
static constexpr u64 kSign = 0x8000000000000000ull;

// Sign-bit operations kept as integer instructions: written as plain integer
// code, the compiler may recognise them as floating-point negation / absolute
// value / copysign and give them to the FP64 pipe.
MCFD_IA_FN u64 sign_xor(u64 b, u64 s) {
#if defined(__CUDA_ARCH__)
  u64 r;
  asm("xor.b64 %0, %1, %2;" : "=l"(r) : "l"(b), "l"(s));
  return r;
#else
  return b ^ s;
#endif
}
MCFD_IA_FN u64 bits_and(u64 b, u64 m) {
#if defined(__CUDA_ARCH__)
  u64 r;
  asm("and.b64 %0, %1, %2;" : "=l"(r) : "l"(b), "l"(m));
  return r;
#else
  return b & m;
#endif
}

// Round the 55-bit truncated significand q (53 bits, guard bit, one more bit)
// with the remainder's sticky bit; returns the 53-bit significand and bumps e
// when rounding carries into the next binade.
MCFD_IA_FN u64 round_q55(u64 q, bool inexact_tail, int& e) {
  u64 m = q >> 2;
  const u64 guard = (q >> 1) & 1ull;
  const u64 sticky = (q & 1ull) | (u64)inexact_tail;
  m += guard & (sticky | (m & 1ull));
  const unsigned carry = (unsigned)(m >> 53);
  e += (int)carry;
  return m >> carry;
}

// The fixed-point reciprocal X ~ 2^116 / mb of the divisor's 53-bit
// significand mb that div_rn divides with: the fp32 seed refined by two
// Newton steps.  It depends on b alone, so quotients by one divisor can share
// it (div_rn_recip); for zero, subnormal or non-finite b it is unused (those
// divisions take the FP64 unit).
MCFD_IA_FN u64 recip_fixed(double b) {
  const u64 mb = (bits(b) & kMant) | kImpl;
  // seed: x32 ~ 2^87 / (mb >> 29) ~ 2^84 / mb (the float conversion is exact)
  const unsigned x32 = to_u32(rcp_seed((float)(unsigned)(mb >> 29)) * 0x1p55f);
  // Newton step 1 on X = x32 2^32 (~2^116 / mb): D = 2^84 - mb x32 (mod 2^64,
  // |D| < 2^62), X += X D / 2^84
  long long D = -(long long)(mb * (u64)x32);
  u64 ad = D < 0 ? (u64)(-D) : (u64)D;
  u64 h = (mulhi((u64)x32, ad) << 12) | (((u64)x32 * ad) >> 52);
  u64 X = (u64)x32 << 32;
  X = D < 0 ? X - h : X + h;
  // Newton step 2: D = 2^84 - (mb X >> 32), X += X D / 2^84
  {
    const u64 ph = mulhi(mb, X), pl = mb * X;
    D = -(long long)((ph << 32) | (pl >> 32));
    ad = D < 0 ? (u64)(-D) : (u64)D;
    h = mulhi(X, ad) >> 20;
    X = D < 0 ? X - h : X + h;
  }
  return X;
}

// a / b given X = recip_fixed(b): the same bits as div_rn(a, b).
MCFD_IA_FN double div_rn_recip(double a, double b, u64 X) {
  const u64 ia = bits(a), ib = bits(b);
  const unsigned ea = (unsigned)(ia >> 52) & 0x7ffu, eb = (unsigned)(ib >> 52) & 0x7ffu;
  const u64 ma = (ia & kMant) | kImpl, mb = (ib & kMant) | kImpl;
  const unsigned sh = ma < mb ? 1u : 0u;
  const u64 A = ma << sh;  // A / mb in [1, 2)
  int e = (int)ea - (int)eb + 1023 - (int)sh;
  // Q = floor(A 2^54 / mb) in [2^54, 2^55), corrected by the exact remainder
  u64 Q = (mulhi(A, X) << 2) | ((A * X) >> 62);
  long long R = (long long)((A << 54) - Q * mb);
  const long long B = (long long)mb;
  if (R < 0) {
    Q -= 1; R += B;
    if (R < 0) { Q -= 1; R += B; }
  } else if (R >= B) {
    Q += 1; R -= B;
    if (R >= B) { Q += 1; R -= B; }
  }
  const bool in_range = R >= 0 && R < B;
  const bool underflow = e < 1;
  const u64 m = round_q55(Q, R != 0, e);
  // a zero dividend over a normal divisor gives a signed zero (a limiter
  // ratio's numerator is zero at every local extremum)
  const bool a_zero = (ia << 1) == 0ull;
  if (eb - 1u >= 0x7feu || (!a_zero && (ea - 1u >= 0x7feu || underflow || e > 2046 || !in_range)))
    return div_fp64(a, b);
  return from_bits(a_zero ? ((ia ^ ib) & kSign) : (((ia ^ ib) & kSign) | ((u64)e << 52) | (m & kMant)));
}

MCFD_IA_FN double div_rn(double a, double b) { return div_rn_recip(a, b, recip_fixed(b)); }

// a / b, the same bits as div_rn, in fewer dependent steps, from y =
// RN(1/b) (div_rn_recip(1.0, b, X)) and X = recip_fixed(b), both of which
// depend on b alone.  A candidate from one Markstein correction of the
// product a y (q0 = RN(a y), q = RN(q0 + RN(a - b q0) y); P. Markstein,
// "Computation of elementary functions on the IBM RISC System/6000
// processor", IBM J. Res. Dev. 34(1), 1990) is accepted only when the
// remainder r = a - b q, an FMA that is exact for q within an ulp of a/b
// (and is large otherwise), lies strictly inside (-|b| u / 2, |b| u / 2),
// u the spacing of the doubles next to q on the side of a/b: then q is the
// double nearest a/b, which is never a midpoint of two doubles (a rounding
// test in the manner of Tuckerman's for square roots).  The bounds |b| u / 2
// are powers-of-two multiples of |b|, formed exactly in the exponent field
// and compared as bit patterns.  Zero, subnormal or non-finite operands,
// quotients near either end of the normal range, and a rejected candidate
// take div_rn_recip.  Four dependent FP64 operations and integer tests
// instead of div_rn_recip's chain of 64-bit integer products.
MCFD_IA_FN double fma_rn(double x, double y, double z) {
#if defined(__CUDA_ARCH__)
  return __fma_rn(x, y, z);
#else
  return fma(x, y, z);
#endif
}
MCFD_IA_FN double mul_rn_fp64(double x, double y) {
#if defined(__CUDA_ARCH__)
  return __dmul_rn(x, y);
#else
  return x * y;
#endif
}

MCFD_IA_FN double div_rn_fma(double a, double b, double y, u64 X) {
  const double q0 = mul_rn_fp64(a, y);
  const double q = fma_rn(fma_rn(-b, q0, a), y, q0);
  const double r = fma_rn(-b, q, a);
  const u64 ia = bits(a), ib = bits(b), iq = bits(q), ir = bits(r);
  const unsigned ea = (unsigned)(ia >> 52) & 0x7ffu, eb = (unsigned)(ib >> 52) & 0x7ffu;
  const unsigned eq = (unsigned)(iq >> 52) & 0x7ffu;
  // |b| u / 2 with u = 2^(eq - 1075) away from zero; toward zero the same,
  // or half of it when |q| is a power of two
  const bool away = ((ir ^ ib ^ iq) >> 63) == 0ull;  // sign(r / b) == sign(q)
  const int eh = (int)eb + (int)eq - 1076 - ((!away && (iq & kMant) == 0ull) ? 1 : 0);
  const bool in_range = ea - 1u < 0x7feu && eb - 1u < 0x7feu && eq - 2u < 0x7fcu && eh >= 1 && eh <= 2046;
  const u64 half = ((u64)(eh < 1 ? 1 : (eh > 2046 ? 2046 : eh)) << 52) | (ib & kMant);
  if (in_range && (ir << 1) < (half << 1)) return q;  // |r| < |b| u / 2 (or r = 0)
  return div_rn_recip(a, b, X);
}

// a * b, round to nearest even, in 32-bit words.  With the significands
// split as a = a1 2^32 + a0 (a1 21 bits), the 106-bit product is summed by
// columns with 32 x 32 + 64 -> 64-bit multiply-adds; its top 53 bits (from
// bit 52 + top, top = product >= 2^105) are funnel-shifted out and rounded
// from the guard bit and the sticky OR of the bits below.  A rounding carry
// out of 53 bits leaves exactly 2^53, whose stored significand field is zero,
// so only the exponent moves.  A zero operand times a finite one gives the
// signed zero; other zeros, subnormals, infinities, NaN and products that
// overflow or underflow go to the FP64 unit.
MCFD_IA_FN double mul_rn(double a, double b) {
  const u64 ia = bits(a), ib = bits(b);
  const unsigned ahi = (unsigned)(ia >> 32), bhi = (unsigned)(ib >> 32);
  const unsigned a0 = (unsigned)ia, b0 = (unsigned)ib;
  const unsigned ea = (ahi >> 20) & 0x7ffu, eb = (bhi >> 20) & 0x7ffu;
  const unsigned a1 = (ahi & 0xfffffu) | 0x100000u, b1 = (bhi & 0xfffffu) | 0x100000u;
  // columns: product = w3:w2 2^64 + w1 2^32 + w0
  const u64 p00 = (u64)a0 * b0;
  const u64 t = (u64)a0 * b1 + (p00 >> 32);
  const u64 u = (u64)a1 * b0 + (unsigned)t;
  const unsigned w0 = (unsigned)p00, w1 = (unsigned)u;
  const u64 w23 = (u64)a1 * b1 + (t >> 32) + (u >> 32);  // < 2^42
  const unsigned w2 = (unsigned)w23, w3 = (unsigned)(w23 >> 32);
  const unsigned top = w3 >> 9;  // product >= 2^105
  const unsigned sh = 20u + top;  // the significand starts at bit 52 + top = 32 + sh
  const unsigned m_lo = shr_funnel(w1, w2, sh), m_hi = shr_funnel(w2, w3, sh);
  const unsigned guard = (w1 >> (sh - 1u)) & 1u;
  const unsigned sticky = ((w1 & ((1u << (sh - 1u)) - 1u)) | w0) != 0u ? 1u : 0u;
  const unsigned inc = guard & (sticky | m_lo);
  const unsigned r_lo = m_lo + inc;
  const unsigned r_hi = m_hi + (r_lo < inc ? 1u : 0u);  // 2^20 <= r_hi <= 2^21
  const unsigned carry = r_hi >> 21;
  const int e0 = (int)ea + (int)eb - 1023 + (int)top;
  const int e = e0 + (int)carry;
  const unsigned sign = (ahi ^ bhi) & 0x80000000u;
  const bool zero = ((ahi << 1) | a0) == 0u || ((bhi << 1) | b0) == 0u;
  const bool special = ea - 1u >= 0x7feu || eb - 1u >= 0x7feu;
  if (zero ? (ea == 0x7ffu || eb == 0x7ffu) : (special || e0 < 1 || e > 2046)) return mul_fp64(a, b);
  const unsigned hi_word = zero ? sign : (sign | ((unsigned)e << 20) | (r_hi & 0xfffffu));
  return from_bits(((u64)hi_word << 32) | (zero ? 0u : r_lo));
}

MCFD_IA_FN double sqrt_rn(double x) {
  const u64 ix = bits(x);
  const unsigned ex = (unsigned)(ix >> 52);   // a set sign bit puts ex out of range
  const unsigned odd = (ex & 1u) ^ 1u;        // the unbiased exponent is odd
  const u64 M = ((ix & kMant) | kImpl) << odd;  // [2^52, 2^54), even exponent left
  int e = (((int)ex - 1023 - (int)odd) >> 1) + 1023;
  // seed: y32 ~ 2^43 / sqrt(M >> 30) ~ 2^31 / sqrt(M / 2^54)
  const unsigned y32 = to_u32(rsqrt_seed((float)(unsigned)(M >> 30)) * 0x1p43f);
  // Newton step 1 on Y = y32 2^32: D = 2^80 - (M y32^2 >> 36) (|D| < 2^60),
  // Y += Y D / 2^81
  u64 S2 = (u64)y32 * y32;
  long long D = -(long long)((mulhi(M, S2) << 28) | ((M * S2) >> 36));
  u64 ad = D < 0 ? (u64)(-D) : (u64)D;
  u64 h = (mulhi((u64)y32, ad) << 15) | (((u64)y32 * ad) >> 49);
  u64 Y = (u64)y32 << 32;
  Y = D < 0 ? Y - h : Y + h;
  // Newton step 2: S2 = Y^2 / 2^64, D = 2^80 - (M S2 >> 36), Y += Y D / 2^81
  {
    S2 = mulhi(Y, Y);
    D = -(long long)((mulhi(M, S2) << 28) | ((M * S2) >> 36));
    ad = D < 0 ? (u64)(-D) : (u64)D;
    h = mulhi(Y, ad) >> 17;
    Y = D < 0 ? Y - h : Y + h;
  }
  // S = floor(sqrt(M 2^56)) in [2^54, 2^55), corrected by R = M 2^56 - S^2
  u64 S = (mulhi(M, Y) << 2) | ((M * Y) >> 62);
  long long R = (long long)((M << 56) - S * S);
  if (R < 0) {
    S -= 1; R += (long long)(2 * S + 1);
    if (R < 0) { S -= 1; R += (long long)(2 * S + 1); }
  } else if (R > (long long)(2 * S)) {
    R -= (long long)(2 * S + 1); S += 1;
    if (R > (long long)(2 * S)) { R -= (long long)(2 * S + 1); S += 1; }
  }
  const bool in_range = R >= 0 && R <= (long long)(2 * S);
  const u64 m = round_q55(S, R != 0, e);
  if (ex - 1u >= 0x7feu || !in_range) return sqrt_fp64(x);
  return from_bits(((u64)e << 52) | (m & kMant));
}

// -x (IEEE negation is exact: the sign bit flips, also for zeros and NaN)
MCFD_IA_FN double negate(double x) { return from_bits(sign_xor(bits(x), kSign)); }

// copysign(m, s) for m >= +0: m with the sign of s
MCFD_IA_FN double with_sign_of(double m, double s) { return from_bits(bits(m) | bits_and(bits(s), kSign)); }

// |x| (clears the sign bit, as the IEEE abs operation does)
MCFD_IA_FN double abs_of(double x) { return from_bits(bits_and(bits(x), ~kSign)); }

// 2 x, exact, on integers: the exponent field steps by one for normal x below
// the top binade; zeros and subnormals shift their significand left (which
// carries into the exponent field where 2 x is normal); the top binade
// overflows to infinity; infinities stay, NaN is returned quiet.
MCFD_IA_FN double twice(double x) {
  const u64 b = bits(x), sign = b & kSign, mag = b & ~kSign;
  const unsigned e = (unsigned)(mag >> 52);
  u64 r;
  if (e == 0u) r = sign | (mag << 1);
  else if (e < 2046u) r = b + (1ull << 52);
  else if (e == 2046u) r = sign | 0x7ff0000000000000ull;
  else r = (mag & kMant) ? (b | 0x0008000000000000ull) : b;
  return from_bits(r);
}

// 0.0 + x, exact: x itself except that -0 becomes +0
MCFD_IA_FN double plus_zero(double x) { return bits(x) == kSign ? 0.0 : x; }

}  // namespace ia

using ia::abs_of;
using ia::div_rn;
using ia::div_rn_recip;
using ia::div_rn_fma;
using ia::recip_fixed;
using ia::mul_rn;
using ia::negate;
using ia::plus_zero;
using ia::with_sign_of;
using ia::sqrt_rn;
using ia::twice;

}  // namespace mcfd

#undef MCFD_IA_FN
#undef MCFD_IA_SLOW
