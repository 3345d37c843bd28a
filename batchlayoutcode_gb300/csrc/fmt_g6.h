// fmt_g6.h -- the %g conversion of printf (6 significant digits, no flags)
// for one double, byte for byte, without printf: the reference's output
// files write every coordinate with the default stream formatting, which is
// %g (sample/algorithms.cpp:1244-1256), and the writer formats a million of
// them.
//
// A finite |v| in [2^-30, 2^60) is m 2^e with an integer m < 2^53; the
// 6-digit decimal significand of v is v 10^(5 - X) = m 5^s 2^(e + s)
// (s = 5 - X, X the decimal exponent) rounded to an integer, computed as an
// exact ratio of 128-bit integers and rounded half to even, as glibc rounds
// the exact binary value in the default rounding mode.  X comes from log10
// and is corrected by one when the exact significand falls outside
// [10^5, 10^6).  Other values (zero excepted) go to snprintf.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>

namespace bl {

// Writes the %g form of v at out (at least 32 bytes); returns its length.
inline int fmt_g6(double v, char *out) {
  if (v == 0.0) {  // +0 and -0
    if (std::signbit(v)) {
      out[0] = '-';
      out[1] = '0';
      return 2;
    }
    out[0] = '0';
    return 1;
  }
  const double a = std::fabs(v);
  if (!(a >= 0x1p-30 && a < 0x1p60)) return std::snprintf(out, 32, "%g", v);  // also inf, nan
  uint64_t bits;
  std::memcpy(&bits, &a, 8);                                   // a is normal here
  const uint64_t m = (bits & ((1ull << 52) - 1)) | (1ull << 52);  // 53 significant bits
  const int e = (int)(bits >> 52) - 1075;                      // a = m 2^e
  static const uint64_t p5[] = {1ull, 5ull, 25ull, 125ull, 625ull, 3125ull, 15625ull, 78125ull, 390625ull,
                                1953125ull, 9765625ull, 48828125ull, 244140625ull, 1220703125ull,
                                6103515625ull, 30517578125ull, 152587890625ull, 762939453125ull,
                                3814697265625ull, 19073486328125ull, 95367431640625ull};
  int X = (int)std::floor(std::log10(a));
  uint32_t D = 0;
  // Fast path: t = a 10^(5 - X) in one correctly rounded operation (10^k is
  // exact in a double for k <= 22), so |t - exact| <= 2^-53 2^20 < 1.2e-10.
  // The rounded significand is then certain unless t lies within 1e-9 of a
  // half or of the ends of [10^5, 10^6); those take the exact path below.
  {
    static const double p10[] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                                 1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};
    const int s = 5 - X;
    if (s >= -22 && s <= 22) {
      const double t = s >= 0 ? a * p10[s] : a / p10[-s];
      if (t > 100000.0 + 1e-9 && t < 1000000.0 - 1e-9) {
        const double fl = std::floor(t);
        const double fr2 = t - fl;  // exact: t and fl are within a factor 2 of each other
        if (fr2 < 0.5 - 1e-9) D = (uint32_t)fl;
        else if (fr2 > 0.5 + 1e-9) D = (uint32_t)fl + 1u;
      }
    }
  }
  unsigned __int128 q = 0, r = 0, den = 1;
  for (int tries = 0; tries < 3 && D == 0; tries++) {  // bounded: the estimate is off by at most one
    const int s = 5 - X;                     // s in [-13, 15] for this range of a
    unsigned __int128 num = m;
    den = 1;
    if (s >= 0) num *= p5[s];
    else den *= p5[-s];
    const int sh = e + s;
    if (sh >= 0) num <<= sh;
    else den <<= -sh;
    q = num / den;
    r = num % den;
    if (q >= 1000000u) {
      X++;
    } else if (q < 100000u) {
      X--;
    } else {
      break;
    }
  }
  if (D == 0) {
    if (q < 100000u || q >= 1000000u) return std::snprintf(out, 32, "%g", v);  // not reached
    D = (uint32_t)q;
    const unsigned __int128 twice = r * 2;
    if (twice > den || (twice == den && (D & 1u))) D++;  // half to even on the exact value
  }
  if (D == 1000000u) {
    D = 100000u;
    X++;
  }
  char dig[6];
  for (int k = 5; k >= 0; k--) {
    dig[k] = (char)('0' + D % 10u);
    D /= 10u;
  }
  int nd = 6;  // significant digits left after dropping trailing zeros
  while (nd > 1 && dig[nd - 1] == '0') nd--;
  int len = 0;
  if (v < 0) out[len++] = '-';
  if (X < -4 || X >= 6) {  // d.ddddde+XX
    out[len++] = dig[0];
    if (nd > 1) {
      out[len++] = '.';
      for (int k = 1; k < nd; k++) out[len++] = dig[k];
    }
    out[len++] = 'e';
    int ex = X;
    out[len++] = ex < 0 ? '-' : '+';
    if (ex < 0) ex = -ex;
    if (ex >= 100) out[len++] = (char)('0' + ex / 100);
    out[len++] = (char)('0' + (ex / 10) % 10);
    out[len++] = (char)('0' + ex % 10);
  } else if (X >= 0) {  // X + 1 integer digits, then the rest
    for (int k = 0; k <= X; k++) out[len++] = dig[k];
    if (nd > X + 1) {
      out[len++] = '.';
      for (int k = X + 1; k < nd; k++) out[len++] = dig[k];
    }
  } else {  // 0.000ddd
    out[len++] = '0';
    out[len++] = '.';
    for (int k = 0; k < -X - 1; k++) out[len++] = '0';
    for (int k = 0; k < nd; k++) out[len++] = dig[k];
  }
  return len;
}

// Decimal digits of a positive integer at out; returns the length.
inline int fmt_u64(uint64_t x, char *out) {
  char t[24];
  int n = 0;
  do {
    t[n++] = (char)('0' + x % 10u);
    x /= 10u;
  } while (x);
  for (int k = 0; k < n; k++) out[k] = t[n - 1 - k];
  return n;
}

}  // namespace bl
