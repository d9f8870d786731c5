// Decimal text to FP64, correctly rounded (round to nearest, ties to even), as a Fortran
// list-directed read of a real (and C's strtod) gives it; the same code runs on the host
// and on the GPU.
//
// A number is [+|-]digits[.digits][(e|E|d|D)[+|-]digits].  Its first 38 significant digits
// form an integer W (< 2^127) with a decimal exponent q: the value is W 10^q (digits beyond
// the 38th set a sticky flag).  When W <= 2^53 and |q| <= 22 both W and 10^|q| are exact
// FP64 numbers and one IEEE multiplication or division is the correctly rounded result
// (Clinger's fast path).  Otherwise the result is exact by construction:
//   * an FP64 estimate of W 10^q (within a few ulp) gives a candidate m 2^e (m of 53 bits);
//   * the candidate is moved until w 10^q lies between its lower and upper midpoints,
//     decided by exact comparisons of 256-bit integers (W 10^q against a midpoint num 2^sh,
//     with 10^-q and 2^-sh moved to the side where they are integers); a value exactly on a
//     midpoint goes to the even mantissa;
//   * with a sticky flag the true value lies strictly between W 10^q and (W + 1) 10^q: the
//     result is the rounding of both when they agree.
// The exact comparisons need the shifted operands within 256 bits, which holds for normal
// results from about 1e-20 to 1e38 (far more than atom coordinates need); outside that
// range, and for malformed text, the parser reports failure instead of guessing.
#pragma once

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define PN_HD __host__ __device__ __forceinline__
#else
#define PN_HD inline
#endif

namespace stem {
namespace pn {

struct U256 {
  uint64_t w[4];  // little-endian limbs
};

PN_HD void mul64(uint64_t a, uint64_t b, uint64_t& hi, uint64_t& lo) {
#ifdef __CUDA_ARCH__
  lo = a * b;
  hi = __umul64hi(a, b);
#else
  const unsigned __int128 p = (unsigned __int128)a * b;
  lo = (uint64_t)p;
  hi = (uint64_t)(p >> 64);
#endif
}

PN_HD U256 u256(uint64_t v) {
  U256 r;
  r.w[0] = v;
  r.w[1] = r.w[2] = r.w[3] = 0;
  return r;
}

// r = a * m (m < 2^64); false on overflow beyond 256 bits
PN_HD bool mul_small(U256& a, uint64_t m) {
  uint64_t carry = 0;
  for (int i = 0; i < 4; ++i) {
    uint64_t hi, lo;
    mul64(a.w[i], m, hi, lo);
    const uint64_t s = lo + carry;
    carry = hi + (s < lo ? 1 : 0);
    a.w[i] = s;
  }
  return carry == 0;
}

// a <<= s; false on overflow
PN_HD bool shl(U256& a, int s) {
  if (s <= 0) return true;
  if (s >= 256) {
    const bool zero = !(a.w[0] | a.w[1] | a.w[2] | a.w[3]);
    a = u256(0);
    return zero;
  }
  const int limbs = s >> 6, bits = s & 63;
  for (int i = 3; i >= 4 - limbs; --i)
    if (a.w[i]) return false;
  if (bits && (a.w[3 - limbs] >> (64 - bits))) return false;
  U256 r = u256(0);
  for (int i = 3; i >= limbs; --i) {
    uint64_t v = a.w[i - limbs] << bits;
    if (bits && i - limbs - 1 >= 0) v |= a.w[i - limbs - 1] >> (64 - bits);
    r.w[i] = v;
  }
  a = r;
  return true;
}

PN_HD int cmp(const U256& a, const U256& b) {
  for (int i = 3; i >= 0; --i) {
    if (a.w[i] < b.w[i]) return -1;
    if (a.w[i] > b.w[i]) return 1;
  }
  return 0;
}

// a *= 10^k; false on overflow
PN_HD bool mul_pow10(U256& a, int k) {
  while (k > 0) {
    const int s = k > 19 ? 19 : k;
    uint64_t p = 1;
    for (int i = 0; i < s; ++i) p *= 10;
    if (!mul_small(a, p)) return false;
    k -= s;
  }
  return true;
}

PN_HD double pow10_exact(int k) {  // 10^k for 0 <= k <= 22: exact in FP64
  double r = 1.0;
  for (int i = 0; i < k; ++i) r *= 10.0;  // every partial product is exact
  return r;
}

PN_HD double pow10_est(int k) {  // 10^k in FP64 (exact up to 10^22), for the estimate only
  double r = 1.0, b = 10.0;
  int e = k < 0 ? -k : k;
  while (e) {
    if (e & 1) r *= b;
    b *= b;
    e >>= 1;
  }
  return k < 0 ? 1.0 / r : r;
}

// Sign of W 10^q - num 2^sh; 2 when the comparison does not fit in 256 bits.
PN_HD int cmp_value(const U256& W, int q, uint64_t num, int sh) {
  U256 L = W, R = u256(num);
  // move 10^-q (q < 0) to R and 2^-sh (sh < 0) to L, so both sides are integers
  if (q >= 0) {
    if (!mul_pow10(L, q)) return 2;
  } else {
    if (!mul_pow10(R, -q)) return 2;
  }
  if (sh >= 0) {
    if (!shl(R, sh)) return 2;
  } else {
    if (!shl(L, -sh)) return 2;
  }
  return cmp(L, R);
}

// The midpoints around the candidate m 2^e (2^52 <= m < 2^53): upper (2m + 1) 2^(e-1);
// lower (2m - 1) 2^(e-1), or (4m - 1) 2^(e-2) at the bottom of the binade, where the
// predecessor is (2^53 - 1) 2^(e-1).
PN_HD int cmp_upper(const U256& W, int q, uint64_t m, int e) { return cmp_value(W, q, 2 * m + 1, e - 1); }
PN_HD int cmp_lower(const U256& W, int q, uint64_t m, int e) {
  return m == (1ULL << 52) ? cmp_value(W, q, 4 * m - 1, e - 2) : cmp_value(W, q, 2 * m - 1, e - 1);
}

PN_HD double make_double(uint64_t m, int e) {  // m 2^e, m < 2^53, a normal number
  // exact scaling by powers of two
  double r = (double)m;
  while (e > 0) {
    const int s = e > 60 ? 60 : e;
    r *= (double)(1ULL << s);
    e -= s;
  }
  while (e < 0) {
    const int s = -e > 60 ? 60 : -e;
    r /= (double)(1ULL << s);
    e += s;
  }
  return r;
}

// Correctly rounded W 10^q (W > 0, an integer of up to 38 digits; est its FP64 value);
// false outside the exact range.
PN_HD bool round_exact(const U256& W, double est, int q, double& out) {
  if (q > 38 || q < -76) return false;
  // estimate, then the candidate m 2^e with 2^52 <= m < 2^53 (normal numbers)
  est = q >= 0 ? est * pow10_est(q) : est / pow10_est(-q);
  if (!(est > 0.0) || est > 1.0e300) return false;
  uint64_t bits;
  memcpy(&bits, &est, 8);
  const int be = (int)((bits >> 52) & 0x7FF);
  if (be == 0) return false;  // subnormal estimate: outside the range handled here
  int e = be - 1075;          // est = m 2^e
  uint64_t m = (bits & ((1ULL << 52) - 1)) | (1ULL << 52);
  // move m (keeping 2^52 <= m < 2^53) until the value lies within its half-ulp interval
  for (int it = 0;; ++it) {
    if (it == 8) return false;
    const int up = cmp_upper(W, q, m, e);  // value vs upper midpoint
    const int dn = cmp_lower(W, q, m, e);  // value vs lower midpoint
    if (up == 2 || dn == 2) return false;
    if (up < 0 && dn > 0) break;  // strictly inside
    if (up == 0) {                // exactly half-way: to the even mantissa
      if (m & 1) {
        ++m;
        if (m == (1ULL << 53)) { m >>= 1; ++e; }
      }
      break;
    }
    if (dn == 0) {
      if (m & 1) {
        if (m == (1ULL << 52)) { m = (1ULL << 53) - 1; --e; }
        else --m;
      }
      break;
    }
    if (up > 0) {
      ++m;
      if (m == (1ULL << 53)) { m >>= 1; ++e; }
    } else {
      if (m == (1ULL << 52)) { m = (1ULL << 53) - 1; --e; }
      else --m;
    }
  }
  if (e + 52 > 1023 || e + 52 < -1022) return false;  // overflow or subnormal: not handled
  out = make_double(m, e);
  return true;
}

// Parse one number from [p, end); used = characters consumed.  Returns false on malformed
// text or outside the exact range.
PN_HD bool parse_real(const char* p, const char* end, double& out, int& used) {
  const char* s = p;
  bool neg = false;
  if (s < end && (*s == '+' || *s == '-')) {
    neg = *s == '-';
    ++s;
  }
  // significant digits: the first 19 in w1, the next up to 19 in w2 (n2 of them)
  uint64_t w1 = 0, w2 = 0;
  int nd = 0, n2 = 0, q = 0, digits = 0;
  bool sticky = false, dot = false;
  for (; s < end; ++s) {
    const char c = *s;
    if (c >= '0' && c <= '9') {
      ++digits;
      if (nd == 0 && c == '0') {
        if (dot) --q;  // leading zeros after the point
        continue;
      }
      if (nd < 38) {
        if (nd < 19) w1 = w1 * 10 + (uint64_t)(c - '0');
        else {
          w2 = w2 * 10 + (uint64_t)(c - '0');
          ++n2;
        }
        ++nd;
        if (dot) --q;
      } else {
        if (c != '0') sticky = true;
        if (!dot) ++q;
      }
    } else if (c == '.' && !dot) {
      dot = true;
    } else {
      break;
    }
  }
  if (digits == 0) return false;
  if (s < end && (*s == 'e' || *s == 'E' || *s == 'd' || *s == 'D')) {
    ++s;
    bool eneg = false;
    if (s < end && (*s == '+' || *s == '-')) {
      eneg = *s == '-';
      ++s;
    }
    int ev = 0, ed = 0;
    for (; s < end && *s >= '0' && *s <= '9'; ++s) {
      if (ev < 100000) ev = ev * 10 + (*s - '0');
      ++ed;
    }
    if (ed == 0) return false;
    q += eneg ? -ev : ev;
  }
  used = (int)(s - p);
  if (w1 == 0) {
    out = neg ? -0.0 : 0.0;
    return true;
  }
  // Clinger's fast path: an integer significand below 2^53 and a power of ten below 10^23
  // are both exact in FP64, so one IEEE multiplication or division rounds correctly
  if (n2 == 0 && !sticky && w1 <= (1ULL << 53) && q >= -22 && q <= 22) {
    const double wd = (double)w1, p10 = pow10_exact(q < 0 ? -q : q);
    const double r = q < 0 ? wd / p10 : wd * p10;
    out = neg ? -r : r;
    return true;
  }
  // W = w1 10^n2 + w2, and its FP64 estimate
  U256 W = u256(w1);
  if (!mul_pow10(W, n2)) return false;
  {
    uint64_t c = 0;
    uint64_t s0 = W.w[0] + w2;
    c = s0 < W.w[0] ? 1 : 0;
    W.w[0] = s0;
    for (int i = 1; i < 4 && c; ++i) {
      W.w[i] += 1;
      c = W.w[i] == 0 ? 1 : 0;
    }
  }
  const double est = (double)w1 * pow10_est(n2) + (double)w2;
  double r;
  if (!round_exact(W, est, q, r)) return false;
  if (sticky) {  // the value lies strictly between W 10^q and (W + 1) 10^q
    U256 W1 = W;
    uint64_t c = 1;
    for (int i = 0; i < 4 && c; ++i) {
      W1.w[i] += 1;
      c = W1.w[i] == 0 ? 1 : 0;
    }
    double r2;
    if (!round_exact(W1, est, q, r2) || r2 != r) return false;
  }
  out = neg ? -r : r;
  return true;
}

PN_HD bool is_blank(char c) { return c == ' ' || c == '\t' || c == '\r' || c == ','; }

// Parse a (possibly signed) integer token; false if it has no digits.
PN_HD bool parse_int(const char* p, const char* end, long long& out, int& used) {
  const char* s = p;
  bool neg = false;
  if (s < end && (*s == '+' || *s == '-')) {
    neg = *s == '-';
    ++s;
  }
  long long v = 0;
  int nd = 0;
  for (; s < end && *s >= '0' && *s <= '9'; ++s, ++nd)
    if (v < 1000000000000000000LL) v = v * 10 + (*s - '0');
  if (nd == 0) return false;
  used = (int)(s - p);
  out = neg ? -v : v;
  return true;
}

}  // namespace pn
}  // namespace stem
