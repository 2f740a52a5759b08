// Shortest round-trip decimal text of an IEEE double, as Python's repr(float)
// and "{}".format(float) print it: the fewest significant digits that read
// back as the same double, the one nearest the value among those, positional
// notation for 1e-4 <= |v| < 1e16 ("0.0001", "123.0", "1234567890123456.0")
// and scientific otherwise ("1e-05", "1.5e+16", "5e-324"); "inf", "-inf",
// "nan", "0.0", "-0.0".  The reference writes every number of its solution
// files this way (BVPDAEReadWriteData.py:337-364).
//
// Digits: the free-format algorithm of Steele & White and of Burger & Dybvig
// ("Printing floating-point numbers quickly and accurately", PLDI 1996),
// restated here on exact fixed-size integers.  v = f 2^e is held as r / s with
// the half-gaps to the neighbouring doubles m+ / s and m- / s; digits are
// generated until the remaining interval contains a shorter decimal.  With
// an even mantissa the interval's ends read back as v (round half to even),
// so they count as inside.
//
// Host and device code: the library formats solution files on the GPU with it
// and exports it for the host as cs_format_double.
#pragma once
#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define CS_HD __host__ __device__ __forceinline__
#else
#define CS_HD static inline
#endif

// longest text: "-1.2345678901234567e-308" (24 characters)
#define CS_DTOA_MAX 24

CS_HD int cs_clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)x);
#else
  return __builtin_clzll(x);
#endif
}

// little-endian unsigned integer of up to CS_BN_LIMBS 32-bit limbs
#define CS_BN_LIMBS 40
struct CsBig {
  uint32_t w[CS_BN_LIMBS];
  int n;  // limbs in use (w[n-1] != 0, or n == 0 for zero)
};

CS_HD void cs_bn_set(CsBig& a, uint64_t v) {
  a.n = 0;
  while (v) {
    a.w[a.n++] = (uint32_t)v;
    v >>= 32;
  }
}

CS_HD void cs_bn_mul_small(CsBig& a, uint32_t m) {
  uint64_t c = 0;
  for (int i = 0; i < a.n; ++i) {
    const uint64_t t = (uint64_t)a.w[i] * m + c;
    a.w[i] = (uint32_t)t;
    c = t >> 32;
  }
  if (c) a.w[a.n++] = (uint32_t)c;
}

// a *= 2^k
CS_HD void cs_bn_shl(CsBig& a, int k) {
  if (a.n == 0 || k <= 0) return;
  const int q = k >> 5, b = k & 31;
  if (b) {
    uint32_t c = 0;
    for (int i = 0; i < a.n; ++i) {
      const uint32_t x = a.w[i];
      a.w[i] = (x << b) | c;
      c = x >> (32 - b);
    }
    if (c) a.w[a.n++] = c;
  }
  if (q) {
    for (int i = a.n - 1; i >= 0; --i) a.w[i + q] = a.w[i];
    for (int i = 0; i < q; ++i) a.w[i] = 0;
    a.n += q;
  }
}

// a *= 10^k (k >= 0)
CS_HD void cs_bn_mul_pow10(CsBig& a, int k) {
  while (k >= 9) {
    cs_bn_mul_small(a, 1000000000u);
    k -= 9;
  }
  uint32_t m = 1;
  while (k-- > 0) m *= 10;
  if (m > 1) cs_bn_mul_small(a, m);
}

CS_HD int cs_bn_cmp(const CsBig& a, const CsBig& b) {
  if (a.n != b.n) return a.n < b.n ? -1 : 1;
  for (int i = a.n - 1; i >= 0; --i)
    if (a.w[i] != b.w[i]) return a.w[i] < b.w[i] ? -1 : 1;
  return 0;
}

// compare a + b with c
CS_HD int cs_bn_cmp_sum(const CsBig& a, const CsBig& b, const CsBig& c) {
  const int n = a.n > b.n ? a.n : b.n;
  if (n + 1 < c.n) return -1;
  if (n > c.n) return 1;  // a + b >= 2^(32(n-1)) > c
  // sum limb by limb, then compare from the top
  uint32_t s[CS_BN_LIMBS + 1];
  uint64_t cy = 0;
  for (int i = 0; i < n; ++i) {
    const uint64_t t = (uint64_t)(i < a.n ? a.w[i] : 0u) + (i < b.n ? b.w[i] : 0u) + cy;
    s[i] = (uint32_t)t;
    cy = t >> 32;
  }
  int sn = n;
  if (cy) s[sn++] = (uint32_t)cy;
  while (sn > 0 && s[sn - 1] == 0) --sn;
  if (sn != c.n) return sn < c.n ? -1 : 1;
  for (int i = sn - 1; i >= 0; --i)
    if (s[i] != c.w[i]) return s[i] < c.w[i] ? -1 : 1;
  return 0;
}

// a -= b (a >= b)
CS_HD void cs_bn_sub(CsBig& a, const CsBig& b) {
  int64_t br = 0;
  for (int i = 0; i < a.n; ++i) {
    int64_t t = (int64_t)a.w[i] - (i < b.n ? (int64_t)b.w[i] : 0) - br;
    br = t < 0;
    a.w[i] = (uint32_t)(t + (br << 32));
  }
  while (a.n > 0 && a.w[a.n - 1] == 0) --a.n;
}

// Significant digits of v > 0 (finite) into dig[], returns their count;
// *k10: v = 0.d1 d2 ... x 10^k10.
CS_HD int cs_shortest_digits(double v, char* dig, int* k10) {
  union {
    double d;
    uint64_t u;
  } bits;
  bits.d = v;
  const int be = (int)((bits.u >> 52) & 0x7ff);
  const uint64_t frac = bits.u & ((1ull << 52) - 1);
  const uint64_t f = be ? (frac | (1ull << 52)) : frac;
  const int e = be ? be - 1075 : -1074;
  const bool even = (f & 1) == 0;
  const bool pow2 = be > 1 && frac == 0;  // the gap below is half the gap above
  CsBig r, s, mp, mm;
  // v = r / s, upper half-gap mp / s, lower half-gap mm / s
  if (e >= 0) {
    cs_bn_set(r, f);
    cs_bn_shl(r, e + (pow2 ? 2 : 1));
    cs_bn_set(s, pow2 ? 4 : 2);
    cs_bn_set(mp, 1);
    cs_bn_shl(mp, e + (pow2 ? 1 : 0));
    cs_bn_set(mm, 1);
    cs_bn_shl(mm, e);
  } else {
    cs_bn_set(r, f);
    cs_bn_shl(r, pow2 ? 2 : 1);
    cs_bn_set(s, 1);
    cs_bn_shl(s, -e + (pow2 ? 2 : 1));
    cs_bn_set(mp, pow2 ? 2 : 1);
    cs_bn_set(mm, 1);
  }
  // Scale by 10^-k so that the digits start right after the point: k is the
  // smallest integer with (r + mp) / s < 10^k (<= with an odd mantissa, whose
  // upper end does not read back).  Start from floor(log10 v) + 1, which is
  // off by one at most, and step.
  const int top = 63 - cs_clz64(f);  // v in [2^(top+e), 2^(top+e+1))
  int kexp = (int)floor((double)(top + e) * 0.30102999566398119521) + 1;
  if (kexp >= 0) {
    cs_bn_mul_pow10(s, kexp);
  } else {
    cs_bn_mul_pow10(r, -kexp);
    cs_bn_mul_pow10(mp, -kexp);
    cs_bn_mul_pow10(mm, -kexp);
  }
  for (;;) {  // too small a scale: 10^k itself (or more) is in the interval
    const int c = cs_bn_cmp_sum(r, mp, s);
    if (!(even ? c >= 0 : c > 0)) break;
    cs_bn_mul_small(s, 10);
    ++kexp;
  }
  for (;;) {  // too large a scale: k - 1 would also do
    CsBig t = r, u = mp;
    cs_bn_mul_small(t, 10);
    cs_bn_mul_small(u, 10);
    const int c = cs_bn_cmp_sum(t, u, s);
    if (!(even ? c < 0 : c <= 0)) break;
    r = t;
    mp = u;
    cs_bn_mul_small(mm, 10);
    --kexp;
  }
  *k10 = kexp;
  int n = 0;
  for (;;) {
    cs_bn_mul_small(r, 10);
    cs_bn_mul_small(mp, 10);
    cs_bn_mul_small(mm, 10);
    int d = 0;
    while (cs_bn_cmp(r, s) >= 0) {
      cs_bn_sub(r, s);
      ++d;
    }
    const int cl = cs_bn_cmp(r, mm);
    const bool low = even ? cl <= 0 : cl < 0;
    const int ch = cs_bn_cmp_sum(r, mp, s);
    const bool high = even ? ch >= 0 : ch > 0;
    if (!low && !high) {
      dig[n++] = (char)('0' + d);
      if (n >= 20) break;  // cannot happen for a double; bounds the loop
      continue;
    }
    if (low && high) {
      // both neighbours read back: the nearer one; on a tie the even digit
      const int c2 = cs_bn_cmp_sum(r, r, s);
      if (c2 > 0 || (c2 == 0 && (d & 1))) ++d;
    } else if (high) {
      ++d;
    }
    dig[n++] = (char)('0' + d);
    break;
  }
  return n;
}

// Text of v into out (at most CS_DTOA_MAX characters, no terminator);
// returns the length.
CS_HD int cs_format_double_text(double v, char* out) {
  union {
    double d;
    uint64_t u;
  } bits;
  bits.d = v;
  const bool neg = (bits.u >> 63) != 0;
  const int be = (int)((bits.u >> 52) & 0x7ff);
  const uint64_t frac = bits.u & ((1ull << 52) - 1);
  int p = 0;
  if (be == 0x7ff) {
    if (frac) {
      out[0] = 'n'; out[1] = 'a'; out[2] = 'n';
      return 3;
    }
    if (neg) out[p++] = '-';
    out[p++] = 'i'; out[p++] = 'n'; out[p++] = 'f';
    return p;
  }
  if (neg) out[p++] = '-';
  if (be == 0 && frac == 0) {
    out[p++] = '0'; out[p++] = '.'; out[p++] = '0';
    return p;
  }
  char dig[24];
  int k = 0;
  const int n = cs_shortest_digits(neg ? -v : v, dig, &k);
  if (k > -4 && k <= 16) {
    // positional: k digits before the point (zeros if k <= 0)
    if (k <= 0) {
      out[p++] = '0';
      out[p++] = '.';
      for (int i = 0; i < -k; ++i) out[p++] = '0';
      for (int i = 0; i < n; ++i) out[p++] = dig[i];
    } else {
      for (int i = 0; i < k; ++i) out[p++] = i < n ? dig[i] : '0';
      out[p++] = '.';
      if (n > k)
        for (int i = k; i < n; ++i) out[p++] = dig[i];
      else
        out[p++] = '0';
    }
    return p;
  }
  out[p++] = dig[0];
  if (n > 1) {
    out[p++] = '.';
    for (int i = 1; i < n; ++i) out[p++] = dig[i];
  }
  out[p++] = 'e';
  int x = k - 1;
  if (x < 0) {
    out[p++] = '-';
    x = -x;
  } else {
    out[p++] = '+';
  }
  if (x >= 100) {
    out[p++] = (char)('0' + x / 100);
    x %= 100;
    out[p++] = (char)('0' + x / 10);
    out[p++] = (char)('0' + x % 10);
  } else {
    out[p++] = (char)('0' + x / 10);
    out[p++] = (char)('0' + x % 10);
  }
  return p;
}
