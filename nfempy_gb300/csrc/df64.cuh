// Double-float arithmetic for the FP64 assembly: a value is the unevaluated
// sum hi + lo of two FP32 numbers, |lo| <= ulp(hi) / 2 after normalisation,
// which carries about 48 significant bits.  GB300 issues FP64 operations at
// a small fraction of its FP32 rate; these routines keep the FP64 path's
// arithmetic on the FP32 pipes and FP64 only where a value enters or leaves.
//
// Building blocks (published methods):
//   two_sum        Knuth, TAOCP vol. 2, 4.2.2: s + e == a + b exactly;
//   quick_two_sum  Dekker (1971): the same for |a| >= |b|;
//   exact products with a fused multiply-add: p = a * b, e = fma(a, b, -p)
//                  gives p + e == a * b exactly;
//   reciprocal     one Newton step r' = r + r (1 - x r) from the FP32
//                  reciprocal, evaluated in double-float.
// Conversions FP64 <-> double-float are done on the bit patterns with
// integer operations (no FP64 instruction):
//   df_from_double  hi = x with its significand cut to 24 bits, lo = the rest
//                   (the remaining 29 bits rounded to 24): |hi + lo - x| <=
//                   2^-48 |x|;
//   df_to_double    the FP64 bit pattern of hi, plus lo counted in units of
//                   the FP64 ulp of hi, rounded: the nearest FP64 value to
//                   hi + lo up to half an ulp.
// Exact integer products for lattice cells: a 32-bit integer times a 64-bit
// fixed-point factor through the high 64 bits of their 96-bit product,
// packed into FP64 bits (df_i32_times_q63).
// The header compiles for the device and for the host (tests check it there
// against long double).
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define DF_HD __host__ __device__ __forceinline__
#else
#define DF_HD inline
#endif

#if !defined(__CUDA_ARCH__)
#include <cmath>
#include <cstring>
#endif

namespace nfem {

struct dfloat {
  float hi, lo;
};

DF_HD uint32_t df_bits(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t u;
  std::memcpy(&u, &x, 4);
  return u;
#endif
}
DF_HD float df_float(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float x;
  std::memcpy(&x, &u, 4);
  return x;
#endif
}
DF_HD uint64_t df_bits64(double x) {
#if defined(__CUDA_ARCH__)
  return static_cast<uint64_t>(__double_as_longlong(x));
#else
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return u;
#endif
}
DF_HD double df_double(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(static_cast<long long>(u));
#else
  double x;
  std::memcpy(&x, &u, 8);
  return x;
#endif
}
// Rounded FP32 operations that the compiler may not fuse or reorder.
DF_HD float df_add_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fadd_rn(a, b);
#else
  volatile float s = a + b;
  return s;
#endif
}
DF_HD float df_sub_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fsub_rn(a, b);
#else
  volatile float s = a - b;
  return s;
#endif
}
DF_HD float df_mul_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  volatile float s = a * b;
  return s;
#endif
}
DF_HD float df_fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return std::fmaf(a, b, c);
#endif
}
DF_HD float df_u32_to_float(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint2float_rn(u);
#else
  return static_cast<float>(u);  // round to nearest (default mode)
#endif
}
DF_HD int32_t df_float_to_i32(float x) {
#if defined(__CUDA_ARCH__)
  return __float2int_rn(x);
#else
  return static_cast<int32_t>(std::nearbyint(x));
#endif
}

DF_HD dfloat two_sum(float a, float b) {
  const float s = df_add_rn(a, b);
  const float bb = df_sub_rn(s, a);
  const float e = df_add_rn(df_sub_rn(a, df_sub_rn(s, bb)), df_sub_rn(b, bb));
  return {s, e};
}
DF_HD dfloat quick_two_sum(float a, float b) {
  const float s = df_add_rn(a, b);
  return {s, df_sub_rn(b, df_sub_rn(s, a))};
}
DF_HD dfloat df_make(float x) { return {x, 0.f}; }
DF_HD dfloat df_neg(dfloat x) { return {-x.hi, -x.lo}; }
DF_HD dfloat df_abs(dfloat x) { return x.hi < 0.f ? df_neg(x) : x; }

// x + y; error below 2^-47 (|x| + |y|)
DF_HD dfloat df_add(dfloat x, dfloat y) {
  dfloat s = two_sum(x.hi, y.hi);
  return quick_two_sum(s.hi, df_add_rn(s.lo, df_add_rn(x.lo, y.lo)));
}
DF_HD dfloat df_sub(dfloat x, dfloat y) { return df_add(x, df_neg(y)); }
// x * y; relative error below 2^-46
DF_HD dfloat df_mul(dfloat x, dfloat y) {
  const float p = df_mul_rn(x.hi, y.hi);
  float e = df_fma(x.hi, y.hi, -p);
  e = df_fma(x.hi, y.lo, e);
  e = df_fma(x.lo, y.hi, e);
  return quick_two_sum(p, e);
}
// x * f for an FP32 f (exact for the small integers used as weights)
DF_HD dfloat df_mul_f(dfloat x, float f) {
  const float p = df_mul_rn(x.hi, f);
  float e = df_fma(x.hi, f, -p);
  e = df_fma(x.lo, f, e);
  return quick_two_sum(p, e);
}
// sum_k sgn_k a_k b_k over N terms (sgn_k = +-1): exact products of the high
// parts, their rounding errors and the cross terms collected in FP32
template <int N>
DF_HD dfloat df_dot(const dfloat (&a)[N], const dfloat (&b)[N], const float (&sgn)[N]) {
  float p[N], e[N];
#pragma unroll
  for (int k = 0; k < N; ++k) {
    const float ah = a[k].hi * sgn[k], al = a[k].lo * sgn[k];  // sign flips are exact
    p[k] = df_mul_rn(ah, b[k].hi);
    e[k] = df_fma(ah, b[k].hi, -p[k]);
    e[k] = df_fma(ah, b[k].lo, e[k]);
    e[k] = df_fma(al, b[k].hi, e[k]);
  }
  dfloat s = {p[0], e[0]};
#pragma unroll
  for (int k = 1; k < N; ++k) {
    const dfloat t = two_sum(s.hi, p[k]);
    s.hi = t.hi;
    s.lo = df_add_rn(s.lo, df_add_rn(t.lo, e[k]));
  }
  return quick_two_sum(s.hi, s.lo);
}
// 1 / x; relative error below 2^-45
DF_HD dfloat df_recip(dfloat x) {
  const float r = 1.0f / x.hi;
  const dfloat xr = df_mul_f(x, r);            // ~ 1
  const dfloat e = df_sub(df_make(1.0f), xr);  // 1 - x r
  return df_add(df_make(r), df_mul_f(e, r));   // r + r (1 - x r)
}

// FP64 -> double-float by bits.  Magnitudes outside the FP32 normal range
// (below 2^-126 or from 2^128) become 0 and +-inf; the callers' values
// (coordinates, edge vectors, coefficients) lie well inside it.
DF_HD dfloat df_from_double(double x) {
  const uint64_t b = df_bits64(x);
  const uint32_t sgn = static_cast<uint32_t>(b >> 32) & 0x80000000u;
  const int32_t e = static_cast<int32_t>((b >> 52) & 0x7ff);
  const uint64_t m = b & 0xFFFFFFFFFFFFFull;
  const int32_t fe = e - 896;  // FP32 biased exponent of the same binade
  if (fe < 1) return {0.f, 0.f};
  if (fe > 254) return {df_float(sgn | 0x7f800000u), 0.f};
  const float hi = df_float(sgn | (static_cast<uint32_t>(fe) << 23) | static_cast<uint32_t>(m >> 29));
  const uint32_t rem = static_cast<uint32_t>(m & 0x1FFFFFFFull);  // rem * 2^(e - 1075)
  float lo = 0.f;
  if (rem) {
    const uint32_t rb = df_bits(df_u32_to_float(rem));
    const int32_t le = static_cast<int32_t>(rb >> 23) + (e - 1075);
    if (le > 0) lo = df_float(sgn | (static_cast<uint32_t>(le) << 23) | (rb & 0x7fffffu));
  }
  return {hi, lo};
}

DF_HD int df_clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return __clzll(static_cast<long long>(x));
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

// The integer d times 2^-shift as a double-float, by integer operations:
// hi = the leading 24 bits of |d|, lo = the next 24 (both truncated, so
// |hi + lo - d 2^-shift| < 2^-47 |d 2^-shift|).  Results below the FP32
// normal range become 0.
DF_HD dfloat df_from_i64(int64_t d, int shift) {
  if (d == 0) return {0.f, 0.f};
  const uint32_t sgn = d < 0 ? 0x80000000u : 0u;
  const uint64_t a = d < 0 ? static_cast<uint64_t>(-(d + 1)) + 1u : static_cast<uint64_t>(d);
  const int lz = df_clz64(a);
  const uint64_t n = a << lz;            // leading bit at position 63
  const int e = 63 - lz - shift + 127;   // FP32 biased exponent of the leading bit
  if (e < 1) return {0.f, 0.f};
  const float hi = df_float(sgn | (static_cast<uint32_t>(e) << 23) | static_cast<uint32_t>((n >> 40) & 0x7fffffu));
  const uint64_t rem = n << 24;          // the 40 bits after the leading 24
  float lo = 0.f;
  if (rem) {
    const int lz2 = df_clz64(rem);
    const uint64_t n2 = rem << lz2;
    const int e2 = e - 24 - lz2;
    if (e2 >= 1) lo = df_float(sgn | (static_cast<uint32_t>(e2) << 23) | static_cast<uint32_t>((n2 >> 40) & 0x7fffffu));
  }
  return {hi, lo};
}

// Bit tests on an FP64 value (no FP64 instruction): finite; finite and > 0
// with a magnitude inside the FP32 normal range of the double-float code.
DF_HD bool df_bits_finite(double x) { return ((df_bits64(x) >> 52) & 0x7ff) != 0x7ff; }
DF_HD bool df_bits_positive(double x) {
  const uint64_t b = df_bits64(x);
  const int e = static_cast<int>((b >> 52) & 0x7ff);
  return (b >> 63) == 0 && e > 896 && e < 1151;
}

// Normalised double-float (|lo| <= ulp(hi) / 2) -> FP64 by bits.
DF_HD double df_to_double(dfloat x) {
  const uint32_t hb = df_bits(x.hi);
  const int32_t he = static_cast<int32_t>((hb >> 23) & 0xff);
  if (he == 0) return 0.0;     // |hi| < 2^-126: treated as zero
  if (he == 255)  // inf / nan pass through (by bits: no conversion instruction)
    return df_double((static_cast<uint64_t>(hb & 0x80000000u) << 32) | 0x7FF0000000000000ull |
                     (static_cast<uint64_t>(hb & 0x7fffffu) << 29));
  uint64_t db = (static_cast<uint64_t>(hb & 0x80000000u) << 32) | (static_cast<uint64_t>(he + 896) << 52) |
                (static_cast<uint64_t>(hb & 0x7fffffu) << 29);
  const uint32_t lb = df_bits(x.lo);
  const int32_t le = static_cast<int32_t>((lb >> 23) & 0xff);
  if (le == 0) return df_double(db);
  // lo in units of the FP64 ulp of hi, 2^(he - 127 - 52); one binade lower
  // (half that unit) when hi is a power of two and lo points below it.  A
  // normalised lo is below 2^28 such units, less than the distance from the
  // largest FP32 significand to the next binade, so no carry crosses upward.
  const bool opposite = ((hb ^ lb) & 0x80000000u) != 0;
  const bool down = opposite && (hb & 0x7fffffu) == 0;
  const int32_t ne = le + 179 - he + (down ? 1 : 0);
  if (ne <= 0) return df_double(db);  // below half an FP64 ulp
  const int32_t k = df_float_to_i32(df_float((lb & 0x807fffffu) | (static_cast<uint32_t>(ne) << 23)));
  const int32_t ak = k < 0 ? -k : k;
  const int64_t step = opposite ? -static_cast<int64_t>(ak) : static_cast<int64_t>(ak);
  const uint64_t mag = (db & 0x7FFFFFFFFFFFFFFFull) + static_cast<uint64_t>(step);
  return df_double((db & 0x8000000000000000ull) | mag);
}

// floor(v 2^q) of a positive normalised double-float as a 64-bit integer,
// by integer operations; needs 2^24 <= hi 2^q < 2^64 (lo's bits below
// 2^-q are cut, and lo < 0 is subtracted).  Larger values (and inf)
// saturate, smaller ones give 0.
DF_HD uint64_t df_to_u64_scaled(dfloat v, int q) {
  const uint32_t hb = df_bits(v.hi);
  const int eh = static_cast<int>((hb >> 23) & 0xff);
  const uint64_t mh = (hb & 0x7fffffu) | 0x800000u;  // hi = mh 2^(eh - 150)
  const int sh = eh - 150 + q;
  if (sh > 40) return ~0ull;
  if (sh < 0) return 0ull;
  uint64_t r = mh << sh;
  const uint32_t lb = df_bits(v.lo);
  const int el = static_cast<int>((lb >> 23) & 0xff);
  if (el != 0) {
    const uint64_t ml = (lb & 0x7fffffu) | 0x800000u;
    const int sl = el - 150 + q;
    const uint64_t lv = sl >= 0 ? (ml << sl) : (sl > -64 ? (ml >> -sl) : 0u);
    r = (lb >> 31) ? r - lv : r + lv;
  }
  return r;
}

DF_HD int df_clz32(uint32_t x) {
#if defined(__CUDA_ARCH__)
  return __clz(static_cast<int>(x));
#else
  return x ? __builtin_clz(x) : 32;
#endif
}
DF_HD uint32_t df_umulhi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __umulhi(a, b);
#else
  return static_cast<uint32_t>((static_cast<uint64_t>(a) * b) >> 32);
#endif
}

// t vq 2^e as FP64 for a 32-bit integer t and a normalised fixed-point
// factor vq in [2^63, 2^64), within one ulp: h = (|t| 2^lz vq) / 2^32 (a
// 32 x 64-bit product, exact down to the cut low word) rounded to 53 bits
// m, and the FP64 bits formed as ((biased exponent - 1) << 52) + m, where
// the leading bit of m carries into the exponent field.  The caller keeps
// e in [-1080, 920], so every result is a normal FP64 number.
DF_HD double df_i32_times_q63(int32_t t, uint64_t vq, int e) {
  const uint32_t a = t < 0 ? 0u - static_cast<uint32_t>(t) : static_cast<uint32_t>(t);
  const int lz = df_clz32(a);
  const uint32_t an = a << (lz & 31);
  const uint64_t h = static_cast<uint64_t>(an) * static_cast<uint32_t>(vq >> 32) +
                     df_umulhi32(an, static_cast<uint32_t>(vq));  // in [2^62, 2^64)
  const int top = static_cast<int>(h >> 63);
  const uint64_t m = (h >> (10 + top)) + ((h >> (9 + top)) & 1u);  // in [2^52, 2^53]
  const uint64_t bexp = static_cast<uint64_t>(1023 + 94 - 1 + top + e - lz);
  const uint64_t bits = (bexp << 52) + m;
  return t == 0 ? 0.0 : df_double(bits | (t < 0 ? 0x8000000000000000ull : 0ull));
}

// A 32-bit integer as FP64, exactly, by bits (no conversion instruction).
DF_HD double df_i32_to_double(int32_t t) {
  if (t == 0) return 0.0;
  const uint32_t a = t < 0 ? 0u - static_cast<uint32_t>(t) : static_cast<uint32_t>(t);
  const int lz = df_clz32(a);
  const uint64_t frac = static_cast<uint64_t>(a << lz << 1) << 20;  // bits below the leading one
  return df_double((t < 0 ? 0x8000000000000000ull : 0ull) | (static_cast<uint64_t>(1023 + 31 - lz) << 52) | frac);
}

// x 2^e as FP64 for a normalised double-float x (df_to_double, then the
// exponent moved on the bits): results beyond the FP64 range become +-inf,
// results below the normal range +-0 (no FP64 instruction).
DF_HD double df_to_double_scaled(dfloat x, int e) {
  const double d = df_to_double(x);
  const uint64_t b = df_bits64(d);
  const int be = static_cast<int>((b >> 52) & 0x7ff);
  if (be == 0 || be == 0x7ff) return d;
  const int ne = be + e;
  const uint64_t sign = b & 0x8000000000000000ull;
  if (ne > 2046) return df_double(sign | 0x7FF0000000000000ull);
  if (ne < 1) return df_double(sign);
  return df_double((b & 0x800FFFFFFFFFFFFFull) | (static_cast<uint64_t>(ne) << 52));
}

}  // namespace nfem
