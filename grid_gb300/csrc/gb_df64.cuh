// Double-float ("df64") arithmetic: a value is hi + lo, two floats, about 48 significant
// bits.  The FP64 hopping term can run in it on the FP32 pipes, which GB300 issues at 64
// times its FP64 rate, while the fields keep their FP64 storage: each double is split
// into (hi, lo) on load and hi + lo is rounded back to a double on store.
//
// The split and the widening use integer operations only, so no FP64 instruction is
// spent on them.  Error-free transformations (Knuth's TwoSum, Dekker's FastTwoSum and the
// FMA-based TwoProduct) give sums and products whose relative error is a few units of
// 2^-48; dot products accumulate the rounding errors of the two-term expansion in a
// separate float (Ogita, Rump and Oishi, "Accurate sum and dot product", SIAM J. Sci.
// Comput. 26 (2005), algorithm Dot2).
//
// The same code compiles for the host (g++) so that a CPU test can check it.
#pragma once
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define GB_HD __host__ __device__ __forceinline__
#else
#include <cmath>
#define GB_HD inline
#endif

namespace gb {

struct dfloat {
  float hi, lo;
  dfloat() = default;
  GB_HD constexpr dfloat(float h, float l) : hi(h), lo(l) {}
  GB_HD explicit constexpr dfloat(int v) : hi(float(v)), lo(0.f) {}
};

namespace df {

GB_HD uint64_t bits64(double d) {
#ifdef __CUDA_ARCH__
  return uint64_t(__double_as_longlong(d));
#else
  uint64_t u;
  std::memcpy(&u, &d, 8);
  return u;
#endif
}
GB_HD double from_bits64(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double d;
  std::memcpy(&d, &u, 8);
  return d;
#endif
}
GB_HD uint32_t bits32(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
#endif
}
GB_HD float from_bits32(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}
GB_HD float fmaf_(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fmaf(a, b, c);
#endif
}
GB_HD float add_rn(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);  // never contracted into an FMA
#else
  return a + b;
#endif
}
GB_HD float sub_rn(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
GB_HD float mul_rn(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}

// TwoSum: s + e == a + b exactly
GB_HD dfloat two_sum(float a, float b) {
  const float s = add_rn(a, b);
  const float bb = sub_rn(s, a);
  const float e = add_rn(sub_rn(a, sub_rn(s, bb)), sub_rn(b, bb));
  return dfloat(s, e);
}
// FastTwoSum (|a| >= |b|, or a == 0)
GB_HD dfloat fast_two_sum(float a, float b) {
  const float s = add_rn(a, b);
  return dfloat(s, sub_rn(b, sub_rn(s, a)));
}

// The split of a double: hi = the double rounded to 24 significant bits, lo = the rest
// rounded to a float.  Integer work only: hi takes bits 29..63 of the double rounded at
// bit 28 (the exponent re-biased by flipping bit 30), and lo is the signed remainder
// (|r| <= 2^28 units of the double's last place) converted to float and scaled by that
// place.  Exact to 2^-48 for |d| in [2^-74, 2^127); below 2^-74 lo is dropped (an error
// under 2^-98 absolute), below 2^-126 the value becomes a signed zero, and infinities and
// NaNs stay infinities and NaNs.  No branch: every lane runs the same instructions.
GB_HD dfloat split(double d) {
  const uint64_t u = bits64(d);
  const uint32_t hw = uint32_t(u >> 32);
  const uint32_t e = (hw >> 20) & 0x7FFu;
  const uint32_t sign = hw & 0x80000000u;
  const uint64_t ur = u + (uint64_t(1) << 28);
  uint32_t hb = ((uint32_t(ur >> 29) & 0x7FFFFFFFu) ^ 0x40000000u) | sign;
  const uint32_t low29 = uint32_t(u) & 0x1FFFFFFFu;
  const int32_t r = int32_t(low29) - int32_t((low29 & 0x10000000u) << 1);
  const uint32_t sb = e >= 949u ? ((e - 948u) << 23) | sign : sign;  // +-2^(E - 52), or +-0
  hb = e < 897u ? sign : hb;
  const bool nan = e == 0x7FFu && (u << 12) != 0;
  hb = e >= 1150u ? (sign | (nan ? 0x7FC00000u : 0x7F800000u)) : hb;
  const float lo = e >= 1150u ? 0.f : mul_rn(float(r), from_bits32(sb));
  return dfloat(from_bits32(hb), lo);
}

// A float widened to a double by integer operations (float subnormals become signed
// zeros; infinities and NaNs stay so).
GB_HD double widen(float f) {
  const uint32_t b = bits32(f);
  const uint32_t ef = (b >> 23) & 0xFFu;
  const uint64_t sign = uint64_t(b & 0x80000000u) << 32;
  const uint64_t mant = uint64_t(b & 0x7FFFFFu) << 29;
  const uint64_t normal = sign | (uint64_t(ef + 896u) << 52) | mant;
  const uint64_t special = sign | (uint64_t(0x7FFu) << 52) | mant;
  return from_bits64(ef == 0u ? sign : (ef == 0xFFu ? special : normal));
}

// hi + lo rounded once to a double
GB_HD double to_double(dfloat a) { return widen(a.hi) + widen(a.lo); }

}  // namespace df

// Sum without renormalisation: (s, e + a.lo + b.lo) with s + e == a.hi + b.hi.  The low
// part stays within a few units of the high part's last place along the Dhop's short
// chains (one projection, eight accumulations), and the store rounds hi + lo exactly.
GB_HD dfloat operator+(dfloat a, dfloat b) {
  const dfloat s = df::two_sum(a.hi, b.hi);
  return dfloat(s.hi, df::add_rn(s.lo, df::add_rn(a.lo, b.lo)));
}
GB_HD dfloat operator-(dfloat a) { return dfloat(-a.hi, -a.lo); }
GB_HD dfloat operator-(dfloat a, dfloat b) { return a + (-b); }
GB_HD dfloat& operator+=(dfloat& a, dfloat b) {
  a = a + b;
  return a;
}
// s times a value for s = +1 or -1 only (the projector and reconstruction signs); any
// other s is treated as its sign
GB_HD dfloat operator*(int s, dfloat a) { return s < 0 ? -a : a; }

// Dot2: sum of a_k b_k with TwoProduct on the high parts, the cross terms and the
// products' and sums' rounding errors gathered in one float, renormalised at the end.
struct DfDot {
  float s, c;
  GB_HD void first(dfloat a, dfloat b) {
    s = df::mul_rn(a.hi, b.hi);
    c = df::fmaf_(a.hi, b.hi, -s);
    c = df::fmaf_(a.hi, b.lo, c);
    c = df::fmaf_(a.lo, b.hi, c);
  }
  GB_HD void mac(dfloat a, dfloat b) {
    const float p = df::mul_rn(a.hi, b.hi);
    float t = df::fmaf_(a.hi, b.hi, -p);
    t = df::fmaf_(a.hi, b.lo, t);
    t = df::fmaf_(a.lo, b.hi, t);
    const dfloat q = df::two_sum(s, p);
    s = q.hi;
    c = df::add_rn(c, df::add_rn(t, q.lo));
  }
  GB_HD dfloat result() const { return df::fast_two_sum(s, c); }
};

}  // namespace gb
