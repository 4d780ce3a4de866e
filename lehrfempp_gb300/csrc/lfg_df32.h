// Double-float ("df32") arithmetic: a value is an unevaluated sum hi + lo of
// two IEEE binary32 numbers with |lo| <= ulp(hi)/2, i.e. ~48 significant bits.
//
// GB300 executes FP32 FMAs ~60x faster than FP64 operations, and converting
// between binary32 and binary64 runs on the slow FP64 pipe as well.  The
// element kernels therefore keep FP64 only for the few coordinate
// differences of a cell and do everything else in df32 on the FP32 pipes.
// Conversions in and out are done with integer bit manipulation.
// Error-free transformations follow Dekker (1971) / Knuth TwoSum and the FMA
// TwoProduct (Ogita, Rump, Oishi 2005).
//
// The same code compiles for the device and for the host (the CPU precision
// test in tests/ builds it with g++), so what the test measures is what the
// kernels execute.  Device adds/multiplies use the _rn intrinsics so that the
// compiler cannot fuse them into FMAs, which would break the error-free
// transformations.
#pragma once

#include <cstdint>
#include <cstring>

#include <math.h>

#if defined(__CUDACC__)
#define DF_HD __host__ __device__ __forceinline__
#else
#include <cmath>
#define DF_HD inline
#endif

namespace lfg {
namespace df {

struct f2 {
  float h, l;
};

DF_HD float Add(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fadd_rn(a, b);
#else
  volatile float r = a + b;
  return r;
#endif
}
DF_HD float Sub(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fsub_rn(a, b);
#else
  volatile float r = a - b;
  return r;
#endif
}
DF_HD float Mul(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  volatile float r = a * b;
  return r;
#endif
}
DF_HD float Fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return std::fmaf(a, b, c);
#endif
}

DF_HD uint64_t DBits(double d) {
#if defined(__CUDA_ARCH__)
  return static_cast<uint64_t>(__double_as_longlong(d));
#else
  uint64_t u;
  std::memcpy(&u, &d, 8);
  return u;
#endif
}
DF_HD double BitsD(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(static_cast<long long>(u));
#else
  double d;
  std::memcpy(&d, &u, 8);
  return d;
#endif
}
DF_HD uint32_t FBits(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
#endif
}
DF_HD float BitsF(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}
DF_HD float U32ToF(uint32_t u) {  // round to nearest
#if defined(__CUDA_ARCH__)
  return __uint2float_rn(u);
#else
  return static_cast<float>(u);
#endif
}

// s + e == a + b exactly (Knuth TwoSum, 6 flops, no magnitude condition).
DF_HD f2 TwoSum(float a, float b) {
  const float s = Add(a, b);
  const float bb = Sub(s, a);
  const float e = Add(Sub(a, Sub(s, bb)), Sub(b, bb));
  return {s, e};
}
// |a| >= |b| (or a == 0): s + e == a + b exactly (3 flops).
DF_HD f2 FastTwoSum(float a, float b) {
  const float s = Add(a, b);
  return {s, Sub(b, Sub(s, a))};
}

DF_HD f2 Make(float h) { return {h, 0.0f}; }
DF_HD f2 Neg(f2 a) { return {-a.h, -a.l}; }

// binary64 -> df32 without FP64 instructions: hi keeps the top 24 significant
// bits (truncated), lo the next 29 rounded to 24.  Finite inputs with
// 2^-100 < |d| < 2^100 (or d == 0) convert with relative error <= 2^-48;
// smaller non-zero inputs keep only hi.
DF_HD f2 FromDouble(double d) {
  const uint64_t u = DBits(d);
  const uint32_t sign = static_cast<uint32_t>(u >> 63) << 31;
  const int E = static_cast<int>((u >> 52) & 0x7ff);
  if (E < 1023 - 100 || E > 1023 + 100) return {0.0f, 0.0f};  // zero, or outside the supported range
  const uint64_t m = u & ((uint64_t(1) << 52) - 1);
  const float h = BitsF(sign | (static_cast<uint32_t>(E - 1023 + 127) << 23) | static_cast<uint32_t>(m >> 29));
  const uint32_t rem = static_cast<uint32_t>(m & ((uint64_t(1) << 29) - 1));
  const int se = E - 1075 + 127;  // exponent of 2^(E-1075) in binary32
  if (rem == 0 || se < 1) return {h, 0.0f};
  const float l = Mul(U32ToF(rem), BitsF(static_cast<uint32_t>(se) << 23));
  return {h, sign ? -l : l};
}

// binary32 -> binary64 bit pattern, exact, without FP64 instructions (normal
// floats and zero; df32 values here never hold subnormals or inf/nan).
DF_HD double FloatToDoubleExact(float f) {
  const uint32_t b = FBits(f);
  const uint64_t sign = static_cast<uint64_t>(b >> 31) << 63;
  const uint32_t e = (b >> 23) & 0xff;
  if (e == 0) return BitsD(sign);
  return BitsD(sign | (static_cast<uint64_t>(e - 127 + 1023) << 52) | (static_cast<uint64_t>(b & 0x7fffff) << 29));
}

// df32 -> binary64 (hi + lo rounded once to nearest): one FP64 add.
DF_HD double ToDouble(f2 a) { return FloatToDoubleExact(a.h) + FloatToDoubleExact(a.l); }

DF_HD f2 Add(f2 a, f2 b) {
  f2 s = TwoSum(a.h, b.h);
  const float t = Add(Add(a.l, b.l), s.l);
  return FastTwoSum(s.h, t);
}
DF_HD f2 Sub(f2 a, f2 b) { return Add(a, Neg(b)); }

DF_HD f2 Mul(f2 a, f2 b) {
  const float p = Mul(a.h, b.h);
  float e = Fma(a.h, b.h, -p);
  e = Fma(a.h, b.l, e);
  e = Fma(a.l, b.h, e);
  return FastTwoSum(p, e);
}
DF_HD f2 Mul(f2 a, float b) {
  const float p = Mul(a.h, b);
  float e = Fma(a.h, b, -p);
  e = Fma(a.l, b, e);
  return FastTwoSum(p, e);
}
// a*b + c
DF_HD f2 MulAdd(f2 a, f2 b, f2 c) { return Add(Mul(a, b), c); }

// 1/a by one Newton step on the binary32 reciprocal: r1 = r0 + r0 (1 - a r0).
DF_HD f2 Rcp(f2 a) {
#if defined(__CUDA_ARCH__)
  const float r0 = __frcp_rn(a.h);
#else
  volatile float r0 = 1.0f / a.h;
#endif
  const f2 ar = Mul(a, r0);
  const f2 one_minus = Sub(Make(1.0f), ar);
  return Add(Make(r0), Mul(one_minus, r0));
}

DF_HD f2 Abs(f2 a) { return a.h < 0.0f ? Neg(a) : a; }

// Accumulator for sums of df32 products: the binary32 leading parts are
// summed exactly with TwoSum (s + c), all rounding errors go to e.
struct Acc {
  float s = 0.0f, e = 0.0f;
  DF_HD void AddProd(f2 a, f2 b) {
    const float p = Mul(a.h, b.h);
    float err = Fma(a.h, b.h, -p);
    err = Fma(a.h, b.l, err);
    err = Fma(a.l, b.h, err);
    const f2 t = TwoSum(s, p);
    s = t.h;
    e = Add(e, Add(t.l, err));
  }
  DF_HD f2 Value() const { return FastTwoSum(s, e); }
};

}  // namespace df
}  // namespace lfg
