// Double-float ("df64") arithmetic on the FP32 pipe.
//
// A df64 value is the unevaluated sum hi + lo of two FP32 numbers with |lo| <= ulp(hi) / 2, which
// carries about 48 significant bits. The operations are built from the classical error-free
// transformations: TwoSum (Knuth, TAOCP vol. 2, 4.2.2), Fast2Sum (Dekker, 1971) and the exact
// product through a fused multiply-add (a * b = p + fma(a, b, -p)). Products drop the lo * lo term
// and sums use the "sloppy" double-word addition (one TwoSum on the high words), as analysed by
// Joldes, Muller and Popescu, "Tight and rigorous error bounds for basic building blocks of
// double-word arithmetic", ACM TOMS 44(2), 2017: the absolute error of a sum is a small multiple of
// 2^-46 (|a| + |b|), which is what an accumulation of many terms needs.
//
// On GB300 the FP32 pipe issues 59x the FP64 pipe's FMAs; a df64 FMA costs about 12 FP32
// instructions, so FP64-grade coupling sums run several times faster in df64 than in FP64.
#pragma once

#include <cuda_runtime.h>

namespace sg {
// The type and its operations live in a nested namespace: argument-dependent lookup finds this fma()
// for df64 arguments only, and an unqualified fma() on double or float arguments inside namespace sg
// still resolves to the CUDA math overloads.
namespace dfw {

struct df64 {
  float hi, lo;
  __host__ __device__ df64() {}
  __host__ __device__ df64(float h, float l) : hi(h), lo(l) {}
  __device__ df64(int v) : hi((float)v), lo(0.f) {}
  __device__ df64(float v) : hi(v), lo(0.f) {}
  __device__ df64(double d) {
    hi = (float)d;
    lo = (float)(d - (double)hi);
  }
  __device__ explicit operator double() const { return (double)hi + (double)lo; }
  __device__ explicit operator float() const { return hi + lo; }
};

struct df64x2 {
  df64 x, y;
};

// s + e == a + b exactly
__device__ __forceinline__ df64 df_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return df64(s, e);
}

// s + e == a + b exactly when |a| >= |b|
__device__ __forceinline__ df64 df_fast_two_sum(float a, float b) {
  const float s = a + b;
  const float e = b - (s - a);
  return df64(s, e);
}

__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }

__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  const df64 s = df_two_sum(a.hi, b.hi);
  return df_fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}

__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }

__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return df_fast_two_sum(p, e);
}

// a * b + c, as compensated accumulation: the high words are added exactly (TwoSum) and every
// rounding error goes into the low word, which is not renormalised. The low word stays a tiny
// fraction of the high word over the lengths used here (it grows by at most about one ulp of the
// high word per call), so the pair remains an accurate unevaluated sum and is accepted as an
// operand by the operations above; conversion to double adds the two words exactly.
__device__ __forceinline__ df64 fma(df64 a, df64 b, df64 c) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  const df64 s = df_two_sum(c.hi, p);
  return df64(s.hi, s.lo + (c.lo + e));
}

// ---- two double-float values at once on the packed FP32x2 instructions (sm_100 and later)
__device__ __forceinline__ float2 f2_add(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "add.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
__device__ __forceinline__ float2 f2_sub(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
__device__ __forceinline__ float2 f2_mul(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "mul.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
__device__ __forceinline__ float2 f2_fma(float2 a, float2 b, float2 c) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%6, %7};\n\t"
      "fma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return d;
}

// two double-float values: (hi.x, lo.x) and (hi.y, lo.y)
struct df64p {
  float2 hi, lo;
};

// a double-float multiplier broadcast to both lanes, with its negated high word
struct df64b {
  float2 hi, lo, nhi;
};

__device__ __forceinline__ df64b df_bcast(df64 a) {
  df64b r;
  r.hi = make_float2(a.hi, a.hi);
  r.lo = make_float2(a.lo, a.lo);
  r.nhi = make_float2(-a.hi, -a.hi);
  return r;
}

// fma(a, b, c) above on two values at once, with the same operations in the same order, so each
// lane's result equals the scalar one bit for bit: the product's negation np = -p is exact, so
// fma(a.hi, b.hi, -p) = fma(a.hi, b.hi, np), c.hi + p = c.hi - np and p - bb = -(np + bb).
__device__ __forceinline__ df64p fma_p(const df64b &a, df64p b, df64p c) {
  const float2 np = f2_mul(a.nhi, b.hi);
  float2 e = f2_fma(a.hi, b.hi, np);
  e = f2_fma(a.hi, b.lo, e);
  e = f2_fma(a.lo, b.hi, e);
  const float2 s = f2_sub(c.hi, np);
  const float2 bb = f2_sub(s, c.hi);
  const float2 err = f2_sub(f2_sub(c.hi, f2_sub(s, bb)), f2_add(np, bb));
  df64p r;
  r.hi = s;
  r.lo = f2_add(err, f2_add(c.lo, e));
  return r;
}

// FP64 complex -> df64 complex (hi = nearest float, lo = nearest float of the remainder)
__device__ __forceinline__ df64x2 df_from_double2(double2 v) {
  df64x2 r;
  r.x = df64(v.x);
  r.y = df64(v.y);
  return r;
}

}  // namespace dfw
using dfw::df64;
using dfw::df64b;
using dfw::df64p;
using dfw::df64x2;
using dfw::df_from_double2;
}  // namespace sg
