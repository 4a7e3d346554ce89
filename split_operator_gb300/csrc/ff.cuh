// Float-float arithmetic for the float-float state precision: a real value is the
// unevaluated sum hi + lo of two FP32 numbers with |lo| <= ulp(hi) / 2 (about 48
// significand bits, FP32's exponent range), a complex value four FP32 numbers (16 bytes,
// the size of a double2).  GB300 runs FP32 at 64 times its FP64 rate, so a few FP32
// operations per float-float operation still beat FP64 arithmetic by a wide margin.
//
// Building blocks (all published error-free transformations):
//   two_sum       Knuth's TwoSum: s + e = a + b exactly (6 operations)
//   fast_two_sum  Dekker's FastTwoSum, |a| >= |b| (3 operations)
//   two_prod      p + e = a b exactly, e from one FMA
// and from them, following Joldes, Muller and Popescu, "Tight and rigorous error bounds
// for basic building blocks of double-word arithmetic", ACM TOMS 44(2), 2017:
//   operator+     AccurateDWPlusDW (their Algorithm 6), relative error <= 3u^2 + 13u^3
//   operator*     DWTimesDW3 (their Algorithm 12), relative error <= 4u^2
// with u = 2^-24.  The FP32 operations are the _rn intrinsics, which the compiler neither
// contracts into FMAs nor reassociates, so every step rounds exactly as written.
#pragma once
#include <cuda_runtime.h>

namespace so {

struct ff {
  float hi, lo;
  ff() = default;
  __host__ __device__ constexpr ff(float h, float l) : hi(h), lo(l) {}
  // the nearest float-float to d: hi = d rounded to FP32, lo = the remainder rounded
  // (d - hi is exact in FP64)
  __host__ __device__ constexpr ff(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
  __host__ __device__ constexpr ff(int i) : hi((float)i), lo(0.0f) {}  // exact for |i| < 2^24
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
  __host__ __device__ explicit operator float() const { return hi; }
};

// a complex float-float value: re, im (16-byte aligned like double2)
struct __align__(16) ffc {
  ff x, y;
};

#ifdef __CUDACC__

__device__ __forceinline__ ff two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

__device__ __forceinline__ ff fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ ff two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ ff operator+(ff x, ff y) {
  const ff s = two_sum(x.hi, y.hi), t = two_sum(x.lo, y.lo);
  const ff v = fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
  return fast_two_sum(v.hi, __fadd_rn(t.lo, v.lo));
}

__device__ __forceinline__ ff operator-(ff x) { return {-x.hi, -x.lo}; }
__device__ __forceinline__ ff operator-(ff x, ff y) { return x + (-y); }

__device__ __forceinline__ ff operator*(ff x, ff y) {
  const ff c = two_prod(x.hi, y.hi);
  const float t = __fmaf_rn(x.hi, y.lo, __fmul_rn(x.lo, y.lo));
  return fast_two_sum(c.hi, __fadd_rn(c.lo, __fmaf_rn(x.lo, y.hi, t)));
}

// s x for a sign or power of two s (the butterflies' direction factors): exact
__device__ __forceinline__ ff operator*(int s, ff x) {
  const float f = (float)s;
  return {__fmul_rn(f, x.hi), __fmul_rn(f, x.lo)};
}

__device__ __forceinline__ ff& operator+=(ff& a, ff b) { return a = a + b; }
__device__ __forceinline__ ff& operator-=(ff& a, ff b) { return a = a - b; }
__device__ __forceinline__ ff& operator*=(ff& a, ff b) { return a = a * b; }

// read-only cached loads of float-float values (the FP32 words through __ldg)
__device__ __forceinline__ ff ldg_ff(const ff* p) {
  const float2 v = __ldg(reinterpret_cast<const float2*>(p));
  return {v.x, v.y};
}
__device__ __forceinline__ ffc ldg_ff(const ffc* p) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(p));
  return {{v.x, v.y}, {v.z, v.w}};
}

// Compensated dot-product accumulator (the Dot2 scheme of Ogita, Rump and Oishi, "Accurate
// sum and dot product", SIAM J. Sci. Comput. 26(6), 2005, with float-float factors): the
// running sum s is an FP32 value, every product's and every addition's rounding error is
// collected exactly (two_prod, two_sum) into the FP32 correction c together with the
// cross terms of the factors' lo parts.  The result s + c is as accurate as a sum computed
// in about twice FP32's precision, at 12 FP32 operations per term instead of the ~28 of a
// float-float multiply and add.
struct FfDot {
  float s = 0.0f, c = 0.0f;
  __device__ __forceinline__ void add(ff a, ff b) {
    const ff p = two_prod(a.hi, b.hi);
    const ff t = two_sum(s, p.hi);
    s = t.hi;
    c = __fadd_rn(c, __fadd_rn(t.lo, __fadd_rn(p.lo, __fmaf_rn(a.hi, b.lo, __fmul_rn(a.lo, b.hi)))));
  }
  __device__ __forceinline__ ff value() const { return two_sum(s, c); }  // c may exceed s after cancellation
};

#endif  // __CUDACC__

}  // namespace so
