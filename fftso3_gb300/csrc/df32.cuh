// Double-FP32 ("double-float") arithmetic: a value is the unevaluated sum h + l
// of two floats, about 48 significant bits, computed on the FP32 pipes.  On
// GB300 the FP64 units are a small fraction of the FP32 ones, so the
// refinement's FFT runs in this arithmetic instead of FP64.
//
// The operations are the classical error-free transformations: two_sum
// (Knuth), quick_two_sum (Dekker, for |a| >= |b|) and the FMA-based exact
// product a*b = p + fma(a, b, -p).  The operators + and * are "lazy": the
// rounding error of h is folded into l (a + b: h = fl(a.h + b.h),
// l = err + a.l + b.l; a * b: h = fl(a.h b.h), l = err + a.h b.l + a.l b.h, the
// l*l term dropped) but the pair is not renormalised after each operation, which
// saves 3 of 11 and 3 of 7 instructions.  |l| then stays a small multiple of
// ulp(h) over the short chains of an FFT butterfly network (one step of growth
// per operation), so h + l keeps about 44 bits relative to the operands -- the
// error an FFT's analysis is stated in.  df_two_sum / df_quick_two_sum give
// normalised pairs where a caller needs them.  No fast-math flags are used.
#pragma once
#include <cuda_runtime.h>

namespace fftso3 {

struct df32 {
    float h, l;
    df32() = default;
    __host__ __device__ constexpr df32(float hh, float ll) : h(hh), l(ll) {}
    // nearest pair to a double: h = fl(d), l = fl(d - h)
    __host__ __device__ df32(double d) : h((float)d), l((float)(d - (double)(float)d)) {}
};

__device__ __forceinline__ df32 df_two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    const float e = (a - (s - bb)) + (b - bb);
    return df32(s, e);
}

__device__ __forceinline__ df32 df_quick_two_sum(float a, float b)
{
    const float s = a + b;
    return df32(s, b - (s - a));
}

__device__ __forceinline__ df32 operator+(df32 a, df32 b)
{
    const df32 s = df_two_sum(a.h, b.h);
    return df32(s.h, s.l + (a.l + b.l));
}

__device__ __forceinline__ df32 operator-(df32 a) { return df32(-a.h, -a.l); }
__device__ __forceinline__ df32 operator-(df32 a, df32 b) { return a + (-b); }

__device__ __forceinline__ df32 operator*(df32 a, df32 b)
{
    const float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return df32(p, e);
}

__device__ __forceinline__ df32& operator+=(df32& a, df32 b) { return a = a + b; }
__device__ __forceinline__ df32& operator-=(df32& a, df32 b) { return a = a - b; }

// complex double-float; in memory (re.h, re.l, im.h, im.l), one 16-byte access
struct __align__(16) dfc32 {
    df32 x, y;
};

}  // namespace fftso3
