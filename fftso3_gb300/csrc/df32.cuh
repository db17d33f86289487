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

// ---- quantised double-float: a pair (h, l) whose high part h is a multiple of a quantum q = 2^e that a whole
// block of data shares, with |h| < 2^24 q.  Sums and differences of high parts are then exact, so adding two
// values costs two FP32 additions instead of a two-sum (2 instead of 8 instructions); l holds the rest in plain
// FP32.  Products round the exact product of the high parts to the quantum in one FMA with the magic constant
// magic = 1.5 * 2^23 q (valid while |product| < 2^22 q) and keep the remainder, exact to 2^-24 q, in l.  With
// the block's values bounded by 2^E and q = 2^(E - G), every result is exact to about 2^-24 q plus the FP32
// error of l: at most ~2^(-24 - G) of the block's largest value per operation, once l is folded back onto the
// quantum (q_renorm) whenever it may have grown.
struct qf32 {
    float h, l;
};
__device__ __forceinline__ qf32 operator+(qf32 a, qf32 b) { return qf32{a.h + b.h, a.l + b.l}; }
__device__ __forceinline__ qf32 operator-(qf32 a, qf32 b) { return qf32{a.h - b.h, a.l - b.l}; }
__device__ __forceinline__ qf32 operator-(qf32 a) { return qf32{-a.h, -a.l}; }
__device__ __forceinline__ qf32& operator+=(qf32& a, qf32 b) { return a = a + b; }
__device__ __forceinline__ qf32& operator-=(qf32& a, qf32 b) { return a = a - b; }

struct __align__(16) qc32 {
    qf32 x, y;
};

// x rounded to the quantum (|x| < 2^22 q)
__device__ __forceinline__ float q_round(float x, float magic) { return __fsub_rn(__fadd_rn(x, magic), magic); }
// a.h c rounded to the quantum, from the exact product
__device__ __forceinline__ float q_round_prod(float a, float c, float magic)
{
    return __fsub_rn(__fmaf_rn(a, c, magic), magic);
}
// any double-float value onto the quantum
__device__ __forceinline__ qf32 q_from(df32 a, float magic)
{
    const float p = q_round(a.h, magic);
    return qf32{p, __fadd_rn(__fsub_rn(a.h, p), a.l)};
}
// fold the quantum part of l into h
__device__ __forceinline__ qf32 q_renorm(qf32 a, float magic)
{
    const float p = q_round(a.l, magic);
    return qf32{__fadd_rn(a.h, p), __fsub_rn(a.l, p)};
}
__device__ __forceinline__ qc32 q_renorm(qc32 a, float magic) { return qc32{q_renorm(a.x, magic), q_renorm(a.y, magic)}; }
__device__ __forceinline__ qc32 q_from(dfc32 a, float magic) { return qc32{q_from(a.x, magic), q_from(a.y, magic)}; }
// a c for a double-float constant c (the a.l c.l term dropped)
__device__ __forceinline__ qf32 q_mul(qf32 a, df32 c, float magic)
{
    const float P = q_round_prod(a.h, c.h, magic);
    float r = __fmaf_rn(a.h, c.h, -P);
    r = __fmaf_rn(a.h, c.l, r);
    r = __fmaf_rn(a.l, c.h, r);
    return qf32{P, r};
}
// complex a w for a double-float twiddle w
__device__ __forceinline__ qc32 q_cmul(qc32 a, dfc32 w, float magic)
{
    const float P1 = q_round_prod(a.x.h, w.x.h, magic), P2 = q_round_prod(a.y.h, w.y.h, magic);
    const float P3 = q_round_prod(a.x.h, w.y.h, magic), P4 = q_round_prod(a.y.h, w.x.h, magic);
    float re = __fsub_rn(__fmaf_rn(a.x.h, w.x.h, -P1), __fmaf_rn(a.y.h, w.y.h, -P2));
    float im = __fadd_rn(__fmaf_rn(a.x.h, w.y.h, -P3), __fmaf_rn(a.y.h, w.x.h, -P4));
    re = __fmaf_rn(a.x.h, w.x.l, re);
    re = __fmaf_rn(a.x.l, w.x.h, re);
    re = __fmaf_rn(-a.y.h, w.y.l, re);
    re = __fmaf_rn(-a.y.l, w.y.h, re);
    im = __fmaf_rn(a.x.h, w.y.l, im);
    im = __fmaf_rn(a.x.l, w.y.h, im);
    im = __fmaf_rn(a.y.h, w.x.l, im);
    im = __fmaf_rn(a.y.l, w.x.h, im);
    return qc32{qf32{__fsub_rn(P1, P2), re}, qf32{__fadd_rn(P3, P4), im}};
}

}  // namespace fftso3
