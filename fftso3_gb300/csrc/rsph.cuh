// The real-harmonic basis change matrix2rsph (fdcl_FFTSO3.cpp:1107-1139) as
// device helpers shared by the basis conversions and the Clebsch-Gordan tables.
#pragma once
#include <cuda_runtime.h>

namespace fftso3 {

// matrix2rsph T(l; a, c) (fdcl_FFTSO3.cpp:1107-1139), row a, column c, in the
// arithmetic type A (double for the FP64 path, float for the tensor-core path).
template <typename A> struct c2t { A x, y; };

// 1/sqrt(2): the FP64 path forms it as the reference does, 1./sqrt(2.).
template <typename A> __device__ __forceinline__ A inv_sqrt2();
template <> __device__ __forceinline__ double inv_sqrt2<double>() { return 1. / sqrt(2.); }
template <> __device__ __forceinline__ float inv_sqrt2<float>() { return 0.70710678118654752440f; }

template <typename A>
__device__ __forceinline__ c2t<A> tmat_t(int a, int c)
{
    const A s = inv_sqrt2<A>();
    if (a < 0) {
        if (c == a) return {(A)0, s};
        if (c == -a) return {(A)0, -s * ((a & 1) ? (A)-1 : (A)1)};
    } else if (a == 0) {
        if (c == 0) return {(A)1, (A)0};
    } else {
        if (c == -a) return {s, (A)0};
        if (c == a) return {((a & 1) ? (A)-1 : (A)1) * s, (A)0};
    }
    return {(A)0, (A)0};
}

template <typename A>
__device__ __forceinline__ c2t<A> cmul_t(c2t<A> a, c2t<A> b)
{
    return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename A>
__device__ __forceinline__ c2t<A> conj_t(c2t<A> a) { return {a.x, -a.y}; }

}  // namespace fftso3
