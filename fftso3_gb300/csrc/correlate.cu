// S^2 -> SO(3) correlation (spherical shape matching) and grid arg-max.
//
// The reference's shape-matching example (example/example3.cpp:28-95,
// example/example3_SSM.hpp J(R)) scores a rotation R of a real spherical
// function F against another, G, by
//   J(R) = sum_l G[l]^T U^l(R) F[l],
// U^l the real harmonics of R (fdcl_FFTSO3.cpp:1062-1105), and evaluates it one
// rotation at a time while descending its gradient.  J is a real SO(3) function
// whose real-basis coefficients are outer products of the two S^2 coefficient
// vectors: with the real inverse f(R) = sum_l (2l+1) sum_mn Fr(l,m,n) U^l_mn(R)
// (fdcl_FFTSO3.cpp:1141-1156),
//   Fr(l, m, n) = G_l(m) F_l(n) / (2l + 1),
// so one SO(3) inverse transform gives J at every rotation of the Euler grid,
// and the grid's arg-max is the best rotation to the grid's resolution.
#include <cfloat>

#include "common.cuh"
#include "contract.cuh"

namespace fftso3 {

template <typename T>
__global__ void corr_coeffs_kernel(const T* __restrict__ F, const T* __restrict__ G, T* __restrict__ C, int L)
{
    const int l = blockIdx.x, b = blockIdx.y;
    const int W = 2 * l + 1;
    const long long s2c = (long long)(L + 1) * (L + 1), so3c = so3_off(L + 1);
    const T* f = F + (long long)b * s2c + (long long)l * l;  // F_l(n) at n + l
    const T* g = G + (long long)b * s2c + (long long)l * l;
    T* c = C + (long long)b * so3c + so3_off(l);
    const T inv = (T)1 / (T)W;
    for (int i = threadIdx.x; i < W * W; i += blockDim.x) {
        const int mi = i % W, ni = i / W;  // column-major (m + l) + (n + l)(2l + 1)
        c[i] = g[mi] * f[ni] * inv;
    }
}

cudaError_t launch_corr_coeffs(const void* F, const void* G, void* C, bool fp64, int L, int batch, cudaStream_t st)
{
    dim3 grid(L + 1, batch);
    if (fp64)
        corr_coeffs_kernel<double><<<grid, 256, 0, st>>>((const double*)F, (const double*)G, (double*)C, L);
    else
        corr_coeffs_kernel<float><<<grid, 256, 0, st>>>((const float*)F, (const float*)G, (float*)C, L);
    return cudaGetLastError();
}

// Two-stage arg-max of nb real arrays of n elements: stage 1 reduces chunks of
// each array to (value, index) pairs, stage 2 reduces the pairs of one array.
// Ties keep the smallest index.
__device__ __forceinline__ void better(double& v, long long& i, double v2, long long i2)
{
    if (v2 > v || (v2 == v && i2 < i)) {
        v = v2;
        i = i2;
    }
}

template <typename T>
__global__ void argmax_stage1(const T* __restrict__ x, long long n, int chunks, double* __restrict__ pv,
                              long long* __restrict__ pi)
{
    const int b = blockIdx.y, c = blockIdx.x;
    const long long per = (n + chunks - 1) / chunks;
    const long long lo = (long long)c * per, hi = lo + per < n ? lo + per : n;
    const T* xb = x + (long long)b * n;
    double v = -DBL_MAX;
    long long idx = n;
    for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) better(v, idx, (double)xb[i], i);
    __shared__ double sv[256];
    __shared__ long long si[256];
    sv[threadIdx.x] = v;
    si[threadIdx.x] = idx;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            double v2 = sv[threadIdx.x + s];
            long long i2 = si[threadIdx.x + s];
            double v1 = sv[threadIdx.x];
            long long i1 = si[threadIdx.x];
            better(v1, i1, v2, i2);
            sv[threadIdx.x] = v1;
            si[threadIdx.x] = i1;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        pv[(long long)b * chunks + c] = sv[0];
        pi[(long long)b * chunks + c] = si[0];
    }
}

__global__ void argmax_stage2(const double* __restrict__ pv, const long long* __restrict__ pi, int chunks,
                              double* __restrict__ ov, long long* __restrict__ oi)
{
    const int b = blockIdx.x;
    double v = -DBL_MAX;
    long long idx = 0x7fffffffffffffffLL;
    for (int c = threadIdx.x; c < chunks; c += blockDim.x)
        better(v, idx, pv[(long long)b * chunks + c], pi[(long long)b * chunks + c]);
    __shared__ double sv[256];
    __shared__ long long si[256];
    sv[threadIdx.x] = v;
    si[threadIdx.x] = idx;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            double v1 = sv[threadIdx.x];
            long long i1 = si[threadIdx.x];
            better(v1, i1, sv[threadIdx.x + s], si[threadIdx.x + s]);
            sv[threadIdx.x] = v1;
            si[threadIdx.x] = i1;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        ov[b] = sv[0];
        oi[b] = si[0];
    }
}

// scratch: chunks * nb doubles + chunks * nb long longs + nb doubles + nb long longs
size_t argmax_scratch_bytes(int nb, int chunks) { return (size_t)(nb * (size_t)chunks + nb) * 16; }

cudaError_t launch_argmax(const void* x, bool fp64, long long n, int nb, int chunks, void* scratch, double* ov,
                          long long* oi, cudaStream_t st)
{
    double* pv = (double*)scratch;
    long long* pi = (long long*)(pv + (size_t)nb * chunks);
    dim3 g1(chunks, nb);
    if (fp64)
        argmax_stage1<double><<<g1, 256, 0, st>>>((const double*)x, n, chunks, pv, pi);
    else
        argmax_stage1<float><<<g1, 256, 0, st>>>((const float*)x, n, chunks, pv, pi);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    argmax_stage2<<<nb, 256, 0, st>>>(pv, pi, chunks, ov, oi);
    return cudaGetLastError();
}

}  // namespace fftso3
