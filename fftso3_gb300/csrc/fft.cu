// Batched 1-D complex FFT along one axis of a strided array, for the (alpha,gamma)
// transforms of the SO(3) path and the phi transform of the S^2 path.
//
// Replaces the per-row / per-column Eigen::FFT<double>::fwd calls of
// fdcl_FFTSO3.cpp:689-698 and fdcl_FFTS2.cpp:153 (unscaled forward DFT,
// X[p] = sum_j x[j] e^{-2 pi i p j / N}).
//
// Design: one CTA transforms `lpb` lines held in shared memory with a
// Stockham auto-sort FFT (mixed radix 8/4/2, small odd radices 3/5/7 and a
// generic O(p^2) pass for larger prime factors, so any N = 2B works).  Lines
// are addressed as  base(i) = (i / inner) * ostride + (i % inner) * istride,
// element j at base + j * es; when consecutive lines are adjacent in memory
// (the column pass) the global loads/stores run line-fastest so each warp
// touches contiguous segments.  Twiddles come from an FP64 host table
// W[i] = e^{-2 pi i i / N} staged in shared memory.
#include "common.cuh"
#include "fft.cuh"

namespace fftso3 {

template <typename T> struct V2;
template <> struct V2<double> {
    using t = double2;
    __device__ static inline double2 mk(double a, double b) { return make_double2(a, b); }
};
template <> struct V2<float> {
    using t = float2;
    __device__ static inline float2 mk(float a, float b) { return make_float2(a, b); }
};

template <typename C> __device__ __forceinline__ C cadd(C a, C b) { a.x += b.x; a.y += b.y; return a; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { a.x -= b.x; a.y -= b.y; return a; }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
    C r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
// multiply by -i
template <typename C> __device__ __forceinline__ C mul_mi(C a) { C r; r.x = a.y; r.y = -a.x; return r; }

template <typename T, int R>
__device__ __forceinline__ void dft_small(typename V2<T>::t* v, const typename V2<T>::t* w, int Nr)
{
    using C = typename V2<T>::t;
    if constexpr (R == 2) {
        C a = v[0], b = v[1];
        v[0] = cadd(a, b); v[1] = csub(a, b);
    } else if constexpr (R == 4) {
        C a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
        C b0 = cadd(v[1], v[3]), b1 = mul_mi(csub(v[1], v[3]));
        v[0] = cadd(a0, b0); v[2] = csub(a0, b0);
        v[1] = cadd(a1, b1); v[3] = csub(a1, b1);
    } else if constexpr (R == 8) {
        const T h = (T)0.70710678118654752440;
        // radix-2 first level across distance 4
        C a[4], b[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) { a[t] = cadd(v[t], v[t + 4]); b[t] = csub(v[t], v[t + 4]); }
        // b[t] *= W8^t
        b[1] = V2<T>::mk(h * (b[1].x + b[1].y), h * (b[1].y - b[1].x));
        b[2] = mul_mi(b[2]);
        b[3] = V2<T>::mk(h * (b[3].y - b[3].x), -h * (b[3].x + b[3].y));
        // two radix-4 on a (even outputs) and b (odd outputs)
        C a0 = cadd(a[0], a[2]), a1 = csub(a[0], a[2]);
        C a2 = cadd(a[1], a[3]), a3 = mul_mi(csub(a[1], a[3]));
        v[0] = cadd(a0, a2); v[4] = csub(a0, a2);
        v[2] = cadd(a1, a3); v[6] = csub(a1, a3);
        C b0 = cadd(b[0], b[2]), b1 = csub(b[0], b[2]);
        C b2 = cadd(b[1], b[3]), b3 = mul_mi(csub(b[1], b[3]));
        v[1] = cadd(b0, b2); v[5] = csub(b0, b2);
        v[3] = cadd(b1, b3); v[7] = csub(b1, b3);
    } else {
        // odd radix: out[q] = sum_t v[t] w^{tq}, w = e^{-2 pi i / R} = W_N^{N/R}
        C o[R];
#pragma unroll
        for (int q = 0; q < R; ++q) {
            C s = v[0];
#pragma unroll
            for (int t = 1; t < R; ++t) s = cadd(s, cmul(v[t], w[((t * q) % R) * Nr]));
            o[q] = s;
        }
#pragma unroll
        for (int q = 0; q < R; ++q) v[q] = o[q];
    }
}

template <typename T, int R>
__device__ __forceinline__ void stockham_stage(const typename V2<T>::t* __restrict__ src,
                                               typename V2<T>::t* __restrict__ dst,
                                               const typename V2<T>::t* __restrict__ w,
                                               int N, int Ns, int lpb, int LS)
{
    using C = typename V2<T>::t;
    const int Nr = N / R;
    const int total = lpb * Nr;
    const int tstride = N / (Ns * R);
    for (int b = threadIdx.x; b < total; b += blockDim.x) {
        int l = b / Nr, j = b - l * Nr;
        int k = j % Ns;
        const C* s = src + l * LS;
        C v[R];
#pragma unroll
        for (int t = 0; t < R; ++t) v[t] = s[j + t * Nr];
        if (Ns > 1) {
            int e = k * tstride;
#pragma unroll
            for (int t = 1; t < R; ++t) v[t] = cmul(v[t], w[t * e]);
        }
        dft_small<T, R>(v, w, Nr);
        C* d = dst + l * LS + (j - k) * R + k;
#pragma unroll
        for (int t = 0; t < R; ++t) d[t * Ns] = v[t];
    }
}

// Generic radix (any prime R): one output per thread, O(R) work each.
template <typename T>
__device__ void stockham_generic(const typename V2<T>::t* __restrict__ src, typename V2<T>::t* __restrict__ dst,
                                 const typename V2<T>::t* __restrict__ w, int N, int Ns, int R, int lpb, int LS)
{
    using C = typename V2<T>::t;
    const int Nr = N / R;
    const int total = lpb * N;
    const int tstride = N / (Ns * R);
    for (int b = threadIdx.x; b < total; b += blockDim.x) {
        int l = b / N, o = b - l * N;
        int k = o % Ns;
        int q = (o / Ns) % R;
        int jb = o / (Ns * R);
        int j = jb * Ns + k;
        const C* s = src + l * LS;
        C acc = s[j];
        for (int t = 1; t < R; ++t) {
            // twiddle W_N^{t k N/(Ns R)} times DFT factor W_N^{t q N/R}
            long long e = ((long long)t * k * tstride + (long long)((t * q) % R) * Nr) % N;
            acc = cadd(acc, cmul(s[j + t * Nr], w[e]));
        }
        dst[l * LS + o] = acc;
    }
}

template <typename T, typename TIN, bool REAL_IN, bool REAL_OUT>
__global__ void __launch_bounds__(256) fft_lines_kernel(const TIN* __restrict__ in, void* __restrict__ out, FFTFactors fac,
                                                        long long nlines, int lpb_log2, long long inner, long long ostride,
                                                        long long istride, long long es, const void* __restrict__ twg,
                                                        int lines_fastest)
{
    using C = typename V2<T>::t;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int N = fac.N;
    const int LS = N + 1;
    const int lpb = 1 << lpb_log2;
    C* w = reinterpret_cast<C*>(smem_raw);
    C* buf0 = w + N;
    C* buf1 = buf0 + lpb * LS;
    long long* base = reinterpret_cast<long long*>(buf1 + lpb * LS);
    const double2* tw = reinterpret_cast<const double2*>(twg);
    for (int i = threadIdx.x; i < N; i += blockDim.x) w[i] = V2<T>::mk((T)tw[i].x, (T)tw[i].y);

    const long long line0 = (long long)blockIdx.x * lpb;
    const int nl = (int)min((long long)lpb, nlines - line0);
    if (threadIdx.x < lpb) {
        long long i = line0 + threadIdx.x;
        base[threadIdx.x] = (i / inner) * ostride + (i % inner) * istride;
    }
    __syncthreads();
    const int tot = lpb * N;
    // load (per-line base offsets precomputed; no per-element 64-bit division)
    if (lines_fastest) {
        for (int e = threadIdx.x; e < tot; e += blockDim.x) {
            const int l = e & (lpb - 1), j = e >> lpb_log2;
            if (l >= nl) continue;
            const long long off = base[l] + (long long)j * es;
            if constexpr (REAL_IN) buf0[l * LS + j] = V2<T>::mk((T)in[off], (T)0);
            else buf0[l * LS + j] = in[off];
        }
    } else {
        for (int l = 0; l < nl; ++l) {
            const long long b0 = base[l];
            for (int j = threadIdx.x; j < N; j += blockDim.x) {
                const long long off = b0 + (long long)j * es;
                if constexpr (REAL_IN) buf0[l * LS + j] = V2<T>::mk((T)in[off], (T)0);
                else buf0[l * LS + j] = in[off];
            }
        }
    }
    __syncthreads();
    C* src = buf0;
    C* dst = buf1;
    int Ns = 1;
    for (int s = 0; s < fac.n; ++s) {
        const int R = fac.r[s];
        switch (R) {
            case 2: stockham_stage<T, 2>(src, dst, w, N, Ns, lpb, LS); break;
            case 3: stockham_stage<T, 3>(src, dst, w, N, Ns, lpb, LS); break;
            case 4: stockham_stage<T, 4>(src, dst, w, N, Ns, lpb, LS); break;
            case 5: stockham_stage<T, 5>(src, dst, w, N, Ns, lpb, LS); break;
            case 7: stockham_stage<T, 7>(src, dst, w, N, Ns, lpb, LS); break;
            case 8: stockham_stage<T, 8>(src, dst, w, N, Ns, lpb, LS); break;
            default: stockham_generic<T>(src, dst, w, N, Ns, R, lpb, LS); break;
        }
        __syncthreads();
        C* t = src; src = dst; dst = t;
        Ns *= R;
    }
    // store
    if (lines_fastest) {
        for (int e = threadIdx.x; e < tot; e += blockDim.x) {
            const int l = e & (lpb - 1), j = e >> lpb_log2;
            if (l >= nl) continue;
            const long long off = base[l] + (long long)j * es;
            const C v = src[l * LS + j];
            if constexpr (REAL_OUT) reinterpret_cast<T*>(out)[off] = v.x;
            else reinterpret_cast<C*>(out)[off] = v;
        }
    } else {
        for (int l = 0; l < nl; ++l) {
            const long long b0 = base[l];
            for (int j = threadIdx.x; j < N; j += blockDim.x) {
                const long long off = b0 + (long long)j * es;
                const C v = src[l * LS + j];
                if constexpr (REAL_OUT) reinterpret_cast<T*>(out)[off] = v.x;
                else reinterpret_cast<C*>(out)[off] = v;
            }
        }
    }
}

void make_fft_factors(int N, FFTFactors& f)
{
    f.N = N;
    f.n = 0;
    int r = N;
    while (r % 8 == 0) { f.r[f.n++] = 8; r /= 8; }
    while (r % 4 == 0) { f.r[f.n++] = 4; r /= 4; }
    while (r % 2 == 0) { f.r[f.n++] = 2; r /= 2; }
    for (int p = 3; r > 1; p += 2) {
        while (r % p == 0) { f.r[f.n++] = p; r /= p; }
    }
}

size_t fft_smem_bytes(int N, int lpb, bool fp64)
{
    size_t c = fp64 ? 16 : 8;
    return c * ((size_t)N + 2 * (size_t)lpb * (N + 1)) + 8 * (size_t)lpb;
}

template <typename T, typename TIN, bool RI, bool RO>
static cudaError_t launch_one(const void* in, void* out, const FFTFactors& fac, long long nlines, int lpb,
                              long long inner, long long ostride, long long istride, long long es,
                              const void* tw, bool lines_fastest, cudaStream_t st)
{
    size_t smem = fft_smem_bytes(fac.N, lpb, sizeof(T) == 8);
    auto kern = fft_lines_kernel<T, TIN, RI, RO>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int lg = 0;
    while ((1 << lg) < lpb) ++lg;
    if ((1 << lg) != lpb || lpb > 256) return cudaErrorInvalidValue;  // lines per CTA: power of two
    long long nblk = (nlines + lpb - 1) / lpb;
    kern<<<(unsigned)nblk, 256, smem, st>>>(reinterpret_cast<const TIN*>(in), out, fac, nlines, lg, inner, ostride,
                                            istride, es, tw, lines_fastest ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_fft_lines(const FFTLaunch& L, cudaStream_t st)
{
    if (L.fp64) {
        if (L.real_in && L.real_out) return cudaErrorInvalidValue;
        if (L.real_in)
            return launch_one<double, double, true, false>(L.in, L.out, L.fac, L.nlines, L.lpb, L.inner, L.ostride,
                                                           L.istride, L.es, L.tw, L.lines_fastest, st);
        if (L.real_out)
            return launch_one<double, double2, false, true>(L.in, L.out, L.fac, L.nlines, L.lpb, L.inner, L.ostride,
                                                            L.istride, L.es, L.tw, L.lines_fastest, st);
        return launch_one<double, double2, false, false>(L.in, L.out, L.fac, L.nlines, L.lpb, L.inner, L.ostride,
                                                         L.istride, L.es, L.tw, L.lines_fastest, st);
    } else {
        if (L.real_in && L.real_out) return cudaErrorInvalidValue;
        if (L.real_in)
            return launch_one<float, float, true, false>(L.in, L.out, L.fac, L.nlines, L.lpb, L.inner, L.ostride,
                                                         L.istride, L.es, L.tw, L.lines_fastest, st);
        if (L.real_out)
            return launch_one<float, float2, false, true>(L.in, L.out, L.fac, L.nlines, L.lpb, L.inner, L.ostride,
                                                          L.istride, L.es, L.tw, L.lines_fastest, st);
        return launch_one<float, float2, false, false>(L.in, L.out, L.fac, L.nlines, L.lpb, L.inner, L.ostride,
                                                       L.istride, L.es, L.tw, L.lines_fastest, st);
    }
}

}  // namespace fftso3
