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
#include "df32.cuh"
#include "fft.cuh"
#include "fused.cuh"

namespace fftso3 {

template <typename T> struct V2;
template <> struct V2<df32> {
    using t = dfc32;
    __device__ static inline dfc32 mk(df32 a, df32 b) { return dfc32{a, b}; }
};
template <> struct V2<double> {
    using t = double2;
    __device__ static inline double2 mk(double a, double b) { return make_double2(a, b); }
};
template <> struct V2<float> {
    using t = float2;
    __device__ static inline float2 mk(float a, float b) { return make_float2(a, b); }
};
template <> struct V2<qf32> {
    using t = qc32;
    __device__ static inline qc32 mk(qf32 a, qf32 b) { return qc32{a, b}; }
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

// Position of element i of a staged line: plain, or (PAD) one padding slot after every 8 elements, so that the
// stride-R writes of a Stockham stage (and the other strided walks) spread over the shared-memory banks.
template <bool PAD> __device__ __forceinline__ int lpos(int i) { return PAD ? i + (i >> 3) : i; }

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
        // odd radix R = 3, 5, 7 in the symmetric form (P = (R-1)/2):
        //   out[q], out[R-q] = v0 + sum_{t<=P} a_t cos(2 pi t q / R) -/+ i b_t sin(2 pi t q / R),
        //   a_t = v_t + v_{R-t}, b_t = v_t - v_{R-t};  w[((t q) mod R) Nr] = (cos, -sin)
        constexpr int P = (R - 1) / 2;
        C a[P + 1], b[P + 1];
        C o0 = v[0];
#pragma unroll
        for (int t = 1; t <= P; ++t) {
            a[t] = cadd(v[t], v[R - t]);
            b[t] = csub(v[t], v[R - t]);
            o0 = cadd(o0, a[t]);
        }
        C o[R];
        o[0] = o0;
#pragma unroll
        for (int q = 1; q <= P; ++q) {
            C cs = v[0], sn = V2<T>::mk((T)0, (T)0);
#pragma unroll
            for (int t = 1; t <= P; ++t) {
                const C wv = w[((t * q) % R) * Nr];
                cs.x += a[t].x * wv.x;
                cs.y += a[t].y * wv.x;
                sn.x -= b[t].x * wv.y;
                sn.y -= b[t].y * wv.y;
            }
            o[q] = V2<T>::mk(cs.x + sn.y, cs.y - sn.x);
            o[R - q] = V2<T>::mk(cs.x - sn.y, cs.y + sn.x);
        }
#pragma unroll
        for (int q = 0; q < R; ++q) v[q] = o[q];
    }
}

// The radix-8 DFT of dft_small in quantised double-float (df32.cuh): the W8 factors are products with the
// double-float constant 1/sqrt(2), everything else exact sums of the high parts.
__device__ __forceinline__ void dft8_q(qc32* v, float magic)
{
    const df32 h(0.70710678118654752440);
    qc32 a[4], b[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) { a[t] = cadd(v[t], v[t + 4]); b[t] = csub(v[t], v[t + 4]); }
    b[1] = qc32{q_mul(b[1].x + b[1].y, h, magic), q_mul(b[1].y - b[1].x, h, magic)};
    b[2] = mul_mi(b[2]);
    b[3] = qc32{q_mul(b[3].y - b[3].x, h, magic), -q_mul(b[3].x + b[3].y, h, magic)};
    qc32 a0 = cadd(a[0], a[2]), a1 = csub(a[0], a[2]);
    qc32 a2 = cadd(a[1], a[3]), a3 = mul_mi(csub(a[1], a[3]));
    v[0] = cadd(a0, a2); v[4] = csub(a0, a2);
    v[2] = cadd(a1, a3); v[6] = csub(a1, a3);
    qc32 b0 = cadd(b[0], b[2]), b1 = csub(b[0], b[2]);
    qc32 b2 = cadd(b[1], b[3]), b3 = mul_mi(csub(b[1], b[3]));
    v[1] = cadd(b0, b2); v[5] = csub(b0, b2);
    v[3] = cadd(b1, b3); v[7] = csub(b1, b3);
}

template <int R> __device__ __forceinline__ void dft_q(qc32* v, float magic)
{
    if constexpr (R == 8) dft8_q(v, magic);
    else dft_small<qf32, R>(v, nullptr, 0);
}

// The quantum of a CTA's block of data (df32.cuh): m = this thread's largest |component|, red 8 floats of shared
// memory; returns magic = 1.5 * 2^23 q with q = 2^(E - G), 2^E > the block's largest |component| and
// G = 20 - log2 N: a pass of N points grows a component at most N sqrt(2)-fold, which keeps every value below
// 2^(E + log2 N + 1/2) < 2^22 q (the range of the rounding to the quantum) with a bit to spare.
template <int N> __device__ __forceinline__ float q_block_magic(float m, float* red)
{
    constexpr int G = 20 - (N == 512 ? 9 : N == 256 ? 8 : N == 128 ? 7 : 6);
#pragma unroll
    for (int s = 16; s; s >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, s));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    m = red[0];
#pragma unroll
    for (int i = 1; i < 8; ++i) m = fmaxf(m, red[i]);
    const int eb = (__float_as_int(m) >> 23) & 0xff;  // biased exponent (0: zero or subnormal)
    int e = eb - 126 - G + 23;                        // exponent of 2^23 q
    e = e < -100 ? -100 : e > 120 ? 120 : e;
    return 1.5f * __int_as_float((e + 127) << 23);
}

// One Stockham pass of radix R over the lpb lines in shared memory.  Thread
// items b = threadIdx.x + i blockDim.x map to (line l, butterfly j) and the
// twiddle class k = j mod Ns; they advance by constant steps (Nr is a
// multiple of Ns, so k survives the wrap of j), so the loop does no division.
template <typename T, int R, bool PAD = false>
__device__ __forceinline__ void stockham_stage(const typename V2<T>::t* __restrict__ src,
                                               typename V2<T>::t* __restrict__ dst,
                                               const typename V2<T>::t* __restrict__ w,
                                               int N, int Ns, int lpb, int LS)
{
    using C = typename V2<T>::t;
    const int Nr = N / R;
    const int total = lpb * Nr;
    const int tstride = N / (Ns * R);
    const int nt = blockDim.x;
    const int linc = nt / Nr, jinc = nt - linc * Nr, kinc = jinc % Ns;
    int l = threadIdx.x / Nr, j = threadIdx.x - l * Nr, k = j % Ns;
    for (int b = threadIdx.x; b < total; b += nt) {
        const C* s = src + l * LS;
        C v[R];
#pragma unroll
        for (int t = 0; t < R; ++t) v[t] = s[lpos<PAD>(j + t * Nr)];
        if (Ns > 1) {
            int e = k * tstride;
#pragma unroll
            for (int t = 1; t < R; ++t) v[t] = cmul(v[t], w[t * e]);
        }
        dft_small<T, R>(v, w, Nr);
        C* d = dst + l * LS;
        const int o = (j - k) * R + k;
#pragma unroll
        for (int t = 0; t < R; ++t) d[lpos<PAD>(o + t * Ns)] = v[t];
        l += linc;
        j += jinc;
        k += kinc;
        if (k >= Ns) k -= Ns;
        if (j >= Nr) {
            j -= Nr;
            ++l;
        }
    }
}

// Generic radix (any prime R): each thread forms GQ outputs q of one
// (line, j) group, sharing the R loads; the twiddle exponent of term t,
// t (k tstride + q Nr) mod N, advances by one add and one conditional
// subtract per term (no division in the inner loop).  Terms are summed in
// ascending t, the plain DFT order.
template <typename T, bool PAD = false>
__device__ void stockham_generic(const typename V2<T>::t* __restrict__ src, typename V2<T>::t* __restrict__ dst,
                                 const typename V2<T>::t* __restrict__ w, int N, int Ns, int R, int lpb, int LS)
{
    using C = typename V2<T>::t;
    constexpr int GQ = 4;
    const int Nr = N / R;
    const int nqb = (R + GQ - 1) / GQ;
    const int per_line = Nr * nqb;
    const int total = lpb * per_line;
    const int tstride = N / (Ns * R);
    for (int b = threadIdx.x; b < total; b += blockDim.x) {
        const int l = b / per_line, rem = b - l * per_line;
        const int qb = rem / Nr, j = rem - qb * Nr;
        const int k = j % Ns;
        const C* s = src + l * LS;
        C acc[GQ];
        int e[GQ], step[GQ];
        const C x0 = s[lpos<PAD>(j)];
#pragma unroll
        for (int u = 0; u < GQ; ++u) {
            acc[u] = x0;
            int st = k * tstride + (qb * GQ + u) * Nr;
            st = st >= N ? st - N : st;
            step[u] = st;
            e[u] = st;
        }
        for (int t = 1; t < R; ++t) {
            const C v = s[lpos<PAD>(j + t * Nr)];
#pragma unroll
            for (int u = 0; u < GQ; ++u) {
                acc[u] = cadd(acc[u], cmul(v, w[e[u]]));
                const int ne = e[u] + step[u];
                e[u] = ne >= N ? ne - N : ne;
            }
        }
        C* d = dst + l * LS;
        const int o = (j - k) * R + k;
#pragma unroll
        for (int u = 0; u < GQ; ++u) {
            const int q = qb * GQ + u;
            if (q < R) d[lpos<PAD>(o + q * Ns)] = acc[u];
        }
    }
}

// First stage (Ns = 1) of a prime radix R > 8: the plain R-point DFTs of the
// stride-Nr subsequences, X[j R + q] = sum_t x[j + t Nr] e^{-2 pi i t q / R},
// in the symmetric form (P = (R-1)/2, a_t = x_t + x_{R-t}, b_t = x_t - x_{R-t}):
//   X[q]     = x_0 + sum_{t<=P} a_t cos(2 pi t q / R) - i b_t sin(2 pi t q / R)
//   X[R - q] = x_0 + sum_{t<=P} a_t cos(2 pi t q / R) + i b_t sin(2 pi t q / R)
// which takes about R real FMAs per output instead of 4R.  The (cos, sin)
// matrix of the R-point DFT, mat[(t-1) P4 + (q-1)], is built per CTA in shared
// memory.  Each thread forms the outputs q and R - q of GP consecutive q for
// LPT lines (l and l + lpb/2 when lpb >= 2), so one matrix read feeds
// 4 LPT FMAs; work items run (j, line) fastest, so the lanes of a warp share
// one block of q and every matrix read is a broadcast.
template <typename T, int LPT, int GP = 4, bool PAD = false>
__device__ void dft_prime_first_t(const typename V2<T>::t* __restrict__ src, typename V2<T>::t* __restrict__ dst,
                                  const typename V2<T>::t* __restrict__ mat, int N, int R, int lpb, int LS)
{
    using C = typename V2<T>::t;
    const int Nr = N / R;
    const int P = (R - 1) / 2;
    const int MS = (P + 3) / 4 * 4;             // row stride of the matrix (as built: a multiple of 4)
    const int nblk = (P + GP - 1) / GP;
    const int lgroups = lpb / LPT;               // line l and l + lgroups share each matrix read
    const int per_blk = Nr * lgroups;
    const int total = per_blk * nblk;
    for (int b = threadIdx.x; b < total; b += blockDim.x) {
        const int blk = b / per_blk, rem = b - blk * per_blk;
        const int l = rem / Nr, j = rem - l * Nr;
        const C* s[LPT];
        C x0[LPT], acc0[LPT], Cs[LPT][GP], Ss[LPT][GP];
#pragma unroll
        for (int u = 0; u < LPT; ++u) {
            s[u] = src + (l + u * lgroups) * LS;
            x0[u] = s[u][lpos<PAD>(j)];
            acc0[u] = x0[u];
#pragma unroll
            for (int g = 0; g < GP; ++g) {
                Cs[u][g] = V2<T>::mk((T)0, (T)0);
                Ss[u][g] = V2<T>::mk((T)0, (T)0);
            }
        }
        const C* m = mat + blk * GP;
        for (int t = 1; t <= P; ++t, m += MS) {
            C a[LPT], bb[LPT];
#pragma unroll
            for (int u = 0; u < LPT; ++u) {
                const C xt = s[u][lpos<PAD>(j + t * Nr)], xr = s[u][lpos<PAD>(j + (R - t) * Nr)];
                a[u] = cadd(xt, xr);
                bb[u] = csub(xt, xr);
                acc0[u] = cadd(acc0[u], a[u]);
            }
#pragma unroll
            for (int g = 0; g < GP; ++g) {
                const C cs = m[g];  // (cos, sin)
#pragma unroll
                for (int u = 0; u < LPT; ++u) {
                    Cs[u][g].x += a[u].x * cs.x;
                    Cs[u][g].y += a[u].y * cs.x;
                    Ss[u][g].x += bb[u].x * cs.y;
                    Ss[u][g].y += bb[u].y * cs.y;
                }
            }
        }
#pragma unroll
        for (int u = 0; u < LPT; ++u) {
            C* d = dst + (l + u * lgroups) * LS;
            const int o = j * R;
            if (blk == 0) d[lpos<PAD>(o)] = acc0[u];
#pragma unroll
            for (int g = 0; g < GP; ++g) {
                const int q = 1 + blk * GP + g;
                if (q <= P) {
                    const C base = cadd(x0[u], Cs[u][g]);
                    d[lpos<PAD>(o + q)] = V2<T>::mk(base.x + Ss[u][g].y, base.y - Ss[u][g].x);
                    d[lpos<PAD>(o + R - q)] = V2<T>::mk(base.x - Ss[u][g].y, base.y + Ss[u][g].x);
                }
            }
        }
    }
}

template <typename T>
__device__ void dft_prime_first(const typename V2<T>::t* __restrict__ src, typename V2<T>::t* __restrict__ dst,
                                const typename V2<T>::t* __restrict__ mat, int N, int R, int lpb, int LS)
{
    if (lpb >= 2)
        dft_prime_first_t<T, 2>(src, dst, mat, N, R, lpb, LS);
    else
        dft_prime_first_t<T, 1>(src, dst, mat, N, R, lpb, LS);
}

// entries of the (cos, sin) matrix used by dft_prime_first for prime radix R
__host__ __device__ inline int prime_mat_entries(int R)
{
    const int P = (R - 1) / 2;
    return P * ((P + 3) / 4 * 4);
}

// Real data, two lines per transform: with REAL_IN the real lines 2p and 2p+1
// are transformed together as z = x_{2p} + i x_{2p+1} and separated with
// X[k] = (Z[k] + conj Z[-k]) / 2, Y[k] = (Z[k] - conj Z[-k]) / 2i; with REAL_OUT
// (the input spectra are those of real lines) z = X_{2p} + i X_{2p+1} and the
// real and imaginary parts of its transform are the two lines.  Either way the
// CTA transforms lpb / 2 complex lines.
template <typename T, typename TIN, bool REAL_IN, bool REAL_OUT>
__global__ void __launch_bounds__(256) fft_lines_kernel(const TIN* __restrict__ in, void* __restrict__ out, FFTFactors fac,
                                                        long long nlines, int lpb_log2, long long inner, long long ostride,
                                                        long long istride, long long es, const void* __restrict__ twg,
                                                        int lines_fastest)
{
    using C = typename V2<T>::t;
    constexpr bool PACK = REAL_IN || REAL_OUT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int N = fac.N;
    const int LS = N + 1;
    const int lpb = 1 << lpb_log2;
    const int lbuf = PACK ? lpb / 2 : lpb;  // complex lines transformed by the CTA
    C* w = reinterpret_cast<C*>(smem_raw);
    C* buf0 = w + N;
    C* buf1 = buf0 + lbuf * LS;
    long long* base = reinterpret_cast<long long*>(buf1 + lbuf * LS);
    C* mat = reinterpret_cast<C*>(base + lpb);  // prime-first DFT matrix (only when fac.r[0] > 8)
    const double2* tw = reinterpret_cast<const double2*>(twg);
    for (int i = threadIdx.x; i < N; i += blockDim.x) w[i] = V2<T>::mk((T)tw[i].x, (T)tw[i].y);
    if (fac.r[0] > 8) {
        const int R = fac.r[0], P = (R - 1) / 2, P4 = (P + 3) / 4 * 4, Nr = N / R;
        for (int i = threadIdx.x; i < P * P4; i += blockDim.x) {
            const int t = i / P4 + 1, q = i - (t - 1) * P4 + 1;
            T c = 0, sn = 0;
            if (q <= P) {
                const double2 v = tw[((t * q) % R) * Nr];  // e^{-2 pi i t q / R}
                c = (T)v.x;
                sn = (T)(-v.y);
            }
            mat[i] = V2<T>::mk(c, sn);
        }
    }

    const long long line0 = (long long)blockIdx.x * lpb;
    const int nl = (int)min((long long)lpb, nlines - line0);  // even when PACK (nlines, lpb even)
    for (int t = threadIdx.x; t < lpb; t += blockDim.x) {
        const long long i = line0 + t;
        base[t] = (i / inner) * ostride + (i % inner) * istride;
    }
    __syncthreads();
    // load (per-line base offsets precomputed; no per-element 64-bit division)
    if (REAL_OUT) {
        // pairs (2p, 2p+1) of complex spectra -> X_{2p} + i X_{2p+1}
        const int np2 = nl / 2;
        for (int e = threadIdx.x; e < lbuf * N; e += blockDim.x) {
            int p2, j;
            if (lines_fastest) {
                p2 = e & (lbuf - 1);
                j = e >> (lpb_log2 - 1);
            } else {
                p2 = e / N;
                j = e - p2 * N;
            }
            if (p2 >= np2) continue;
            const C a = reinterpret_cast<const C*>(in)[base[2 * p2] + (long long)j * es];
            const C b = reinterpret_cast<const C*>(in)[base[2 * p2 + 1] + (long long)j * es];
            buf0[p2 * LS + j] = V2<T>::mk(a.x - b.y, a.y + b.x);
        }
    } else if (lines_fastest) {
        for (int e = threadIdx.x; e < lpb * N; e += blockDim.x) {
            const int l = e & (lpb - 1), j = e >> lpb_log2;
            if (l >= nl) continue;
            const long long off = base[l] + (long long)j * es;
            if constexpr (REAL_IN) reinterpret_cast<T*>(buf0)[2 * ((l >> 1) * LS + j) + (l & 1)] = (T)in[off];
            else buf0[l * LS + j] = reinterpret_cast<const C*>(in)[off];
        }
    } else {
        const int linc = blockDim.x / N, jinc = blockDim.x - linc * N;
        int l = threadIdx.x / N, j = threadIdx.x - l * N;
        for (int e = threadIdx.x; e < nl * N; e += blockDim.x) {
            const long long off = base[l] + (long long)j * es;
            if constexpr (REAL_IN) reinterpret_cast<T*>(buf0)[2 * ((l >> 1) * LS + j) + (l & 1)] = (T)in[off];
            else buf0[l * LS + j] = reinterpret_cast<const C*>(in)[off];
            l += linc;
            j += jinc;
            if (j >= N) {
                j -= N;
                ++l;
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
            case 2: stockham_stage<T, 2>(src, dst, w, N, Ns, lbuf, LS); break;
            case 3: stockham_stage<T, 3>(src, dst, w, N, Ns, lbuf, LS); break;
            case 4: stockham_stage<T, 4>(src, dst, w, N, Ns, lbuf, LS); break;
            case 5: stockham_stage<T, 5>(src, dst, w, N, Ns, lbuf, LS); break;
            case 7: stockham_stage<T, 7>(src, dst, w, N, Ns, lbuf, LS); break;
            case 8: stockham_stage<T, 8>(src, dst, w, N, Ns, lbuf, LS); break;
            default:
                if (Ns == 1) dft_prime_first<T>(src, dst, mat, N, R, lbuf, LS);
                else stockham_generic<T>(src, dst, w, N, Ns, R, lbuf, LS);
                break;
        }
        __syncthreads();
        C* t = src; src = dst; dst = t;
        Ns *= R;
    }
    // store
    auto value = [&](int l, int j) -> C {
        if constexpr (REAL_IN) {
            const C z = src[(l >> 1) * LS + j], zm = src[(l >> 1) * LS + (j == 0 ? 0 : N - j)];
            return (l & 1) ? V2<T>::mk((T)0.5 * (z.y + zm.y), (T)-0.5 * (z.x - zm.x))
                           : V2<T>::mk((T)0.5 * (z.x + zm.x), (T)0.5 * (z.y - zm.y));
        } else if constexpr (REAL_OUT) {
            const C z = src[(l >> 1) * LS + j];
            return V2<T>::mk((l & 1) ? z.y : z.x, (T)0);
        } else {
            return src[l * LS + j];
        }
    };
    if (lines_fastest) {
        for (int e = threadIdx.x; e < lpb * N; e += blockDim.x) {
            const int l = e & (lpb - 1), j = e >> lpb_log2;
            if (l >= nl) continue;
            const long long off = base[l] + (long long)j * es;
            const C v = value(l, j);
            if constexpr (REAL_OUT) reinterpret_cast<T*>(out)[off] = v.x;
            else reinterpret_cast<C*>(out)[off] = v;
        }
    } else {
        const int linc = blockDim.x / N, jinc = blockDim.x - linc * N;
        int l = threadIdx.x / N, j = threadIdx.x - l * N;
        for (int e = threadIdx.x; e < nl * N; e += blockDim.x, l += linc, j += jinc) {
            if (j >= N) {
                j -= N;
                ++l;
            }
            const long long off = base[l] + (long long)j * es;
            const C v = value(l, j);
            if constexpr (REAL_OUT) reinterpret_cast<T*>(out)[off] = v.x;
            else reinterpret_cast<C*>(out)[off] = v;
        }
    }
}

// ---- double-float FFT along a strided axis of k-contiguous arrays (the refinement's forward FFT and the exact
// inverse's synthesis FFT)
//
// Arithmetic: quantised double-float (df32.cuh), the quantum set per CTA from the largest component of its TK
// lines, so the butterflies' sums need no two-sum; data in and out of the kernel are ordinary double-float pairs.
// The high parts are renormalised after the first stages, so a pass keeps about 2^(-24 - G) of the CTA's
// largest input per operation (G = 20 - log2 N, q_block_magic).
//
// Line (o, k): element j at obase(o) + k + j S, obase(o) = (o / oinner) oouter + (o % oinner) oistride.  One CTA
// transforms TK = 2048 / N consecutive k of one o (N = 64..512, a power of two) with 256 threads: radix-8
// Stockham stages (a last radix-4 or 2 stage when log2 N is not a multiple of 3), each thread holding the 8
// values of one butterfly in registers.  The first stage reads its butterflies straight from global memory and
// the last one writes them straight back, with the threads of a warp on consecutive k (TK consecutive elements
// per j); the stages in between exchange through shared memory with the threads of a line side by side.
// Shared-memory layout, so that the accesses of a warp fill whole 16-byte bank groups:
//   rows padded by one element per 8 (phys(i) = i + i / 8): a stage's strided reads and scattered writes;
//   row stride N + N / 8 + 1 elements (+ 2 at N = 512, four rows per CTA): the k-fastest first / last stages;
//   twiddles per stage as [r - 1][kt] (kt = butterfly index mod Ns): consecutive lanes, consecutive entries.
// LOAD 1 / 2: the first pass of the forward FFT of sample grids [fn][k][j1][j2] (complex64 / float32), lines
// o = (fn, j1) along j2 (S = N, oinner = N, oouter = N^3, oistride = N^2): the TK lines are TK grid rows (index
// rbase + kk N^2 + j), staged through shared memory with row-contiguous reads.
// STORE 3: the lines are written renormalised as two complex64 arrays at buf's index: hi (the FP32 rounding) and
// lo (the remainder).
// STORE 4 / 5: the last pass of a synthesis, lines o = (fn, j1) along j2 (S = N, oinner = N, oouter = N^3,
// oistride = N^2): the TK lines are written as TK grid rows [fn][k][j1][j2] (the mirror of LOAD 1 / 2) into hi,
// rounded once to complex64 (4) or to the real part as float32 (5).  Each butterfly of the last stage reads and
// writes the same places of its line, so the results go back into the line in shared memory and leave it as
// row-contiguous writes after one barrier.
// STORE 4 / 5: after the last stage, the TK lines (in shared memory, padded rows) as grid rows
template <int N, int TK, int ROW, bool REAL_OUT>
__device__ __forceinline__ void synth_rows_out(const qc32* sm, long long o, long long oinner, float2* out)
{
    constexpr long long NN = (long long)N * N;
    __syncthreads();
    const long long rbase = (o / oinner) * NN * N + (o % oinner) * N + (long long)blockIdx.x * TK * NN;
#pragma unroll
    for (int u = 0; u < N * TK / 256; ++u) {
        const int e = threadIdx.x + 256 * u, kk2 = e / N, j = e % N;
        const long long i = rbase + kk2 * NN + j;
        const qc32 x = sm[kk2 * ROW + j + (j >> 3)];
        if constexpr (REAL_OUT) reinterpret_cast<float*>(out)[i] = x.x.h + x.x.l;
        else out[i] = make_float2(x.x.h + x.x.l, x.y.h + x.y.l);
    }
}

template <int N, int LOAD, int STORE>
__global__ void __launch_bounds__(256, 4) fft_df32_k_kernel(dfc32* __restrict__ buf, long long S, long long oinner,
                                                             long long oouter, long long oistride,
                                                             const double2* __restrict__ twg, const void* fin,
                                                             float2* __restrict__ hi, float2* __restrict__ lo)
{
    constexpr int TK = 2048 / N;         // lines per CTA
    constexpr int TPL = N / 8;           // threads per line
    constexpr int ROW = N + N / 8 + (N == 512 ? 2 : 1);
    __shared__ qc32 sm[TK * ROW];
    __shared__ dfc32 w[N];               // stage twiddle tables (at most N - 8 entries)
    __shared__ float red[8];
    auto phys = [](int i) { return i + (i >> 3); };
    const int tid = threadIdx.x;
    const long long o = blockIdx.y;
    const long long obase = (o / oinner) * oouter + (o % oinner) * oistride + (long long)blockIdx.x * TK;
    // stage tables: radix-8 stages with Ns = 8, 64 (when present) and the last radix-4 / 2 stage with Ns = 64
    {
        int off = 0;
        for (int Ns = 8; Ns < N; Ns *= 8) {
            const int R = Ns * 8 <= N ? 8 : N / Ns;
            for (int i = tid; i < (R - 1) * Ns; i += 256) {
                const int r = i / Ns + 1, kt = i % Ns;
                const double2 v = twg[r * kt * (N / (R * Ns))];
                w[off + i] = dfc32{df32(v.x), df32(v.y)};
            }
            off += (R - 1) * Ns;
        }
    }
    const int kq = tid % TK, tq = tid / TK;  // k-fastest thread of the first / last stage
    const int kk = tid / TPL, t = tid % TPL;  // line-major thread of the middle stages
    // the CTA's block of TK lines: loaded as double-float, then put on the block's quantum
    dfc32 d[8];
    float mx = 0.f;
    if constexpr (LOAD == 0) {
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            d[r] = buf[obase + (long long)(tq + r * (N / 8)) * S + kq];
            mx = fmaxf(mx, fmaxf(fabsf(d[r].x.h), fabsf(d[r].y.h)));
        }
    } else {
        constexpr long long NN = (long long)N * N;
        const long long rbase = (o / oinner) * NN * N + (o % oinner) * N + (long long)blockIdx.x * TK * NN;
        dfc32* st = reinterpret_cast<dfc32*>(sm);
#pragma unroll
        for (int u = 0; u < N * TK / 256; ++u) {
            const int e = tid + 256 * u, kk2 = e / N, j = e % N;
            const long long i = rbase + kk2 * NN + j;
            dfc32 x;
            if constexpr (LOAD == 2) {
                x = dfc32{df32(reinterpret_cast<const float*>(fin)[i], 0.f), df32(0.f, 0.f)};
            } else {
                const float2 y = reinterpret_cast<const float2*>(fin)[i];
                x = dfc32{df32(y.x, 0.f), df32(y.y, 0.f)};
            }
            mx = fmaxf(mx, fmaxf(fabsf(x.x.h), fabsf(x.y.h)));
            st[kk2 * ROW + phys(j)] = x;
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < 8; ++r) d[r] = st[kq * ROW + phys(tq + r * (N / 8))];
    }
    const float magic = q_block_magic<N>(mx, red);  // (its barrier also orders the staging reads above)
    qc32 v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = q_from(d[r], magic);
    // stage 0 (Ns = 1)
    dft8_q(v, magic);
#pragma unroll
    for (int r = 0; r < 8; ++r) sm[kq * ROW + phys(tq * 8 + r)] = q_renorm(v[r], magic);
    __syncthreads();
    auto store = [&](int j, const qc32& x) {  // element j of line kq, from the last stage's registers
        if constexpr (STORE >= 4) {
            sm[kq * ROW + phys(j)] = x;
            return;
        }
        const long long i = obase + (long long)j * S + kq;
        if constexpr (STORE == 3) {
            const df32 a = df_two_sum(x.x.h, x.x.l), b = df_two_sum(x.y.h, x.y.l);
            hi[i] = make_float2(a.h, b.h);
            lo[i] = make_float2(a.l, b.l);
        } else {
            buf[i] = dfc32{df32(x.x.h, x.x.l), df32(x.y.h, x.y.l)};
        }
    };
    // stage 1 (Ns = 8): the last stage at N = 64
    if constexpr (N == 64) {
        const int kt = tq % 8;
#pragma unroll
        for (int r = 0; r < 8; ++r) v[r] = sm[kq * ROW + phys(tq + r * 8)];
#pragma unroll
        for (int r = 1; r < 8; ++r) v[r] = q_cmul(v[r], w[(r - 1) * 8 + kt], magic);
        dft8_q(v, magic);
#pragma unroll
        for (int r = 0; r < 8; ++r) store(tq + r * 8, v[r]);  // (tq - kt) 8 + kt + 8 r with tq < 8
        if constexpr (STORE >= 4) synth_rows_out<N, TK, ROW, STORE == 5>(sm, o, oinner, hi);
        return;
    } else {
        qc32* line = sm + kk * ROW;
        const int kt = t % 8;
#pragma unroll
        for (int r = 0; r < 8; ++r) v[r] = line[phys(t + r * (N / 8))];
        __syncthreads();
#pragma unroll
        for (int r = 1; r < 8; ++r) v[r] = q_cmul(v[r], w[(r - 1) * 8 + kt], magic);
        dft8_q(v, magic);
#pragma unroll
        for (int r = 0; r < 8; ++r) line[phys((t - kt) * 8 + kt + r * 8)] = q_renorm(v[r], magic);
        __syncthreads();
    }
    // last stage (Ns = 64): radix 8 (N = 512), 4 (256) or 2 (128); outputs j + 64 r of butterfly j < 64
    constexpr int R = N == 512 ? 8 : N == 256 ? 4 : 2;
    constexpr int PER = 8 / R;
    constexpr int BPL = N / R;  // butterflies per line (= 64)
    qc32* lq = sm + kq * ROW;
#pragma unroll
    for (int b = 0; b < PER; ++b) {
        const int j = tq + b * (256 / TK);  // butterfly of line kq
        qc32 x[R];
#pragma unroll
        for (int r = 0; r < R; ++r) x[r] = lq[phys(j + r * BPL)];
#pragma unroll
        for (int r = 1; r < R; ++r) x[r] = q_cmul(x[r], w[56 + (r - 1) * 64 + j], magic);
        dft_q<R>(x, magic);
#pragma unroll
        for (int r = 0; r < R; ++r) store(j + r * 64, x[r]);
    }
    if constexpr (STORE >= 4) synth_rows_out<N, TK, ROW, STORE == 5>(sm, o, oinner, hi);
}

// ---- both FFT passes of the beta slices of an uneven batch, every bucket in one launch
//
// A CTA takes spc consecutive beta slices (N x N each, N = 2B) of one bucket and holds them in shared memory;
// each pass moves groups of G lines into a line buffer, runs the same Stockham stages as fft_lines_kernel
// (prime-first factors) between two line buffers and writes the lines back, so the grid slab is read (or
// written) once and the pencils written (or read) once.  Real data keep only the columns q = 0..N/2 of the
// Hermitian half-spectrum: the forward transforms two real rows per complex line (z = x_a + i x_b, separated
// as in fft_lines_kernel) and N/2 + 1 columns, and writes each pencil (p, q), 0 < q < N/2, a second time as
// its mirror (-p, -q) = conj; the inverse takes the Hermitian part H = (P(p, q) + conj P(-p, -q)) / 2 of the
// pencils (the real part of the complex synthesis is the synthesis of H), transforms N/2 + 1 columns and then
// two rows per complex line (z = Y_a + i Y_b, the real and imaginary parts of its transform are the rows).
// Column lines are ordered slice-fastest, so the pencil accesses of neighbouring lines are consecutive k.
__device__ float2* run_line_stages(float2* src, float2* dst, const float2* w, const float2* mat,
                                   const FFTFactors& fac, int N, int nl, int LS)
{
    int Ns = 1;
    const int ns = fac.n;
    for (int s = 0; s < ns; ++s) {
        const int R = fac.r[s];
        switch (R) {
            case 2: stockham_stage<float, 2, SLICE_PAD>(src, dst, w, N, Ns, nl, LS); break;
            case 3: stockham_stage<float, 3, SLICE_PAD>(src, dst, w, N, Ns, nl, LS); break;
            case 4: stockham_stage<float, 4, SLICE_PAD>(src, dst, w, N, Ns, nl, LS); break;
            case 5: stockham_stage<float, 5, SLICE_PAD>(src, dst, w, N, Ns, nl, LS); break;
            case 7: stockham_stage<float, 7, SLICE_PAD>(src, dst, w, N, Ns, nl, LS); break;
            case 8: stockham_stage<float, 8, SLICE_PAD>(src, dst, w, N, Ns, nl, LS); break;
            default:
                // prime first stage: four outputs q per work item (two measured slower)
                if (Ns == 1) dft_prime_first_t<float, 2, 4, SLICE_PAD>(src, dst, mat, N, R, nl, LS);
                else stockham_generic<float, SLICE_PAD>(src, dst, w, N, Ns, R, nl, LS);
                break;
        }
        __syncthreads();
        float2* t = src;
        src = dst;
        dst = t;
        Ns *= R;
    }
    return src;
}

static int slice_prime_entries(const FFTFactors& f) { return f.r[0] > 8 ? prime_mat_entries(f.r[0]) : 0; }

// Per-line (or per-slice) tables of a CTA: two 64-bit global offsets and one shared-memory offset per entry.
__host__ __device__ inline int slice_table_entries(int G, int spc) { return G > spc ? G : spc; }

size_t slice_fft_smem_bytes(int N, int spc, bool real, bool wide)
{
    FFTFactors f;
    make_fft_factors_prime_first(N, f);
    const size_t sst = (size_t)N * slice_row_stride(N, real) + 1;
    const size_t G = (size_t)slice_lines_per_group(N, wide);
    const size_t tb = (size_t)slice_table_entries((int)G, spc);
    return sizeof(float2) * (spc * sst + 2 * G * slice_line_stride(N) + N + slice_prime_entries(f)) + tb * (8 + 8 + 4);
}

// Every element walk below advances its indices by constant steps (one division per walk, none per element).
template <bool FWD, bool REAL, int NT>
__global__ void __launch_bounds__(NT, NT == 256 ? 2 : 1) slice_fft_kernel(const BucketSeg* __restrict__ segs, int nseg,
                                                                    const void* __restrict__ in,
                                                                    void* __restrict__ out)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int sb;
    const long long blk = blockIdx.x;
    if (threadIdx.x == 0) {
        int lo = 0, hi = nseg - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (segs[mid].blk0 <= blk) lo = mid;
            else hi = mid - 1;
        }
        sb = lo;
    }
    __syncthreads();
    const BucketSeg& S = segs[sb];
    const int N = S.N, B = N / 2, LS = slice_line_stride(N), G = S.G, spc = S.spc;
    const int RS = slice_row_stride(N, REAL), NC = REAL ? B + 1 : N;
    const int SSt = N * RS + 1;
    const long long NN = (long long)N * N, NNN = NN * N;
    const long long s0 = (blk - S.blk0) * spc;
    const int ns = (int)min((long long)spc, (long long)S.batch * N - s0);
    constexpr int T = NT;
    const int tid = threadIdx.x;
    const int R0 = S.fac.r[0];
    const int nmat = R0 > 8 ? prime_mat_entries(R0) : 0;
    float2* X = reinterpret_cast<float2*>(smem_raw);
    float2* A = X + (size_t)spc * SSt;
    float2* Bf = A + G * LS;
    float2* w = Bf + G * LS;
    float2* mat = w + N;
    const int TB = slice_table_entries(G, spc);
    long long* lg = reinterpret_cast<long long*>(mat + nmat);  // per line: global offset
    long long* lm = lg + TB;                                    // per line: mirrored pencil offset (real), or -1
    int* lx = reinterpret_cast<int*>(lm + TB);                  // per line: offset in the slices
    const float2* __restrict__ Pin = S.pencil;
    float2* __restrict__ Pout = S.pencil;
    const double2* tw = S.tw;
    for (int i = tid; i < N; i += T) w[i] = make_float2((float)tw[i].x, (float)tw[i].y);
    if (R0 > 8) {
        const int P = (R0 - 1) / 2, P4 = (P + 3) / 4 * 4, Nr = N / R0;
        for (int i = tid; i < P * P4; i += T) {
            const int t = i / P4 + 1, q = i - (t - 1) * P4 + 1;
            float c = 0.f, sn = 0.f;
            if (q <= P) {
                const double2 v = tw[((t * q) % R0) * Nr];  // e^{-2 pi i t q / R}
                c = (float)v.x;
                sn = (float)(-v.y);
            }
            mat[i] = make_float2(c, sn);
        }
    }
    const int NR = REAL ? B : N;           // row lines per slice
    const int rl = T / N, rj = T - rl * N;  // walk (l, j) over rows of N
    const int cl = T / NC, cq = T - cl * NC;  // walk (l, q) over rows of NC
    // row lines [l0, l0 + nl): global row offset and slice row offset
    auto row_tables = [&](int l0, int nl) {
        for (int i = tid; i < nl; i += T) {
            const int line = l0 + i, s = line / NR, r = line - s * NR, rr = REAL ? 2 * r : r;
            lg[i] = S.g0 + (s0 + s) * NN + (long long)rr * N;
            lx[i] = s * SSt + rr * RS;
        }
    };
    // column lines [l0, l0 + nl) (slice fastest): slice column offset, pencil offsets of (q) and (-q)
    auto col_tables = [&](int l0, int nl) {
        for (int i = tid; i < nl; i += T) {
            const int line = l0 + i, q = line / ns, s = line - q * ns;
            lx[i] = s * SSt + q;
            const long long sl = s0 + s, f = sl / N, pb = f * NNN + (sl - f * N);
            lg[i] = pb + (long long)q * N;
            lm[i] = (REAL && q > 0 && q < B) ? pb + (long long)(N - q) * N : -1;
        }
    };
    if (FWD) {
        // rows: grid -> line buffer -> slice rows (real: the two half-spectra of each row pair)
        const int nlr = ns * NR;
        for (int l0 = 0; l0 < nlr; l0 += G) {
            const int nl = min(G, nlr - l0), nle = (nl + 1) & ~1;
            row_tables(l0, nl);
            __syncthreads();
            {
                int l = tid / N, j = tid - l * N;
#pragma unroll 4
                for (int e = tid; e < nl * N; e += T) {
                    if (REAL) {
                        const float* g = reinterpret_cast<const float*>(in) + lg[l] + j;
                        A[l * LS + lpos<SLICE_PAD>(j)] = make_float2(g[0], g[N]);
                    } else {
                        A[l * LS + lpos<SLICE_PAD>(j)] = reinterpret_cast<const float2*>(in)[lg[l] + j];
                    }
                    j += rj;
                    l += rl;
                    if (j >= N) { j -= N; ++l; }
                }
            }
            __syncthreads();
            const float2* res = run_line_stages(A, Bf, w, mat, S.fac, N, nle, LS);
            {
                int l = tid / NC, q = tid - l * NC;
                for (int e = tid; e < nl * NC; e += T) {
                    float2* x = X + lx[l];
                    if (REAL) {
                        const float2 z = res[l * LS + lpos<SLICE_PAD>(q)], zm = res[l * LS + lpos<SLICE_PAD>(q == 0 ? 0 : N - q)];
                        x[q] = make_float2(0.5f * (z.x + zm.x), 0.5f * (z.y - zm.y));
                        x[RS + q] = make_float2(0.5f * (z.y + zm.y), -0.5f * (z.x - zm.x));
                    } else {
                        x[q] = res[l * LS + lpos<SLICE_PAD>(q)];
                    }
                    q += cq;
                    l += cl;
                    if (q >= NC) { q -= NC; ++l; }
                }
            }
            __syncthreads();
        }
        // columns: slice -> line buffer -> pencils
        const int nlc = ns * NC;
        for (int l0 = 0; l0 < nlc; l0 += G) {
            const int nl = min(G, nlc - l0), nle = (nl + 1) & ~1;
            col_tables(l0, nl);
            __syncthreads();
            const int gj = T / nl, gl = T - gj * nl;  // walk (j, l), l fastest
            {
                int j = tid / nl, l = tid - j * nl;
                for (int e = tid; e < nl * N; e += T) {
                    A[l * LS + lpos<SLICE_PAD>(j)] = X[lx[l] + j * RS];
                    l += gl;
                    j += gj;
                    if (l >= nl) { l -= nl; ++j; }
                }
            }
            __syncthreads();
            const float2* res = run_line_stages(A, Bf, w, mat, S.fac, N, nle, LS);
            {
                int p = tid / nl, l = tid - p * nl;
                for (int e = tid; e < nl * N; e += T) {
                    const float2 v = res[l * LS + lpos<SLICE_PAD>(p)];
                    Pout[lg[l] + p * NN] = v;
                    if (REAL && lm[l] >= 0) Pout[lm[l] + (p == 0 ? 0 : N - p) * NN] = make_float2(v.x, -v.y);
                    l += gl;
                    p += gj;
                    if (l >= nl) { l -= nl; ++p; }
                }
            }
            __syncthreads();
        }
    } else {
        // pencils -> slice (Nyquist bins zero; real: the Hermitian part), walk e = (p NC + q) ns + s
        for (int i = tid; i < ns; i += T) {
            const long long sl = s0 + i, f = sl / N;
            lg[i] = f * NNN + (sl - f * N);
        }
        __syncthreads();
        {
            const int sinc = T % ns, pqinc = T / ns, qinc = pqinc % NC, pinc = pqinc / NC;
            int s = tid % ns, q = (tid / ns) % NC, p = (tid / ns) / NC;
#pragma unroll 4
            for (int e = tid; e < ns * N * NC; e += T) {
                float2 v = make_float2(0.f, 0.f);
                if (p != B && q != B) {
                    v = Pin[lg[s] + ((long long)p * N + q) * N];
                    if (REAL) {
                        const float2 u = Pin[lg[s] + ((long long)(p == 0 ? 0 : N - p) * N + (q == 0 ? 0 : N - q)) * N];
                        v = make_float2(0.5f * (v.x + u.x), 0.5f * (v.y - u.y));
                    }
                }
                X[s * SSt + p * RS + q] = v;
                s += sinc;
                int c = 0;
                if (s >= ns) { s -= ns; c = 1; }
                q += qinc + c;
                c = 0;
                if (q >= NC) { q -= NC; c = 1; }
                p += pinc + c;
            }
        }
        __syncthreads();
        // columns (along p), in place in the slice
        const int nlc = ns * NC;
        for (int l0 = 0; l0 < nlc; l0 += G) {
            const int nl = min(G, nlc - l0), nle = (nl + 1) & ~1;
            col_tables(l0, nl);
            __syncthreads();
            const int gj = T / nl, gl = T - gj * nl;
            {
                int j = tid / nl, l = tid - j * nl;
                for (int e = tid; e < nl * N; e += T) {
                    A[l * LS + lpos<SLICE_PAD>(j)] = X[lx[l] + j * RS];
                    l += gl;
                    j += gj;
                    if (l >= nl) { l -= nl; ++j; }
                }
            }
            __syncthreads();
            const float2* res = run_line_stages(A, Bf, w, mat, S.fac, N, nle, LS);
            {
                int j = tid / nl, l = tid - j * nl;
                for (int e = tid; e < nl * N; e += T) {
                    X[lx[l] + j * RS] = res[l * LS + lpos<SLICE_PAD>(j)];
                    l += gl;
                    j += gj;
                    if (l >= nl) { l -= nl; ++j; }
                }
            }
            __syncthreads();
        }
        // rows: slice -> line buffer -> grid (real: two rows per complex line)
        const int nlr = ns * NR;
        for (int l0 = 0; l0 < nlr; l0 += G) {
            const int nl = min(G, nlr - l0), nle = (nl + 1) & ~1;
            row_tables(l0, nl);
            __syncthreads();
            {
                int l = tid / N, j = tid - l * N;
                for (int e = tid; e < nl * N; e += T) {
                    const float2* x = X + lx[l];
                    if (REAL) {
                        float2 ya, yb;
                        if (j <= B) {
                            ya = x[j];
                            yb = x[RS + j];
                        } else {
                            ya = x[N - j];
                            yb = x[RS + N - j];
                            ya.y = -ya.y;
                            yb.y = -yb.y;
                        }
                        A[l * LS + lpos<SLICE_PAD>(j)] = make_float2(ya.x - yb.y, ya.y + yb.x);
                    } else {
                        A[l * LS + lpos<SLICE_PAD>(j)] = x[j];
                    }
                    j += rj;
                    l += rl;
                    if (j >= N) { j -= N; ++l; }
                }
            }
            __syncthreads();
            const float2* res = run_line_stages(A, Bf, w, mat, S.fac, N, nle, LS);
            {
                int l = tid / N, j = tid - l * N;
                for (int e = tid; e < nl * N; e += T) {
                    const float2 v = res[l * LS + lpos<SLICE_PAD>(j)];
                    if (REAL) {
                        float* g = reinterpret_cast<float*>(out) + lg[l] + j;
                        g[0] = v.x;
                        g[N] = v.y;
                    } else {
                        reinterpret_cast<float2*>(out)[lg[l] + j] = v;
                    }
                    j += rj;
                    l += rl;
                    if (j >= N) { j -= N; ++l; }
                }
            }
            __syncthreads();
        }
    }
}

template <int NT>
static cudaError_t slice_launch(const BucketSeg* segs, int nseg, long long nblk, size_t smem, bool fwd, bool real,
                                const void* in, void* out, cudaStream_t st)
{
    auto kern = fwd ? (real ? slice_fft_kernel<true, true, NT> : slice_fft_kernel<true, false, NT>)
                    : (real ? slice_fft_kernel<false, true, NT> : slice_fft_kernel<false, false, NT>);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<(unsigned)nblk, NT, smem, st>>>(segs, nseg, in, out);
    return cudaGetLastError();
}

cudaError_t launch_slice_fft(const BucketSeg* segs, int nseg, long long nblk, size_t smem, bool fwd, bool real,
                             bool wide, const void* in, void* out, cudaStream_t st)
{
    if (nblk <= 0) return cudaSuccess;
    if (nblk > 0x7fffffffLL || nseg <= 0) return cudaErrorInvalidValue;
    return wide ? slice_launch<512>(segs, nseg, nblk, smem, fwd, real, in, out, st)
                : slice_launch<256>(segs, nseg, nblk, smem, fwd, real, in, out, st);
}

bool fft_df32_k_supported(int N) { return N == 64 || N == 128 || N == 256 || N == 512; }

template <int LOAD, int STORE>
static void df32_k_launch(int N, dim3 grid, dfc32* b, long long S, long long oinner, long long oouter,
                          long long oistride, const double2* t, const void* fin, float2* hi, float2* lo,
                          cudaStream_t st)
{
    switch (N) {
        case 64:
            fft_df32_k_kernel<64, LOAD, STORE><<<grid, 256, 0, st>>>(b, S, oinner, oouter, oistride, t, fin, hi, lo);
            break;
        case 128:
            fft_df32_k_kernel<128, LOAD, STORE><<<grid, 256, 0, st>>>(b, S, oinner, oouter, oistride, t, fin, hi, lo);
            break;
        case 256:
            fft_df32_k_kernel<256, LOAD, STORE><<<grid, 256, 0, st>>>(b, S, oinner, oouter, oistride, t, fin, hi, lo);
            break;
        default:
            fft_df32_k_kernel<512, LOAD, STORE><<<grid, 256, 0, st>>>(b, S, oinner, oouter, oistride, t, fin, hi, lo);
            break;
    }
}

cudaError_t launch_fft_df32_k(void* buf, int N, long long S, long long nouter, long long oinner, long long oouter,
                              long long oistride, const void* tw, cudaStream_t st)
{
    if (!fft_df32_k_supported(N) || nouter < 1 || nouter > 65535 || oinner < 1) return cudaErrorInvalidValue;
    const dim3 grid((unsigned)(N / (2048 / N)), (unsigned)nouter);
    df32_k_launch<0, 0>(N, grid, (dfc32*)buf, S, oinner, oouter, oistride, (const double2*)tw, nullptr, nullptr,
                        nullptr, st);
    return cudaGetLastError();
}

cudaError_t launch_fft_df32_k_forward(void* buf, int N, long long nb, const void* f, bool real, float2* hi,
                                      float2* lo, const void* tw, cudaStream_t st)
{
    if (!fft_df32_k_supported(N) || nb < 1 || nb * N > 65535) return cudaErrorInvalidValue;
    const dim3 grid((unsigned)(N / (2048 / N)), (unsigned)(nb * N));
    const long long NN = (long long)N * N;
    const double2* t = (const double2*)tw;
    dfc32* b = (dfc32*)buf;
    // along j2, from the grid rows, into buf [fn][j1][q][k]
    if (real)
        df32_k_launch<2, 0>(N, grid, b, N, N, NN * N, NN, t, f, nullptr, nullptr, st);
    else
        df32_k_launch<1, 0>(N, grid, b, N, N, NN * N, NN, t, f, nullptr, nullptr, st);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    // along j1 (stride N^2), lines (fn, q), into the pencils [fn][p][q][k] as hi + lo
    df32_k_launch<0, 3>(N, grid, b, NN, N, NN * N, N, t, nullptr, hi, lo, st);
    return cudaGetLastError();
}

cudaError_t launch_fft_df32_k_synth_pass(int pass, void* buf, int N, long long nb, void* out, bool real,
                                         const void* tw, cudaStream_t st)
{
    if (!fft_df32_k_supported(N) || nb < 1 || nb * N > 65535 || (pass != 1 && pass != 2)) return cudaErrorInvalidValue;
    const dim3 grid((unsigned)(N / (2048 / N)), (unsigned)(nb * N));
    const long long NN = (long long)N * N;
    const double2* t = (const double2*)tw;
    dfc32* b = (dfc32*)buf;
    if (pass == 1) {
        // along p (stride N^2), lines (fn, q), in place
        df32_k_launch<0, 0>(N, grid, b, NN, N, NN * N, N, t, nullptr, nullptr, nullptr, st);
    } else if (real) {
        // along q, lines (fn, p), out as the grid rows [fn][k][j1][j2]
        df32_k_launch<0, 5>(N, grid, b, N, N, NN * N, NN, t, nullptr, (float2*)out, nullptr, st);
    } else {
        df32_k_launch<0, 4>(N, grid, b, N, N, NN * N, NN, t, nullptr, (float2*)out, nullptr, st);
    }
    return cudaGetLastError();
}

cudaError_t launch_fft_df32_k_synth(void* buf, int N, long long nb, void* out, bool real, const void* tw,
                                    cudaStream_t st)
{
    cudaError_t e = launch_fft_df32_k_synth_pass(1, buf, N, nb, out, real, tw, st);
    return e != cudaSuccess ? e : launch_fft_df32_k_synth_pass(2, buf, N, nb, out, real, tw, st);
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

void make_fft_factors_prime_first(int N, FFTFactors& f)
{
    FFTFactors g;
    make_fft_factors(N, g);
    f.N = N;
    f.n = 0;
    for (int i = g.n - 1; i >= 0; --i)
        if (g.r[i] > 8) f.r[f.n++] = g.r[i];
    for (int i = 0; i < g.n; ++i)
        if (g.r[i] <= 8) f.r[f.n++] = g.r[i];
}

size_t fft_smem_bytes(int N, int lpb, bool fp64)
{
    size_t c = fp64 ? 16 : 8;
    // the largest prime factor above 8 may head the factor list (prime-first order)
    int r = N, pmax = 0;
    for (int p = 2; r > 1; ++p)
        while (r % p == 0) {
            r /= p;
            pmax = p;
        }
    // (only FP32 plans order factors prime-first; N = 2B keeps FP64 lists starting with 8, 4 or 2)
    const size_t mat = (!fp64 && pmax > 8) ? (size_t)prime_mat_entries(pmax) : 0;
    return c * ((size_t)N + 2 * (size_t)lpb * (N + 1)) + 8 * (size_t)lpb + c * mat;
}

template <typename T, typename TIN, bool RI, bool RO>
static cudaError_t launch_one(const void* in, void* out, const FFTFactors& fac, long long nlines, int lpb,
                              long long inner, long long ostride, long long istride, long long es,
                              const void* tw, bool lines_fastest, int threads, cudaStream_t st)
{
    if (threads < 32 || threads > 256 || threads % 32 != 0) return cudaErrorInvalidValue;
    if ((RI || RO) && lpb < 2) lpb = 2;  // real data: lines transformed in pairs
    if ((RI || RO) && nlines % 2) return cudaErrorInvalidValue;
    const int lbuf = (RI || RO) ? lpb / 2 : lpb;
    size_t smem = fft_smem_bytes(fac.N, lbuf, sizeof(T) == 8) + 8 * (size_t)(lpb - lbuf);
    auto kern = fft_lines_kernel<T, TIN, RI, RO>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int lg = 0;
    while ((1 << lg) < lpb) ++lg;
    if ((1 << lg) != lpb || lpb > 256) return cudaErrorInvalidValue;  // lines per CTA: power of two
    long long nblk = (nlines + lpb - 1) / lpb;
    kern<<<(unsigned)nblk, threads, smem, st>>>(reinterpret_cast<const TIN*>(in), out, fac, nlines, lg, inner, ostride,
                                            istride, es, tw, lines_fastest ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_fft_lines(const FFTLaunch& L, cudaStream_t st)
{
    if (L.df32) {  // double-float complex lines (16 bytes per element), complex in and out only
        if (L.real_in || L.real_out) return cudaErrorInvalidValue;
        return launch_one<df32, dfc32, false, false>(L.in, L.out, L.fac, L.nlines, L.lpb, L.inner, L.ostride,
                                                     L.istride, L.es, L.tw, L.lines_fastest, L.threads, st);
    }
    if (L.fp64) {
        if (L.real_in && L.real_out) return cudaErrorInvalidValue;
        if (L.real_in)
            return launch_one<double, double, true, false>(L.in, L.out, L.fac, L.nlines, L.lpb, L.inner, L.ostride,
                                                           L.istride, L.es, L.tw, L.lines_fastest, L.threads, st);
        if (L.real_out)
            return launch_one<double, double2, false, true>(L.in, L.out, L.fac, L.nlines, L.lpb, L.inner, L.ostride,
                                                            L.istride, L.es, L.tw, L.lines_fastest, L.threads, st);
        return launch_one<double, double2, false, false>(L.in, L.out, L.fac, L.nlines, L.lpb, L.inner, L.ostride,
                                                         L.istride, L.es, L.tw, L.lines_fastest, L.threads, st);
    } else {
        if (L.real_in && L.real_out) return cudaErrorInvalidValue;
        if (L.real_in)
            return launch_one<float, float, true, false>(L.in, L.out, L.fac, L.nlines, L.lpb, L.inner, L.ostride,
                                                         L.istride, L.es, L.tw, L.lines_fastest, L.threads, st);
        if (L.real_out)
            return launch_one<float, float2, false, true>(L.in, L.out, L.fac, L.nlines, L.lpb, L.inner, L.ostride,
                                                          L.istride, L.es, L.tw, L.lines_fastest, L.threads, st);
        return launch_one<float, float2, false, false>(L.in, L.out, L.fac, L.nlines, L.lpb, L.inner, L.ostride,
                                                       L.istride, L.es, L.tw, L.lines_fastest, L.threads, st);
    }
}

}  // namespace fftso3
