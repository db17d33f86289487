// FP64 beta-sum contractions (the plain method) and the coefficient-basis
// conversions of the real transforms.
//
// SO(3) forward (fdcl_FFTSO3.cpp:704-740):
//   F(l,m,n) = sum_k w_k d^l_mn(beta_k) G_k(-m mod N, -n mod N),
// where G_k is the unscaled 2-D DFT of the beta_k slice.  One CTA per
// (symmetry group, function): the group's <= 4 (m,n) pairs share one table
// block d_g[l][k], so X[p][k] = w_k G_k(pair p) is staged in shared memory and
// each warp walks one row l with its lanes over k (coalesced table reads),
// finishing with a shuffle reduction.
//
// SO(3) inverse (grid form of fdcl_FFTSO3.cpp:498-531):
//   H_k(m,n) = sum_l (2l+1) F(l,m,n) d^l_mn(beta_k), placed at bin
//   (m mod N, n mod N) of slice k; a forward 2-D DFT of the slice then gives
//   f(alpha_j1, beta_k, gamma_j2) = sum_mn H_k(m,n) e^{-i m alpha_j1} e^{-i n gamma_j2}.
//   Threads over k (coalesced table reads), (2l+1) F staged in shared memory.
//
// S^2 is the same pattern with the Legendre table and groups m >= 0 serving
// the pairs (m, -m) (fdcl_FFTS2.cpp:157-173 forward, :194-230 inverse).
#include "common.cuh"
#include "contract.cuh"
#include "rsph.cuh"

namespace fftso3 {

__device__ __forceinline__ int mod_n(int a, int N) { int r = a % N; return r < 0 ? r + N : r; }

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Reduce-scatter of 8 (4) per-lane partial sums over the warp: every lane gets the full sum of value
// 4 b4 + 2 b3 + b2 (2 b4 + b3), b_i = bit i of the lane; each level halves the values a lane carries,
// so it costs 9 (6) shuffles and additions instead of 40 (20) for separate butterflies.
__device__ __forceinline__ double warp_reduce_scatter8(const double (&v)[8], int lane)
{
    const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
    double w[4], x[2];
#pragma unroll
    for (int j = 0; j < 4; ++j) w[j] = (b4 ? v[j + 4] : v[j]) + __shfl_xor_sync(0xffffffffu, b4 ? v[j] : v[j + 4], 16);
#pragma unroll
    for (int j = 0; j < 2; ++j) x[j] = (b3 ? w[j + 2] : w[j]) + __shfl_xor_sync(0xffffffffu, b3 ? w[j] : w[j + 2], 8);
    double y = (b2 ? x[1] : x[0]) + __shfl_xor_sync(0xffffffffu, b2 ? x[0] : x[1], 4);
    y += __shfl_xor_sync(0xffffffffu, y, 2);
    y += __shfl_xor_sync(0xffffffffu, y, 1);
    return y;
}
__device__ __forceinline__ double warp_reduce_scatter4(const double (&v)[4], int lane)
{
    const bool b4 = lane & 16, b3 = lane & 8;
    double w[2];
#pragma unroll
    for (int j = 0; j < 2; ++j) w[j] = (b4 ? v[j + 2] : v[j]) + __shfl_xor_sync(0xffffffffu, b4 ? v[j] : v[j + 2], 16);
    double y = (b3 ? w[1] : w[0]) + __shfl_xor_sync(0xffffffffu, b3 ? w[0] : w[1], 8);
    y += __shfl_xor_sync(0xffffffffu, y, 4);
    y += __shfl_xor_sync(0xffffffffu, y, 2);
    y += __shfl_xor_sync(0xffffffffu, y, 1);
    return y;
}

// ------------------------------------------------------------------ SO(3)

template <int NT>
__global__ void __launch_bounds__(NT) so3_fwd_fp64_kernel(const double* __restrict__ table,
                                                          const long long* __restrict__ goff,
                                                          const double2* __restrict__ G, const double* __restrict__ w,
                                                          double2* __restrict__ F, int L, int N, long long gstride,
                                                          long long cstride)
{
    extern __shared__ double2 X[];  // [4][N]
    const int g = blockIdx.x, b = blockIdx.y;
    int m0, n0;
    group_mn(g, m0, n0);
    const GroupPairs P = group_pairs(m0, n0);
    const double2* Gb = G + (long long)b * gstride;
    const long long NN = (long long)N * N;
    for (int i = threadIdx.x; i < P.np * N; i += NT) {
        int p = i / N, k = i - p * N;
        int pi = mod_n(-P.m[p], N), qi = mod_n(-P.n[p], N);
        double2 v = Gb[(long long)k * NN + (long long)pi * N + qi];
        double wk = w[k];
        X[p * N + k] = make_double2(wk * v.x, wk * v.y);
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const double* tg = table + goff[g];
    double* Fb = reinterpret_cast<double*>(F + (long long)b * cstride);
    // after the reduce-scatter lane holds value vi = 2 p + (re, im) of pair p; lanes 4j write
    const int vi = ((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1), wp = vi >> 1;
    const bool writer = (lane & 3) == 0 && wp < P.np;
    const int wm = wp < P.np ? P.m[wp] : 0, wn = wp < P.np ? P.n[wp] : 0;
    const double wsign = wp < P.np ? (double)P.sign[wp] : 0.;
    for (int l = m0 + warp; l <= L; l += NT / 32) {
        const double* drow = tg + (long long)(l - m0) * N;
        double v[8] = {0., 0., 0., 0., 0., 0., 0., 0.};
        for (int k = lane; k < N; k += 32) {
            double d = drow[k];
#pragma unroll
            for (int p = 0; p < 4; ++p)
                if (p < P.np) {
                    double2 x = X[p * N + k];
                    v[2 * p] += d * x.x;
                    v[2 * p + 1] += d * x.y;
                }
        }
        const double y = warp_reduce_scatter8(v, lane);
        if (writer) Fb[2 * so3_idx(l, wm, wn) + (vi & 1)] = wsign * y;
    }
}

template <int NT>
__global__ void __launch_bounds__(NT) so3_inv_fp64_kernel(const double* __restrict__ table,
                                                          const long long* __restrict__ goff,
                                                          const double2* __restrict__ F, double2* __restrict__ H,
                                                          int L, int N, long long gstride, long long cstride)
{
    extern __shared__ double2 Y[];  // [4][B]
    const int g = blockIdx.x, b = blockIdx.y;
    const int B = L + 1;
    int m0, n0;
    group_mn(g, m0, n0);
    const GroupPairs P = group_pairs(m0, n0);
    const int nl = B - m0;
    const double2* Fb = F + (long long)b * cstride;
    for (int i = threadIdx.x; i < P.np * nl; i += NT) {
        int p = i / nl, l = m0 + (i - p * nl);
        double2 c = Fb[so3_idx(l, P.m[p], P.n[p])];
        double s = (double)(2 * l + 1) * P.sign[p];
        Y[p * B + (l - m0)] = make_double2(s * c.x, s * c.y);
    }
    __syncthreads();
    const double* tg = table + goff[g];
    double2* Hb = H + (long long)b * gstride;
    const long long NN = (long long)N * N;
    for (int k = threadIdx.x; k < N; k += NT) {
        double ar[4] = {0., 0., 0., 0.}, ai[4] = {0., 0., 0., 0.};
        for (int j = 0; j < nl; ++j) {
            double d = tg[(long long)j * N + k];
#pragma unroll
            for (int p = 0; p < 4; ++p)
                if (p < P.np) {
                    double2 y = Y[p * B + j];
                    ar[p] += d * y.x;
                    ai[p] += d * y.y;
                }
        }
#pragma unroll
        for (int p = 0; p < 4; ++p)
            if (p < P.np) {
                int pi = mod_n(P.m[p], N), qi = mod_n(P.n[p], N);
                Hb[(long long)k * NN + (long long)pi * N + qi] = make_double2(ar[p], ai[p]);
            }
    }
}

// Zero the Nyquist row p = B and column q = B of every N x N slice (the bins
// no (m, n) with |m|, |n| <= L maps to).
template <typename C>
__global__ void zero_nyquist_so3_kernel(C* __restrict__ H, int N, long long nslices)
{
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nslices * 2 * N) return;
    long long s = idx / (2 * N);
    int r = (int)(idx % (2 * N));
    int B = N / 2;
    C z;
    z.x = 0;
    z.y = 0;
    C* slice = H + s * N * N;
    if (r < N)
        slice[(long long)B * N + r] = z;
    else
        slice[(long long)(r - N) * N + B] = z;
}

__device__ __forceinline__ double2 tmat(int a, int c)
{
    c2t<double> t = tmat_t<double>(a, c);
    return make_double2(t.x, t.y);
}
__device__ __forceinline__ double2 cmul2(double2 a, double2 b)
{
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 conj2(double2 a) { return make_double2(a.x, -a.y); }

// F_r = Re(T F_c T^H) per l (fdcl_FFTSO3.cpp:1169-1181): the real-basis
// coefficients of a real function from its complex coefficients.
template <typename CIN, typename ROUT, typename A>
__global__ void so3_c2r_kernel(const CIN* __restrict__ Fc, ROUT* __restrict__ Fr, int L, long long cstride)
{
    const int l = blockIdx.x, b = blockIdx.y;
    const int W = 2 * l + 1;
    const CIN* fc = Fc + (long long)b * cstride;
    ROUT* fr = Fr + (long long)b * cstride;
    for (int i = threadIdx.x; i < W * W; i += blockDim.x) {
        int m = i % W - l, n = i / W - l;
        int am[2] = {-m, m}, bn[2] = {-n, n};
        int na = (m == 0) ? 1 : 2, nb = (n == 0) ? 1 : 2;
        A acc = 0;
        for (int ia = 0; ia < na; ++ia)
            for (int ib = 0; ib < nb; ++ib) {
                c2t<A> t1 = tmat_t<A>(m, am[ia]), t2 = conj_t(tmat_t<A>(n, bn[ib]));
                CIN v = fc[so3_idx(l, am[ia], bn[ib])];
                c2t<A> c = cmul_t(cmul_t(t1, c2t<A>{(A)v.x, (A)v.y}), t2);
                acc += c.x;
            }
        fr[so3_idx(l, m, n)] = (ROUT)acc;
    }
}

// F_c = T^H F_r T per l: the complex coefficients whose synthesis equals the
// real-basis synthesis sum (2l+1) F_r U (U = Re(conj(T) D T^T), fdcl_FFTSO3.cpp:1010-1022).
template <typename RIN, typename COUT, typename A>
__global__ void so3_r2c_kernel(const RIN* __restrict__ Fr, COUT* __restrict__ Fc, int L, long long cstride)
{
    const int l = blockIdx.x, b = blockIdx.y;
    const int W = 2 * l + 1;
    const RIN* fr = Fr + (long long)b * cstride;
    COUT* fc = Fc + (long long)b * cstride;
    for (int i = threadIdx.x; i < W * W; i += blockDim.x) {
        int m = i % W - l, n = i / W - l;
        int am[2] = {m, -m}, bn[2] = {n, -n};
        int na = (m == 0) ? 1 : 2, nb = (n == 0) ? 1 : 2;
        c2t<A> acc = {(A)0, (A)0};
        for (int ia = 0; ia < na; ++ia)
            for (int ib = 0; ib < nb; ++ib) {
                c2t<A> c = cmul_t(conj_t(tmat_t<A>(am[ia], m)), tmat_t<A>(bn[ib], n));
                A v = (A)fr[so3_idx(l, am[ia], bn[ib])];
                acc.x += c.x * v;
                acc.y += c.y * v;
            }
        COUT o;
        o.x = acc.x;
        o.y = acc.y;
        fc[so3_idx(l, m, n)] = o;
    }
}

// ------------------------------------------------------------------- S^2

template <int NT>
__global__ void __launch_bounds__(NT) s2_fwd_fp64_kernel(const double* __restrict__ table,
                                                         const long long* __restrict__ moff,
                                                         const double2* __restrict__ G, const double* __restrict__ w,
                                                         double2* __restrict__ F, int L, int N, long long gstride,
                                                         long long cstride, int is_real)
{
    extern __shared__ double2 X[];  // [2][N]
    const int m = blockIdx.x, b = blockIdx.y;
    const int np = (m > 0 && !is_real) ? 2 : 1;
    const double2* Gb = G + (long long)b * gstride;
    for (int i = threadIdx.x; i < np * N; i += NT) {
        int p = i / N, k = i - p * N;
        int bin = (p == 0) ? m : N - m;  // F_k(m) and F_k(2B + (-m)), fdcl_FFTS2.cpp:162,165
        double2 v = Gb[(long long)k * N + bin];
        double wk = w[k];
        X[p * N + k] = make_double2(wk * v.x, wk * v.y);
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const double* tg = table + moff[m];
    double2* Fb = F + (long long)b * cstride;
    const double sg = (m & 1) ? -1. : 1.;
    // after the reduce-scatter lane holds value vi = 2 p + (re, im) of pair p (p = 1: -m); lanes 8j write
    const int vi = ((lane >> 4) & 1) * 2 + ((lane >> 3) & 1), wp = vi >> 1, wc = vi & 1;
    const bool writer = (lane & 7) == 0 && wp < np;
    double* Fd = reinterpret_cast<double*>(Fb);
    for (int l = m + warp; l <= L; l += NT / 32) {
        const double* prow = tg + (long long)(l - m) * N;
        double v[4] = {0., 0., 0., 0.};
        for (int k = lane; k < N; k += 32) {
            double d = prow[k];
            double2 x0 = X[k];
            v[0] += d * x0.x;
            v[1] += d * x0.y;
            if (np == 2) {
                double2 x1 = X[N + k];
                v[2] += d * x1.x;
                v[3] += d * x1.y;
            }
        }
        const double y = warp_reduce_scatter4(v, lane);
        if (writer) {
            if (wp == 0) {
                Fd[2 * s2_idx(l, m) + wc] = y;
                if (m > 0 && is_real)  // Hermitian fill, fdcl_FFTS2.cpp:182-188
                    Fd[2 * s2_idx(l, -m) + wc] = sg * (wc ? -y : y);
            } else {
                Fd[2 * s2_idx(l, -m) + wc] = sg * y;
            }
        }
    }
}

template <int NT>
__global__ void __launch_bounds__(NT) s2_inv_fp64_kernel(const double* __restrict__ table,
                                                         const long long* __restrict__ moff,
                                                         const double2* __restrict__ F, double2* __restrict__ H,
                                                         int L, int N, long long gstride, long long cstride)
{
    extern __shared__ double2 Y[];  // [2][B]
    const int m = blockIdx.x, b = blockIdx.y;
    const int B = L + 1;
    const int nl = B - m;
    const int np = (m > 0) ? 2 : 1;
    const double sg = (m & 1) ? -1. : 1.;
    const double2* Fb = F + (long long)b * cstride;
    for (int i = threadIdx.x; i < np * nl; i += NT) {
        int p = i / nl, l = m + (i - p * nl);
        double2 c = Fb[s2_idx(l, p == 0 ? m : -m)];
        double s = (p == 0) ? 1. : sg;
        Y[p * B + (l - m)] = make_double2(s * c.x, s * c.y);
    }
    __syncthreads();
    const double* tg = table + moff[m];
    double2* Hb = H + (long long)b * gstride;
    for (int k = threadIdx.x; k < N; k += NT) {
        double ar[2] = {0., 0.}, ai[2] = {0., 0.};
        for (int j = 0; j < nl; ++j) {
            double d = tg[(long long)j * N + k];
            double2 y0 = Y[j];
            ar[0] += d * y0.x;
            ai[0] += d * y0.y;
            if (np == 2) {
                double2 y1 = Y[B + j];
                ar[1] += d * y1.x;
                ai[1] += d * y1.y;
            }
        }
        // f = sum_m H(m) e^{+i m phi}: H(m) goes to bin -m mod N of a forward DFT
        Hb[(long long)k * N + mod_n(-m, N)] = make_double2(ar[0], ai[0]);
        if (np == 2) Hb[(long long)k * N + mod_n(m, N)] = make_double2(ar[1], ai[1]);
    }
}

template <typename C>
__global__ void zero_nyquist_s2_kernel(C* __restrict__ H, int N, long long nrows)
{
    long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrows) return;
    C z;
    z.x = 0;
    z.y = 0;
    H[r * N + N / 2] = z;
}

// degree l of packed S^2 index i = l^2 + l + m (integer fix-up of a float square root)
__device__ __forceinline__ int s2_degree(long long i)
{
    int l = (int)sqrtf((float)i);
    while ((long long)l * l > i) --l;
    while ((long long)(l + 1) * (l + 1) <= i) ++l;
    return l;
}

// F_r(l) = Re(conj(T(l)) F_c(l)) (fdcl_FFTS2.cpp:424-436), arithmetic in A
// (double for the FP64 path, float for the tensor-core path).
template <typename CIN, typename ROUT, typename A>
__global__ void s2_c2r_kernel(const CIN* __restrict__ Fc, ROUT* __restrict__ Fr, int L, long long cstride)
{
    const int b = blockIdx.y;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long C = (long long)(L + 1) * (L + 1);
    if (i >= C) return;
    const int l = s2_degree(i);
    const int m = (int)(i - (long long)l * l) - l;
    const CIN* fc = Fc + (long long)b * cstride;
    int cs[2] = {-m, m};
    if (m > 0) { cs[0] = -m; cs[1] = m; } else if (m < 0) { cs[0] = m; cs[1] = -m; }
    const int nc = (m == 0) ? 1 : 2;
    A acc = 0;
    for (int j = 0; j < nc; ++j) {
        const c2t<A> t = conj_t(tmat_t<A>(m, cs[j]));
        const CIN v = fc[s2_idx(l, cs[j])];
        acc += t.x * (A)v.x - t.y * (A)v.y;
    }
    Fr[(long long)b * cstride + i] = (ROUT)acc;
}

// F_c = T^T F_r: the complex coefficients whose synthesis is the real-basis
// synthesis sum F_r(l,m) y(l,m), y = T Y (fdcl_FFTS2.cpp:383-422).
template <typename RIN, typename COUT, typename A>
__global__ void s2_r2c_kernel(const RIN* __restrict__ Fr, COUT* __restrict__ Fc, int L, long long cstride)
{
    const int b = blockIdx.y;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long C = (long long)(L + 1) * (L + 1);
    if (i >= C) return;
    const int l = s2_degree(i);
    const int c = (int)(i - (long long)l * l) - l;
    const RIN* fr = Fr + (long long)b * cstride;
    const int as[2] = {c, -c};
    const int na = (c == 0) ? 1 : 2;
    c2t<A> acc = {(A)0, (A)0};
    for (int j = 0; j < na; ++j) {
        const c2t<A> t = tmat_t<A>(as[j], c);
        const A v = (A)fr[s2_idx(l, as[j])];
        acc.x += t.x * v;
        acc.y += t.y * v;
    }
    COUT o;
    o.x = acc.x;
    o.y = acc.y;
    Fc[(long long)b * cstride + i] = o;
}

// S^2 real coefficients straight from the tensor-core group-major layout
// (Fg[f][goff2[g] + p (B - g) + (l - g)] = F_c(l, m) for g = |m|, p = (m < 0)):
// the gather to the packed complex layout and s2_c2r_kernel in one pass, with
// the same arithmetic.  A CTA stages a 32 (l) x 32 (m) tile of F_c(l, +-m) in
// shared memory, so the group-major side is read along l and the packed real
// side written along m, both in runs of 32.
constexpr int S2T = 32;

__global__ void __launch_bounds__(256) s2_group_to_real_kernel(const float2* __restrict__ Fg, float* __restrict__ Fr,
                                                              const long long* __restrict__ goff2, int L,
                                                              long long cstride)
{
    __shared__ float2 tp[S2T][S2T + 1];  // F_c(l0 + li, +(mb + mi)) as [mi][li]
    __shared__ float2 tn[S2T][S2T + 1];  // F_c(l0 + li, -(mb + mi))
    const int B = L + 1;
    const int l0 = blockIdx.x * S2T, mb = (int)blockIdx.y * S2T, b = blockIdx.z;  // |m| tile [mb, mb + 32)
    if (mb > l0 + S2T - 1 || mb > L) return;  // every |m| of the tile exceeds every l
    const float2* fg = Fg + (long long)b * cstride;
    for (int e = threadIdx.x; e < S2T * S2T; e += 256) {
        const int mi = e / S2T, li = e % S2T, g = mb + mi, l = l0 + li;
        if (g > L || l > L || l < g) continue;
        const long long o = goff2[g] + (l - g);
        tp[mi][li] = fg[o];
        tn[mi][li] = g > 0 ? fg[o + (B - g)] : fg[o];
    }
    __syncthreads();
    float* fr = Fr + (long long)b * cstride;
    // outputs (l, m) for |m| in the tile, m = +g and m = -g: runs along m (packed l^2 + l + m)
    for (int e = threadIdx.x; e < 2 * S2T * S2T; e += 256) {
        const int li = e / (2 * S2T), r = e % (2 * S2T), neg = r < S2T, mi = neg ? S2T - 1 - r : r - S2T;
        const int g = mb + mi, l = l0 + li;
        if (g > L || l > L || l < g || (neg && g == 0)) continue;
        const int m = neg ? -g : g;
        int cs[2] = {-m, m};
        if (m > 0) { cs[0] = -m; cs[1] = m; } else if (m < 0) { cs[0] = m; cs[1] = -m; }
        const int nc = (m == 0) ? 1 : 2;
        float acc = 0.f;
        for (int j = 0; j < nc; ++j) {
            const c2t<float> t = conj_t(tmat_t<float>(m, cs[j]));
            const float2 v = cs[j] < 0 ? tn[mi][li] : tp[mi][li];
            acc += t.x * v.x - t.y * v.y;
        }
        fr[(long long)l * l + l + m] = acc;
    }
}

// S^2 real coefficients straight into the scaled group-major layout of the
// inverse GEMM (pair 0: F_c(l, m), pair 1: (-1)^m F_c(l, -m), m >= 0):
// s2_r2c_kernel and the packed -> group-major permutation in one pass, with
// the same arithmetic.  A CTA stages F_r(l, +-m) for a 32 (l) x 32 (m) tile,
// read along m (packed) and written along l (group-major).
__global__ void __launch_bounds__(256) s2_real_to_group_kernel(const float* __restrict__ Fr, float2* __restrict__ Y,
                                                              const long long* __restrict__ goff2, int L,
                                                              long long cstride)
{
    __shared__ float tp[S2T][S2T + 1];  // F_r(l0 + li, +(mb + mi)) as [li][mi]
    __shared__ float tn[S2T][S2T + 1];  // F_r(l0 + li, -(mb + mi))
    const int B = L + 1;
    const int l0 = blockIdx.x * S2T, mb = (int)blockIdx.y * S2T, b = blockIdx.z;
    if (mb > l0 + S2T - 1 || mb > L) return;
    const float* fr = Fr + (long long)b * cstride;
    for (int e = threadIdx.x; e < 2 * S2T * S2T; e += 256) {
        const int li = e / (2 * S2T), r = e % (2 * S2T), neg = r < S2T, mi = neg ? S2T - 1 - r : r - S2T;
        const int g = mb + mi, l = l0 + li;
        if (g > L || l > L || l < g) continue;
        const float v = fr[(long long)l * l + l + (neg ? -g : g)];
        if (neg) tn[li][mi] = v; else tp[li][mi] = v;
    }
    __syncthreads();
    float2* y = Y + (long long)b * cstride;
    for (int e = threadIdx.x; e < 2 * S2T * S2T; e += 256) {
        const int p = e / (S2T * S2T), r = e % (S2T * S2T), mi = r / S2T, li = r % S2T;
        const int m = mb + mi, l = l0 + li;
        if (m > L || l > L || l < m || (p == 1 && m == 0)) continue;
        const int c = p == 0 ? m : -m;
        const int as[2] = {c, -c};
        const int na = (c == 0) ? 1 : 2;
        c2t<float> acc = {0.f, 0.f};
        for (int j = 0; j < na; ++j) {
            const c2t<float> t = tmat_t<float>(as[j], c);
            const float v = as[j] < 0 ? tn[li][mi] : tp[li][mi];
            acc.x += t.x * v;
            acc.y += t.y * v;
        }
        const float sc = (p == 0 || !(m & 1)) ? 1.f : -1.f;
        y[goff2[m] + (long long)p * (B - m) + (l - m)] = make_float2(sc * acc.x, sc * acc.y);
    }
}

// ---------------------------------------------------------------- launchers

cudaError_t launch_so3_fwd_fp64(const double* table, const long long* goff, const double2* G, const double* w,
                                double2* F, int L, int N, int batch, cudaStream_t st)
{
    const int B = L + 1;
    size_t smem = sizeof(double2) * 4 * N;
    auto k = so3_fwd_fp64_kernel<256>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid(B * B, batch);
    k<<<grid, 256, smem, st>>>(table, goff, G, w, F, L, N, (long long)N * N * N, so3_off(B));
    return cudaGetLastError();
}

cudaError_t launch_so3_inv_fp64(const double* table, const long long* goff, const double2* F, double2* H, int L,
                                int N, int batch, cudaStream_t st)
{
    const int B = L + 1;
    size_t smem = sizeof(double2) * 4 * B;
    dim3 grid(B * B, batch);
    so3_inv_fp64_kernel<256><<<grid, 256, smem, st>>>(table, goff, F, H, L, N, (long long)N * N * N, so3_off(B));
    return cudaGetLastError();
}

cudaError_t launch_zero_nyquist_so3(void* H, bool fp64, int N, long long nslices, cudaStream_t st)
{
    long long tot = nslices * 2 * N;
    unsigned nb = (unsigned)((tot + 255) / 256);
    if (fp64)
        zero_nyquist_so3_kernel<double2><<<nb, 256, 0, st>>>((double2*)H, N, nslices);
    else
        zero_nyquist_so3_kernel<float2><<<nb, 256, 0, st>>>((float2*)H, N, nslices);
    return cudaGetLastError();
}

cudaError_t launch_so3_c2r(const void* Fc, void* Fr, bool fp64, int L, int batch, cudaStream_t st)
{
    dim3 grid(L + 1, batch);
    long long cs = so3_off(L + 1);
    if (fp64)
        so3_c2r_kernel<double2, double, double><<<grid, 256, 0, st>>>((const double2*)Fc, (double*)Fr, L, cs);
    else
        so3_c2r_kernel<float2, float, float><<<grid, 256, 0, st>>>((const float2*)Fc, (float*)Fr, L, cs);
    return cudaGetLastError();
}

cudaError_t launch_so3_r2c(const void* Fr, void* Fc, bool fp64, int L, int batch, cudaStream_t st)
{
    dim3 grid(L + 1, batch);
    long long cs = so3_off(L + 1);
    if (fp64)
        so3_r2c_kernel<double, double2, double><<<grid, 256, 0, st>>>((const double*)Fr, (double2*)Fc, L, cs);
    else
        so3_r2c_kernel<float, float2, float><<<grid, 256, 0, st>>>((const float*)Fr, (float2*)Fc, L, cs);
    return cudaGetLastError();
}

cudaError_t launch_s2_fwd_fp64(const double* table, const long long* moff, const double2* G, const double* w,
                               double2* F, int L, int N, int batch, bool is_real, cudaStream_t st)
{
    size_t smem = sizeof(double2) * 2 * N;
    dim3 grid(L + 1, batch);
    s2_fwd_fp64_kernel<256><<<grid, 256, smem, st>>>(table, moff, G, w, F, L, N, (long long)N * N,
                                                     (long long)(L + 1) * (L + 1), is_real ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_s2_inv_fp64(const double* table, const long long* moff, const double2* F, double2* H, int L,
                               int N, int batch, cudaStream_t st)
{
    size_t smem = sizeof(double2) * 2 * (L + 1);
    dim3 grid(L + 1, batch);
    s2_inv_fp64_kernel<256><<<grid, 256, smem, st>>>(table, moff, F, H, L, N, (long long)N * N,
                                                     (long long)(L + 1) * (L + 1));
    return cudaGetLastError();
}

cudaError_t launch_zero_nyquist_s2(void* H, bool fp64, int N, long long nrows, cudaStream_t st)
{
    unsigned nb = (unsigned)((nrows + 255) / 256);
    if (fp64)
        zero_nyquist_s2_kernel<double2><<<nb, 256, 0, st>>>((double2*)H, N, nrows);
    else
        zero_nyquist_s2_kernel<float2><<<nb, 256, 0, st>>>((float2*)H, N, nrows);
    return cudaGetLastError();
}

cudaError_t launch_s2_c2r(const void* Fc, void* Fr, bool fp64, int L, int batch, cudaStream_t st)
{
    long long C = (long long)(L + 1) * (L + 1);
    dim3 grid((unsigned)((C + 255) / 256), batch);
    if (fp64)
        s2_c2r_kernel<double2, double, double><<<grid, 256, 0, st>>>((const double2*)Fc, (double*)Fr, L, C);
    else
        s2_c2r_kernel<float2, float, float><<<grid, 256, 0, st>>>((const float2*)Fc, (float*)Fr, L, C);
    return cudaGetLastError();
}

cudaError_t launch_s2_group_to_real(const void* Fg, void* Fr, const long long* goff2, int L, int batch,
                                   cudaStream_t st)
{
    const long long C = (long long)(L + 1) * (L + 1);
    const unsigned nt = (unsigned)((L + 1 + S2T - 1) / S2T);
    s2_group_to_real_kernel<<<dim3(nt, nt, batch), 256, 0, st>>>((const float2*)Fg, (float*)Fr, goff2, L, C);
    return cudaGetLastError();
}

cudaError_t launch_s2_real_to_group(const void* Fr, void* Y, const long long* goff2, int L, int batch,
                                   cudaStream_t st)
{
    const long long C = (long long)(L + 1) * (L + 1);
    const unsigned nt = (unsigned)((L + 1 + S2T - 1) / S2T);
    s2_real_to_group_kernel<<<dim3(nt, nt, batch), 256, 0, st>>>((const float*)Fr, (float2*)Y, goff2, L, C);
    return cudaGetLastError();
}

cudaError_t launch_s2_r2c(const void* Fr, void* Fc, bool fp64, int L, int batch, cudaStream_t st)
{
    long long C = (long long)(L + 1) * (L + 1);
    dim3 grid((unsigned)((C + 255) / 256), batch);
    if (fp64)
        s2_r2c_kernel<double, double2, double><<<grid, 256, 0, st>>>((const double*)Fr, (double2*)Fc, L, C);
    else
        s2_r2c_kernel<float, float2, float><<<grid, 256, 0, st>>>((const float*)Fr, (float2*)Fc, L, C);
    return cudaGetLastError();
}

// ---- residual refinement of the FP32-data plans (F += forward(f - inverse(F)), the inverse in FP64)

__global__ void widen_kernel(const float* __restrict__ in, double* __restrict__ out, long long n)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (double)in[i];
}

// r = f - g with f the FP32 samples the forward transformed and g the FP64
// synthesis of its first result: the subtraction is done in FP64 (f is exact
// there), only the small difference is rounded to FP32.  f may be r itself.
__global__ void resid_fp64_kernel(const float* f, const double* __restrict__ g, float* r, long long n)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) r[i] = (float)((double)f[i] - g[i]);
}

__global__ void add_real_kernel(float* __restrict__ F, const float* __restrict__ d, long long n)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) F[i] += d[i];
}

cudaError_t launch_widen(const float* in, double* out, long long n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    widen_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, out, n);
    return cudaGetLastError();
}

__global__ void narrow_kernel(const double* __restrict__ in, float* __restrict__ out, long long n)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (float)in[i];
}

cudaError_t launch_narrow(const double* in, float* out, long long n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    narrow_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, out, n);
    return cudaGetLastError();
}

cudaError_t launch_resid_fp64(const float* f, const double* g, float* r, long long n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    resid_fp64_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(f, g, r, n);
    return cudaGetLastError();
}

cudaError_t launch_add_real(float* F, const float* d, long long n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    add_real_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(F, d, n);
    return cudaGetLastError();
}

}  // namespace fftso3
