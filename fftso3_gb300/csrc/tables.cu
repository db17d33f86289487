// Wigner-d / Legendre table kernels and FP64 point-evaluation kernels.
//
// Compiled with -fmad=false (see wigner_rec.cuh): the reference-faithful
// recursions must not be contracted into fused multiply-adds.
//
// Table layout (both tables): one block per symmetry group, rows l from the
// group's first degree l0, the beta index k contiguous:
//     table[goff(g) + (l - l0) * N + k]
//   Wigner:   g <-> (m0, n0), m0 >= |n0|, l0 = m0 (the lower triangle the
//             reference fills by recursion, fdcl_FFTSO3.cpp:150-171; every
//             other (m, n) is a signed copy, :173-190).
//   Legendre: g = m >= 0, l0 = m; nP(l,-m) = (-1)^m nP(l,m) (fdcl_FFTS2.cpp:95-97).
#include "common.cuh"
#include "tables.cuh"
#include "wigner_rec.cuh"

namespace fftso3 {

// One thread per (group, k); consecutive threads write consecutive k.
__global__ void wigner_table_kernel(double* __restrict__ table, const long long* __restrict__ goff,
                                    const WignerSeeds* __restrict__ seeds, const double* __restrict__ lfact, int L,
                                    int N, int ngroups, int stable)
{
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)ngroups * N) return;
    int g = (int)(idx / N), k = (int)(idx % N);
    int m0, n0;
    group_mn(g, m0, n0);
    const WignerSeeds s = seeds[k];
    double* out = table + goff[g] + k;
    auto emit = [&](int l, double v) { out[(long long)(l - m0) * N] = v; };
    if (stable)
        wigner_column_stable(m0, n0, L, s, lfact, emit);
    else
        wigner_column_faithful(m0, n0, L, s, emit);
}

// One thread per (m, k).
__global__ void legendre_table_kernel(double* __restrict__ table, const long long* __restrict__ moff,
                                      const double* __restrict__ xs, int L, int N)
{
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)(L + 1) * N) return;
    int m = (int)(idx / N), k = (int)(idx % N);
    double* out = table + moff[m] + k;
    auto emit = [&](int l, double v) { out[(long long)(l - m) * N] = v; };
    legendre_column_faithful(m, L, xs[k], emit);
}

cudaError_t launch_wigner_table(double* table, const long long* goff, const WignerSeeds* seeds, const double* lfact,
                                int L, int N, int ngroups, bool stable, cudaStream_t st)
{
    long long tot = (long long)ngroups * N;
    int th = 128;
    wigner_table_kernel<<<(unsigned)((tot + th - 1) / th), th, 0, st>>>(table, goff, seeds, lfact, L, N, ngroups,
                                                                       stable ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_legendre_table(double* table, const long long* moff, const double* xs, int L, int N,
                                  cudaStream_t st)
{
    long long tot = (long long)(L + 1) * N;
    int th = 128;
    legendre_table_kernel<<<(unsigned)((tot + th - 1) / th), th, 0, st>>>(table, moff, xs, L, N);
    return cudaGetLastError();
}

// ----------------------------------------------------------- point kernels

template <int NT>
__device__ __forceinline__ double2 block_sum(double2 v)
{
    __shared__ double2 red[NT];
    red[threadIdx.x] = v;
    __syncthreads();
    for (int s = NT / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            red[threadIdx.x].x += red[threadIdx.x + s].x;
            red[threadIdx.x].y += red[threadIdx.x + s].y;
        }
        __syncthreads();
    }
    return red[0];
}

// f(alpha,beta,gamma) = sum_{m,n} e^{-i m alpha} e^{-i n gamma} sum_l (2l+1) F(l,m,n) d^l_mn(beta)
// (fdcl_FFTSO3.cpp:498-531), one CTA per point, threads over symmetry groups.
template <int NT>
__global__ void __launch_bounds__(NT) so3_points_kernel(const double2* __restrict__ F, const WignerSeeds* __restrict__ pseeds,
                                                        const double* __restrict__ pts, const double* __restrict__ lfact,
                                                        int L, int stable, double2* __restrict__ out)
{
    const int pt = blockIdx.x;
    const WignerSeeds s = pseeds[pt];
    const double alpha = pts[3 * pt], gamma = pts[3 * pt + 2];
    const int B = L + 1;
    double2 acc = make_double2(0., 0.);
    for (int g = threadIdx.x; g < B * B; g += NT) {
        int m0, n0;
        group_mn(g, m0, n0);
        GroupPairs P = group_pairs(m0, n0);
        double sr[4] = {0., 0., 0., 0.}, si[4] = {0., 0., 0., 0.};
        auto emit = [&](int l, double d) {
            const double w = (double)(2 * l + 1);
#pragma unroll
            for (int p = 0; p < 4; ++p) {
                if (p < P.np) {
                    double2 c = F[so3_idx(l, P.m[p], P.n[p])];
                    sr[p] += w * c.x * d;
                    si[p] += w * c.y * d;
                }
            }
        };
        if (stable)
            wigner_column_stable(m0, n0, L, s, lfact, emit);
        else
            wigner_column_faithful(m0, n0, L, s, emit);
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            if (p < P.np) {
                double sa, ca, sg, cg;
                sincos(-(double)P.m[p] * alpha, &sa, &ca);
                sincos(-(double)P.n[p] * gamma, &sg, &cg);
                double er = ca * cg - sa * sg, ei = ca * sg + sa * cg;
                double vr = P.sign[p] * sr[p], vi = P.sign[p] * si[p];
                acc.x += vr * er - vi * ei;
                acc.y += vr * ei + vi * er;
            }
        }
    }
    double2 t = block_sum<NT>(acc);
    if (threadIdx.x == 0) out[pt] = t;
}

// y(theta,phi) = sum_{l,m} F(l,m) nP(l,m)(cos theta) e^{i m phi} (fdcl_FFTS2.cpp:17-46, :194-230).
template <int NT>
__global__ void __launch_bounds__(NT) s2_points_kernel(const double2* __restrict__ F, const double* __restrict__ xs,
                                                       const double* __restrict__ pts, int L, double2* __restrict__ out)
{
    const int pt = blockIdx.x;
    const double phi = pts[2 * pt + 1];
    double2 acc = make_double2(0., 0.);
    for (int m = threadIdx.x; m <= L; m += NT) {
        double pr = 0., pi = 0., qr = 0., qi = 0.;
        auto emit = [&](int l, double v) {
            double2 a = F[s2_idx(l, m)];
            pr += a.x * v;
            pi += a.y * v;
            if (m > 0) {
                double2 b = F[s2_idx(l, -m)];
                qr += b.x * v;
                qi += b.y * v;
            }
        };
        legendre_column_faithful(m, L, xs[pt], emit);
        double sp, cp;
        sincos((double)m * phi, &sp, &cp);
        acc.x += pr * cp - pi * sp;
        acc.y += pr * sp + pi * cp;
        if (m > 0) {
            double sg = (m & 1) ? -1.0 : 1.0;  // nP(l,-m) = (-1)^m nP(l,m), e^{-i m phi}
            qr *= sg;
            qi *= sg;
            acc.x += qr * cp + qi * sp;
            acc.y += qi * cp - qr * sp;
        }
    }
    double2 t = block_sum<NT>(acc);
    if (threadIdx.x == 0) out[pt] = t;
}

cudaError_t launch_so3_points(const double2* F, const WignerSeeds* pseeds, const double* pts, const double* lfact,
                              int L, bool stable, int n, double2* out, cudaStream_t st)
{
    so3_points_kernel<128><<<n, 128, 0, st>>>(F, pseeds, pts, lfact, L, stable ? 1 : 0, out);
    return cudaGetLastError();
}

cudaError_t launch_s2_points(const double2* F, const double* xs, const double* pts, int L, int n, double2* out,
                             cudaStream_t st)
{
    s2_points_kernel<128><<<n, 128, 0, st>>>(F, xs, pts, L, out);
    return cudaGetLastError();
}

// Full packed d^l_mn(beta) for all l <= L at one angle: each thread computes
// one group's column and writes every member of the orbit with its sign
// (fdcl_FFTSO3.cpp:173-190).
__global__ void wigner_full_kernel(const WignerSeeds* __restrict__ seed, const double* __restrict__ lfact, int L,
                                   int stable, double* __restrict__ out)
{
    const int B = L + 1;
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= B * B) return;
    int m0, n0;
    group_mn(g, m0, n0);
    const GroupPairs P = group_pairs(m0, n0);
    const WignerSeeds s = seed[0];
    auto emit = [&](int l, double v) {
        for (int p = 0; p < P.np; ++p) out[so3_idx(l, P.m[p], P.n[p])] = P.sign[p] * v;
    };
    if (stable)
        wigner_column_stable(m0, n0, L, s, lfact, emit);
    else
        wigner_column_faithful(m0, n0, L, s, emit);
}

cudaError_t launch_wigner_full(const WignerSeeds* seed, const double* lfact, int L, bool stable, double* out,
                               cudaStream_t st)
{
    int ng = (L + 1) * (L + 1);
    wigner_full_kernel<<<(ng + 127) / 128, 128, 0, st>>>(seed, lfact, L, stable ? 1 : 0, out);
    return cudaGetLastError();
}

}  // namespace fftso3
