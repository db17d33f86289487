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
#include <algorithm>

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

// ------------------------------------------------- SO(3) point evaluation
//
// f(alpha,beta,gamma) = sum_{m,n} e^{-i m alpha} e^{-i n gamma} sum_l (2l+1) F(l,m,n) d^l_mn(beta)
// (fdcl_FFTSO3.cpp:498-531).  FP64 is a small unit on this part, so the kernel spends its FP64
// operations on the O(B^3) core only:
//   * one warp evaluates 32 points (lane = point): the loops over (m0, n0, l) are the same for every
//     point, so each coefficient load is one broadcast per warp and no lane waits on another;
//   * the beta-independent factors of the recursion (64) come from a per-plan table (below), so a
//     recursion step is five multiplies / subtractions instead of two square roots and two divisions;
//   * the seeds (65)-(68) of all groups of one m0 are the prefixes of one chain over n0 (the
//     reference's loops over n run from m0 - 1 down to n0), so they cost O(B^2) per point, not O(B^3);
//   * e^{-i m0 alpha} comes from sincos once per m0, e^{-i n0 alpha} by one complex step per group.
// The Wigner-d values are the same doubles as the table kernel's (same operations, this unit's
// -fmad=false), so a reference-recursion plan keeps the reference's underflow near beta = pi.
// The degrees m0 split into parts of equal work (blockIdx.y) whose partial sums are added in a fixed
// order by a second kernel.

// beta-independent factors of (64) per (group, l), l = m0 + 1..L, as {a, c, P2, P1}:
//   a = 1/sqrt((l^2-m^2)(l^2-n^2)),  c = sqrt(((l-1)^2-m^2)((l-1)^2-n^2)) l/(l-1),
//   P2 = (2l-1) m n/(l-1),  P1 = l(2l-1),  d^l = a ((P1 cos(beta) - P2) d^{l-1} - c d^{l-2}),
// with the expressions of rec64_faithful and of the stable column (so the same doubles); row (0, 1)
// is unused (d^1_00 = cos(beta)) and zero.  Group (m0, n0) starts at rec_row0(m0) + (n0 + m0)(L - m0).
// sq[l (l - 1) + n + l] = sqrt(((l + n) + 1) / (l - n)), 1 <= l <= L + 1, -l <= n < l: the seed factors.
__host__ __device__ inline long long rec_row0(int m0, int L)
{
    long long o = 0;
    for (int m = 0; m < m0; ++m) o += (long long)(2 * m + 1) * (L - m);
    return o;
}
__host__ __device__ inline long long sq_idx(int l, int n) { return (long long)l * (l - 1) + n + l; }

size_t wigner_rec_elems(int L) { return (size_t)rec_row0(L + 1, L); }
size_t wigner_sq_elems(int L) { return (size_t)(L + 1) * (L + 2); }

__global__ void wigner_rec_factors_kernel(double4* __restrict__ rec, double* __restrict__ sq, int L)
{
    const int B = L + 1;
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < B * B) {
        int m0, n0;
        group_mn(g, m0, n0);
        double4* row = rec + rec_row0(m0, L) + (long long)(n0 + m0) * (L - m0);
        const double mm = (double)m0 * (double)m0, nn = (double)n0 * (double)n0;
        for (int l = m0 + 1; l <= L; ++l) {
            double4 f = make_double4(0., 0., 0., 0.);
            if (l >= 2) {
                const double ll = (double)l * (double)l, lm1 = (double)l - 1.;
                f.x = 1. / sqrt((ll - mm) * (ll - nn));
                f.y = sqrt(fmax((lm1 * lm1 - mm) * (lm1 * lm1 - nn), 0.0)) * (double)l / lm1;
                f.z = (2. * (double)l - 1.) * (double)m0 * (double)n0 / lm1;
                f.w = (double)l * (2. * (double)l - 1.);
            }
            row[l - m0 - 1] = f;
        }
    }
    if (g >= 1 && g <= L + 1)
        for (int n = -g; n < g; ++n) sq[sq_idx(g, n)] = sqrt(((double)(g + n) + 1.) / (double)(g - n));
}

cudaError_t launch_wigner_rec_factors(double4* rec, double* sq, int L, cudaStream_t st)
{
    const int nt = std::max((L + 1) * (L + 1), L + 2);
    wigner_rec_factors_kernel<<<(nt + 127) / 128, 128, 0, st>>>(rec, sq, L);
    return cudaGetLastError();
}

struct PointParts {
    int m0[MAX_POINT_PARTS + 1];  // part s covers the degrees m0 in [m0[s], m0[s + 1])
};

constexpr int PW = 4;  // warps (batches of 32 points) per CTA

__device__ __forceinline__ double4 ld_rec(const double4* p)
{
    const double2* q = reinterpret_cast<const double2*>(p);
    const double2 a = __ldg(q), b = __ldg(q + 1);
    return make_double4(a.x, a.y, b.x, b.y);
}

__device__ __forceinline__ double2 cmul2(double2 a, double2 b)
{
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

template <bool STABLE>
__global__ void __launch_bounds__(32 * PW) so3_points_kernel(const double2* __restrict__ F,
                                                             const WignerSeeds* __restrict__ pseeds,
                                                             const double* __restrict__ pts,
                                                             const double4* __restrict__ rec,
                                                             const double* __restrict__ sq,
                                                             const double* __restrict__ lfact, int L, int n,
                                                             const PointParts parts, double2* __restrict__ part)
{
    extern __shared__ double wl[];  // wl[l] = 2l + 1
    for (int l = threadIdx.x; l <= L; l += blockDim.x) wl[l] = (double)(2 * l + 1);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * PW + (threadIdx.x >> 5);
    if (b * 32 >= n) return;
    const int pt = b * 32 + lane;
    const int pq = pt < n ? pt : n - 1;  // lanes past n evaluate a copy of the last point, not written
    const WignerSeeds s = pseeds[pq];
    const double alpha = pts[3 * pq], gamma = pts[3 * pq + 2], cb = s.cb;
    double sa1, ca1, sg1, cg1;
    sincos(alpha, &sa1, &ca1);
    sincos(gamma, &sg1, &cg1);
    const double2 upa = make_double2(ca1, sa1), upg = make_double2(cg1, sg1);  // n0 -> n0 - 1 steps
    const int mb = parts.m0[blockIdx.y], me = parts.m0[blockIdx.y + 1];
    long long row0 = rec_row0(mb, L);
    double dd = s.d111;  // d(m0, m0, m0) = d111^m0 (65), as the reference's loop forms it
    if (!STABLE)
        for (int m = 2; m < mb; ++m) dd = s.d111 * dd;
    double2 acc = make_double2(0., 0.);
    for (int m0 = mb; m0 < me; ++m0) {
        if (m0 == 0) {
            // group (0, 0), both modes: d^0 = 1, d^1 = cos(beta), then (64)
            double2 D = __ldg(&F[0]);
            if (L >= 1) {
                const double2 c = __ldg(&F[so3_idx(1, 0, 0)]);
                D.x = __fma_rn(c.x, wl[1] * cb, D.x);
                D.y = __fma_rn(c.y, wl[1] * cb, D.y);
            }
            double d2 = 1., d1 = cb;
            for (int l = 2; l <= L; ++l) {
                const double4 f = ld_rec(&rec[row0 + (l - 1)]);
                const double v = f.x * ((f.w * cb - f.z) * d1 - f.y * d2);
                const double wv = wl[l] * v;
                const double2 c = __ldg(&F[so3_idx(l, 0, 0)]);
                D.x = __fma_rn(c.x, wv, D.x);
                D.y = __fma_rn(c.y, wv, D.y);
                d2 = d1;
                d1 = v;
            }
            acc.x += D.x;
            acc.y += D.y;
            row0 += L;
            continue;
        }
        double sm, cm, sgm, cgm;
        sincos((double)m0 * alpha, &sm, &cm);
        sincos((double)m0 * gamma, &sgm, &cgm);
        const double2 Ema = make_double2(cm, -sm), Emg = make_double2(cgm, -sgm);
        double2 Ena = Ema, Eng = Emg;  // e^{-i n0 alpha}, e^{-i n0 gamma} at n0 = m0
        if (!STABLE && m0 >= 2) dd = s.d111 * dd;
        const int l1 = m0 + 1, rows = L - m0;
        const double lcb = (double)l1 * cb;
        double v0 = dd;                           // (67) chain at l = m0 (m0 >= 2), n0 = m0
        double v1 = (lcb - (double)l1 + 1.) * dd;  // (66), then the (68) chain at l = m0 + 1
        long long grow = row0 + (long long)(2 * m0) * rows;
        for (int n0 = m0; n0 >= -m0; --n0) {
            if (n0 < m0) {
                if (!STABLE) {
                    if (m0 >= 2) v0 = (-__ldg(&sq[sq_idx(m0, n0)]) * s.tb2) * v0;
                    if (l1 <= L)
                        v1 = (-(lcb - (double)n0)) / (lcb - (double)n0 - 1.) * __ldg(&sq[sq_idx(l1, n0)]) * s.tb2 * v1;
                }
                Ena = cmul2(Ena, upa);
                Eng = cmul2(Eng, upg);
                grow -= rows;
            }
            const bool four = n0 != m0 && n0 != -m0;
            double2 D0 = make_double2(0., 0.), D1 = D0, D2 = D0, D3 = D0;
            auto emit = [&](int l, double v) {
                const double wv = wl[l] * v;
                const long long o = so3_off(l);
                const long long w = 2 * l + 1;
                const double2 c0 = __ldg(&F[o + (m0 + l) + (n0 + l) * w]);
                const double2 c1 = __ldg(&F[o + (l - m0) + (l - n0) * w]);
                D0.x = __fma_rn(c0.x, wv, D0.x);
                D0.y = __fma_rn(c0.y, wv, D0.y);
                D1.x = __fma_rn(c1.x, wv, D1.x);
                D1.y = __fma_rn(c1.y, wv, D1.y);
                if (four) {
                    const double2 c2 = __ldg(&F[o + (n0 + l) + (m0 + l) * w]);
                    const double2 c3 = __ldg(&F[o + (l - n0) + (l - m0) * w]);
                    D2.x = __fma_rn(c2.x, wv, D2.x);
                    D2.y = __fma_rn(c2.y, wv, D2.y);
                    D3.x = __fma_rn(c3.x, wv, D3.x);
                    D3.y = __fma_rn(c3.y, wv, D3.y);
                }
            };
            if (STABLE) {
                // closed-form seed and renormalised (64), as wigner_column_stable
                const double LN2 = 0.69314718055994530942;
                double lg = 0.5 * (lfact[2 * m0] - lfact[m0 + n0] - lfact[m0 - n0]);
                if (m0 + n0 > 0) lg += (double)(m0 + n0) * s.lc2;
                if (m0 - n0 > 0) lg += (double)(m0 - n0) * s.ls2;
                int E = 0;
                double d1 = 0.;  // beta = 0 or pi: the whole column is exactly zero
                if (lg > -1.0e300) {
                    double sgn = ((m0 - n0) & 1) ? -1.0 : 1.0;
                    if (((m0 + n0) & 1) && s.c2 < 0.0) sgn = -sgn;
                    if (((m0 - n0) & 1) && s.s2 < 0.0) sgn = -sgn;
                    const double e2 = lg / LN2;
                    if (e2 >= -900.0) {
                        d1 = sgn * exp2(e2);
                    } else {
                        E = 600 * (int)floor((e2 + 300.0) / 600.0);
                        d1 = sgn * exp2(e2 - (double)E);
                    }
                }
                double d2 = 0.;
                emit(m0, (E == 0) ? d1 : ldexp(d1, E));
                for (int l = l1; l <= L; ++l) {
                    const double4 f = ld_rec(&rec[grow + (l - l1)]);
                    const double v = f.x * ((f.w * cb - f.z) * d1 - f.y * d2);
                    d2 = d1;
                    d1 = v;
                    if (E < 0 && fabs(d1) > 0x1p600) {
                        d1 = ldexp(d1, -600);
                        d2 = ldexp(d2, -600);
                        E += 600;
                    }
                    emit(l, (E == 0) ? d1 : ldexp(d1, E));
                }
            } else {
                const double v0g = m0 == 1 ? (n0 == 1 ? s.d111 : (n0 == 0 ? s.d110 : s.d11m1)) : v0;
                emit(m0, v0g);
                if (l1 <= L) {
                    emit(l1, v1);
                    double d2 = v0g, d1 = v1;
                    for (int l = l1 + 1; l <= L; ++l) {
                        const double4 f = ld_rec(&rec[grow + (l - l1)]);
                        const double v = f.x * ((f.w * cb - f.z) * d1 - f.y * d2);
                        emit(l, v);
                        d2 = d1;
                        d1 = v;
                    }
                }
            }
            // p0 (m0, n0), p1 (-m0, -n0) sign (-1)^(m0+n0), p2 (n0, m0) same sign, p3 (-n0, -m0)
            const double sg = ((m0 + n0) & 1) ? -1. : 1.;
            const double2 ph0 = cmul2(Ema, Eng);
            const double2 t0 = cmul2(D0, ph0), t1 = cmul2(D1, make_double2(ph0.x, -ph0.y));
            acc.x += t0.x + sg * t1.x;
            acc.y += t0.y + sg * t1.y;
            if (four) {
                const double2 ph2 = cmul2(Ena, Emg);
                const double2 t2 = cmul2(D2, ph2), t3 = cmul2(D3, make_double2(ph2.x, -ph2.y));
                acc.x += sg * t2.x + t3.x;
                acc.y += sg * t2.y + t3.y;
            }
        }
        row0 += (long long)(2 * m0 + 1) * rows;
    }
    if (pt < n) part[(long long)blockIdx.y * n + pt] = acc;
}

__global__ void sum_parts_kernel(const double2* __restrict__ part, int S, int n, double2* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double2 a = part[i];
    for (int s = 1; s < S; ++s) {
        const double2 v = part[(long long)s * n + i];
        a.x += v.x;
        a.y += v.y;
    }
    out[i] = a;
}

// Degree parts of about equal work ((2 m0 + 1)(L - m0 + 2) per m0 for SO(3), L - m + 2 per order m for
// S^2), enough of them that the launch has about 16 warps per SM; returns their number S, bounds in m0b[0..S].
int points_parts(bool so3, int L, int n, int nsm, int* m0b)
{
    const long long nb = ((long long)n + 31) / 32;
    long long S = (16LL * std::max(nsm, 1) + nb - 1) / nb;
    S = std::max(1LL, std::min<long long>({S, (long long)MAX_POINT_PARTS, (long long)L + 1}));
    auto work = [&](int m) { return (so3 ? 2.0 * m + 1.0 : 1.0) * (L - m + 2); };
    double total = 0.;
    for (int m = 0; m <= L; ++m) total += work(m);
    int k = 0;
    m0b[0] = 0;
    double cum = 0.;
    for (int m = 0; m <= L && k + 1 < S; ++m) {
        cum += work(m);
        if (cum >= total * (double)(k + 1) / (double)S && m + 1 <= L) m0b[++k] = m + 1;
    }
    m0b[++k] = L + 1;
    return k;
}

cudaError_t launch_so3_points(const double2* F, const WignerSeeds* pseeds, const double* pts, const double4* rec,
                              const double* sq, const double* lfact, int L, bool stable, int n, const int* m0b,
                              int S, double2* part, double2* out, cudaStream_t st)
{
    if (S < 1 || S > MAX_POINT_PARTS) return cudaErrorInvalidValue;
    PointParts P;
    for (int s = 0; s <= S; ++s) P.m0[s] = m0b[s];
    const long long nb = ((long long)n + 31) / 32;
    const dim3 grid((unsigned)((nb + PW - 1) / PW), (unsigned)S);
    const size_t smem = sizeof(double) * (size_t)(L + 1);
    if (stable)
        so3_points_kernel<true><<<grid, 32 * PW, smem, st>>>(F, pseeds, pts, rec, sq, lfact, L, n, P, part);
    else
        so3_points_kernel<false><<<grid, 32 * PW, smem, st>>>(F, pseeds, pts, rec, sq, lfact, L, n, P, part);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    sum_parts_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(part, S, n, out);
    return cudaGetLastError();
}

// ------------------------------------------------- S^2 point evaluation
//
// y(theta,phi) = sum_{l,m} F(l,m) nP(l,m)(cos theta) e^{i m phi} (fdcl_FFTS2.cpp:17-46, :194-230), in the
// layout of the SO(3) point kernel: one warp per 32 points, the orders m split into parts of equal work.
// The Legendre recursion of fdcl_FFTS2.cpp:48-100 runs with its beta-independent factors from a per-plan
// table: step l uses fact(l, m) = sqrt((4l^2 - 1)/(l^2 - m^2)) and 1/fact(l - 1, m) (the reference
// divides by fact(l - 1, m), so values agree with it to rounding, not bit for bit); the seed pmm(m) keeps
// the reference's operations, chained over m.  Table: per m, rows l = m + 2..L of {fact, 1/previous
// fact}, starting at s2_row0(m) (the first previous fact is sqrt(2m + 3)).
__host__ __device__ inline long long s2_row0(int m, int L)
{
    long long o = 0;
    for (int k = 0; k < m; ++k) o += (L - k - 1 > 0) ? L - k - 1 : 0;
    return o;
}
size_t legendre_rec_elems(int L) { return (size_t)std::max<long long>(s2_row0(L + 1, L), 1); }

__global__ void legendre_rec_factors_kernel(double2* __restrict__ rec, int L)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m > L) return;
    double2* row = rec + s2_row0(m, L);
    double oldfact = sqrt(2.0 * (double)m + 3.0);
    for (int l = m + 2; l <= L; ++l) {
        const double fact = sqrt((4.0 * (double)l * (double)l - 1.0) / (double)(l * l - m * m));
        row[l - m - 2] = make_double2(fact, 1.0 / oldfact);
        oldfact = fact;
    }
}

cudaError_t launch_legendre_rec_factors(double2* rec, int L, cudaStream_t st)
{
    legendre_rec_factors_kernel<<<(L + 1 + 127) / 128, 128, 0, st>>>(rec, L);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(32 * PW) s2_points_kernel(const double2* __restrict__ F, const double* __restrict__ xs,
                                                            const double* __restrict__ pts,
                                                            const double2* __restrict__ rec, int L, int n,
                                                            const PointParts parts, double2* __restrict__ part)
{
    const double fourpi = 4.0 * 3.14159265358979323846;
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * PW + (threadIdx.x >> 5);
    if (b * 32 >= n) return;
    const int pt = b * 32 + lane;
    const int pq = pt < n ? pt : n - 1;  // lanes past n evaluate a copy of the last point, not written
    const double x = xs[pq], phi = pts[2 * pq + 1];
    const double omx2 = (1.0 - x) * (1.0 + x);
    const int mb = parts.m0[blockIdx.y], me = parts.m0[blockIdx.y + 1];
    // pmm before its sqrt: prod_{i <= m} omx2 (2i - 1) / (2i), the reference's loop chained over m
    double praw = 1.0;
    for (int i = 1; i < mb; ++i) {
        const double fact = (double)(2 * i - 1);
        praw *= omx2 * fact / (fact + 1.0);
    }
    long long row = s2_row0(mb, L);
    double2 acc = make_double2(0., 0.);
    for (int m = mb; m < me; ++m) {
        double pmm;
        if (m == 0) {
            pmm = sqrt(1. / fourpi);
        } else {
            const double fact = (double)(2 * m - 1);
            praw *= omx2 * fact / (fact + 1.0);
            pmm = sqrt((double)(2 * m + 1) * praw / fourpi);
            if (m & 1) pmm = -pmm;
        }
        double2 Dp = make_double2(0., 0.), Dn = Dp;
        auto emit = [&](int l, double v) {
            const double2 a = __ldg(&F[s2_idx(l, m)]);
            Dp.x = __fma_rn(a.x, v, Dp.x);
            Dp.y = __fma_rn(a.y, v, Dp.y);
            if (m > 0) {
                const double2 c = __ldg(&F[s2_idx(l, -m)]);
                Dn.x = __fma_rn(c.x, v, Dn.x);
                Dn.y = __fma_rn(c.y, v, Dn.y);
            }
        };
        emit(m, pmm);
        if (m + 1 <= L) {
            double p1 = x * sqrt(2.0 * (double)m + 3.0) * pmm, p0 = pmm;
            emit(m + 1, p1);
            for (int l = m + 2; l <= L; ++l) {
                const double2 f = __ldg(&rec[row + (l - m - 2)]);
                const double v = (x * p1 - p0 * f.y) * f.x;
                emit(l, v);
                p0 = p1;
                p1 = v;
            }
        }
        row += (L - m - 1 > 0) ? L - m - 1 : 0;
        double sp, cp;
        sincos((double)m * phi, &sp, &cp);
        acc.x += Dp.x * cp - Dp.y * sp;  // F(l, m) nP e^{i m phi}
        acc.y += Dp.x * sp + Dp.y * cp;
        if (m > 0) {
            const double sg = (m & 1) ? -1.0 : 1.0;  // nP(l,-m) = (-1)^m nP(l,m), e^{-i m phi}
            acc.x += sg * (Dn.x * cp + Dn.y * sp);
            acc.y += sg * (Dn.y * cp - Dn.x * sp);
        }
    }
    if (pt < n) part[(long long)blockIdx.y * n + pt] = acc;
}

cudaError_t launch_s2_points(const double2* F, const double* xs, const double* pts, const double2* rec, int L, int n,
                             const int* m0b, int S, double2* part, double2* out, cudaStream_t st)
{
    if (S < 1 || S > MAX_POINT_PARTS) return cudaErrorInvalidValue;
    PointParts P;
    for (int s = 0; s <= S; ++s) P.m0[s] = m0b[s];
    const long long nb = ((long long)n + 31) / 32;
    const dim3 grid((unsigned)((nb + PW - 1) / PW), (unsigned)S);
    s2_points_kernel<<<grid, 32 * PW, 0, st>>>(F, xs, pts, rec, L, n, P, part);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    sum_parts_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(part, S, n, out);
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
