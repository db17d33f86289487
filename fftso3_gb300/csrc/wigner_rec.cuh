// Column recursions for the Wigner-d and normalized associated Legendre
// functions, shared by the table kernels and the point-evaluation kernels.
//
// A "column" is one symmetry group at one angle: d^l_{m0 n0}(beta) for
// l = m0..L (m0 >= |n0|), or nP(l, m)(x) for l = m..L.  Each value is handed
// to emit(l, value) in increasing l.
//
// The *_faithful functions keep the operation order of the reference
// (fdcl_FFTSO3.cpp:127-194, fdcl_FFTS2.cpp:48-100); translation units that
// include them are compiled with -fmad=false so the values are bit-for-bit the
// reference's on the same machine (host-computed seeds, IEEE +,-,*,/,sqrt).
#pragma once
#include "common.cuh"
#include "tables.cuh"

namespace fftso3 {

__device__ __forceinline__ double rec64_faithful(int l, int m, int n, double cb, double d1, double d2)
{
    // (64): 1/sqrt((l^2-m^2)(l^2-n^2)) * ((l(2l-1)cb - (2l-1)mn/(l-1)) d1
    //        - sqrt(((l-1)^2-m^2)((l-1)^2-n^2)) l/(l-1) d2)
    double ll = (double)l * (double)l, mm = (double)m * (double)m, nn = (double)n * (double)n;
    double lm1 = (double)l - 1.;
    double a = 1. / sqrt((ll - mm) * (ll - nn));
    double b = (double)l * (2. * (double)l - 1.) * cb - (2. * (double)l - 1.) * (double)m * (double)n / lm1;
    double c = sqrt((lm1 * lm1 - mm) * (lm1 * lm1 - nn)) * (double)l / lm1;
    return a * (b * d1 - c * d2);
}

// fdcl_FFTSO3.cpp:127-194 restricted to one (m0, n0), m0 >= |n0|.  Rows l = m0
// and l = m0 + 1 come from the reference's seed formulas (65)-(68) (or the
// explicit l = 1 values), rows l >= m0 + 2 from (64).
template <class Emit>
__device__ __forceinline__ void wigner_column_faithful(int m0, int n0, int L, const WignerSeeds& s, Emit&& emit)
{
    if (m0 == 0) {
        emit(0, 1.);
        if (L < 1) return;
        emit(1, s.cb);
        double d2 = 1., d1 = s.cb;
        for (int l = 2; l <= L; ++l) {
            double v = rec64_faithful(l, 0, 0, s.cb, d1, d2);
            emit(l, v);
            d2 = d1;
            d1 = v;
        }
        return;
    }
    double dd = s.d111;  // d(l,l,l) = d(1,1,1) d(l-1,l-1,l-1), (65)
    for (int l = 2; l <= m0; ++l) dd = s.d111 * dd;
    double v0;
    if (m0 == 1) {
        v0 = (n0 == 1) ? s.d111 : (n0 == 0 ? s.d110 : s.d11m1);
    } else {
        const int l = m0;
        v0 = dd;
        for (int n = l - 1; n >= n0; --n)
            v0 = -sqrt(((double)(l + n) + 1.) / (double)(l - n)) * s.tb2 * v0;  // (67)
    }
    emit(m0, v0);
    if (m0 + 1 > L) return;
    double v1;
    {
        const int l = m0 + 1;
        v1 = ((double)l * s.cb - (double)l + 1.) * dd;  // (66), dd = d(l-1,l-1,l-1)
        for (int n = l - 2; n >= n0; --n)
            v1 = -((double)l * s.cb - (double)n) / ((double)l * s.cb - (double)n - 1.) *
                 sqrt(((double)(l + n) + 1.) / (double)(l - n)) * s.tb2 * v1;  // (68)
    }
    emit(m0 + 1, v1);
    double d2 = v0, d1 = v1;
    for (int l = m0 + 2; l <= L; ++l) {
        double v = rec64_faithful(l, m0, n0, s.cb, d1, d2);
        emit(l, v);
        d2 = d1;
        d1 = v;
    }
}

// Stable column: closed-form log-domain seed at l = m0,
//   d^{m0}_{m0,n0} = (-1)^{m0-n0} sqrt(C(2m0, m0-n0)) cos(b/2)^{m0+n0} sin(b/2)^{m0-n0},
// then (64) upward with the value carried as mantissa * 2^E (E <= 0,
// renormalised by 2^-600 whenever the mantissa exceeds 2^600) so that an
// underflowing seed recovers when the true values grow back to O(1).
template <class Emit>
__device__ __forceinline__ void wigner_column_stable(int m0, int n0, int L, const WignerSeeds& s,
                                                     const double* __restrict__ lfact, Emit&& emit)
{
    const double LN2 = 0.69314718055994530942;
    double lg = 0.5 * (lfact[2 * m0] - lfact[m0 + n0] - lfact[m0 - n0]);
    if (m0 + n0 > 0) lg += (double)(m0 + n0) * s.lc2;
    if (m0 - n0 > 0) lg += (double)(m0 - n0) * s.ls2;
    if (!(lg > -1.0e300)) {  // beta = 0 or pi: the whole column is exactly zero
        for (int l = m0; l <= L; ++l) emit(l, 0.0);
        return;
    }
    double sgn = ((m0 - n0) & 1) ? -1.0 : 1.0;
    if (((m0 + n0) & 1) && s.c2 < 0.0) sgn = -sgn;
    if (((m0 - n0) & 1) && s.s2 < 0.0) sgn = -sgn;
    const double e2 = lg / LN2;
    int E = 0;
    double d1;
    if (e2 >= -900.0) {
        d1 = sgn * exp2(e2);
    } else {
        E = 600 * (int)floor((e2 + 300.0) / 600.0);
        d1 = sgn * exp2(e2 - (double)E);
    }
    double d2 = 0.0;
    emit(m0, (E == 0) ? d1 : ldexp(d1, E));
    const double cb = s.cb;
    for (int l = m0 + 1; l <= L; ++l) {
        double v;
        if (l == 1) {
            v = cb * d1;  // d^1_00 = cos(beta)
        } else {
            double ll = (double)l * l, mm = (double)m0 * m0, nn = (double)n0 * n0;
            double lm1 = (double)l - 1.0;
            double a = 1.0 / sqrt((ll - mm) * (ll - nn));
            double b = (double)l * (2.0 * l - 1.0) * cb - (2.0 * l - 1.0) * (double)m0 * (double)n0 / lm1;
            double c = sqrt(fmax((lm1 * lm1 - mm) * (lm1 * lm1 - nn), 0.0)) * (double)l / lm1;
            v = a * (b * d1 - c * d2);
        }
        d2 = d1;
        d1 = v;
        if (E < 0 && fabs(d1) > 0x1p600) {
            d1 = ldexp(d1, -600);
            d2 = ldexp(d2, -600);
            E += 600;
        }
        emit(l, (E == 0) ? d1 : ldexp(d1, E));
    }
}

// fdcl_FFTS2.cpp:48-100 restricted to one m >= 0 (Numerical Recipes 6.7).
template <class Emit>
__device__ __forceinline__ void legendre_column_faithful(int m, int L, double x, Emit&& emit)
{
    const double fourpi = 4.0 * 3.14159265358979323846;
    double pmm;
    if (m == 0) {
        pmm = sqrt(1. / fourpi);
    } else {
        pmm = 1.0;
        double omx2 = (1.0 - x) * (1.0 + x);
        double fact = 1.0;
        for (int i = 1; i <= m; ++i) {
            pmm *= omx2 * fact / (fact + 1.0);
            fact += 2.0;
        }
        pmm = sqrt((double)(2 * m + 1) * pmm / fourpi);
        if (m & 1) pmm = -pmm;
    }
    emit(m, pmm);
    if (m + 1 > L) return;
    double p1 = x * sqrt(2.0 * (double)m + 3.0) * pmm;
    emit(m + 1, p1);
    double p0 = pmm;
    double oldfact = sqrt(2.0 * (double)m + 3.0);
    for (int l = m + 2; l <= L; ++l) {
        double fact = sqrt((4.0 * (double)l * (double)l - 1.0) / (double)(l * l - m * m));
        double v = (x * p1 - p0 / oldfact) * fact;
        oldfact = fact;
        emit(l, v);
        p0 = p1;
        p1 = v;
    }
}

}  // namespace fftso3
