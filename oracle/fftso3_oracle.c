/*
 * fftso3_oracle.c -- CPU oracle for the SO(3) / S^2 harmonic-transform hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is a plain-C restatement of the
 * fdcl-gwu/FFTSO3 algorithms (file:line citations below, paths relative to the
 * reference project).  It exists to check the CUDA library and to time the
 * reference's CPU algorithm; the product (fftso3_gb300/) never links, loads or
 * calls it.
 *
 * Why a restatement and not the reference itself: the reference needs Eigen
 * (an un-vendored git submodule, extern/eigen3, no pinned commit; CMakeLists.txt
 * comments "Eigen3 3.3") for its containers and FFT (Eigen's kissfft backend),
 * so it cannot be compiled from its own sources here.  The arithmetic of the
 * path is restated with the reference's operation order (so that, compiled with
 * -ffp-contract=off, the Wigner-d and Legendre tables are bit-for-bit what the
 * reference computes on the same machine); Eigen's FFT is restated as its
 * published algorithm (unscaled forward DFT, e^{-2 pi i jk/N}, mixed radix).
 *
 * Conventions shared with the product:
 *   B = l_max+1, N = 2B.
 *   SO(3) coefficients, packed:  off(l) = l(4l^2-1)/3, element (l,m,n) at
 *     off(l) + (m+l) + (n+l)(2l+1)   (column-major (2l+1)^2 block per l, as
 *     fdcl_FFTSO3_matrix.cpp:43-47 stores M[l](m+l,n+l)).
 *   S^2 coefficients, packed: l^2 + (m+l)   (fdcl_FFTS2_matrix.cpp:43-47).
 *   SO(3) grid: [k][j1][j2]  (beta_k slowest, alpha_j1, gamma_j2 fastest),
 *     the loop order of fdcl_FFTSO3.cpp:676-685.
 *   S^2 grid: [k][j]  (theta_k, phi_j), fdcl_FFTS2.cpp:146-152.
 *   Complex arrays are interleaved (re, im) doubles.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static inline long so3_off(int l) { return (long)l * (4L * l * l - 1) / 3; }
static inline long so3_idx(int l, int m, int n) { return so3_off(l) + (m + l) + (long)(n + l) * (2 * l + 1); }
static inline long s2_idx(int l, int m) { return (long)l * l + m + l; }

long orc_so3_ncoeff(int L) { return so3_off(L + 1); }
long orc_s2_ncoeff(int L) { return (long)(L + 1) * (L + 1); }

/* ------------------------------------------------------------------ grid */

/* fdcl_FFTSO3.cpp:578-591 */
double orc_beta_k(int B, int k) { return ((double)(2 * k + 1)) * M_PI / 4. / ((double)B); }
double orc_alpha_j(int B, int j) { return ((double)j) * M_PI / ((double)B); }

/* fdcl_FFTSO3.cpp:236-256 (compute_weight) */
void orc_so3_weights(int l_max, double *weight)
{
    int B = l_max + 1, j, k;
    double factor = M_PI / ((double)(4 * B));
    for (j = 0; j < 2 * B; j++) {
        double sum = 0.0;
        for (k = 0; k < B; k++)
            sum += 1. / ((double)(2 * k + 1)) * sin((double)((2 * j + 1) * (2 * k + 1)) * factor);
        sum *= 1. / ((double)4 * B * B * B) * sin((double)(2 * j + 1) * factor);
        weight[j] = sum;
    }
}

/* fdcl_FFTS2.cpp:102-123 (compute_weight) */
void orc_s2_weights(int l_max, double *weight)
{
    int B = l_max + 1, j, k;
    double factor = M_PI / ((double)(4 * B));
    for (j = 0; j < 2 * B; j++) {
        double sum = 0.0;
        for (k = 0; k < B; k++)
            sum += 1. / ((double)(2 * k + 1)) * sin((double)((2 * j + 1) * (2 * k + 1)) * factor);
        sum *= 2. * M_PI / ((double)B * B) * sin((double)(2 * j + 1) * factor);
        weight[j] = sum;
    }
}

/* ------------------------------------------------------- Wigner small-d */

#define D(l, m, n) d[so3_idx((l), (m), (n))]

/* fdcl_FFTSO3.cpp:127-194 (wigner_d(beta, L)), Blanco-Florez-Bermejo recursion
 * (64)-(68) for the lower triangle m >= |n|, then the symmetric fills.  The
 * expressions keep the reference's evaluation order. */
void orc_wigner_d(double beta, int L, double *d)
{
    double cb, sb, sb2, cb2, tb2;
    int l, m, n;
    memset(d, 0, sizeof(double) * so3_off(L + 1));
    cb = cos(beta);
    sb = sin(beta);
    sb2 = sin(beta / 2.);
    cb2 = cos(beta / 2.);
    tb2 = tan(beta / 2.);

    D(0, 0, 0) = 1.;
    if (L >= 1) {
        D(1, 0, 0) = cb;
        D(1, 1, -1) = pow(sb2, 2.);
        D(1, 1, 0) = -1. / sqrt(2.) * sb;
        D(1, 1, 1) = pow(cb2, 2.);
    }
    for (l = 2; l <= L; l++) {
        for (m = 0; m <= l - 2; m++) {
            for (n = -m; n <= m; n++) {
                D(l, m, n) = 1. / sqrt((pow(l, 2.) - pow(m, 2.)) * (pow(l, 2.) - pow(n, 2.))) *
                    ((l * (2. * l - 1.) * D(1, 0, 0) - (2. * l - 1.) * m * n / (l - 1.)) * D(l - 1, m, n)
                     - sqrt((pow(l - 1., 2.) - pow(m, 2.)) * (pow(l - 1., 2) - pow(n, 2.))) * l / (l - 1.) * D(l - 2, m, n)); /* (64) */
            }
        }
        D(l, l, l) = D(1, 1, 1) * D(l - 1, l - 1, l - 1);                 /* (65) */
        D(l, l - 1, l - 1) = (l * D(1, 0, 0) - l + 1.) * D(l - 1, l - 1, l - 1); /* (66) */
        for (n = l - 1; n >= -l; n--)
            D(l, l, n) = -sqrt((l + n + 1.) / (l - n)) * tb2 * D(l, l, n + 1); /* (67) */
        for (n = l - 2; n >= 1 - l; n--)
            D(l, l - 1, n) = -(l * cb - n) / (l * cb - n - 1.) * sqrt((l + n + 1.) / (l - n)) * tb2 * D(l, l - 1, n + 1); /* (68) */
    }
    for (l = 1; l <= L; l++) {
        for (m = -l; m < 0; m++)              /* upper triangle */
            for (n = m; n <= -m; n++)
                D(l, m, n) = pow(-1., m + n) * D(l, -m, -n);
        for (n = -l; n < 0; n++)              /* left triangle */
            for (m = n + 1; m < -n; m++)
                D(l, m, n) = D(l, -n, -m);
        for (n = 1; n <= l; n++)              /* right triangle */
            for (m = -n + 1; m <= n - 1; m++)
                D(l, m, n) = pow(-1., m + n) * D(l, n, m);
    }
}

/* fdcl_FFTSO3.cpp:16-120 (wigner_d_explicit): closed forms for l <= 3, the
 * known-answer table the reference's check_wigner_d compares against. */
void orc_wigner_d_explicit(double beta, double *d)
{
    double cb = cos(beta), sb = sin(beta);
    memset(d, 0, sizeof(double) * so3_off(4));
    D(0, 0, 0) = 1.;
    D(1, 1, 1) = (1. + cb) / 2.;   D(1, 1, 0) = -sb / sqrt(2.);  D(1, 1, -1) = (1. - cb) / 2.;
    D(1, 0, 1) = sb / sqrt(2.);    D(1, 0, 0) = cb;              D(1, 0, -1) = -sb / sqrt(2.);
    D(1, -1, 1) = (1 - cb) / 2.;   D(1, -1, 0) = sb / sqrt(2.);  D(1, -1, -1) = (1. + cb) / 2.;

    D(2, 2, 2) = pow(1 + cb, 2) / 4.;  D(2, 2, 1) = -sb * (1. + cb) / 2.;
    D(2, 2, 0) = 1. / 2. * sqrt(3. / 2.) * pow(sb, 2);
    D(2, 2, -1) = -sb * (1. - cb) / 2.; D(2, 2, -2) = pow(1 - cb, 2) / 4.;
    D(2, 1, 2) = sb * (1. + cb) / 2.;   D(2, 1, 1) = (2. * pow(cb, 2) + cb - 1.) / 2.;
    D(2, 1, 0) = -sqrt(3. / 2.) * sb * cb; D(2, 1, -1) = -(2. * pow(cb, 2) - cb - 1.) / 2.;
    D(2, 1, -2) = -sb * (1 - cb) / 2.;
    D(2, 0, 2) = 1. / 2. * sqrt(3. / 2.) * pow(sb, 2); D(2, 0, 1) = sqrt(3. / 2.) * sb * cb;
    D(2, 0, 0) = (3. * pow(cb, 2) - 1.) / 2.; D(2, 0, -1) = -sqrt(3. / 2.) * sb * cb;
    D(2, 0, -2) = 1. / 2. * sqrt(3. / 2.) * pow(sb, 2);
    D(2, -1, 2) = sb * (1. - cb) / 2.;  D(2, -1, 1) = -(2. * pow(cb, 2) - cb - 1.) / 2.;
    D(2, -1, 0) = sqrt(3. / 2.) * sb * cb; D(2, -1, -1) = (2 * pow(cb, 2) + cb - 1.) / 2.;
    D(2, -1, -2) = -sb * (1 + cb) / 2.;
    D(2, -2, 2) = pow(1. - cb, 2) / 4.; D(2, -2, 1) = sb * (1. - cb) / 2.;
    D(2, -2, 0) = 1. / 2. * sqrt(3. / 2.) * pow(sb, 2); D(2, -2, -1) = sb * (1. + cb) / 2.;
    D(2, -2, -2) = pow(1 + cb, 2) / 4.;

    D(3, 3, 3) = 1. / 8. * pow(1. + cb, 3);
    D(3, 3, 2) = -sqrt(6.) / 8. * sb * pow(1. + cb, 2);
    D(3, 3, 1) = sqrt(15.) / 8. * pow(sb, 2) * (1. + cb);
    D(3, 3, 0) = -sqrt(5.) / 4. * pow(sb, 3);
    D(3, 3, -1) = sqrt(15.) / 8. * pow(sb, 2) * (1 - cb);
    D(3, 3, -2) = -sqrt(6.) / 8. * sb * pow(1 - cb, 2);
    D(3, 3, -3) = 1. / 8. * pow(1 - cb, 3);
    D(3, 2, 3) = pow(-1, 2 - 3) * D(3, 3, 2);
    D(3, 2, 2) = -1. / 4. * pow(1 + cb, 2) * (2. - 3. * cb);
    D(3, 2, 1) = sqrt(10.) / 8. * sb * (1. - 2. * cb - 3. * pow(cb, 2));
    D(3, 2, 0) = sqrt(30.) / 4. * pow(sb, 2) * cb;
    D(3, 2, -1) = -sqrt(10.) / 8. * sb * (1. + 2. * cb - 3 * pow(cb, 2));
    D(3, 2, -2) = 1. / 4. * pow(1 - cb, 2) * (2. + 3. * cb);
    D(3, 2, -3) = D(3, 3, -2);
    D(3, 1, 3) = pow(-1, 1 - 3) * D(3, 3, 1);
    D(3, 1, 2) = pow(-1, 1 - 2) * D(3, 2, 1);
    D(3, 1, 1) = -1. / 8. * (1. + cb) * (1. + 10. * cb - 15. * pow(cb, 2));
    D(3, 1, 0) = sqrt(3.) / 4. * sb * (1. - 5. * pow(cb, 2));
    D(3, 1, -1) = -1. / 8. * (1. - cb) * (1. - 10. * cb - 15. * pow(cb, 2));
    D(3, 1, -2) = D(3, 2, -1);
    D(3, 1, -3) = D(3, 3, -1);
    D(3, 0, 3) = pow(-1, 0 - 3) * D(3, 3, 0);
    D(3, 0, 2) = pow(-1, 0 - 2) * D(3, 2, 0);
    D(3, 0, 1) = pow(-1, 0 - 1) * D(3, 1, 0);
    D(3, 0, 0) = -1. / 2. * cb * (3. - 5. * pow(cb, 2));
    D(3, 0, -1) = D(3, 1, 0);
    D(3, 0, -2) = D(3, 2, 0);
    D(3, 0, -3) = D(3, 3, 0);
    D(3, -1, 3) = pow(-1, -1 - 3) * D(3, 3, -1);
    D(3, -1, 2) = pow(-1, -1 - 2) * D(3, 2, -1);
    D(3, -1, 1) = pow(-1, -1 - 1) * D(3, 1, -1);
    D(3, -1, 0) = D(3, 0, 1);
    D(3, -1, -1) = D(3, 1, 1);
    D(3, -1, -2) = D(3, 2, 1);
    D(3, -1, -3) = D(3, 3, 1);
    D(3, -2, 3) = pow(-1, -2 - 3) * D(3, 3, -2);
    D(3, -2, 2) = pow(-1, -2 - 2) * D(3, 2, -2);
    D(3, -2, 1) = D(3, -1, 2);
    D(3, -2, 0) = D(3, 0, 2);
    D(3, -2, -1) = D(3, 1, 2);
    D(3, -2, -2) = D(3, 2, 2);
    D(3, -2, -3) = D(3, 3, 2);
    D(3, -3, 3) = pow(-1, -3 - 3) * D(3, 3, -3);
    D(3, -3, 2) = pow(-1, -3 - 2) * D(3, 2, -3);
    D(3, -3, 1) = D(3, -1, 3);
    D(3, -3, 0) = D(3, 0, 3);
    D(3, -3, -1) = D(3, 1, 3);
    D(3, -3, -2) = D(3, 2, 3);
    D(3, -3, -3) = D(3, 3, 3);
}
#undef D

/* ----------------------------------------------- normalized Legendre P_l^m */

/* fdcl_FFTS2.cpp:48-100 (nor_assoc_Legendre_poly): Numerical Recipes 6.7
 * recursion, packed S^2 layout, nP(l,-m) = (-1)^m nP(l,m). */
void orc_nor_assoc_legendre(double x, int L, double *nP)
{
    double fact, oldfact, pmm, omx2;
    int l, m, i;
    memset(nP, 0, sizeof(double) * (size_t)(L + 1) * (L + 1));
    nP[s2_idx(0, 0)] = sqrt(1. / (4.0 * M_PI));
    for (l = 1; l <= L; l++) {
        pmm = 1.0;
        omx2 = (1.0 - x) * (1.0 + x);
        fact = 1.0;
        for (i = 1; i <= l; i++) {
            pmm *= omx2 * fact / (fact + 1.0);
            fact += 2.0;
        }
        pmm = sqrt((2 * l + 1) * pmm / (4.0 * M_PI));
        if (l & 1)
            pmm = -pmm;
        nP[s2_idx(l, l)] = pmm;
    }
    for (l = 0; l < L; l++)
        nP[s2_idx(l + 1, l)] = x * sqrt(2.0 * l + 3.0) * nP[s2_idx(l, l)];
    for (m = 0; m <= L; m++) {
        oldfact = sqrt(2.0 * m + 3.0);
        for (l = m + 2; l <= L; l++) {
            fact = sqrt((4.0 * l * l - 1.0) / (l * l - m * m));
            nP[s2_idx(l, m)] = (x * nP[s2_idx(l - 1, m)] - nP[s2_idx(l - 2, m)] / oldfact) * fact;
            oldfact = fact;
        }
    }
    for (l = 1; l <= L; l++)
        for (m = 1; m <= l; m++)
            nP[s2_idx(l, -m)] = pow(-1., m) * nP[s2_idx(l, m)];
}

/* ------------------------------------------------------------------- DFT */

/* Restatement of the published algorithm of Eigen::FFT<double>::fwd (kissfft
 * backend, Eigen's unsupported/Eigen/FFT): unscaled forward DFT
 *   X[p] = sum_j x[j] exp(-2 pi i p j / N),
 * computed by mixed-radix decimation in time (smallest prime factor first,
 * generic O(p^2) butterfly for each prime p). */
static void dft_rec(const double *x, long xs, double *X, int N, int Ntot, const double *tw)
{
    int p = 2, M, q, r, k;
    if (N == 1) { X[0] = x[0]; X[1] = x[1]; return; }
    while (N % p) p++;
    M = N / p;
    /* sub-transforms of the p decimated sequences, stored contiguously */
    double *Y = (double *)malloc(sizeof(double) * 2 * N);
    for (r = 0; r < p; r++)
        dft_rec(x + 2 * r * xs, xs * p, Y + 2 * (long)r * M, M, Ntot, tw);
    long step = Ntot / N; /* tw[i*step] = exp(-2 pi i i / N) */
    for (q = 0; q < p; q++) {
        for (k = 0; k < M; k++) {
            int kk = k + M * q;
            double sr = 0., si = 0.;
            for (r = 0; r < p; r++) {
                long e = ((long)r * kk) % N;
                double wr = tw[2 * e * step], wi = tw[2 * e * step + 1];
                double yr = Y[2 * ((long)r * M + k)], yi = Y[2 * ((long)r * M + k) + 1];
                sr += wr * yr - wi * yi;
                si += wr * yi + wi * yr;
            }
            X[2 * kk] = sr;
            X[2 * kk + 1] = si;
        }
    }
    free(Y);
}

static double *make_twiddles(int N)
{
    double *tw = (double *)malloc(sizeof(double) * 2 * N);
    for (int i = 0; i < N; i++) {
        double a = -2. * M_PI * (double)i / (double)N;
        tw[2 * i] = cos(a);
        tw[2 * i + 1] = sin(a);
    }
    return tw;
}

/* unscaled forward DFT of one complex line (in/out element strides in complex units) */
void orc_dft(int N, const double *in, long in_stride, double *out, long out_stride)
{
    double *tw = make_twiddles(N);
    double *X = (double *)malloc(sizeof(double) * 2 * N);
    dft_rec(in, in_stride, X, N, N, tw);
    for (int i = 0; i < N; i++) {
        out[2 * i * out_stride] = X[2 * i];
        out[2 * i * out_stride + 1] = X[2 * i + 1];
    }
    free(X);
    free(tw);
}

/* 2-D transform of one N x N slice: rows (fft over j2) then columns (over j1),
 * as fdcl_FFTSO3.cpp:689-698. In-place on a complex N*N array. */
static void dft2_slice(int N, double *s, const double *tw)
{
    double *X = (double *)malloc(sizeof(double) * 2 * N);
    double *c = (double *)malloc(sizeof(double) * 2 * N);
    for (int j1 = 0; j1 < N; j1++) {
        dft_rec(s + 2L * j1 * N, 1, X, N, N, tw);
        memcpy(s + 2L * j1 * N, X, sizeof(double) * 2 * N);
    }
    for (int j2 = 0; j2 < N; j2++) {
        for (int j1 = 0; j1 < N; j1++) { c[2 * j1] = s[2L * (j1 * N + j2)]; c[2 * j1 + 1] = s[2L * (j1 * N + j2) + 1]; }
        dft_rec(c, 1, X, N, N, tw);
        for (int j1 = 0; j1 < N; j1++) { s[2L * (j1 * N + j2)] = X[2 * j1]; s[2L * (j1 * N + j2) + 1] = X[2 * j1 + 1]; }
    }
    free(c);
    free(X);
}

/* ------------------------------------------------- SO(3) complex forward */

/* fdcl_FFTSO3.cpp:659-763 (forward_transform(func, is_real)).  The callback is
 * replaced by the sampled grid f[k][j1][j2] (complex); the OpenMP structure is
 * the reference's: per-k local coefficients zeroed, accumulated, then merged
 * into F under a critical section. */
static void so3_forward_complex_range(int l_max, const double *grid, int is_real, double *F, int k0, int kstride,
                                      int count);

void orc_so3_forward_complex(int l_max, const double *grid, int is_real, double *F)
{
    so3_forward_complex_range(l_max, grid, is_real, F, 0, 1, 2 * (l_max + 1));
}

/* The slices k in [k0, k1) of the forward sum (bounded CPU timing samples);
 * grid holds only those slices, grid[(k - k0)][j1][j2]. */
void orc_so3_forward_complex_slices(int l_max, const double *grid, double *F, int k0, int k1)
{
    so3_forward_complex_range(l_max, grid, 0, F, k0, 1, k1 - k0);
}

/* The slices k = k0 + i kstride, i < count, of the forward sum (CPU timing samples spread over
 * beta); grid holds only those slices, grid[i][j1][j2]. */
void orc_so3_forward_complex_strided(int l_max, const double *grid, double *F, int k0, int kstride, int count)
{
    so3_forward_complex_range(l_max, grid, 0, F, k0, kstride, count);
}

/* grid[i] is slice k = k0 + i kstride, i < count */
static void so3_forward_complex_range(int l_max, const double *grid, int is_real, double *F, int k0, int kstride,
                                      int count)
{
    int B = l_max + 1, N = 2 * B;
    long C = so3_off(l_max + 1);
    double *weight = (double *)malloc(sizeof(double) * N);
    double *tw = make_twiddles(N);
    orc_so3_weights(l_max, weight);
    memset(F, 0, sizeof(double) * 2 * C);

#pragma omp parallel
    {
        double *F_local = (double *)malloc(sizeof(double) * 2 * C);
        double *d = (double *)malloc(sizeof(double) * C);
        double *F_k = (double *)malloc(sizeof(double) * 2L * N * N);
        int i;
#pragma omp for schedule(static)
        for (i = 0; i < count; i++) {
            const int k = k0 + i * kstride;
            double beta = orc_beta_k(B, k);
            memcpy(F_k, grid + 2L * i * N * N, sizeof(double) * 2L * N * N);
            dft2_slice(N, F_k, tw);
            orc_wigner_d(beta, l_max, d);
            memset(F_local, 0, sizeof(double) * 2 * C);
#define ACC(l, m, n, p, q)                                                   \
    do {                                                                     \
        double wd = weight[k] * d[so3_idx(l, m, n)];                         \
        long o = 2 * so3_idx(l, m, n), s = 2L * ((long)(p) * N + (q));       \
        F_local[o] += wd * F_k[s];                                           \
        F_local[o + 1] += wd * F_k[s + 1];                                   \
    } while (0)
            for (int l = 0; l <= l_max; l++) {
                for (int m = 1; m <= l; m++) {
                    for (int n = 1; n <= l; n++) ACC(l, m, n, N - m, N - n);
                    for (int n = -l; n <= 0; n++) ACC(l, m, n, N - m, -n);
                }
                if (!is_real) {
                    for (int m = -l; m <= 0; m++) {
                        for (int n = 1; n <= l; n++) ACC(l, m, n, -m, N - n);
                        for (int n = -l; n <= 0; n++) ACC(l, m, n, -m, -n);
                    }
                } else {
                    for (int n = -l; n <= 0; n++) ACC(l, 0, n, 0, -n);
                }
            }
#undef ACC
#pragma omp critical
            for (long i = 0; i < 2 * C; i++) F[i] += F_local[i];
        }
        free(F_k);
        free(d);
        free(F_local);
    }
    if (is_real) { /* fdcl_FFTSO3.cpp:746-758 Hermitian fill */
        for (int l = 0; l <= l_max; l++) {
            for (int m = -l; m < 0; m++)
                for (int n = -l; n <= l; n++) {
                    double s = pow(-1., m - n);
                    long o = 2 * so3_idx(l, m, n), p = 2 * so3_idx(l, -m, -n);
                    F[o] = s * F[p];
                    F[o + 1] = s * -F[p + 1];
                }
            for (int n = 1; n <= l; n++) {
                double s = pow(-1., 0 - n);
                long o = 2 * so3_idx(l, 0, n), p = 2 * so3_idx(l, 0, -n);
                F[o] = s * F[p];
                F[o + 1] = s * -F[p + 1];
            }
        }
    }
    free(tw);
    free(weight);
}

/* ---------------------------------------------------- SO(3) real forward */

static int signum_i(int x) { return x > 0 ? 1 : (x < 0 ? -1 : 0); }

/* fdcl_FFTSO3.cpp:1431-1471 (compute_Psi) */
static void compute_psi(double beta, int L, double *d, double *Psi)
{
    orc_wigner_d(beta, L, d);
    memset(Psi, 0, sizeof(double) * so3_off(L + 1));
#define P(l, m, n) Psi[so3_idx((l), (m), (n))]
#define DD(l, m, n) d[so3_idx((l), (m), (n))]
    for (int l = 0; l <= L; l++) {
        int m, n;
        double A, Bv, Cv;
        P(l, 0, 0) = DD(l, 0, 0);
        m = 0;
        for (n = 1; n <= l; n++) {
            Cv = sqrt(2.) * DD(l, abs(m), abs(n));
            P(l, m, n) = pow(-1, m - n) * Cv;
            P(l, m, -n) = P(l, m, n);
        }
        for (m = 1; m <= l; m++) {
            n = 0;
            Cv = sqrt(2.) * DD(l, abs(m), abs(n));
            P(l, m, n) = pow(-1., m - n) * Cv;
            P(l, -m, n) = P(l, m, n);
            for (n = 1; n <= l; n++) {
                A = pow(-1., m - n) * DD(l, abs(m), abs(n));
                Bv = pow(-1., m) * signum_i(m) * DD(l, abs(m), -abs(n));
                P(l, m, n) = A + Bv;
                P(l, -m, n) = A - Bv;
                P(l, m, -n) = P(l, m, n);
                P(l, -m, -n) = P(l, -m, n);
            }
        }
    }
#undef P
#undef DD
}

/* fdcl_FFTSO3.cpp:765-772 (index_fft) */
static int index_fft(int i, int B) { return i <= 0 ? -i : 2 * B - i; }

/* fdcl_FFTSO3.cpp:774-850 (FFTSO3_real::forward_transform): real grid, real
 * coefficients through Psi^l_mn(beta_k) and the Re/Im parts of the FFT at +-n. */
void orc_so3_forward_real(int l_max, const double *grid, double *F)
{
    int B = l_max + 1, N = 2 * B;
    long C = so3_off(l_max + 1);
    double *weight = (double *)malloc(sizeof(double) * N);
    double *tw = make_twiddles(N);
    orc_so3_weights(l_max, weight);
    memset(F, 0, sizeof(double) * C);
#pragma omp parallel
    {
        double *F_local = (double *)calloc(C, sizeof(double));
        double *Psi = (double *)malloc(sizeof(double) * C);
        double *d = (double *)malloc(sizeof(double) * C);
        double *F_k = (double *)malloc(sizeof(double) * 2L * N * N);
        int k;
#pragma omp for schedule(static)
        for (k = 0; k < N; k++) {
            double beta = orc_beta_k(B, k);
            for (long i = 0; i < (long)N * N; i++) {
                F_k[2 * i] = grid[(long)k * N * N + i];
                F_k[2 * i + 1] = 0.;
            }
            dft2_slice(N, F_k, tw);
            compute_psi(beta, l_max, d, Psi);
            for (int l = 0; l <= l_max; l++)
                for (int m = -l; m <= l; m++) {
                    int im = index_fft(m, B);
                    for (int n = -l; n <= l; n++) {
                        int in = index_fft(n, B), i_n = index_fft(-n, B);
                        double cos_mang = F_k[2L * (im * N + in)];
                        double cos_ma_ng = F_k[2L * (im * N + i_n)];
                        double sin_mang = F_k[2L * (im * N + in) + 1];
                        double sin_ma_ng = F_k[2L * (im * N + i_n) + 1];
                        double sin_ma_sin_ng = 0.5 * (cos_ma_ng - cos_mang);
                        double cos_ma_cos_ng = 0.5 * (cos_ma_ng + cos_mang);
                        double sin_ma_cos_ng = 0.5 * (sin_mang + sin_ma_ng);
                        double cos_ma_sin_ng = 0.5 * (sin_mang - sin_ma_ng);
                        if ((m >= 0 && n >= 0) || (m < 0 && n < 0))
                            F_local[so3_idx(l, m, n)] += weight[k] * (-sin_ma_sin_ng * Psi[so3_idx(l, -m, n)] + cos_ma_cos_ng * Psi[so3_idx(l, m, n)]);
                        else
                            F_local[so3_idx(l, m, n)] += weight[k] * (-sin_ma_cos_ng * Psi[so3_idx(l, -m, n)] + cos_ma_sin_ng * Psi[so3_idx(l, m, n)]);
                    }
                }
        }
#pragma omp critical
        for (long i = 0; i < C; i++) F[i] += F_local[i];
        free(F_k);
        free(d);
        free(Psi);
        free(F_local);
    }
    free(tw);
    free(weight);
}

/* ------------------------------------------------- SO(3) point inverses */

/* fdcl_FFTSO3.cpp:498-531 (inverse_transform(F, alpha, beta, gamma)):
 * Fmn(m,n) = sum_l (2l+1) F(l,m,n) d(l,m,n), then expIMA^T Fmn expING. */
void orc_so3_inverse_complex_point(int l_max, const double *F, double alpha, double beta, double gamma, double *out)
{
    int B = l_max + 1, W = 2 * l_max + 1;
    double *d = (double *)malloc(sizeof(double) * so3_off(l_max + 1));
    double *Fmn = (double *)calloc(2L * W * W, sizeof(double));
    double *ea = (double *)malloc(sizeof(double) * 2 * W), *eg = (double *)malloc(sizeof(double) * 2 * W);
    (void)B;
    orc_wigner_d(beta, l_max, d);
    for (int m = -l_max; m <= l_max; m++) {
        /* exp(-I*(double)m*alpha) = (cos(m alpha), -sin(m alpha)) */
        ea[2 * (m + l_max)] = cos(-((double)m) * alpha);
        ea[2 * (m + l_max) + 1] = sin(-((double)m) * alpha);
        eg[2 * (m + l_max)] = cos(-((double)m) * gamma);
        eg[2 * (m + l_max) + 1] = sin(-((double)m) * gamma);
    }
    for (int m = -l_max; m <= l_max; m++)
        for (int n = -l_max; n <= l_max; n++) {
            double sr = 0., si = 0.;
            int l0 = abs(m) > abs(n) ? abs(m) : abs(n);
            for (int l = l0; l <= l_max; l++) {
                long o = so3_idx(l, m, n);
                double cr = (double)(2 * l + 1) * F[2 * o], ci = (double)(2 * l + 1) * F[2 * o + 1];
                sr += cr * d[o];
                si += ci * d[o];
            }
            Fmn[2L * ((m + l_max) * W + (n + l_max))] = sr;
            Fmn[2L * ((m + l_max) * W + (n + l_max)) + 1] = si;
        }
    /* (expIMA^T Fmn) expING */
    double fr = 0., fi = 0.;
    for (int n = 0; n < W; n++) {
        double tr = 0., ti = 0.;
        for (int m = 0; m < W; m++) {
            double ar = ea[2 * m], ai = ea[2 * m + 1];
            double br = Fmn[2L * (m * W + n)], bi = Fmn[2L * (m * W + n) + 1];
            tr += ar * br - ai * bi;
            ti += ar * bi + ai * br;
        }
        fr += tr * eg[2 * n] - ti * eg[2 * n + 1];
        fi += tr * eg[2 * n + 1] + ti * eg[2 * n];
    }
    out[0] = fr;
    out[1] = fi;
    free(eg);
    free(ea);
    free(Fmn);
    free(d);
}

/* fdcl_FFTSO3.cpp:1062-1105 (real_harmonics(alpha, beta, gamma, L)) */
void orc_so3_real_harmonics(int L, double alpha, double beta, double gamma, double *U)
{
    double *d = (double *)malloc(sizeof(double) * so3_off(L + 1));
    orc_wigner_d(beta, L, d);
    memset(U, 0, sizeof(double) * so3_off(L + 1));
#define UU(l, m, n) U[so3_idx((l), (m), (n))]
#define DD(l, m, n) d[so3_idx((l), (m), (n))]
    for (int l = 0; l <= L; l++) {
        UU(l, 0, 0) = DD(l, 0, 0);
        for (int m = 1; m <= l; m++) {
            UU(l, -m, 0) = sqrt(2.) * DD(l, -m, 0) * sin(((double)m) * alpha);
            UU(l, m, 0) = pow(-1., m) * sqrt(2.) * DD(l, m, 0) * cos(((double)m) * alpha);
            for (int n = 1; n <= l; n++) {
                double cos_mamg = cos(((double)m) * alpha + ((double)n) * gamma);
                double cos_ma_mg = cos(((double)m) * alpha - ((double)n) * gamma);
                double sin_mamg = sin(((double)m) * alpha + ((double)n) * gamma);
                double sin_ma_mg = sin(((double)m) * alpha - ((double)n) * gamma);
                UU(l, m, n) = pow(-1., m + n) * DD(l, m, n) * cos_mamg + pow(-1., m) * DD(l, m, -n) * cos_ma_mg;
                UU(l, m, -n) = pow(-1., m) * DD(l, m, -n) * sin_ma_mg - pow(-1., m + n) * DD(l, m, n) * sin_mamg;
                UU(l, -m, n) = -pow(-1., n) * DD(l, -m, n) * -sin_ma_mg + DD(l, -m, -n) * sin_mamg;
                UU(l, -m, -n) = DD(l, -m, -n) * cos_mamg - pow(-1., n) * DD(l, -m, n) * cos_ma_mg;
            }
        }
        for (int n = 1; n <= l; n++) {
            UU(l, 0, -n) = -sqrt(2.) * DD(l, 0, -n) * sin(((double)n) * gamma);
            UU(l, 0, n) = pow(-1., n) * sqrt(2.) * DD(l, 0, n) * cos(((double)n) * gamma);
        }
    }
#undef UU
#undef DD
    free(d);
}

/* fdcl_FFTSO3.cpp:1141-1156 (FFTSO3_real::inverse_transform) */
double orc_so3_inverse_real_point(int l_max, const double *F, double alpha, double beta, double gamma)
{
    double *U = (double *)malloc(sizeof(double) * so3_off(l_max + 1));
    double f = 0.;
    orc_so3_real_harmonics(l_max, alpha, beta, gamma, U);
    for (int l = 0; l <= l_max; l++)
        for (int m = -l; m <= l; m++)
            for (int n = -l; n <= l; n++)
                f += ((double)2 * l + 1) * F[so3_idx(l, m, n)] * U[so3_idx(l, m, n)];
    free(U);
    return f;
}

/* ---------------------------------------------------- SO(3) grid inverses */

/* Grid synthesis with the semantics of fdcl_FFTSO3.cpp:498-531 evaluated at
 * every grid point, done separably per beta_k: Fmn(m,n) as the reference
 * forms it, then the alpha and gamma sums with the reference's exponentials
 * exp(-i m alpha_j1), exp(-i n gamma_j2).  O(B^4) instead of O(B^6). */
static void so3_inverse_complex_range(int l_max, const double *F, double *grid, int k0, int kstride, int count);

void orc_so3_inverse_complex_grid(int l_max, const double *F, double *grid)
{
    so3_inverse_complex_range(l_max, F, grid, 0, 1, 2 * (l_max + 1));
}

/* The slices k in [k0, k1) of the grid synthesis, written to grid[(k - k0)][j1][j2]. */
void orc_so3_inverse_complex_slices(int l_max, const double *F, double *grid, int k0, int k1)
{
    so3_inverse_complex_range(l_max, F, grid, k0, 1, k1 - k0);
}

/* The slices k = k0 + i kstride, i < count, of the grid synthesis, written to grid[i][j1][j2]. */
void orc_so3_inverse_complex_strided(int l_max, const double *F, double *grid, int k0, int kstride, int count)
{
    so3_inverse_complex_range(l_max, F, grid, k0, kstride, count);
}

/* grid[i] is slice k = k0 + i kstride, i < count */
static void so3_inverse_complex_range(int l_max, const double *F, double *grid, int k0, int kstride, int count)
{
    int B = l_max + 1, N = 2 * B, W = 2 * l_max + 1;
    double *ex = (double *)malloc(sizeof(double) * 2L * N * W);
    for (int j = 0; j < N; j++) {
        double a = orc_alpha_j(B, j);
        for (int m = -l_max; m <= l_max; m++) {
            ex[2L * (j * W + m + l_max)] = cos(-((double)m) * a);
            ex[2L * (j * W + m + l_max) + 1] = sin(-((double)m) * a);
        }
    }
#pragma omp parallel
    {
        double *d = (double *)malloc(sizeof(double) * so3_off(l_max + 1));
        double *Fmn = (double *)malloc(sizeof(double) * 2L * W * W);
        double *T = (double *)malloc(sizeof(double) * 2L * N * W);
        int i;
#pragma omp for schedule(static)
        for (i = 0; i < count; i++) {
            const int k = k0 + i * kstride;
            orc_wigner_d(orc_beta_k(B, k), l_max, d);
            for (int m = -l_max; m <= l_max; m++)
                for (int n = -l_max; n <= l_max; n++) {
                    double sr = 0., si = 0.;
                    int l0 = abs(m) > abs(n) ? abs(m) : abs(n);
                    for (int l = l0; l <= l_max; l++) {
                        long o = so3_idx(l, m, n);
                        sr += (double)(2 * l + 1) * F[2 * o] * d[o];
                        si += (double)(2 * l + 1) * F[2 * o + 1] * d[o];
                    }
                    Fmn[2L * ((m + l_max) * W + n + l_max)] = sr;
                    Fmn[2L * ((m + l_max) * W + n + l_max) + 1] = si;
                }
            /* T(j1, n) = sum_m e^{-i m alpha_j1} Fmn(m, n) */
            for (int j1 = 0; j1 < N; j1++)
                for (int n = 0; n < W; n++) {
                    double tr = 0., ti = 0.;
                    for (int m = 0; m < W; m++) {
                        double ar = ex[2L * (j1 * W + m)], ai = ex[2L * (j1 * W + m) + 1];
                        double br = Fmn[2L * (m * W + n)], bi = Fmn[2L * (m * W + n) + 1];
                        tr += ar * br - ai * bi;
                        ti += ar * bi + ai * br;
                    }
                    T[2L * (j1 * W + n)] = tr;
                    T[2L * (j1 * W + n) + 1] = ti;
                }
            /* f(j1, j2) = sum_n T(j1, n) e^{-i n gamma_j2} */
            for (int j1 = 0; j1 < N; j1++)
                for (int j2 = 0; j2 < N; j2++) {
                    double fr = 0., fi = 0.;
                    for (int n = 0; n < W; n++) {
                        double ar = T[2L * (j1 * W + n)], ai = T[2L * (j1 * W + n) + 1];
                        double br = ex[2L * (j2 * W + n)], bi = ex[2L * (j2 * W + n) + 1];
                        fr += ar * br - ai * bi;
                        fi += ar * bi + ai * br;
                    }
                    long o = 2L * (((long)i * N + j1) * N + j2);
                    grid[o] = fr;
                    grid[o + 1] = fi;
                }
        }
        free(T);
        free(Fmn);
        free(d);
    }
    free(ex);
}

/* matrix2rsph (fdcl_FFTSO3.cpp:1107-1139): T(l,m,m')  as (row m, col m').
 * Returns the two nonzeros of row m: columns c0, c1 with values v0, v1. */
static void tmat_row(int m, int *c0, double *v0r, double *v0i, int *c1, double *v1r, double *v1i)
{
    double s = 1. / sqrt(2.);
    if (m < 0) {
        *c0 = m;  *v0r = 0.; *v0i = s;                       /* T(l,m,m) = I/sqrt2 */
        *c1 = -m; *v1r = 0.; *v1i = -s * pow(-1., m);        /* T(l,m,-m) = -I/sqrt2 (-1)^m */
    } else if (m == 0) {
        *c0 = 0; *v0r = 1.; *v0i = 0.; *c1 = 0; *v1r = 0.; *v1i = 0.;
    } else {
        *c0 = -m; *v0r = s; *v0i = 0.;                       /* T(l,m,-m) = 1/sqrt2 */
        *c1 = m;  *v1r = pow(-1., m) * s; *v1i = 0.;         /* T(l,m,m) = (-1)^m/sqrt2 */
    }
}

/* Real grid synthesis: f = sum (2l+1) F_r U (fdcl_FFTSO3.cpp:1141-1156) with
 * U = Re(conj(T) D T^T) (fdcl_FFTSO3.cpp:1010-1022), i.e. the complex
 * synthesis of F_c = T^H F_r T.  Checked against orc_so3_inverse_real_point. */
void orc_so3_real_to_complex(int l_max, const double *Fr, double *Fc)
{
    for (int l = 0; l <= l_max; l++)
        for (int m = -l; m <= l; m++)
            for (int n = -l; n <= l; n++) {
                /* Fc(m,n) = sum_{a,b} conj(T(a,m)) Fr(a,b) T(b,n) */
                double sr = 0., si = 0.;
                for (int a = -l; a <= l; a++) {
                    int c0, c1; double v0r, v0i, v1r, v1i;
                    tmat_row(a, &c0, &v0r, &v0i, &c1, &v1r, &v1i);
                    double tar = 0., tai = 0.;
                    if (c0 == m) { tar += v0r; tai += v0i; }
                    if (c1 == m && a != 0) { tar += v1r; tai += v1i; }
                    if (tar == 0. && tai == 0.) continue;
                    for (int b = -l; b <= l; b++) {
                        int e0, e1; double w0r, w0i, w1r, w1i;
                        tmat_row(b, &e0, &w0r, &w0i, &e1, &w1r, &w1i);
                        double tbr = 0., tbi = 0.;
                        if (e0 == n) { tbr += w0r; tbi += w0i; }
                        if (e1 == n && b != 0) { tbr += w1r; tbi += w1i; }
                        if (tbr == 0. && tbi == 0.) continue;
                        double f = Fr[so3_idx(l, a, b)];
                        /* conj(ta) * f * tb */
                        double pr = tar * tbr + tai * tbi, pi = tar * tbi - tai * tbr;
                        sr += f * pr;
                        si += f * pi;
                    }
                }
                Fc[2 * so3_idx(l, m, n)] = sr;
                Fc[2 * so3_idx(l, m, n) + 1] = si;
            }
}

void orc_so3_inverse_real_grid(int l_max, const double *F, double *grid)
{
    int N = 2 * (l_max + 1);
    long C = so3_off(l_max + 1);
    double *Fc = (double *)malloc(sizeof(double) * 2 * C);
    double *g = (double *)malloc(sizeof(double) * 2L * N * N * N);
    orc_so3_real_to_complex(l_max, F, Fc);
    orc_so3_inverse_complex_grid(l_max, Fc, g);
    for (long i = 0; i < (long)N * N * N; i++) grid[i] = g[2 * i];
    free(g);
    free(Fc);
}

/* --------------------------------------------------------------- S^2 */

/* fdcl_FFTS2.cpp:125-192 (FFTS2_complex::forward_transform(func, is_real)) */
void orc_s2_forward_complex(int l_max, const double *grid, int is_real, double *F)
{
    int B = l_max + 1, N = 2 * B;
    long C = (long)B * B;
    double *weight = (double *)malloc(sizeof(double) * N);
    double *tw = make_twiddles(N);
    orc_s2_weights(l_max, weight);
    memset(F, 0, sizeof(double) * 2 * C);
#pragma omp parallel
    {
        double *F_k = (double *)malloc(sizeof(double) * 2 * N);
        double *nP = (double *)malloc(sizeof(double) * C);
        double *F_local = (double *)malloc(sizeof(double) * 2 * C);
        int k;
#pragma omp for schedule(static)
        for (k = 0; k < N; k++) {
            double theta = orc_beta_k(B, k);
            dft_rec(grid + 2L * k * N, 1, F_k, N, N, tw);
            memset(F_local, 0, sizeof(double) * 2 * C);
            orc_nor_assoc_legendre(cos(theta), l_max, nP);
            for (int l = 0; l <= l_max; l++) {
                for (int m = 0; m <= l; m++) {
                    double wp = weight[k] * nP[s2_idx(l, m)];
                    F_local[2 * s2_idx(l, m)] += wp * F_k[2 * m];
                    F_local[2 * s2_idx(l, m) + 1] += wp * F_k[2 * m + 1];
                }
                if (!is_real)
                    for (int m = -l; m < 0; m++) {
                        double wp = weight[k] * nP[s2_idx(l, m)];
                        F_local[2 * s2_idx(l, m)] += wp * F_k[2 * (2 * l_max + 2 + m)];
                        F_local[2 * s2_idx(l, m) + 1] += wp * F_k[2 * (2 * l_max + 2 + m) + 1];
                    }
            }
#pragma omp critical
            for (long i = 0; i < 2 * C; i++) F[i] += F_local[i];
        }
        free(F_local);
        free(nP);
        free(F_k);
    }
    if (is_real)
        for (int l = 0; l <= l_max; l++)
            for (int m = -l; m < 0; m++) {
                double s = pow(-1., m);
                F[2 * s2_idx(l, m)] = s * F[2 * s2_idx(l, -m)];
                F[2 * s2_idx(l, m) + 1] = s * -F[2 * s2_idx(l, -m) + 1];
            }
    free(tw);
    free(weight);
}

/* fdcl_FFTS2.cpp:424-436 (FFTS2_real::forward_transform):
 * F[l] = Re(conj(T[l]) F_complex[l]), T from matrix2rsph (:318-369). */
void orc_s2_forward_real(int l_max, const double *grid, double *F)
{
    int N = 2 * (l_max + 1);
    long C = (long)(l_max + 1) * (l_max + 1);
    double *g = (double *)malloc(sizeof(double) * 2L * N * N);
    double *Fc = (double *)malloc(sizeof(double) * 2 * C);
    for (long i = 0; i < (long)N * N; i++) { g[2 * i] = grid[i]; g[2 * i + 1] = 0.; }
    orc_s2_forward_complex(l_max, g, 1, Fc);
    for (int l = 0; l <= l_max; l++)
        for (int m = -l; m <= l; m++) {
            int c0, c1; double v0r, v0i, v1r, v1i;
            tmat_row(m, &c0, &v0r, &v0i, &c1, &v1r, &v1i);
            /* Re(conj(v0) Fc(c0) + conj(v1) Fc(c1)) */
            double a = v0r * Fc[2 * s2_idx(l, c0)] + v0i * Fc[2 * s2_idx(l, c0) + 1];
            if (m != 0) a += v1r * Fc[2 * s2_idx(l, c1)] + v1i * Fc[2 * s2_idx(l, c1) + 1];
            F[s2_idx(l, m)] = a;
        }
    free(Fc);
    free(g);
}

/* fdcl_FFTS2.cpp:17-46 + :194-230: y = sum_{l,m} F(l,m) Y(l,m),
 * Y(l,m) = nP(l,m) e^{i m phi}, Y(l,-m) = (-1)^m conj Y(l,m). */
void orc_s2_inverse_complex_point(int l_max, const double *F, double theta, double phi, double *out)
{
    long C = (long)(l_max + 1) * (l_max + 1);
    double *nP = (double *)malloc(sizeof(double) * C);
    double yr = 0., yi = 0.;
    orc_nor_assoc_legendre(cos(theta), l_max, nP);
    for (int l = 0; l <= l_max; l++) {
        for (int m = 0; m <= l; m++) {
            double Yr = nP[s2_idx(l, m)] * cos((double)m * phi), Yi = nP[s2_idx(l, m)] * sin((double)m * phi);
            yr += F[2 * s2_idx(l, m)] * Yr - F[2 * s2_idx(l, m) + 1] * Yi;
            yi += F[2 * s2_idx(l, m)] * Yi + F[2 * s2_idx(l, m) + 1] * Yr;
            if (m > 0) {
                double s = pow(-1., m);
                double Zr = s * Yr, Zi = s * -Yi;
                yr += F[2 * s2_idx(l, -m)] * Zr - F[2 * s2_idx(l, -m) + 1] * Zi;
                yi += F[2 * s2_idx(l, -m)] * Zi + F[2 * s2_idx(l, -m) + 1] * Zr;
            }
        }
    }
    out[0] = yr;
    out[1] = yi;
    free(nP);
}

/* fdcl_FFTS2.cpp:383-422 + :500-512: real spherical harmonics
 * y(l,0) = nP(l,0), y(l,m) = sqrt2 (-1)^m nP cos(m phi), y(l,-m) = sqrt2 (-1)^m nP sin(m phi). */
double orc_s2_inverse_real_point(int l_max, const double *F, double theta, double phi)
{
    long C = (long)(l_max + 1) * (l_max + 1);
    double *nP = (double *)malloc(sizeof(double) * C);
    double z = 0.;
    orc_nor_assoc_legendre(cos(theta), l_max, nP);
    for (int l = 0; l <= l_max; l++) {
        z += F[s2_idx(l, 0)] * nP[s2_idx(l, 0)];
        for (int m = 1; m <= l; m++) {
            double tmp = sqrt(2.) * pow(-1., m) * nP[s2_idx(l, m)];
            z += F[s2_idx(l, m)] * (tmp * cos((double)m * phi));
            z += F[s2_idx(l, -m)] * (tmp * sin((double)m * phi));
        }
    }
    free(nP);
    return z;
}

/* Separable S^2 grid synthesis with the semantics of fdcl_FFTS2.cpp:194-230 at
 * every grid point: H_k(m) = sum_l F(l,m) nP(l,m)(cos theta_k), then
 * f(k,j) = sum_m H_k(m) e^{i m phi_j}. */
void orc_s2_inverse_complex_grid(int l_max, const double *F, double *grid)
{
    int B = l_max + 1, N = 2 * B, W = 2 * l_max + 1;
    long C = (long)B * B;
#pragma omp parallel
    {
        double *nP = (double *)malloc(sizeof(double) * C);
        double *H = (double *)malloc(sizeof(double) * 2 * W);
        int k;
#pragma omp for schedule(static)
        for (k = 0; k < N; k++) {
            orc_nor_assoc_legendre(cos(orc_beta_k(B, k)), l_max, nP);
            for (int m = -l_max; m <= l_max; m++) {
                double hr = 0., hi = 0.;
                for (int l = abs(m); l <= l_max; l++) {
                    hr += F[2 * s2_idx(l, m)] * nP[s2_idx(l, m)];
                    hi += F[2 * s2_idx(l, m) + 1] * nP[s2_idx(l, m)];
                }
                H[2 * (m + l_max)] = hr;
                H[2 * (m + l_max) + 1] = hi;
            }
            for (int j = 0; j < N; j++) {
                double phi = orc_alpha_j(B, j), fr = 0., fi = 0.;
                for (int m = -l_max; m <= l_max; m++) {
                    double c = cos((double)m * phi), s = sin((double)m * phi);
                    fr += H[2 * (m + l_max)] * c - H[2 * (m + l_max) + 1] * s;
                    fi += H[2 * (m + l_max)] * s + H[2 * (m + l_max) + 1] * c;
                }
                grid[2L * ((long)k * N + j)] = fr;
                grid[2L * ((long)k * N + j) + 1] = fi;
            }
        }
        free(H);
        free(nP);
    }
}

/* Real S^2 synthesis: f = sum F_r(l,m) y(l,m) with y = T Y, i.e. the complex
 * synthesis of F_c = T^T F_r (T unitary, fdcl_FFTS2.cpp:318-369). */
void orc_s2_real_to_complex(int l_max, const double *Fr, double *Fc)
{
    long C = (long)(l_max + 1) * (l_max + 1);
    memset(Fc, 0, sizeof(double) * 2 * C);
    for (int l = 0; l <= l_max; l++)
        for (int a = -l; a <= l; a++) {
            int c0, c1; double v0r, v0i, v1r, v1i;
            tmat_row(a, &c0, &v0r, &v0i, &c1, &v1r, &v1i);
            double f = Fr[s2_idx(l, a)];
            Fc[2 * s2_idx(l, c0)] += v0r * f;
            Fc[2 * s2_idx(l, c0) + 1] += v0i * f;
            if (a != 0) {
                Fc[2 * s2_idx(l, c1)] += v1r * f;
                Fc[2 * s2_idx(l, c1) + 1] += v1i * f;
            }
        }
}

void orc_s2_inverse_real_grid(int l_max, const double *F, double *grid)
{
    int N = 2 * (l_max + 1);
    long C = (long)(l_max + 1) * (l_max + 1);
    double *Fc = (double *)malloc(sizeof(double) * 2 * C);
    double *g = (double *)malloc(sizeof(double) * 2L * N * N);
    orc_s2_real_to_complex(l_max, F, Fc);
    orc_s2_inverse_complex_grid(l_max, Fc, g);
    for (long i = 0; i < (long)N * N; i++) grid[i] = g[2 * i];
    free(g);
    free(Fc);
}

/* ------------------------------------------------------------ utilities */

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
