// Wigner-d / Legendre tables and FP64 point evaluation (see tables.cu).
#pragma once
#include <cuda_runtime.h>

namespace fftso3 {

// Per-angle seeds, computed on the host with the C library exactly as
// fdcl_FFTSO3.cpp:135-147 forms them (plus the logs used by the stable mode).
struct WignerSeeds {
    double cb;     // cos(beta)
    double sb;     // sin(beta)
    double tb2;    // tan(beta/2)
    double d111;   // pow(cos(beta/2), 2.)
    double d11m1;  // pow(sin(beta/2), 2.)
    double d110;   // -1./sqrt(2.) * sin(beta)
    double lc2;    // log(|cos(beta/2)|)   (stable mode)
    double ls2;    // log(|sin(beta/2)|)   (stable mode)
    double c2;     // cos(beta/2)          (stable mode, sign)
    double s2;     // sin(beta/2)          (stable mode, sign)
};

cudaError_t launch_wigner_table(double* table, const long long* goff, const WignerSeeds* seeds, const double* lfact,
                                int L, int N, int ngroups, bool stable, cudaStream_t st);
cudaError_t launch_legendre_table(double* table, const long long* moff, const double* xs, int L, int N,
                                  cudaStream_t st);
// SO(3) point evaluation (see tables.cu): the beta-independent recursion factors (built once per
// plan: wigner_rec_elems(L) double4 and wigner_sq_elems(L) doubles), the split of the degrees into
// parts (m0b: MAX_POINT_PARTS + 1 ints), and the launch (part: S x n double2 scratch).
constexpr int MAX_POINT_PARTS = 32;
size_t wigner_rec_elems(int L);
size_t wigner_sq_elems(int L);
cudaError_t launch_wigner_rec_factors(double4* rec, double* sq, int L, cudaStream_t st);
int points_parts(bool so3, int L, int n, int nsm, int* m0b);
cudaError_t launch_so3_points(const double2* F, const WignerSeeds* pseeds, const double* pts, const double4* rec,
                              const double* sq, const double* lfact, int L, bool stable, int n, const int* m0b,
                              int S, double2* part, double2* out, cudaStream_t st);
cudaError_t launch_wigner_full(const WignerSeeds* seed, const double* lfact, int L, bool stable, double* out,
                               cudaStream_t st);
// S^2 point evaluation: the per-plan Legendre factors (legendre_rec_elems(L) double2) and the launch
size_t legendre_rec_elems(int L);
cudaError_t launch_legendre_rec_factors(double2* rec, int L, cudaStream_t st);
cudaError_t launch_s2_points(const double2* F, const double* xs, const double* pts, const double2* rec, int L, int n,
                             const int* m0b, int S, double2* part, double2* out, cudaStream_t st);

}  // namespace fftso3
