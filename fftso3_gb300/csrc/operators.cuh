// Operators on SO(3) coefficients and harmonics (see operators.cu).
#pragma once
#include <cuda_runtime.h>

#include <vector>

namespace fftso3 {

// One row of a derivative matrix u_i^l: at most two nonzeros, at columns col[j] (index n + l; -1 unused).
struct DerivEntry {
    int col[2];
    double re[2], im[2];
};

// Rows of u_1^l, u_2^l, u_3^l for l <= L: table [3][(L+1)^2], row l^2 + k + l (k = -l..l); real: the
// real-harmonic matrices of deriv_real_harmonics, else those of deriv_wigner_D.
std::vector<DerivEntry> derivative_table(int L, bool real);
// out = F (u_i^l)^T per degree for `batch` coefficient vectors (tab: the axis's rows); F != out.
cudaError_t launch_derivative(const void* F, void* out, const DerivEntry* tab, bool fp64, bool real, int L,
                              int batch, cudaStream_t st);
// C (n x n, n = (2 l1 + 1)(2 l2 + 1), column-major, device) of the complex harmonics; with creal != null also
// the real-harmonic coefficients (n x n complex, column-major).
cudaError_t launch_clebsch_gordan(int l1, int l2, double* C, double2* creal, cudaStream_t st);

}  // namespace fftso3
