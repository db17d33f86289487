// Beta-sum contraction launchers (see contract_fp64.cu, contract_tc.cu).
#pragma once
#include <cuda_runtime.h>

namespace fftso3 {

cudaError_t launch_so3_fwd_fp64(const double* table, const long long* goff, const double2* G, const double* w,
                                double2* F, int L, int N, int batch, cudaStream_t st);
cudaError_t launch_so3_inv_fp64(const double* table, const long long* goff, const double2* F, double2* H, int L,
                                int N, int batch, cudaStream_t st);
cudaError_t launch_zero_nyquist_so3(void* H, bool fp64, int N, long long nslices, cudaStream_t st);
cudaError_t launch_so3_c2r(const void* Fc, void* Fr, bool fp64, int L, int batch, cudaStream_t st);
cudaError_t launch_so3_r2c(const void* Fr, void* Fc, bool fp64, int L, int batch, cudaStream_t st);

cudaError_t launch_s2_fwd_fp64(const double* table, const long long* moff, const double2* G, const double* w,
                               double2* F, int L, int N, int batch, bool is_real, cudaStream_t st);
cudaError_t launch_s2_inv_fp64(const double* table, const long long* moff, const double2* F, double2* H, int L,
                               int N, int batch, cudaStream_t st);
cudaError_t launch_zero_nyquist_s2(void* H, bool fp64, int N, long long nrows, cudaStream_t st);
cudaError_t launch_s2_c2r(const void* Fc, void* Fr, bool fp64, int L, int batch, cudaStream_t st);
cudaError_t launch_s2_r2c(const void* Fr, void* Fc, bool fp64, int L, int batch, cudaStream_t st);
// tensor-core S^2 real kinds: group-major GEMM output -> real coefficients, and real coefficients ->
// scaled group-major GEMM input, each in one pass (FP32; goff2 the group-major offsets, cstride (L+1)^2)
cudaError_t launch_s2_group_to_real(const void* Fg, void* Fr, const long long* goff2, int L, int batch,
                                   cudaStream_t st);
cudaError_t launch_s2_real_to_group(const void* Fr, void* Y, const long long* goff2, int L, int batch,
                                   cudaStream_t st);

// S^2 -> SO(3) correlation coefficients Fr(l,m,n) = G_l(m) F_l(n) / (2l+1) (correlate.cu)
cudaError_t launch_corr_coeffs(const void* F, const void* G, void* C, bool fp64, int L, int batch, cudaStream_t st);
// per-array arg-max (value, flat index) of nb real arrays of n elements; ov, oi device arrays of nb
size_t argmax_scratch_bytes(int nb, int chunks);
cudaError_t launch_argmax(const void* x, bool fp64, long long n, int nb, int chunks, void* scratch, double* ov,
                          long long* oi, cudaStream_t st);

// residual refinement of the FP32-data plans: FP32 -> FP64 copy; r = f - g (FP64 difference rounded to FP32);
// F += d.  n counts real elements (twice the complex count for interleaved complex data).
cudaError_t launch_widen(const float* in, double* out, long long n, cudaStream_t st);
// FP64 -> FP32 (rounded to nearest); n real elements
cudaError_t launch_narrow(const double* in, float* out, long long n, cudaStream_t st);
cudaError_t launch_resid_fp64(const float* f, const double* g, float* r, long long n, cudaStream_t st);
cudaError_t launch_add_real(float* F, const float* d, long long n, cudaStream_t st);

}  // namespace fftso3
