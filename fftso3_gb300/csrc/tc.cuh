// FP32-data transform state (see contract_tc.cu): tcgen05 split-BF16 or FP32 CUDA-core beta-sum, SO(3) or S^2.
#pragma once
#include <cuda_runtime.h>
#include <string>
#include <vector>

#include "fft.cuh"
#include "timing.cuh"

namespace fftso3 {

struct TCState;

int tc_create(TCState** out, int L, int N, int batch, const double* d_table_fp64, const std::vector<long long>& goff,
              long long table_elems, const double* d_tw, const double* d_w, bool refine, bool real, bool s2,
              bool autotune, bool simt, std::string& err);
void tc_destroy(TCState* s);
long long tc_device_bytes(const TCState* s);
int tc_forward(TCState* s, const void* grid, void* coeffs, cudaStream_t st, StageTimer* T, std::string& err);
int tc_inverse(TCState* s, const void* coeffs, void* grid, cudaStream_t st, StageTimer* T, std::string& err);
// Device error word of the tensor-core kernels (0 = no bounded wait timed out); synchronising read.
int tc_status(TCState* s);

}  // namespace fftso3
