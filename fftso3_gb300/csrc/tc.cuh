// FP32-data transform state (see contract_tc.cu): tcgen05 split-BF16 or FP32 CUDA-core beta-sum, SO(3) or S^2.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <string>
#include <vector>

#include "../../include/fftso3_gb300.h"
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
// Residual refinement (plans created with refine = true): the plan's residual grid buffer (batch grids of the
// plan's sample type), and coeffs += forward(resid) in the coefficients' element type.
void* tc_resid_buffer(TCState* s);
int tc_refine_add(TCState* s, const void* resid, void* coeffs, cudaStream_t st, StageTimer* T, std::string& err);
// Spectral refinement (SO(3)): the plan's pencil buffer (complex64 [fn][p][q][k], batch functions), the forward
// from pencils already there (GEMM + coefficient permutation + real basis), and coeffs += forward(pencils).
float2* tc_pencil_buffer(TCState* s);
// Refinement plans: the pencil and residual buffers as one array of batch x (pencil places) 16-byte elements
// (the exact inverse's double-float synthesis pencils); null otherwise.
void* tc_exact_buffer(TCState* s);
// Complex SO(3) plans: functions f0 .. f0 + nb - 1 of the packed complex64 coefficients, permuted unscaled into
// the group-major buffer (the exact contraction's input order); returns their place there (null on a launch
// error).
const float2* tc_group_from_packed(TCState* s, const void* packed, int f0, int nb, cudaStream_t st);
int tc_forward_pencils(TCState* s, void* coeffs, cudaStream_t st, StageTimer* T, std::string& err);
int tc_refine_add_pencils(TCState* s, void* coeffs, cudaStream_t st, StageTimer* T, std::string& err);
// Complex SO(3) refined plans, group-major form: F0 = the forward GEMM of the pencils, left group-major in the
// plan's group buffer (the exact contraction reads it there); then the correction's GEMM, F0 + correction, and one
// permutation into the packed coefficients.
float2* tc_group_buffer(TCState* s);
int tc_gemm_forward_group(TCState* s, cudaStream_t st, StageTimer* T, std::string& err);
int tc_refine_finish_group(TCState* s, void* coeffs, cudaStream_t st, StageTimer* T, std::string& err);
// Device error word of the tensor-core kernels (0 = no bounded wait timed out); synchronising read.
int tc_status(TCState* s);

// Phases of one direction, so that several plans can share one GEMM launch:
//   forward = tc_forward_fft, GEMM, tc_forward_finish;
//   inverse = tc_inverse_prepare, GEMM, tc_inverse_fft.
int tc_forward_fft(TCState* s, const void* grid, cudaStream_t st, StageTimer* T, std::string& err);
int tc_forward_finish(TCState* s, void* coeffs, cudaStream_t st, StageTimer* T, std::string& err);
int tc_inverse_prepare(TCState* s, const void* coeffs, cudaStream_t st, StageTimer* T, std::string& err);
int tc_inverse_fft(TCState* s, void* grid, cudaStream_t st, StageTimer* T, std::string& err);

// One persistent tensor-core GEMM launch over the work items of several plans.
struct TCFused;
int tc_fused_create(TCFused** out, const std::vector<TCState*>& parts, std::string& err);
void tc_fused_destroy(TCFused* f);
int tc_fused_gemm(TCFused* f, bool fwd, cudaStream_t st, StageTimer* T, std::string& err);
int tc_fused_status(TCFused* f);
// Three launches per direction over SO(3) plans of one kind without refinement (fused.cuh): slice FFT, GEMM,
// conversion (forward) and the mirror image (inverse).  Plan i's functions sit at element offsets g0[i] / c0[i]
// of the caller's grids / coefficients.  FFTSO3_ERR_UNSUPPORTED when one beta slice of the largest N does not
// fit a CTA's shared memory (the per-plan phases then serve).
int tc_fused_phases(TCFused* f, const std::vector<long long>& g0, const std::vector<long long>& c0, std::string& err);
int tc_fused_forward(TCFused* f, const void* grid, void* coeffs, cudaStream_t st, StageTimer* T, std::string& err);
int tc_fused_inverse(TCFused* f, const void* coeffs, void* grid, cudaStream_t st, StageTimer* T, std::string& err);

// Row-major 2-D BF16 tensor map (inner elements per row, outer rows; 128-byte swizzle, boxes of
// box_inner x box_outer), resolved through the runtime's driver entry point.
bool tc_encode_bf16_2d(CUtensorMap* tm, const void* base, unsigned long long inner, unsigned long long outer,
                       unsigned box_inner, unsigned box_outer);

// A plan's tensor-core state (null for FP64 plans) and stage timer (api.cu).
TCState* plan_tc_state(fftso3_plan* p);
StageTimer* plan_timer(fftso3_plan* p);

}  // namespace fftso3
