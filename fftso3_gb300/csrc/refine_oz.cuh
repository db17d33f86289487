// Exact tensor-core inverse of the residual refinement (see refine_oz.cu).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "timing.cuh"

namespace fftso3 {

struct OZState;

// SO(3) with l_max <= 255 (at most 256 degrees per contraction keep the digit sums exact).
bool oz_supported(int L, int N);
// Builds the table's digit planes and exponents from the plan's FP64 Wigner-d table (goff: group offsets into
// it), coefficient buffers for `chunk` functions per contraction and a double-float pencil buffer for pen_fns
// functions (the grid form's synthesis needs pen_fns >= chunk; the spectral form's FFT runs pen_fns at a time).
int oz_create(OZState** out, const double* d_table, const std::vector<long long>& goff, int L, int N, int chunk,
              int pen_fns, const double* d_tw, std::string& err);
void oz_destroy(OZState* o);
long long oz_device_bytes(const OZState* o);
// Error word of the exact contraction kernel (a bounded wait that gave up); synchronising read.
int oz_status(OZState* o);
// For nb <= chunk functions: r = f - inverse(F), F complex coefficients (complex128 when f64, else complex64),
// f the FP32 samples (complex64, or float32 when real), r written like f.
int oz_inverse_resid(OZState* o, const void* F, bool f64, int nb, const void* fgrid, bool real, float* resid,
                     cudaStream_t st, StageTimer* T, std::string& err);
// The exact inverse (FFTSO3_FLAG_EXACT_INVERSE): for nb coefficient sets F (as oz_inverse_resid), the synthesis
// with exact digit sums and a double-float FFT, rounded once into grid (complex64, or the real part as float32
// when real).  The double-float synthesis pencils go to pen (nb <= chunk functions of 16-byte elements), or,
// when pen is null, to the state's own buffer (nb <= oz_fft_functions()).
// host (non-null): the grids go to host memory instead; grid is then the device staging for all nb grids
// (the generic FFT) and ring a device buffer of 2 OZ_SYNTH_PIECE grids (N = 64..512), whose copies to the host
// run under the FFT of the next pieces.
constexpr int OZ_SYNTH_PIECE = 4;
// join = false (host path): st does not wait for the last copies to the host (a later call's join, or the
// caller's synchronisation of the copy stream through oz_host_join, covers them).  group_major: F (complex64) is
// in the tensor-core path's group-major order, unscaled (tc_group_from_packed), read as runs.
int oz_inverse_exact(OZState* o, const void* F, bool f64, int nb, void* grid, bool real, cudaStream_t st,
                     StageTimer* T, std::string& err, void* pen = nullptr, void* host = nullptr,
                     void* ring = nullptr, bool join = true, bool group_major = false);
// st waits for every copy to the host issued so far.
int oz_host_join(OZState* o, cudaStream_t st);
// Functions per contraction chunk.
int oz_chunk(const OZState* o);
// Device bytes of the coefficients' digit image per column tile of 8 functions (the contraction's B operand).
long long oz_image_bytes_per_column_tile(int L);

// The spectral form of the residual step (N = 64..512): the forward's FFT in double-float and the residual in
// the pencil domain, r^ = FFT(f) - N^2 H(F), which is what the forward GEMM consumes -- no FP32 FFT of f or of
// the residual.  oz_forward_fft: nb <= chunk sample grids f (complex64, or float32 when real) -> pencils
// [fn][p][q][k] as hi (complex64) + lo (remainder).  oz_resid_pencils: hi := (hi + lo) - N^2 H(F) at every
// pencil place the forward GEMM reads, for nb <= chunk coefficient sets F (as oz_inverse_resid).
bool oz_spectral(const OZState* o);
int oz_fft_functions(const OZState* o);
int oz_forward_fft(OZState* o, const void* fgrid, bool real, int nb, float2* hi, float2* lo, cudaStream_t st,
                   StageTimer* T, std::string& err);
// group_major: F (complex64) is group-major, the forward GEMM's own output layout, instead of packed.
int oz_resid_pencils(OZState* o, const void* F, bool f64, int nb, float2* hi, const float2* lo, cudaStream_t st,
                     StageTimer* T, std::string& err, bool group_major = false);

}  // namespace fftso3
