// Launches that span every l_max bucket of an uneven SO(3) tensor-core batch (fftso3_batch_*): with the fused
// beta-sum GEMM (contract_tc.cu) a direction is three launches,
//   forward: slice FFT (grid slabs -> pencils), GEMM, group-major -> packed coefficients (+ real basis);
//   inverse: packed (+ real basis) -> scaled group-major, GEMM, slice FFT (pencils -> grid slabs).
#pragma once
#include <cuda_runtime.h>

#include "fft.cuh"

namespace fftso3 {

// One bucket: its sizes, FFT factors and twiddles, the bucket plan's pencils and group-major coefficients, the
// element offsets of its slab in the caller's grid and coefficient buffers, and its first work index in each
// fused launch.  A launch's segment table is ordered by its work index (blk0 and cblk0 ascending).
struct BucketSeg {
    int L, B, N, batch;
    int spc;                     // beta slices per CTA of the slice FFT
    int G;                       // lines per Stockham group of the slice FFT (even)
    FFTFactors fac;              // prime-first factors of N
    const double2* tw;           // W[i] = e^{-2 pi i i / N}
    float2* pencil;              // [fn][p][q][k]
    float2* fg;                  // group-major coefficients [fn][so3_off(B)]
    long long g0, c0;            // slab offsets (elements) in the caller's grids / coefficients
    long long blk0;              // first CTA of the bucket in the slice FFT
    long long cblk0;             // first CTA of the bucket in the coefficient conversions
};

// Two launch shapes: 256 threads per CTA with line buffers of 2048 elements (two CTAs per SM), or "wide":
// 512 threads with 4096-element line buffers (one CTA per SM; twice the lines per Stockham group, so half the
// barrier phases per slice and twice the work items of a prime-radix stage).
__host__ __device__ inline int slice_threads(bool wide) { return wide ? 512 : 256; }
__host__ __device__ inline int slice_line_elems(bool wide) { return wide ? 4096 : 2048; }

// Row stride of a slice in shared memory (complex: all N columns; real: columns 0..N/2 of the Hermitian
// half-spectrum), odd so that column walks meet distinct banks, and the shared memory one CTA of the slice
// FFT needs for spc slices of size N.
__host__ __device__ inline int slice_row_stride(int N, bool real) { return real ? ((N / 2 + 1) | 1) : N + 1; }
// Stockham line buffers: lines of N elements (odd stride N + 1; SLICE_PAD: one padding slot per 8 elements,
// measured slower), groups of an even number of lines within the launch shape's line elements
constexpr bool SLICE_PAD = false;
__host__ __device__ inline int slice_line_stride(int N) { return SLICE_PAD ? (N + (N >> 3) + 1) | 1 : N + 1; }
__host__ __device__ inline int slice_lines_per_group(int N, bool wide)
{
    const int g = (slice_line_elems(wide) / slice_line_stride(N)) & ~1;
    return g < 2 ? 2 : g;
}
size_t slice_fft_smem_bytes(int N, int spc, bool real, bool wide);

// Both FFT passes of the beta slices of every bucket in one launch (nblk CTAs, smem bytes of dynamic shared
// memory each): fwd: grid slabs (complex64, or float32 when real) -> pencils; else pencils (Nyquist bins read
// as zero; real: their Hermitian part) -> grid slabs (float32 when real).
cudaError_t launch_slice_fft(const BucketSeg* segs, int nseg, long long nblk, size_t smem, bool fwd, bool real,
                             bool wide, const void* in, void* out, cudaStream_t st);

// Coefficient conversions of every bucket in one launch (CONVERT_THREADS coefficients of one bucket per CTA,
// nblk CTAs in total, CTA i serving bucket segs[cseg[i]]; l_max <= 255):
//   forward: group-major GEMM output -> packed coefficients (complex64, or the real basis in float32);
//   inverse: packed coefficients (complex64 / real float32) -> group-major (2l + 1) sign F.
constexpr int CONVERT_THREADS = 256;
cudaError_t launch_fused_group_to_packed(const BucketSeg* segs, const unsigned short* cseg, long long nblk,
                                         bool real, void* out, cudaStream_t st);
cudaError_t launch_fused_packed_to_group(const BucketSeg* segs, const unsigned short* cseg, long long nblk,
                                         bool real, const void* in, cudaStream_t st);

}  // namespace fftso3
