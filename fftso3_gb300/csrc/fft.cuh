// Batched strided 1-D FFT launcher (see fft.cu).
#pragma once
#include <cuda_runtime.h>

namespace fftso3 {

struct FFTFactors {
    int N;
    int n;
    int r[24];
};

struct FFTLaunch {
    const void* in;       // complex (or real when real_in) input
    void* out;            // complex (or real part only when real_out) output; may equal in
    FFTFactors fac;
    long long nlines;     // number of transforms
    int lpb;              // lines per CTA
    long long inner, ostride, istride, es;  // line i base = (i/inner)*ostride + (i%inner)*istride; element stride es
    const void* tw;       // device double2 table, W[i] = exp(-2 pi i i / N)
    bool fp64;
    bool df32 = false;    // double-float complex data (dfc32, 16 bytes: re.h, re.l, im.h, im.l); complex only
    bool real_in;
    bool real_out;
    bool lines_fastest;   // consecutive lines adjacent in memory (column pass)
    int threads = 256;    // threads per CTA (<= 256)
};

void make_fft_factors(int N, FFTFactors& f);
// Same factors with the prime radices above 8 first (largest first): the
// first stage is then a plain DFT whose twiddles every lane of a warp shares.
void make_fft_factors_prime_first(int N, FFTFactors& f);
size_t fft_smem_bytes(int N, int lpb, bool fp64);
cudaError_t launch_fft_lines(const FFTLaunch& L, cudaStream_t st);

// Double-float (dfc32) FFT along a strided axis of arrays whose innermost index k (N values) is contiguous,
// in place: line (o, k), o < nouter, has element j at obase(o) + k + j S, obase(o) = (o / oinner) oouter +
// (o % oinner) oistride.  N = 64..512, powers of two (fft.cu).
bool fft_df32_k_supported(int N);
cudaError_t launch_fft_df32_k(void* buf, int N, long long S, long long nouter, long long oinner, long long oouter,
                              long long oistride, const void* tw, cudaStream_t st);
// Double-float forward FFT of nb sample grids f [fn][k][j1][j2] (complex64, or float32 when real) into the
// k-contiguous pencils [fn][p][q][k], written renormalised as hi (complex64, the FP32 rounding) + lo (the
// remainder); buf: nb double-float grids of work space.
cudaError_t launch_fft_df32_k_forward(void* buf, int N, long long nb, const void* f, bool real, float2* hi,
                                      float2* lo, const void* tw, cudaStream_t st);
// The double-float FFT of nb synthesis pencils buf [fn][p][q][k] (dfc32; overwritten) into the grids out
// [fn][k][j1][j2], rounded once to complex64, or to the real part as float32 when real.
cudaError_t launch_fft_df32_k_synth(void* buf, int N, long long nb, void* out, bool real, const void* tw,
                                    cudaStream_t st);
// One of its two passes (1: along p, in place; 2: along q into out), for pipelining pieces of functions.
cudaError_t launch_fft_df32_k_synth_pass(int pass, void* buf, int N, long long nb, void* out, bool real,
                                         const void* tw, cudaStream_t st);

// Register-resident FP32 kernels for N = 64..1024, powers of two (fft_fast.cu).
bool fft_fast_supported(int N);
// nlines contiguous lines of N complex64: out[line][K] = FFT(in[line])[K] (in may equal out)
cudaError_t launch_fft_rows_fast(const void* in, void* out, long long nlines, int N, const void* tw, cudaStream_t st);
// Tiled transposing passes over nf grids of N^3 complex64 (in != out):
//   pass  1: grid [nf][k][j1][j2] -> FFT over j2 -> T1 [nf][k][q][j1]
//   pass  2: T1 [nf][k][q][j1]    -> FFT over j1 -> pencils [nf][p][q][k]
//   pass -2: pencils [nf][p][q][k] -> FFT over p -> T1 [nf][k][q][j1]
//   pass -1: T1 [nf][k][q][j1]     -> FFT over q -> grid [nf][k][j1][j2]
// real_io: pass 1 reads real samples (float), pass -1 writes the real part only.
cudaError_t launch_fft_grid_pass(const void* in, void* out, long long nf, int N, int pass, const void* tw,
                                 cudaStream_t st, bool real_io = false);
// Both passes of one direction in one persistent launch (N = 64..512): dir 1
// grid -> pencils (passes 1, 2), dir -1 pencils -> grid (passes -2, -1), the
// intermediate held in a ring of ring_elems >= fft_grid_fused_ring_elems(N)
// complex64 (sized for the current device) that stays in L2, instead of a
// full-size work grid.  ctl: fft_grid_fused_ctl_ints device ints (zeroed by
// the launch, on st); err: device error word (9 when a wait on another tile
// timed out).  Same arithmetic as the two-pass form: bit-identical results.
bool fft_grid_fused_supported(int N);
size_t fft_grid_fused_ring_elems(int N);
size_t fft_grid_fused_ctl_ints(long long nf, int N);
cudaError_t launch_fft_grid_fused(const void* in, void* out, void* ring, size_t ring_elems, int* ctl, int* err,
                                  long long nf, int N, int dir, const void* tw, cudaStream_t st,
                                  bool real_io = false);
// Tiled pass over nf S^2 grids of N^2 complex64 (in != out):
//   dir  1: grid [nf][k][j]     -> FFT over j -> pencils [nf][p][k]
//   dir -1: pencils [nf][p][k]  -> FFT over p -> grid [nf][k][j]
// real_io: dir 1 reads real samples, dir -1 writes the real part only.
cudaError_t launch_fft_s2_pass(const void* in, void* out, long long nf, int N, int dir, const void* tw,
                               cudaStream_t st, bool real_io = false);

}  // namespace fftso3
