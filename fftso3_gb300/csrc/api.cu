// C ABI of the GB300 SO(3) / S^2 transform library (declared in include/fftso3_gb300.h).
//
// Host side of the plan: argument checks, the FP64 host precompute that the
// reference does inline (quadrature weights fdcl_FFTSO3.cpp:236-256 /
// fdcl_FFTS2.cpp:102-123, grid angles :578-591, recursion seeds :135-147),
// device tables, workspace, and the launch sequence of each transform.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fftso3_gb300.h"
#include "common.cuh"
#include "contract.cuh"
#include "fft.cuh"
#include "operators.cuh"
#include "refine_oz.cuh"
#include "tables.cuh"
#include "tc.cuh"
#include "timing.cuh"

using namespace fftso3;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg)
{
    g_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what)
{
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? FFTSO3_ERR_OOM : FFTSO3_ERR_CUDA;
}

#define CK(call)                                                   \
    do {                                                           \
        cudaError_t _e = (call);                                   \
        if (_e != cudaSuccess) return cuda_fail(_e, #call);        \
    } while (0)

bool valid_kind(int k) { return k >= FFTSO3_SO3_COMPLEX && k <= FFTSO3_S2_REAL; }
bool is_so3(int k) { return k == FFTSO3_SO3_COMPLEX || k == FFTSO3_SO3_REAL; }
bool is_real_kind(int k) { return k == FFTSO3_SO3_REAL || k == FFTSO3_S2_REAL; }

// fdcl_FFTSO3.cpp:578-591 (beta_k, identical expression for theta_k in fdcl_FFTS2.cpp:292-296)
double beta_k(int B, int k) { return ((double)(2 * k + 1)) * M_PI / 4. / ((double)B); }

void host_weights(int kind, int l_max, double* weight)
{
    int B = l_max + 1;
    double factor = M_PI / ((double)(4 * B));
    for (int j = 0; j < 2 * B; j++) {
        double sum = 0.0;
        for (int k = 0; k < B; k++)
            sum += 1. / ((double)(2 * k + 1)) * sin((double)((2 * j + 1) * (2 * k + 1)) * factor);
        if (is_so3(kind))
            sum *= 1. / ((double)4 * B * B * B) * sin((double)(2 * j + 1) * factor);
        else
            sum *= 2. * M_PI / ((double)B * B) * sin((double)(2 * j + 1) * factor);
        weight[j] = sum;
    }
}

WignerSeeds make_seeds(double beta)
{
    WignerSeeds s;
    s.cb = cos(beta);
    s.sb = sin(beta);
    double sb2 = sin(beta / 2.), cb2 = cos(beta / 2.);
    s.tb2 = tan(beta / 2.);
    s.d111 = pow(cb2, 2.);
    s.d11m1 = pow(sb2, 2.);
    s.d110 = -1. / sqrt(2.) * s.sb;
    s.lc2 = log(fabs(cb2));
    s.ls2 = log(fabs(sb2));
    s.c2 = cb2;
    s.s2 = sb2;
    return s;
}

std::vector<double> log_factorials(int n)
{
    std::vector<double> f(n + 1);
    for (int i = 0; i <= n; ++i) f[i] = lgamma((double)i + 1.0);
    return f;
}

}  // namespace

namespace fftso3 {
// Lets other translation units report through fftso3_last_error_string().
void set_last_error(const std::string& msg) { g_err = msg; }
}  // namespace fftso3

struct fftso3_plan {
    int kind = 0, L = 0, B = 0, N = 0, batch = 0, precision = 0, recursion = 0;
    unsigned flags = 0;
    int device = 0;
    bool so3 = true, real = false, fp64 = true;
    long long grid_elems = 0, coeff_elems = 0;  // per function
    FFTFactors fac;
    std::vector<double> weights;
    double* d_tw = nullptr;        // N double2
    double* d_w = nullptr;         // N
    long long* d_goff = nullptr;   // group offsets into the table
    double* d_table = nullptr;
    long long table_elems = 0;
    double* d_lfact = nullptr;
    void* d_work = nullptr;        // FFT workspace: batch * grid_elems complex
    void* d_fc = nullptr;          // complex coefficients of the real kinds
    void* d_io_grid = nullptr;     // staging for the *_host calls
    void* d_io_ring = nullptr;     // exact inverse into host memory: two pieces of grids in flight to the host
    void* d_io_coeff = nullptr;
    void* d_corr = nullptr;        // correlation coefficients (fftso3_correlate_s2)
    void* d_amax = nullptr;        // arg-max scratch (fftso3_grid_argmax)
    void* d_prec = nullptr;        // point evaluation: beta-independent recursion factors (built on first use:
    double* d_psq = nullptr;       //   SO(3) Wigner factors + seed factors here, or S^2 Legendre factors)
    void* d_pscratch = nullptr;    // point evaluation scratch (grows with n)
    size_t pscratch_bytes = 0;
    // residual refinement of FP32-data plans (FFTSO3_FLAG_REFINE): the FP64 table stays, and the FP64 inverse of
    // the first result runs over chunks of rchunk functions
    void* d_rw = nullptr;          // FP64 work grid of one chunk (complex128)
    void* d_rg = nullptr;          // FP64 real grid of one chunk (real kinds)
    void* d_rc = nullptr;          // FP64 copy of one chunk's coefficients
    void* d_rfc = nullptr;         // complex FP64 coefficients of one chunk (real kinds)
    int rchunk = 0;
    OZState* oz = nullptr;         // SO(3), l_max <= 255: the refinement's inverse on the tensor cores, exactly
    DerivEntry* d_deriv = nullptr; // rows of the derivative matrices u_1..u_3 (built on the first derivative call)
    long long bytes = 0;
    TCState* tc = nullptr;         // tensor-core contraction state
    StageTimer timer;              // optional per-stage CUDA-event timing
    // host calls of the refined forward: the samples' copy runs on its own stream, piece by piece, ahead of the
    // double-float FFT of each piece (created on first use)
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t copy_ev[3] = {nullptr, nullptr, nullptr};
};

namespace fftso3 {
TCState* plan_tc_state(fftso3_plan* p) { return p ? p->tc : nullptr; }
StageTimer* plan_timer(fftso3_plan* p) { return p ? &p->timer : nullptr; }
}  // namespace fftso3

namespace {

int plan_alloc(fftso3_plan* p, void** ptr, size_t bytes)
{
    cudaError_t e = cudaMalloc(ptr, bytes);
    if (e != cudaSuccess) {
        *ptr = nullptr;
        return cuda_fail(e, "cudaMalloc");
    }
    p->bytes += (long long)bytes;
    return FFTSO3_SUCCESS;
}

void plan_free(fftso3_plan* p)
{
    void* ptrs[] = {p->d_tw, p->d_w, p->d_goff, p->d_table, p->d_lfact, p->d_work, p->d_fc, p->d_io_grid, p->d_io_ring,
                    p->d_io_coeff, p->d_corr, p->d_amax, p->d_prec, p->d_pscratch, p->d_rw, p->d_rg, p->d_rc,
                    p->d_rfc, p->d_deriv};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    if (p->tc) tc_destroy(p->tc);
    if (p->oz) oz_destroy(p->oz);
    for (cudaEvent_t e : p->copy_ev)
        if (e) cudaEventDestroy(e);
    if (p->copy_stream) cudaStreamDestroy(p->copy_stream);
}

size_t cbytes(const fftso3_plan* p) { return p->fp64 ? 16 : 8; }  // complex element bytes
size_t rbytes(const fftso3_plan* p) { return p->fp64 ? 8 : 4; }   // real element bytes

FFTLaunch fft_rows(const fftso3_plan* p, const void* in, void* out, long long nlines, bool real_in, bool real_out,
                   bool fp64)
{
    FFTLaunch L;
    L.in = in;
    L.out = out;
    L.fac = p->fac;
    L.nlines = nlines;
    int N = p->N;
    int lpb = 1;
    size_t budget = 200 * 1024;
    while (lpb < 4 && fft_smem_bytes(N, lpb * 2, fp64) <= budget) lpb *= 2;
    L.lpb = lpb;
    L.inner = 1;
    L.ostride = N;
    L.istride = 0;
    L.es = 1;
    L.tw = p->d_tw;
    L.fp64 = fp64;
    L.real_in = real_in;
    L.real_out = real_out;
    L.lines_fastest = false;
    return L;
}

// FFT along j1 of [outer][N][N] (lines (outer, j2), element stride N)
FFTLaunch fft_cols(const fftso3_plan* p, const void* in, void* out, long long nouter, bool real_out, bool fp64)
{
    FFTLaunch L;
    L.in = in;
    L.out = out;
    L.fac = p->fac;
    int N = p->N;
    L.nlines = nouter * N;
    int lpb = 16;
    while (lpb > 1 && fft_smem_bytes(N, lpb, fp64) > 200 * 1024) lpb /= 2;
    L.lpb = lpb;
    L.inner = N;
    L.ostride = (long long)N * N;
    L.istride = 1;
    L.es = N;
    L.tw = p->d_tw;
    L.fp64 = fp64;
    L.real_in = false;
    L.real_out = real_out;
    L.lines_fastest = true;
    return L;
}

#define STAGE(id, call)      \
    do {                     \
        T.begin(id, st);     \
        CK(call);            \
        T.end(st);           \
    } while (0)

// FP64 inverse of nb functions of the plan's kind: coefficients Fin (complex128, or float64 for the real kinds)
// -> grid gout (complex128 / float64; may be `work` itself for the complex kinds).  work: nb complex128 grids;
// fc: nb complex128 coefficient vectors (real kinds).  refine: the launches belong to a refinement step (its
// stage names) of an FP32-data plan.
int fp64_inverse(fftso3_plan* p, const void* Fin_, void* gout, int nb, void* work, void* fc, bool refine,
                 cudaStream_t st)
{
    const int N = p->N, L = p->L;
    StageTimer& T = p->timer;
    const int s_con = refine ? ST_REF_CONTRACT : ST_FP64_INV;
    const int s_rows = refine ? ST_REF_FFT : ST_FFT_ROWS, s_cols = refine ? ST_REF_FFT : ST_FFT_COLS;
    const double2* Fin = (const double2*)Fin_;
    if (p->so3) {
        if (p->real) {
            STAGE(ST_BASIS, launch_so3_r2c(Fin_, fc, true, L, nb, st));
            Fin = (const double2*)fc;
        }
        STAGE(ST_NYQUIST, launch_zero_nyquist_so3(work, true, N, (long long)nb * N, st));
        STAGE(s_con, launch_so3_inv_fp64(p->d_table, p->d_goff, Fin, (double2*)work, L, N, nb, st));
        STAGE(s_rows, launch_fft_lines(fft_rows(p, work, work, (long long)nb * N * N, false, false, true), st));
        STAGE(s_cols, launch_fft_lines(fft_cols(p, work, gout, (long long)nb * N, p->real, true), st));
    } else {
        if (p->real) {
            STAGE(ST_BASIS, launch_s2_r2c(Fin_, fc, true, L, nb, st));
            Fin = (const double2*)fc;
        }
        STAGE(ST_NYQUIST, launch_zero_nyquist_s2(work, true, N, (long long)nb * N, st));
        STAGE(s_con, launch_s2_inv_fp64(p->d_table, p->d_goff, Fin, (double2*)work, L, N, nb, st));
        STAGE(s_rows, launch_fft_lines(fft_rows(p, work, gout, (long long)nb * N, false, p->real, true), st));
    }
    return FFTSO3_SUCCESS;
}

// One residual step of an FP32-data plan (FFTSO3_FLAG_REFINE) after its forward wrote F to coeffs:
//   F += forward(f - inverse(F)),
// the inverse in FP64 (chunks of rchunk functions) and the difference f - inverse(F) formed in FP64, so the
// correction carries the errors of the first forward, not those of an FP32 inverse.
int refine_forward(fftso3_plan* p, const void* grid, void* coeffs, cudaStream_t st)
{
    StageTimer& T = p->timer;
    const long long C = p->coeff_elems, G = p->grid_elems;
    const int rc_per = p->real ? 1 : 2;  // reals per element
    float* resid = (float*)tc_resid_buffer(p->tc);
    if (p->oz) {
        // SO(3): the inverse on the tensor cores with exact digit sums, double-float FFT and residual
        for (int f0 = 0; f0 < p->batch; f0 += p->rchunk) {
            const int nb = p->batch - f0 < p->rchunk ? p->batch - f0 : p->rchunk;
            const void* Fc = (const float2*)coeffs + (long long)f0 * C;
            if (p->real) {
                STAGE(ST_REFINE, launch_widen((const float*)coeffs + (long long)f0 * C, (double*)p->d_rc,
                                              (long long)nb * C, st));
                STAGE(ST_BASIS, launch_so3_r2c(p->d_rc, p->d_rfc, true, p->L, nb, st));
                Fc = p->d_rfc;
            }
            const long long off = (long long)f0 * G * rc_per;
            int rc = oz_inverse_resid(p->oz, Fc, p->real, nb, (const float*)grid + off, p->real, resid + off, st, &T,
                                      g_err);
            if (rc) return rc;
        }
        return tc_refine_add(p->tc, resid, coeffs, st, &T, g_err);
    }
    for (int f0 = 0; f0 < p->batch; f0 += p->rchunk) {
        const int nb = p->batch - f0 < p->rchunk ? p->batch - f0 : p->rchunk;
        STAGE(ST_REFINE, launch_widen((const float*)coeffs + (long long)f0 * C * rc_per, (double*)p->d_rc,
                                      (long long)nb * C * rc_per, st));
        void* g64 = p->real ? p->d_rg : p->d_rw;
        int rc = fp64_inverse(p, p->d_rc, g64, nb, p->d_rw, p->d_rfc, true, st);
        if (rc) return rc;
        const long long off = (long long)f0 * G * rc_per;
        STAGE(ST_REFINE, launch_resid_fp64((const float*)grid + off, (const double*)g64, resid + off,
                                           (long long)nb * G * rc_per, st));
    }
    return tc_refine_add(p->tc, resid, coeffs, st, &T, g_err);
}

// The spectral form of the refined forward (SO(3), exact inverse, N = 64..512): the samples' FFT in
// double-float (pencils hi in the plan's pencil buffer, remainders lo in its residual buffer), F0 = the GEMM of
// hi, then per chunk the residual in the pencil domain, r^ = (hi + lo) - N^2 H(F0) (H: the exact synthesis
// contraction, whose FFT is N^2 H), written over hi, and F = F0 + the GEMM of r^.  Equal to the grid form
// F0 + forward(f - inverse(F0)) -- the forward GEMM reads exactly these pencils -- without the FP32 FFTs of the
// samples and of the residual and without the double-float FFT of the synthesis.
//
// host (non-null): the samples are in host memory and `grid` is the plan's staging area for them; they are copied
// there on the plan's copy stream in pieces of a few functions, each piece's FFT waiting only for its own copy,
// so the copy of the next piece runs under the FFT of this one.
int refine_forward_spectral(fftso3_plan* p, const void* grid, void* coeffs, cudaStream_t st, const void* host)
{
    StageTimer& T = p->timer;
    const long long C = p->coeff_elems, G = p->grid_elems;
    float2* hi = tc_pencil_buffer(p->tc);
    float2* lo = (float2*)tc_resid_buffer(p->tc);
    const int per = p->real ? 1 : 2;  // floats per sample
    const int fftn = oz_fft_functions(p->oz);
    const int piece = host ? (fftn < 4 ? fftn : 4) : fftn;
    if (host) {
        if (!p->copy_stream) {
            CK(cudaStreamCreateWithFlags(&p->copy_stream, cudaStreamNonBlocking));
            for (cudaEvent_t& e : p->copy_ev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        }
        // the staging area is free once the caller's earlier work on st is done
        CK(cudaEventRecord(p->copy_ev[2], st));
        CK(cudaStreamWaitEvent(p->copy_stream, p->copy_ev[2], 0));
    }
    for (int f0 = 0, i = 0; f0 < p->batch; f0 += piece, ++i) {
        const int nb = p->batch - f0 < piece ? p->batch - f0 : piece;
        const float* g = (const float*)grid + (long long)f0 * G * per;
        if (host) {
            CK(cudaMemcpyAsync((void*)g, (const float*)host + (long long)f0 * G * per,
                               sizeof(float) * (size_t)nb * G * per, cudaMemcpyHostToDevice, p->copy_stream));
            CK(cudaEventRecord(p->copy_ev[i & 1], p->copy_stream));
            CK(cudaStreamWaitEvent(st, p->copy_ev[i & 1], 0));
        }
        int rc = oz_forward_fft(p->oz, g, p->real, nb, hi + (long long)f0 * G, lo + (long long)f0 * G, st, &T,
                                g_err);
        if (rc) return rc;
    }
    if (!p->real) {
        // complex: F0 stays group-major (the GEMM's layout, which the contraction reads as runs); one permutation
        // of F0 + correction at the end
        const float2* Fg = tc_group_buffer(p->tc);
        int rc = tc_gemm_forward_group(p->tc, st, &T, g_err);
        if (rc) return rc;
        for (int f0 = 0; f0 < p->batch; f0 += p->rchunk) {
            const int nb = p->batch - f0 < p->rchunk ? p->batch - f0 : p->rchunk;
            if ((rc = oz_resid_pencils(p->oz, Fg + (long long)f0 * C, false, nb, hi + (long long)f0 * G,
                                       lo + (long long)f0 * G, st, &T, g_err, true)))
                return rc;
        }
        return tc_refine_finish_group(p->tc, coeffs, st, &T, g_err);
    }
    int rc = tc_forward_pencils(p->tc, coeffs, st, &T, g_err);
    if (rc) return rc;
    for (int f0 = 0; f0 < p->batch; f0 += p->rchunk) {
        const int nb = p->batch - f0 < p->rchunk ? p->batch - f0 : p->rchunk;
        const void* Fc = (const float2*)coeffs + (long long)f0 * C;
        if (p->real) {
            STAGE(ST_REFINE, launch_widen((const float*)coeffs + (long long)f0 * C, (double*)p->d_rc,
                                          (long long)nb * C, st));
            STAGE(ST_BASIS, launch_so3_r2c(p->d_rc, p->d_rfc, true, p->L, nb, st));
            Fc = p->d_rfc;
        }
        if ((rc = oz_resid_pencils(p->oz, Fc, p->real, nb, hi + (long long)f0 * G, lo + (long long)f0 * G, st, &T,
                                   g_err)))
            return rc;
    }
    return tc_refine_add_pencils(p->tc, coeffs, st, &T, g_err);
}

bool spectral_refine(const fftso3_plan* p)
{
    return p->tc && p->oz && (p->flags & FFTSO3_FLAG_REFINE) && oz_spectral(p->oz);
}

int run_forward(fftso3_plan* p, const void* grid, void* coeffs, cudaStream_t st)
{
    const int N = p->N, L = p->L, b = p->batch;
    StageTimer& T = p->timer;
    if (spectral_refine(p)) return refine_forward_spectral(p, grid, coeffs, st, nullptr);
    if (p->tc) {
        int rc = tc_forward(p->tc, grid, coeffs, st, &T, g_err);
        if (rc || !(p->flags & FFTSO3_FLAG_REFINE)) return rc;
        return refine_forward(p, grid, coeffs, st);
    }
    if (p->so3) {
        STAGE(ST_FFT_ROWS, launch_fft_lines(fft_rows(p, grid, p->d_work, (long long)b * N * N, p->real, false, true), st));
        STAGE(ST_FFT_COLS, launch_fft_lines(fft_cols(p, p->d_work, p->d_work, (long long)b * N, false, true), st));
        double2* Fout = p->real ? (double2*)p->d_fc : (double2*)coeffs;
        STAGE(ST_FP64_FWD,
              launch_so3_fwd_fp64(p->d_table, p->d_goff, (const double2*)p->d_work, p->d_w, Fout, L, N, b, st));
        if (p->real) STAGE(ST_BASIS, launch_so3_c2r(p->d_fc, coeffs, true, L, b, st));
    } else {
        STAGE(ST_FFT_ROWS, launch_fft_lines(fft_rows(p, grid, p->d_work, (long long)b * N, p->real, false, true), st));
        double2* Fout = p->real ? (double2*)p->d_fc : (double2*)coeffs;
        STAGE(ST_FP64_FWD, launch_s2_fwd_fp64(p->d_table, p->d_goff, (const double2*)p->d_work, p->d_w, Fout, L, N,
                                              b, p->real, st));
        if (p->real) STAGE(ST_BASIS, launch_s2_c2r(p->d_fc, coeffs, true, L, b, st));
    }
    return FFTSO3_SUCCESS;
}

// FFTSO3_FLAG_EXACT_INVERSE: the synthesis without FP32 rounding -- SO(3), l_max <= 255: exact digit sums on the
// tensor cores and a double-float FFT, a contraction chunk of functions at a time, the double-float pencils in
// the plan's pencil + residual buffers; otherwise the FP64 inverse in chunks of rchunk functions -- rounded once
// into the FP32 grid.  host (non-null): the grids go to host memory; grid is then device staging for them (unused
// by the double-float FFT of N = 64..512, which streams pieces through a small device ring instead).
int exact_inverse(fftso3_plan* p, const void* coeffs, void* grid, cudaStream_t st, void* host = nullptr)
{
    StageTimer& T = p->timer;
    const long long C = p->coeff_elems, G = p->grid_elems;
    const int per = p->real ? 1 : 2;  // floats per element
    if (p->oz) {
        void* pen = tc_exact_buffer(p->tc);
        const int fftn = pen ? p->rchunk : oz_fft_functions(p->oz);
        void* ring = nullptr;
        if (host && oz_spectral(p->oz)) {
            const size_t fn_bytes = (size_t)G * per * sizeof(float);
            int rc = p->d_io_ring ? FFTSO3_SUCCESS : plan_alloc(p, &p->d_io_ring, 2 * (size_t)OZ_SYNTH_PIECE * fn_bytes);
            if (rc) return rc;
            ring = p->d_io_ring;
        }
        for (int f0 = 0; f0 < p->batch; f0 += fftn) {
            const int nb = p->batch - f0 < fftn ? p->batch - f0 : fftn;
            const void* Fc;
            if (p->real) {
                STAGE(ST_BASIS, launch_widen((const float*)coeffs + (long long)f0 * C, (double*)p->d_rc,
                                             (long long)nb * C, st));
                STAGE(ST_BASIS, launch_so3_r2c(p->d_rc, p->d_rfc, true, p->L, nb, st));
                Fc = p->d_rfc;
            } else {
                // complex: permuted into group-major runs first, so the digit image reads contiguous runs
                T.begin(ST_BASIS, st);
                Fc = tc_group_from_packed(p->tc, coeffs, f0, nb, st);
                T.end(st);
                if (!Fc) return cuda_fail(cudaGetLastError(), "tc_group_from_packed");
            }
            const long long off = (long long)f0 * G * per;  // floats
            int rc = oz_inverse_exact(p->oz, Fc, p->real, nb, ring ? nullptr : (float*)grid + off, p->real, st, &T,
                                      g_err, pen, host ? (float*)host + off : nullptr, ring, true, !p->real);
            if (rc) return rc;
        }
        return FFTSO3_SUCCESS;
    }
    for (int f0 = 0; f0 < p->batch; f0 += p->rchunk) {
        const int nb = p->batch - f0 < p->rchunk ? p->batch - f0 : p->rchunk;
        STAGE(ST_BASIS, launch_widen((const float*)coeffs + (long long)f0 * C * per, (double*)p->d_rc,
                                     (long long)nb * C * per, st));
        void* g64 = p->real ? p->d_rg : p->d_rw;
        int rc = fp64_inverse(p, p->d_rc, g64, nb, p->d_rw, p->d_rfc, false, st);
        if (rc) return rc;
        STAGE(ST_BASIS, launch_narrow((const double*)g64, (float*)grid + (long long)f0 * G * per,
                                      (long long)nb * G * per, st));
    }
    if (host) CK(cudaMemcpyAsync(host, grid, (size_t)p->batch * G * per * sizeof(float), cudaMemcpyDeviceToHost, st));
    return FFTSO3_SUCCESS;
}

int run_inverse(fftso3_plan* p, const void* coeffs, void* grid, cudaStream_t st)
{
    if (p->tc && (p->flags & FFTSO3_FLAG_EXACT_INVERSE)) return exact_inverse(p, coeffs, grid, st);
    if (p->tc) return tc_inverse(p->tc, coeffs, grid, st, &p->timer, g_err);
    return fp64_inverse(p, coeffs, grid, p->batch, p->d_work, p->d_fc, false, st);
}
#undef STAGE

int check_plan(const fftso3_plan* p)
{
    if (!p) return fail(FFTSO3_ERR_INVALID_ARG, "plan is NULL");
    int dev = -1;
    cudaGetDevice(&dev);
    if (dev != p->device) {
        cudaError_t e = cudaSetDevice(p->device);
        if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    }
    return FFTSO3_SUCCESS;
}

}  // namespace

extern "C" {

const char* fftso3_last_error_string(void) { return g_err.c_str(); }

int fftso3_version(void) { return 100; }

long long fftso3_grid_elems(int kind, int l_max)
{
    if (!valid_kind(kind) || l_max < 0) return -1;
    long long N = 2LL * (l_max + 1);
    return is_so3(kind) ? N * N * N : N * N;
}

long long fftso3_coeff_elems(int kind, int l_max)
{
    if (!valid_kind(kind) || l_max < 0) return -1;
    long long B = l_max + 1;
    return is_so3(kind) ? so3_off((int)B) : B * B;
}

int fftso3_weights(int kind, int l_max, double* weights_out)
{
    if (!valid_kind(kind)) return fail(FFTSO3_ERR_INVALID_ARG, "unknown transform kind");
    if (l_max < 0) return fail(FFTSO3_ERR_INVALID_ARG, "l_max must be >= 0");
    if (!weights_out) return fail(FFTSO3_ERR_INVALID_ARG, "weights_out is NULL");
    host_weights(kind, l_max, weights_out);
    return FFTSO3_SUCCESS;
}

int fftso3_plan_create(fftso3_plan** out, int kind, int l_max, int batch, int precision, int recursion,
                       unsigned flags)
{
    if (!out) return fail(FFTSO3_ERR_INVALID_ARG, "plan output pointer is NULL");
    *out = nullptr;
    if (!valid_kind(kind)) return fail(FFTSO3_ERR_INVALID_ARG, "unknown transform kind");
    if (l_max < 0) return fail(FFTSO3_ERR_INVALID_ARG, "l_max must be >= 0");
    if (batch < 1) return fail(FFTSO3_ERR_INVALID_ARG, "batch must be >= 1");
    if (precision != FFTSO3_PREC_FP64 && precision != FFTSO3_PREC_TC_BF16X3 && precision != FFTSO3_PREC_FP32)
        return fail(FFTSO3_ERR_INVALID_ARG, "unknown precision");
    if (recursion != FFTSO3_RECURSION_REFERENCE && recursion != FFTSO3_RECURSION_STABLE)
        return fail(FFTSO3_ERR_INVALID_ARG, "unknown recursion mode");
    if ((flags & ~(FFTSO3_FLAG_REFINE | FFTSO3_FLAG_AUTOTUNE | FFTSO3_FLAG_EXACT_INVERSE)) != 0)
        return fail(FFTSO3_ERR_INVALID_ARG, "unknown flag bits");
    if (is_so3(kind) && l_max > 511) return fail(FFTSO3_ERR_UNSUPPORTED, "SO(3) l_max above 511 is not supported");
    if (!is_so3(kind) && l_max > 2047) return fail(FFTSO3_ERR_UNSUPPORTED, "S^2 l_max above 2047 is not supported");
    if (precision != FFTSO3_PREC_FP64 && l_max > 511)
        return fail(FFTSO3_ERR_UNSUPPORTED,
                    "the tensor-core and FP32 paths support l_max <= 511 (2(l_max+1) <= 1024)");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(FFTSO3_ERR_NO_DEVICE, "no CUDA device available");

    fftso3_plan* p = new fftso3_plan();
    p->kind = kind;
    p->L = l_max;
    p->B = l_max + 1;
    p->N = 2 * p->B;
    p->batch = batch;
    p->precision = precision;
    p->recursion = recursion;
    p->flags = flags;
    p->so3 = is_so3(kind);
    p->real = is_real_kind(kind);
    p->fp64 = (precision == FFTSO3_PREC_FP64);
    p->grid_elems = fftso3_grid_elems(kind, l_max);
    p->coeff_elems = fftso3_coeff_elems(kind, l_max);
    cudaGetDevice(&p->device);
    make_fft_factors(p->N, p->fac);

    const int B = p->B, N = p->N, L = p->L;
    int rc;
    auto bail = [&](int code) {
        plan_free(p);
        delete p;
        return code;
    };

    // twiddles and weights
    std::vector<double> tw(2 * N);
    for (int i = 0; i < N; ++i) {
        double a = -2. * M_PI * (double)i / (double)N;
        tw[2 * i] = cos(a);
        tw[2 * i + 1] = sin(a);
    }
    p->weights.resize(N);
    host_weights(kind, l_max, p->weights.data());
    if ((rc = plan_alloc(p, (void**)&p->d_tw, sizeof(double) * 2 * N))) return bail(rc);
    if ((rc = plan_alloc(p, (void**)&p->d_w, sizeof(double) * N))) return bail(rc);
    if (cudaMemcpy(p->d_tw, tw.data(), sizeof(double) * 2 * N, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(p->d_w, p->weights.data(), sizeof(double) * N, cudaMemcpyHostToDevice) != cudaSuccess)
        return bail(cuda_fail(cudaGetLastError(), "upload constants"));

    // tables
    std::vector<long long> goff;
    if (p->so3) {
        int ng = B * B;
        goff.resize(ng + 1);
        long long o = 0;
        for (int g = 0; g < ng; ++g) {
            int m0, n0;
            group_mn(g, m0, n0);
            goff[g] = o;
            o += (long long)(B - m0) * N;
        }
        goff[ng] = o;
        p->table_elems = o;
    } else {
        goff.resize(B + 1);
        long long o = 0;
        for (int m = 0; m < B; ++m) {
            goff[m] = o;
            o += (long long)(B - m) * N;
        }
        goff[B] = o;
        p->table_elems = o;
    }
    if ((rc = plan_alloc(p, (void**)&p->d_goff, sizeof(long long) * goff.size()))) return bail(rc);
    if ((rc = plan_alloc(p, (void**)&p->d_table, sizeof(double) * p->table_elems))) return bail(rc);
    if (cudaMemcpy(p->d_goff, goff.data(), sizeof(long long) * goff.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        return bail(cuda_fail(cudaGetLastError(), "upload offsets"));
    std::vector<double> lf = log_factorials(2 * L + 2);
    if ((rc = plan_alloc(p, (void**)&p->d_lfact, sizeof(double) * lf.size()))) return bail(rc);
    if (cudaMemcpy(p->d_lfact, lf.data(), sizeof(double) * lf.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        return bail(cuda_fail(cudaGetLastError(), "upload log factorials"));
    {
        void* d_tmp = nullptr;
        cudaError_t e;
        if (p->so3) {
            std::vector<WignerSeeds> seeds(N);
            for (int k = 0; k < N; ++k) seeds[k] = make_seeds(beta_k(B, k));
            if ((e = cudaMalloc(&d_tmp, sizeof(WignerSeeds) * N)) != cudaSuccess) return bail(cuda_fail(e, "cudaMalloc"));
            cudaMemcpy(d_tmp, seeds.data(), sizeof(WignerSeeds) * N, cudaMemcpyHostToDevice);
            e = launch_wigner_table(p->d_table, p->d_goff, (const WignerSeeds*)d_tmp, p->d_lfact, L, N, B * B,
                                    recursion == FFTSO3_RECURSION_STABLE, 0);
        } else {
            std::vector<double> xs(N);
            for (int k = 0; k < N; ++k) xs[k] = cos(beta_k(B, k));
            if ((e = cudaMalloc(&d_tmp, sizeof(double) * N)) != cudaSuccess) return bail(cuda_fail(e, "cudaMalloc"));
            cudaMemcpy(d_tmp, xs.data(), sizeof(double) * N, cudaMemcpyHostToDevice);
            e = launch_legendre_table(p->d_table, p->d_goff, (const double*)d_tmp, L, N, 0);
        }
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        cudaFree(d_tmp);
        if (e != cudaSuccess) return bail(cuda_fail(e, "table generation"));
    }

    if (p->fp64) {
        if ((rc = plan_alloc(p, &p->d_work, cbytes(p) * (size_t)batch * p->grid_elems))) return bail(rc);
        if (p->real)
            if ((rc = plan_alloc(p, &p->d_fc, 16 * (size_t)batch * p->coeff_elems))) return bail(rc);
    } else {
        std::string err;
        rc = tc_create(&p->tc, p->L, p->N, batch, p->d_table, goff, p->table_elems, p->d_tw, p->d_w,
                       (flags & (FFTSO3_FLAG_REFINE | FFTSO3_FLAG_EXACT_INVERSE)) != 0, p->real, !p->so3,
                       (flags & FFTSO3_FLAG_AUTOTUNE) != 0,
                       precision == FFTSO3_PREC_FP32, err);
        if (rc) {
            g_err = err;
            return bail(rc);
        }
        p->bytes += tc_device_bytes(p->tc);
        const char* ev_ref = getenv("FFTSO3_REFINE_FP64");
        const unsigned exact_flags = FFTSO3_FLAG_REFINE | FFTSO3_FLAG_EXACT_INVERSE;
        const bool use_oz = (flags & exact_flags) && p->so3 && oz_supported(L, N) && !(ev_ref && ev_ref[0] == '1');
        if (use_oz) {
            // SO(3) refinement on the tensor cores: digit planes of the FP64 table, then the table is freed.
            // Chunks of 16 functions (two column tiles, whose items share each table tile through L2, so the
            // digit planes are read once per 16 functions) when the device has room for them with 16 GB to
            // spare after the FP64 table is freed, else 8 (one column tile), else fewer
            // The spectral form (N = 64..512) needs the double-float pencils only as its FFT's work space
            // (pen_fns = up to 8 functions at a time), so its contraction chunks grow to 32 functions (four column
            // tiles sharing each table tile; the digit planes read once per 32 functions).
            const bool spectral = fft_df32_k_supported(N);
            const size_t pen_fn = 16 * (size_t)p->grid_elems;
            const size_t planes = 4 * 2 * (size_t)(p->table_elems / N) * (size_t)((N + 63) / 64 * 64);
            const size_t tab64 = sizeof(double) * (size_t)p->table_elems;
            size_t freeb = 0, totb = 0;
            cudaMemGetInfo(&freeb, &totb);
            const size_t spare = (size_t)16 << 30, slack = (size_t)2 << 30;
            const size_t img_tile = (size_t)oz_image_bytes_per_column_tile(L);
            auto need = [&](size_t nch) {
                const size_t pens = spectral ? std::min<size_t>(nch, 8) : nch;
                return planes + pens * pen_fn + (nch + 7) / 8 * img_tile;
            };
            size_t nch = spectral ? 32 : 16;
            while (nch > 1 && (need(nch) + slack > freeb || freeb + tab64 < need(nch) + spare))
                nch = nch > 16 ? 16 : nch > 8 ? 8 : nch - 1;
            if (const char* ev = getenv("FFTSO3_REFINE_CHUNK")) {  // cap (1..16), e.g. to exercise several chunks
                const int c = atoi(ev);
                if (c >= 1 && (size_t)c < nch) nch = (size_t)c;
            }
            p->rchunk = (int)(nch < (size_t)batch ? nch : (size_t)batch);
            const int pen_fns = spectral ? std::min(p->rchunk, 8) : p->rchunk;
            std::string err;
            if ((rc = oz_create(&p->oz, p->d_table, goff, L, N, p->rchunk, pen_fns, p->d_tw, err))) {
                g_err = err;
                return bail(rc);
            }
            p->bytes += oz_device_bytes(p->oz);
            if (p->real) {
                const size_t nb = (size_t)p->rchunk;
                if ((rc = plan_alloc(p, &p->d_rc, 8 * (size_t)p->coeff_elems * nb))) return bail(rc);
                if ((rc = plan_alloc(p, &p->d_rfc, 16 * (size_t)p->coeff_elems * nb))) return bail(rc);
            }
            cudaFree(p->d_table);
            p->d_table = nullptr;
            p->bytes -= (long long)sizeof(double) * p->table_elems;
        } else if (flags & exact_flags) {
            // the FP64 inverse of the refinement and of the exact inverse keeps the FP64 table; its buffers hold
            // one chunk of functions, the chunk sized to about 4 GB of FP64 work grid
            const size_t g16 = 16 * (size_t)p->grid_elems;
            size_t nch = (size_t)4 << 30;
            nch = nch / g16 < 1 ? 1 : nch / g16;
            p->rchunk = (int)(nch < (size_t)batch ? nch : (size_t)batch);
            const size_t nb = (size_t)p->rchunk;
            if ((rc = plan_alloc(p, &p->d_rw, g16 * nb))) return bail(rc);
            if ((rc = plan_alloc(p, &p->d_rc, (p->real ? 8 : 16) * (size_t)p->coeff_elems * nb))) return bail(rc);
            if (p->real) {
                if ((rc = plan_alloc(p, &p->d_rg, 8 * (size_t)p->grid_elems * nb))) return bail(rc);
                if ((rc = plan_alloc(p, &p->d_rfc, 16 * (size_t)p->coeff_elems * nb))) return bail(rc);
            }
        } else {
            // the FP32-data paths keep only their BF16 planes / FP32 copy of the table
            cudaFree(p->d_table);
            p->d_table = nullptr;
            p->bytes -= (long long)sizeof(double) * p->table_elems;
        }
    }
    *out = p;
    return FFTSO3_SUCCESS;
}

int fftso3_plan_destroy(fftso3_plan* plan)
{
    if (!plan) return fail(FFTSO3_ERR_INVALID_ARG, "plan is NULL");
    int dev = -1;
    const int pdev = plan->device;
    cudaGetDevice(&dev);
    if (dev != pdev) cudaSetDevice(pdev);
    plan_free(plan);
    delete plan;
    if (dev >= 0 && dev != pdev) cudaSetDevice(dev);
    return FFTSO3_SUCCESS;
}

long long fftso3_plan_device_bytes(const fftso3_plan* plan) { return plan ? plan->bytes : -1; }

int fftso3_plan_set_timing(fftso3_plan* plan, int enable)
{
    int rc = check_plan(plan);
    if (rc) return rc;
    plan->timer.enabled = (enable != 0);
    return FFTSO3_SUCCESS;
}

int fftso3_stage_count(void) { return ST_COUNT; }

const char* fftso3_stage_name(int stage) { return stage_name(stage); }

int fftso3_plan_stage_times(fftso3_plan* plan, double* ms_total, long long* launches, int reset)
{
    int rc = check_plan(plan);
    if (rc) return rc;
    plan->timer.collect();
    for (int i = 0; i < ST_COUNT; ++i) {
        if (ms_total) ms_total[i] = plan->timer.total_ms[i];
        if (launches) launches[i] = plan->timer.launches[i];
    }
    if (reset) plan->timer.reset();
    return FFTSO3_SUCCESS;
}

int fftso3_plan_check(fftso3_plan* plan)
{
    int rc = check_plan(plan);
    if (rc) return rc;
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(e, "device synchronize");
    if (plan->tc) {
        int code = tc_status(plan->tc);
        if (code == 0 && plan->oz) code = oz_status(plan->oz);
        if (code != 0)
            return fail(FFTSO3_ERR_CUDA, "a tensor-core kernel gave up a bounded wait (code " + std::to_string(code) + ")");
    }
    return FFTSO3_SUCCESS;
}

int fftso3_forward(fftso3_plan* plan, const void* grid, void* coeffs, void* stream)
{
    int rc = check_plan(plan);
    if (rc) return rc;
    if (!grid || !coeffs) return fail(FFTSO3_ERR_INVALID_ARG, "grid/coeffs pointer is NULL");
    return run_forward(plan, grid, coeffs, (cudaStream_t)stream);
}

int fftso3_inverse(fftso3_plan* plan, const void* coeffs, void* grid, void* stream)
{
    int rc = check_plan(plan);
    if (rc) return rc;
    if (!grid || !coeffs) return fail(FFTSO3_ERR_INVALID_ARG, "grid/coeffs pointer is NULL");
    return run_inverse(plan, coeffs, grid, (cudaStream_t)stream);
}

static size_t grid_bytes(const fftso3_plan* p)
{
    return (size_t)p->batch * p->grid_elems * (p->real ? rbytes(p) : cbytes(p));
}
static size_t coeff_bytes(const fftso3_plan* p)
{
    return (size_t)p->batch * p->coeff_elems * (p->real ? rbytes(p) : cbytes(p));
}

static int ensure_io_grid(fftso3_plan* p)
{
    return p->d_io_grid ? FFTSO3_SUCCESS : plan_alloc(p, &p->d_io_grid, grid_bytes(p));
}
static int ensure_io_coeff(fftso3_plan* p)
{
    return p->d_io_coeff ? FFTSO3_SUCCESS : plan_alloc(p, &p->d_io_coeff, coeff_bytes(p));
}

// Device address of a pinned (page-locked) host buffer, or null for pageable memory.
// With unified addressing the GPU reads and writes pinned host memory directly
// (over the C2C link on Grace-Blackwell), so a transform can stream its input
// from, and its output to, host memory instead of staging whole copies.
static void* host_device_ptr(const void* p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

int fftso3_forward_host(fftso3_plan* plan, const void* grid_host, void* coeffs_host, void* stream)
{
    int rc = check_plan(plan);
    if (rc) return rc;
    if (!grid_host || !coeffs_host) return fail(FFTSO3_ERR_INVALID_ARG, "grid/coeffs pointer is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    // pinned buffers: read the samples / write the coefficients in place
    const void* gin = host_device_ptr(grid_host);
    void* cout = host_device_ptr(coeffs_host);
    if (plan->tc && (plan->flags & FFTSO3_FLAG_REFINE)) {
        // the refinement reads the samples twice: copy them once into the residual buffer (batch complex64 grids);
        // the residual (grid form) or the FFT remainders (spectral form) then overwrite them chunk by chunk, each
        // chunk's samples read before its outputs are written.  Real samples go to the buffer's upper half, so
        // that a chunk's complex64 remainders never reach the samples of later chunks.  The refined forward
        // passes over the coefficients several times: it writes them to device memory and copies them out once.
        void* stage = (char*)tc_resid_buffer(plan->tc) + (plan->real ? grid_bytes(plan) : 0);
        if ((rc = ensure_io_coeff(plan))) return rc;
        if (spectral_refine(plan)) {
            // the samples' copy pipelined under the double-float FFT, piece by piece
            if ((rc = refine_forward_spectral(plan, stage, plan->d_io_coeff, st, grid_host))) return rc;
        } else {
            CK(cudaMemcpyAsync(stage, grid_host, grid_bytes(plan), cudaMemcpyHostToDevice, st));
            if ((rc = run_forward(plan, stage, plan->d_io_coeff, st))) return rc;
        }
        CK(cudaMemcpyAsync(coeffs_host, plan->d_io_coeff, coeff_bytes(plan), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        return FFTSO3_SUCCESS;
    }
    if ((!gin && (rc = ensure_io_grid(plan))) || (!cout && (rc = ensure_io_coeff(plan)))) return rc;
    if (!gin) {
        CK(cudaMemcpyAsync(plan->d_io_grid, grid_host, grid_bytes(plan), cudaMemcpyHostToDevice, st));
        gin = plan->d_io_grid;
    }
    if ((rc = run_forward(plan, gin, cout ? cout : plan->d_io_coeff, st))) return rc;
    if (!cout) CK(cudaMemcpyAsync(coeffs_host, plan->d_io_coeff, coeff_bytes(plan), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return FFTSO3_SUCCESS;
}

// The exact inverse into host memory (SO(3), N = 64..512), pipelined in chunks of up to 8 functions (one column
// tile of the exact contraction): each chunk's coefficients are copied in, contracted and transformed, and its
// grids stream out through the device ring on the copy stream, so the copies out (the host link bounds the call)
// start after the first chunk instead of after the whole batch.
static int exact_inverse_host(fftso3_plan* p, const void* coeffs_host, void* grid_host, cudaStream_t st)
{
    StageTimer& T = p->timer;
    const long long C = p->coeff_elems, G = p->grid_elems;
    const int per = p->real ? 1 : 2;  // floats per element
    const size_t fn_bytes = (size_t)G * per * sizeof(float), cf_bytes = (size_t)C * per * sizeof(float);
    int rc = p->d_io_ring ? FFTSO3_SUCCESS : plan_alloc(p, &p->d_io_ring, 2 * (size_t)OZ_SYNTH_PIECE * fn_bytes);
    if (rc) return rc;
    void* pen = tc_exact_buffer(p->tc);
    const int cf = std::min(p->rchunk, 8);
    for (int f0 = 0; f0 < p->batch; f0 += cf) {
        const int nb = p->batch - f0 < cf ? p->batch - f0 : cf;
        float* cd = (float*)p->d_io_coeff + (long long)f0 * C * per;
        CK(cudaMemcpyAsync(cd, (const char*)coeffs_host + (size_t)f0 * cf_bytes, (size_t)nb * cf_bytes,
                           cudaMemcpyHostToDevice, st));
        const void* Fc;
        T.begin(ST_BASIS, st);
        if (p->real) {
            CK(launch_widen(cd, (double*)p->d_rc, (long long)nb * C, st));
            CK(launch_so3_r2c(p->d_rc, p->d_rfc, true, p->L, nb, st));
            Fc = p->d_rfc;
        } else {
            Fc = tc_group_from_packed(p->tc, p->d_io_coeff, f0, nb, st);
            if (!Fc) return cuda_fail(cudaGetLastError(), "tc_group_from_packed");
        }
        T.end(st);
        const bool last = f0 + nb >= p->batch;
        if ((rc = oz_inverse_exact(p->oz, Fc, p->real, nb, nullptr, p->real, st, &T, g_err, pen,
                                   (char*)grid_host + (size_t)f0 * fn_bytes, p->d_io_ring, last, !p->real)))
            return rc;
    }
    CK(cudaStreamSynchronize(st));
    return FFTSO3_SUCCESS;
}

int fftso3_inverse_host(fftso3_plan* plan, const void* coeffs_host, void* grid_host, void* stream)
{
    int rc = check_plan(plan);
    if (rc) return rc;
    if (!grid_host || !coeffs_host) return fail(FFTSO3_ERR_INVALID_ARG, "grid/coeffs pointer is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    // the coefficients always go to device memory in bulk copies (the inverse's first kernels gather them in an
    // order that would cross the host link in small pieces)
    if ((rc = ensure_io_coeff(plan))) return rc;
    if (plan->tc && (plan->flags & FFTSO3_FLAG_EXACT_INVERSE) && plan->oz && oz_spectral(plan->oz))
        return exact_inverse_host(plan, coeffs_host, grid_host, st);
    CK(cudaMemcpyAsync(plan->d_io_coeff, coeffs_host, coeff_bytes(plan), cudaMemcpyHostToDevice, st));
    const void* cin = plan->d_io_coeff;
    if (plan->tc && (plan->flags & FFTSO3_FLAG_EXACT_INVERSE)) {
        // the exact inverse copies its grids out itself, piece by piece under its FFT where it can
        if (!(plan->oz && oz_spectral(plan->oz)) && (rc = ensure_io_grid(plan))) return rc;
        if ((rc = exact_inverse(plan, cin, plan->d_io_grid, st, grid_host))) return rc;
        CK(cudaStreamSynchronize(st));
        return FFTSO3_SUCCESS;
    }
    // otherwise a grid in pinned host memory is written in place, by rows
    void* gout = host_device_ptr(grid_host);
    if (!gout && (rc = ensure_io_grid(plan))) return rc;
    if ((rc = run_inverse(plan, cin, gout ? gout : plan->d_io_grid, st))) return rc;
    if (!gout) CK(cudaMemcpyAsync(grid_host, plan->d_io_grid, grid_bytes(plan), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return FFTSO3_SUCCESS;
}

int fftso3_correlate_s2(fftso3_plan* plan, const void* F_s2, const void* G_s2, void* grid, void* stream)
{
    int rc = check_plan(plan);
    if (rc) return rc;
    if (plan->kind != FFTSO3_SO3_REAL)
        return fail(FFTSO3_ERR_INVALID_ARG, "correlation needs an FFTSO3_SO3_REAL plan");
    if (!F_s2 || !G_s2 || !grid) return fail(FFTSO3_ERR_INVALID_ARG, "NULL pointer argument");
    if (!plan->d_corr && (rc = plan_alloc(plan, &plan->d_corr, coeff_bytes(plan)))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    CK(launch_corr_coeffs(F_s2, G_s2, plan->d_corr, plan->fp64, plan->L, plan->batch, st));
    return run_inverse(plan, plan->d_corr, grid, st);
}

int fftso3_grid_argmax(fftso3_plan* plan, const void* grid, long long* index_out, double* value_out, void* stream)
{
    int rc = check_plan(plan);
    if (rc) return rc;
    if (!plan->real) return fail(FFTSO3_ERR_INVALID_ARG, "arg-max needs a real-kind plan");
    if (!grid || !index_out) return fail(FFTSO3_ERR_INVALID_ARG, "NULL pointer argument");
    const int chunks = 256, nb = plan->batch;
    const size_t sb = argmax_scratch_bytes(nb, chunks);
    if (!plan->d_amax && (rc = plan_alloc(plan, &plan->d_amax, sb))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    double* ov = (double*)((char*)plan->d_amax + (size_t)nb * chunks * 16);
    long long* oi = (long long*)(ov + nb);
    CK(launch_argmax(grid, plan->fp64, plan->grid_elems, nb, chunks, plan->d_amax, ov, oi, st));
    CK(cudaMemcpyAsync(index_out, oi, sizeof(long long) * nb, cudaMemcpyDeviceToHost, st));
    if (value_out) CK(cudaMemcpyAsync(value_out, ov, sizeof(double) * nb, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return FFTSO3_SUCCESS;
}

int fftso3_inverse_points(fftso3_plan* plan, const void* coeffs, int index, const double* pts, int n, void* out,
                          void* stream)
{
    int rc = check_plan(plan);
    if (rc) return rc;
    if (!coeffs || !pts || !out) return fail(FFTSO3_ERR_INVALID_ARG, "NULL pointer argument");
    if (index < 0 || index >= plan->batch) return fail(FFTSO3_ERR_INVALID_ARG, "index outside the plan's batch");
    if (n < 0) return fail(FFTSO3_ERR_INVALID_ARG, "n must be >= 0");
    if (n == 0) return FFTSO3_SUCCESS;
    if (!plan->fp64) return fail(FFTSO3_ERR_UNSUPPORTED, "point evaluation needs an FFTSO3_PREC_FP64 plan");
    cudaStream_t st = (cudaStream_t)stream;
    const int L = plan->L;
    const long long C = plan->coeff_elems;
    const int dim = plan->so3 ? 3 : 2;
    cudaError_t e;
    // the plan's recursion factors, once
    if (!plan->d_prec) {
        if (plan->so3) {
            const size_t nrec = wigner_rec_elems(L), nsq = wigner_sq_elems(L);
            if ((rc = plan_alloc(plan, &plan->d_prec, sizeof(double4) * nrec + sizeof(double) * nsq))) return rc;
            plan->d_psq = (double*)((double4*)plan->d_prec + nrec);
            e = launch_wigner_rec_factors((double4*)plan->d_prec, plan->d_psq, L, st);
        } else {
            if ((rc = plan_alloc(plan, &plan->d_prec, sizeof(double2) * legendre_rec_elems(L)))) return rc;
            e = launch_legendre_rec_factors((double2*)plan->d_prec, L, st);
        }
        if (e != cudaSuccess) {  // not built: release it, so a later call builds it again
            cudaFree(plan->d_prec);
            plan->bytes -= (long long)(plan->so3 ? sizeof(double4) * wigner_rec_elems(L) + sizeof(double) * wigner_sq_elems(L)
                                                 : sizeof(double2) * legendre_rec_elems(L));
            plan->d_prec = nullptr;
            plan->d_psq = nullptr;
            return cuda_fail(e, "recursion factors");
        }
    }
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    int m0b[MAX_POINT_PARTS + 1];
    const int S = points_parts(plan->so3, L, n, nsm, m0b);
    // plan-owned scratch (grows, never shrinks; the call synchronises before returning):
    // [points][values][seeds][parts][complex coefficients of a real kind], 256-byte aligned pieces
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t b_pts = up(sizeof(double) * dim * n), b_out = up(sizeof(double2) * n);
    const size_t b_seed = up(plan->so3 ? sizeof(WignerSeeds) * n : sizeof(double) * n);
    const size_t b_part = up(sizeof(double2) * (size_t)S * n), b_c = plan->real ? up(16 * (size_t)C) : 0;
    const size_t need = b_pts + b_out + b_seed + b_part + b_c;
    if (need > plan->pscratch_bytes) {
        if (plan->d_pscratch) {
            cudaFree(plan->d_pscratch);
            plan->bytes -= (long long)plan->pscratch_bytes;
            plan->d_pscratch = nullptr;
            plan->pscratch_bytes = 0;
        }
        if ((rc = plan_alloc(plan, &plan->d_pscratch, need))) return rc;
        plan->pscratch_bytes = need;
    }
    char* base = (char*)plan->d_pscratch;
    double* d_pts = (double*)base;
    double2* d_out = (double2*)(base + b_pts);
    void* d_seed = base + b_pts + b_out;
    double2* d_part = (double2*)(base + b_pts + b_out + b_seed);
    void* d_c = base + b_pts + b_out + b_seed + b_part;
    // complex coefficients of the selected function
    const double2* Fc;
    if (plan->real) {
        const double* src = (const double*)coeffs + (long long)index * C;
        e = plan->so3 ? launch_so3_r2c(src, d_c, true, L, 1, st) : launch_s2_r2c(src, d_c, true, L, 1, st);
        if (e != cudaSuccess) return cuda_fail(e, "real-to-complex coefficients");
        Fc = (const double2*)d_c;
    } else {
        Fc = (const double2*)coeffs + (long long)index * C;
    }
    if ((e = cudaMemcpyAsync(d_pts, pts, sizeof(double) * dim * n, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return cuda_fail(e, "copy points");
    if (plan->so3) {
        std::vector<WignerSeeds> seeds(n);
        for (int i = 0; i < n; ++i) seeds[i] = make_seeds(pts[3 * i + 1]);
        e = cudaMemcpyAsync(d_seed, seeds.data(), sizeof(WignerSeeds) * n, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = launch_so3_points(Fc, (const WignerSeeds*)d_seed, d_pts, (const double4*)plan->d_prec, plan->d_psq,
                                  plan->d_lfact, L, plan->recursion == FFTSO3_RECURSION_STABLE, n, m0b, S, d_part,
                                  d_out, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // seeds vector must outlive the copy
    } else {
        std::vector<double> xs(n);
        for (int i = 0; i < n; ++i) xs[i] = cos(pts[2 * i]);
        e = cudaMemcpyAsync(d_seed, xs.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = launch_s2_points(Fc, (const double*)d_seed, d_pts, (const double2*)plan->d_prec, L, n, m0b, S, d_part,
                                 d_out, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    if (e != cudaSuccess) return cuda_fail(e, "point evaluation");
    if (plan->real) {
        std::vector<double> tmp(2 * (size_t)n);
        if ((e = cudaMemcpy(tmp.data(), d_out, sizeof(double2) * n, cudaMemcpyDeviceToHost)) != cudaSuccess)
            return cuda_fail(e, "copy points");
        for (int i = 0; i < n; ++i) ((double*)out)[i] = tmp[2 * i];
    } else if ((e = cudaMemcpy(out, d_out, sizeof(double2) * n, cudaMemcpyDeviceToHost)) != cudaSuccess) {
        return cuda_fail(e, "copy points");
    }
    return FFTSO3_SUCCESS;
}

int fftso3_derivative(fftso3_plan* plan, const void* coeffs, int axis, void* coeffs_out, void* stream)
{
    int rc = check_plan(plan);
    if (rc) return rc;
    if (!plan->so3) return fail(FFTSO3_ERR_INVALID_ARG, "derivatives need an SO(3) plan");
    if (axis < 1 || axis > 3) return fail(FFTSO3_ERR_INVALID_ARG, "axis must be 1, 2 or 3");
    if (!coeffs || !coeffs_out) return fail(FFTSO3_ERR_INVALID_ARG, "NULL pointer argument");
    if (coeffs == coeffs_out) return fail(FFTSO3_ERR_INVALID_ARG, "coeffs and coeffs_out must be different buffers");
    const long long R = (long long)plan->B * plan->B;
    if (!plan->d_deriv) {
        std::vector<DerivEntry> t = derivative_table(plan->L, plan->real);
        if (t.empty()) return fail(FFTSO3_ERR_CUDA, "internal: derivative table has a row with three nonzeros");
        if ((rc = plan_alloc(plan, (void**)&plan->d_deriv, sizeof(DerivEntry) * t.size()))) return rc;
        cudaError_t e = cudaMemcpy(plan->d_deriv, t.data(), sizeof(DerivEntry) * t.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(plan->d_deriv);
            plan->d_deriv = nullptr;
            plan->bytes -= (long long)(sizeof(DerivEntry) * t.size());
            return cuda_fail(e, "derivative table");
        }
    }
    CK(launch_derivative(coeffs, coeffs_out, plan->d_deriv + (axis - 1) * R, plan->fp64, plan->real, plan->L,
                         plan->batch, (cudaStream_t)stream));
    return FFTSO3_SUCCESS;
}

int fftso3_clebsch_gordan(int l1, int l2, int real, void* out_host)
{
    if (l1 < 0 || l2 < 0) return fail(FFTSO3_ERR_INVALID_ARG, "l1 and l2 must be >= 0");
    if (!out_host) return fail(FFTSO3_ERR_INVALID_ARG, "output pointer is NULL");
    if (l1 > 1023 || l2 > 1023) return fail(FFTSO3_ERR_UNSUPPORTED, "l1, l2 above 1023 are not supported");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(FFTSO3_ERR_NO_DEVICE, "no CUDA device available");
    const size_t n = (size_t)(2 * l1 + 1) * (2 * l2 + 1);
    double* C = nullptr;
    double2* cr = nullptr;
    cudaError_t e = cudaMalloc(&C, sizeof(double) * n * n);
    if (e == cudaSuccess && real) e = cudaMalloc(&cr, sizeof(double2) * n * n);
    if (e == cudaSuccess) e = launch_clebsch_gordan(l1, l2, C, cr, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess)
        e = real ? cudaMemcpy(out_host, cr, sizeof(double2) * n * n, cudaMemcpyDeviceToHost)
                 : cudaMemcpy(out_host, C, sizeof(double) * n * n, cudaMemcpyDeviceToHost);
    if (C) cudaFree(C);
    if (cr) cudaFree(cr);
    if (e != cudaSuccess) return cuda_fail(e, "clebsch_gordan");
    return FFTSO3_SUCCESS;
}

int fftso3_wigner_d(double beta, int l_max, int recursion, double* d_out_host)
{
    if (l_max < 0) return fail(FFTSO3_ERR_INVALID_ARG, "l_max must be >= 0");
    if (!d_out_host) return fail(FFTSO3_ERR_INVALID_ARG, "output pointer is NULL");
    if (recursion != FFTSO3_RECURSION_REFERENCE && recursion != FFTSO3_RECURSION_STABLE)
        return fail(FFTSO3_ERR_INVALID_ARG, "unknown recursion mode");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(FFTSO3_ERR_NO_DEVICE, "no CUDA device available");
    long long C = so3_off(l_max + 1);
    WignerSeeds s = make_seeds(beta);
    std::vector<double> lf = log_factorials(2 * l_max + 2);
    void *d_s = nullptr, *d_lf = nullptr, *d_o = nullptr;
    cudaError_t e = cudaMalloc(&d_s, sizeof(s));
    if (e == cudaSuccess) e = cudaMalloc(&d_lf, sizeof(double) * lf.size());
    if (e == cudaSuccess) e = cudaMalloc(&d_o, sizeof(double) * C);
    if (e == cudaSuccess) e = cudaMemcpy(d_s, &s, sizeof(s), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_lf, lf.data(), sizeof(double) * lf.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = launch_wigner_full((const WignerSeeds*)d_s, (const double*)d_lf, l_max,
                               recursion == FFTSO3_RECURSION_STABLE, (double*)d_o, 0);
    if (e == cudaSuccess) e = cudaMemcpy(d_out_host, d_o, sizeof(double) * C, cudaMemcpyDeviceToHost);
    if (d_s) cudaFree(d_s);
    if (d_lf) cudaFree(d_lf);
    if (d_o) cudaFree(d_o);
    if (e != cudaSuccess) return cuda_fail(e, "wigner_d");
    return FFTSO3_SUCCESS;
}

}  // extern "C"
