/*
 * fftso3_gb300.h -- C ABI of the GB300 (sm_103a) SO(3) / S^2 harmonic-transform library.
 *
 * Each entry point replaces one operation of the fdcl-gwu/FFTSO3 C++ API
 * (cited per declaration as file:line of that project).  The ABI uses plain
 * pointers, sizes and an opaque plan; every call returns an int status
 * (FFTSO3_SUCCESS == 0) and fftso3_last_error_string() describes the last
 * failure on the calling thread.  The reference reports errors with assert()
 * only (fdcl_FFTSO3_matrix.cpp:23-33); this library rejects the same bad
 * inputs (l_max < 0, index ranges, sizes) with FFTSO3_ERR_INVALID_ARG instead.
 *
 * Data layouts (shared by every call):
 *   B = l_max + 1, N = 2B.
 *   SO(3) grid   [batch][k][j1][j2]: f(alpha_j1, beta_k, gamma_j2),
 *                beta_k = (2k+1) pi / (4B), alpha_j = gamma_j = j pi / B
 *                (fdcl_FFTSO3.cpp:578-591, loop order :676-685).
 *   S^2 grid     [batch][k][j]: f(theta_k, phi_j), theta_k = (2k+1) pi / (4B),
 *                phi_j = j pi / B (fdcl_FFTS2.cpp:292-300).
 *   SO(3) coefficients [batch][C], C = B(4B^2-1)/3, F(l,m,n) at
 *                l(4l^2-1)/3 + (m+l) + (n+l)(2l+1): the per-l (2l+1)x(2l+1)
 *                column-major blocks of FFTSO3_matrix (fdcl_FFTSO3_matrix.cpp:43-47)
 *                laid end to end, so each M[l].data() is one contiguous copy.
 *   S^2 coefficients [batch][B^2], F(l,m) at l^2 + m + l (fdcl_FFTS2_matrix.cpp:43-47).
 *   Complex data is interleaved (re, im): complex128 for FFTSO3_PREC_FP64,
 *   complex64 for the tensor-core / FP32 precisions; real data float64 / float32.
 *
 * Streams: `stream` is a cudaStream_t passed as void*; NULL means the legacy
 * default stream.  Device-pointer calls are asynchronous on that stream.
 */
#ifndef FFTSO3_GB300_H
#define FFTSO3_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define FFTSO3_SUCCESS 0
#define FFTSO3_ERR_INVALID_ARG 1
#define FFTSO3_ERR_CUDA 2
#define FFTSO3_ERR_OOM 3
#define FFTSO3_ERR_UNSUPPORTED 4
#define FFTSO3_ERR_NO_DEVICE 5

/* transform kinds: the four reference classes */
#define FFTSO3_SO3_COMPLEX 0 /* fdcl::FFTSO3_complex, include/fdcl_FFTSO3.hpp:27-177 */
#define FFTSO3_SO3_REAL 1    /* fdcl::FFTSO3_real,    include/fdcl_FFTSO3.hpp:184-308 */
#define FFTSO3_S2_COMPLEX 2  /* fdcl::FFTS2_complex,  include/fdcl_FFTS2.hpp:28-100 */
#define FFTSO3_S2_REAL 3     /* fdcl::FFTS2_real,     include/fdcl_FFTS2.hpp:107-160 */

/* arithmetic of the beta-sum contraction */
#define FFTSO3_PREC_FP64 0      /* FP64 end to end (the plain method) */
#define FFTSO3_PREC_TC_BF16X3 1 /* tcgen05 tensor cores, 3-term split-BF16, FP32 accumulate; complex64/float32 data;
                                   all four kinds, l_max <= 511 */
#define FFTSO3_PREC_FP32 2      /* FP32 beta-sum on the CUDA cores (FP32 table, FP32 FMA accumulate), FP32 FFT;
                                   complex64/float32 data; all four kinds, l_max <= 511 */

/* Wigner-d recursion */
#define FFTSO3_RECURSION_REFERENCE 0 /* bit-faithful to fdcl_FFTSO3.cpp:127-194 (underflows near beta=pi, l_max>~90) */
#define FFTSO3_RECURSION_STABLE 1    /* log-domain seeds + extended-exponent recursion */

/* plan flags */
#define FFTSO3_FLAG_REFINE 0x1u /* FP32-data forward: one residual step F += forward(f - inverse(F)); the
                                   inverse of F and the difference f - inverse(F) are formed in FP64 or exactly
                                   (SO(3), l_max <= 255: digit sums on the tensor cores; for N = 64..512 the
                                   step runs in the pencil domain on a double-float FFT of the samples), so the
                                   correction removes the first forward's FP32 FFT and contraction errors.
                                   Environment at plan creation: FFTSO3_REFINE_FP64=1 keeps the FP64 inverse;
                                   FFTSO3_REFINE_CHUNK=n caps the functions per refinement chunk */
#define FFTSO3_FLAG_GRAPH 0x2u  /* batches: capture each direction into a CUDA graph, replay it */
#define FFTSO3_FLAG_AUTOTUNE 0x4u /* tensor-core plans: time the launch shapes of the generic-N FFT passes on
                                     the plan's workspace at creation and keep the fastest (cached per N for
                                     the process); batches: also time 1/2/4/8 bucket streams on the first
                                     call of each direction */
#define FFTSO3_FLAG_EXACT_INVERSE 0x8u /* FP32-data inverse synthesised without FP32 rounding and rounded once to
                                          the output (complex64 / float32): SO(3) with l_max <= 255 by exact digit
                                          sums on the tensor cores and a double-float FFT, otherwise in FP64, in
                                          chunks of functions (the refinement's buffers, shared with
                                          FFTSO3_FLAG_REFINE).  The grid values are the FP64 synthesis of the
                                          coefficients up to that one rounding. */

typedef struct fftso3_plan fftso3_plan;
typedef struct fftso3_batch fftso3_batch;

/* Thread-local description of the last error ("" when none). */
const char* fftso3_last_error_string(void);

/* Library version (major*10000 + minor*100 + patch). */
int fftso3_version(void);

/* Element counts of one function's grid and coefficient vector for a kind
 * (complex or real elements as the kind dictates).  -1 on bad arguments. */
long long fftso3_grid_elems(int kind, int l_max);
long long fftso3_coeff_elems(int kind, int l_max);

/* Quadrature weights w_k, k < 2B, computed on the host in FP64.
 * SO(3): fdcl_FFTSO3.cpp:236-256 (compute_weight); S^2: fdcl_FFTS2.cpp:102-123. */
int fftso3_weights(int kind, int l_max, double* weights_out);

/* Create a plan for `batch` functions of bandwidth l_max on the current CUDA
 * device.  Replaces the constructor / init(l_max) of the reference classes
 * (fdcl_FFTSO3.cpp:3-14, :1000-1008, fdcl_FFTS2.cpp:3-15, :371-381); the plan
 * owns the Wigner-d (SO(3)) or Legendre (S^2) tables, twiddles and workspace.
 * precision: FFTSO3_PREC_*; recursion: FFTSO3_RECURSION_* (SO(3) only).
 * Threads: a plan is not re-entrant (nor are the reference objects, whose
 * init() and weights mutate members).  Calls on one plan share its workspace,
 * and fftso3_inverse_points may free and regrow the plan's point scratch, so
 * two host threads must not use one plan at the same time: give each thread
 * its own plan, or serialise the calls.  Different plans are independent.
 * With FFTSO3_FLAG_REFINE (FP32-data precisions) the plan also keeps the FP64
 * table and FP64 work buffers for one chunk of functions (about 4 GB of work
 * grid) for the refinement's FP64 inverse. */
int fftso3_plan_create(fftso3_plan** plan, int kind, int l_max, int batch, int precision, int recursion,
                       unsigned flags);
int fftso3_plan_destroy(fftso3_plan* plan);

/* Device bytes held by the plan (tables + workspace). */
long long fftso3_plan_device_bytes(const fftso3_plan* plan);

/* Per-stage timing (tracing).  With timing enabled every internal kernel
 * launch of the plan is bracketed by CUDA events on the caller's stream;
 * fftso3_plan_stage_times() waits for them and returns, per stage, the summed
 * milliseconds and the number of launches (arrays of fftso3_stage_count()
 * entries), optionally resetting the totals.  Stage i is named
 * fftso3_stage_name(i).  No reference counterpart (the reference times whole
 * calls with fdcl::tictoc, src/fdcl_tictoc.cpp:4-22). */
int fftso3_plan_set_timing(fftso3_plan* plan, int enable);
int fftso3_stage_count(void);
const char* fftso3_stage_name(int stage);
int fftso3_plan_stage_times(fftso3_plan* plan, double* ms_total, long long* launches, int reset);

/* Synchronise the plan's device and report failures of earlier asynchronous
 * calls, including a tensor-core kernel that gave up one of its bounded waits
 * (its kernels never spin without limit; they record an error code instead).
 * No reference counterpart: the reference has no asynchronous work. */
int fftso3_plan_check(fftso3_plan* plan);

/* Forward transform of `batch` sampled functions (device pointers).
 * Replaces forward_transform(func): fdcl_FFTSO3.cpp:654-763 (complex),
 * :774-850 (real), fdcl_FFTS2.cpp:125-192 (complex), :424-436 (real); the
 * callback is replaced by its samples on the grid above. */
int fftso3_forward(fftso3_plan* plan, const void* grid, void* coeffs, void* stream);

/* Inverse transform onto the full grid (device pointers): f at every grid
 * point, with the semantics of inverse_transform(F, alpha, beta, gamma)
 * (fdcl_FFTSO3.cpp:498-531, :1141-1156; fdcl_FFTS2.cpp:194-230, :500-512)
 * evaluated at each (alpha_j1, beta_k, gamma_j2) / (theta_k, phi_j). */
int fftso3_inverse(fftso3_plan* plan, const void* coeffs, void* grid, void* stream);

/* Host-buffer variants: transform host data and synchronise the stream
 * before returning (the reference's by-value call convention).  Host buffers
 * may be pageable or pinned (page-locked; faster).  The inverse copies the
 * coefficients to the device in bulk; its grids are copied out (or, for plain
 * plans and pinned buffers, written in place by the kernels over the host
 * link).  Refined forwards copy the samples in pieces of a few functions under
 * the FFT of the previous piece; exact inverses (SO(3), N = 64..512) run in
 * chunks of 8 functions whose grids stream out through a small device ring
 * on an internal copy stream while the next chunk is computed. */
int fftso3_forward_host(fftso3_plan* plan, const void* grid_host, void* coeffs_host, void* stream);
int fftso3_inverse_host(fftso3_plan* plan, const void* coeffs_host, void* grid_host, void* stream);

/* Point evaluation of one coefficient set (batch entry `index` of the device
 * array `coeffs`) at n points given in host memory; the n results are written
 * to host memory and the call synchronises `stream` before returning.
 * SO(3): pts = n x (alpha, beta, gamma); S^2: n x (theta, phi).
 * Replaces inverse_transform(F, alpha, beta, gamma) (fdcl_FFTSO3.cpp:498-531,
 * :1141-1156) and inverse_transform(F, theta, phi) (fdcl_FFTS2.cpp:194-230,
 * :500-512).  Output complex128 (complex kinds) or float64 (real kinds);
 * FP64 arithmetic; needs an FFTSO3_PREC_FP64 plan (FFTSO3_ERR_UNSUPPORTED
 * otherwise).  The first call allocates the plan's beta-independent
 * recursion factors and a scratch buffer that later calls reuse. */
int fftso3_inverse_points(fftso3_plan* plan, const void* coeffs, int index, const double* pts, int n, void* out,
                          void* stream);

/* S^2 -> SO(3) correlation (spherical shape matching).  For `batch` pairs of
 * real S^2 coefficient vectors F, G (device, [batch][B^2], packed like
 * FFTS2_matrix_real, float64 for FP64 plans, float32 otherwise), writes to the
 * device grid of a FFTSO3_SO3_REAL plan the score of every grid rotation R,
 *   J(R) = sum_l G[l]^T U^l(R) F[l]
 * (U^l the real harmonics of R, fdcl_FFTSO3.cpp:1062-1105) -- the cost the
 * reference's example evaluates one rotation at a time
 * (example/example3_SSM.hpp, J(R); example/example3.cpp:28-95).  It forms the
 * real SO(3) coefficients Fr(l,m,n) = G_l(m) F_l(n) / (2l+1) and runs the
 * plan's inverse transform.  Asynchronous on `stream`. */
int fftso3_correlate_s2(fftso3_plan* plan, const void* F_s2, const void* G_s2, void* grid, void* stream);

/* Arg-max of each of the plan's `batch` real grids (device): flat grid index
 * (k N^2 + j1 N + j2 for SO(3), k N + j for S^2; ties -> smallest index) and
 * value, written to host arrays of `batch` entries (value_out may be NULL);
 * synchronises `stream`.  With fftso3_correlate_s2 it gives the best rotation
 * (alpha_j1, beta_k, gamma_j2) to the grid's resolution.  No reference
 * counterpart (the reference descends the gradient from an initial guess). */
int fftso3_grid_argmax(fftso3_plan* plan, const void* grid, long long* index_out, double* value_out, void* stream);

/* Wigner-d table d^l_mn(beta) for all l <= l_max at one angle, packed like
 * the SO(3) coefficients, computed on the GPU (host output buffer).
 * Replaces wigner_d(beta) (fdcl_FFTSO3.cpp:122-194). */
int fftso3_wigner_d(double beta, int l_max, int recursion, double* d_out_host);

/* Directional derivative of SO(3) functions: for each of the plan's `batch`
 * coefficient vectors F (device, the plan's kind and element type), writes
 * to coeffs_out (device, a different buffer) the coefficients of
 *   f_i(R) = d/dt f(R exp(t e_i)) at t = 0,   i = axis in {1, 2, 3},
 * i.e. F'^l = F^l (u_i^l)^T per degree, with u_i^l the matrices of
 * deriv_wigner_D (fdcl_FFTSO3.cpp:417-453; complex kind) or
 * deriv_real_harmonics (:1577-1645; real kind), which satisfy
 * d/dt D^l(R exp(t e_i)) = D^l(R) u_i^l.  An inverse transform of the result
 * gives the derivative on the whole grid.  The first call builds the plan's
 * table of the matrices' nonzeros (at most two per row).  Asynchronous on
 * `stream`.  SO(3) kinds only. */
int fftso3_derivative(fftso3_plan* plan, const void* coeffs, int axis, void* coeffs_out, void* stream);

/* Clebsch-Gordan coefficients for the pair (l1, l2), computed on the GPU:
 * real = 0: the n x n matrix C of the complex harmonics (float64), real = 1:
 * the matrix c of the real harmonics (complex128); n = (2 l1 + 1)(2 l2 + 1),
 * column-major, row (l1 + m1)(2 l2 + 1) + l2 + m2, column
 * l^2 - (l2 - l1)^2 + l + m, as Clebsch_Gordon_complex::compute and
 * Clebsch_Gordon_real::compute (src/fdcl_Clebsch_Gordon.cpp:18-26, :41-98,
 * :224-329).  out_host: n * n elements of host memory; the call allocates
 * device scratch of that size and synchronises. */
int fftso3_clebsch_gordan(int l1, int l2, int real, void* out_host);

/* ---- batches of uneven bandwidth ----
 * One object for n_functions functions of one kind whose l_max differs per
 * function (l_max[i]).  It replaces the reference user's loop of
 * forward_transform / inverse_transform calls over functions
 * (fdcl_FFTSO3.cpp:654-763, :774-850, :1141-1167; fdcl_FFTS2.cpp:125-230,
 * :424-512), re-initialising the object whenever l_max changes (:500).
 * Functions are bucketed by l_max and every bucket runs as one batched plan.
 * Tensor-core SO(3) batches without refinement run each direction as three
 * launches over all buckets on the caller's stream (forward: one launch of
 * both FFT passes of every beta slice, one persistent beta-sum GEMM, one
 * coefficient conversion; the inverse mirrors it) whenever one beta slice of
 * the largest l_max fits a CTA's shared memory (l_max <= 77 complex, about
 * <= 105 real); otherwise the buckets run side by side on internal streams forked
 * from and joined into the caller's stream (tensor-core batches still share
 * one GEMM launch).  FFTSO3_BATCH_PHASES=0 in the environment at creation
 * selects the per-bucket form for every batch.
 * Layout: function i's grid starts fftso3_batch_grid_offset(b, i) elements
 * into `grids` and its coefficients fftso3_batch_coeff_offset(b, i) elements
 * into `coeffs` (elements of the kind's and precision's type, as for plans);
 * i = n_functions gives the totals.  The batch chooses the offsets
 * (ascending l_max, caller order within one l_max) so that no gather pass is
 * needed.  flags: FFTSO3_FLAG_REFINE (tensor-core forward refinement),
 * FFTSO3_FLAG_GRAPH (capture each direction once per (input, output) pair of
 * pointers into a CUDA graph and replay it; a new pointer pair re-captures),
 * FFTSO3_FLAG_AUTOTUNE (tune each bucket plan's FFT launch shapes at creation
 * and the number of bucket streams on the first call).
 * Calls on one batch object must not overlap (shared workspaces). */
int fftso3_batch_create(fftso3_batch** batch, int kind, const int* l_max, int n_functions, int precision,
                        int recursion, unsigned flags);
int fftso3_batch_destroy(fftso3_batch* batch);
long long fftso3_batch_grid_offset(const fftso3_batch* batch, int fn);
long long fftso3_batch_coeff_offset(const fftso3_batch* batch, int fn);
int fftso3_batch_bucket_count(const fftso3_batch* batch);
/* Internal streams the buckets are spread over (chosen by FFTSO3_FLAG_AUTOTUNE on the first call). */
int fftso3_batch_stream_count(const fftso3_batch* batch);
/* Kernel nodes of the CUDA graph captured for direction 0 (forward) or 1
 * (inverse) with FFTSO3_FLAG_GRAPH; -1 before the first capture. */
int fftso3_batch_graph_kernels(const fftso3_batch* batch, int direction);
long long fftso3_batch_device_bytes(const fftso3_batch* batch);
int fftso3_batch_forward(fftso3_batch* batch, const void* grids, void* coeffs, void* stream);
int fftso3_batch_inverse(fftso3_batch* batch, const void* coeffs, void* grids, void* stream);
/* Bucket `bucket` (0 <= bucket < fftso3_batch_bucket_count()): its l_max and number of functions. */
int fftso3_batch_bucket_info(const fftso3_batch* batch, int bucket, int* l_max, int* count);
/* Per-stage timing of every bucket's plan (as fftso3_plan_set_timing); while
 * it is on, calls launch eagerly instead of through the CUDA graph, and the
 * buckets run one after another on the caller's stream.  Stage
 * times are summed over all buckets (bucket = -1) or given for one bucket. */
int fftso3_batch_set_timing(fftso3_batch* batch, int enable);
int fftso3_batch_stage_times(fftso3_batch* batch, int bucket, double* ms_total, long long* launches, int reset);
/* Synchronise and report asynchronous failures of every bucket (fftso3_plan_check). */
int fftso3_batch_check(fftso3_batch* batch);

/* Largest l_max accepted by fftso3_forward_noalloc(). */
#define FFTSO3_NOALLOC_MAX_LMAX 31

/* Allocation-free forward transform: FFTSO3_SO3_COMPLEX, FP64, the reference
 * Wigner-d recursion, one function, l_max <= FFTSO3_NOALLOC_MAX_LMAX.  No
 * counterpart in the reference: it is the forward transform of a batch-1
 * FP64 plan (fdcl_FFTSO3.cpp:654-763 semantics) for callers that cannot
 * allocate device memory -- a host that owns all device memory and does not
 * let libraries call cudaMalloc, or a latency-critical loop where
 * cudaMalloc/cudaFree would synchronise the device.  It allocates nothing: its
 * intermediates (tables, seeds, the Wigner-d table and the 64^3 FFT work
 * grid, about 10 MB) live in one file-scope __device__ array that every GPU
 * which loads the library holds until the process exits.  grid (complex128,
 * (2l_max+2)^3) and coeffs (complex128) are device pointers; the call is
 * asynchronous on `stream`.  The first call on a device looks up that array's
 * address (cudaGetSymbolAddress, with the device current): make it before any
 * stream capture.  All calls share the array, so calls that overlap on the GPU
 * race; serialise them.  l_max above the limit returns FFTSO3_ERR_INVALID_ARG. */
int fftso3_forward_noalloc(int l_max, const void* grid, void* coeffs, void* stream);

/* The two-dimensional grid FFT stage of the tensor-core SO(3) transforms on
 * its own (the alpha/gamma FFTs that the reference runs inside its forward
 * transforms, fdcl_FFTSO3.cpp:689-699 and :805-815).  N = 2(l_max+1) in {64, 128, 256,
 * 512}; nf grids; in != out, device buffers, asynchronous on `stream`.
 *   dir = 1:  grids g[f][k][j1][j2] (complex64, or float32 when real != 0) ->
 *             pencils P[f][p][q][k] = sum_{j1,j2} g[f][k][j1][j2] e^{-2 pi i (p j1 + q j2) / N}
 *   dir = -1: pencils P[f][p][q][k] -> grids g[f][k][j1][j2] = sum_{p,q} P[f][p][q][k] e^{-2 pi i (p j1 + q j2) / N}
 *             (complex64; with real != 0 the pencils must be Hermitian, P[f][-p][-q][k] =
 *             conj P[f][p][q][k] indices mod N, as those of a real grid are, and g is written as float32)
 * Both directions use the kernel e^{-2 pi i / N} without normalisation (the
 * inverse SO(3) transform feeds it bin-reversed pencils).  One launch: the
 * intermediate goes through a small ring in L2, not through device memory.
 * workspace: fftso3_grid_fft_workspace_bytes(N, nf) bytes of device memory,
 * 256-byte aligned, zeroed once before first use (its first int is the error
 * word); calls that share a workspace must not overlap on the GPU.  No
 * allocation, so the call may be captured into a CUDA graph.
 * fftso3_grid_fft_check() synchronises `stream` and reports a bounded wait that
 * gave up (FFTSO3_ERR_CUDA); fftso3_grid_fft_reset() clears the error word. */
size_t fftso3_grid_fft_workspace_bytes(int N, long long nf);
int fftso3_grid_fft(int N, long long nf, int dir, int real, const void* in, void* out, void* workspace,
                    void* stream);
int fftso3_grid_fft_check(const void* workspace, void* stream);
int fftso3_grid_fft_reset(void* workspace, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FFTSO3_GB300_H */
