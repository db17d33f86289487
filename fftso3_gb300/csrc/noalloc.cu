// Allocation-free SO(3) forward transform for small bandwidths.
//
// fftso3_forward_noalloc() runs the same FP64 forward transform as an
// FFTSO3_SO3_COMPLEX / FFTSO3_PREC_FP64 / FFTSO3_RECURSION_REFERENCE plan with
// batch 1, but it never allocates device memory: every intermediate (twiddle
// and weight tables, symmetry-group offsets, recursion seeds, the Wigner-d
// table and the FFT work grid) lives in one file-scope __device__ array sized
// for l_max <= FFTSO3_NOALLOC_MAX_LMAX.  That array exists on every GPU that
// loads this library, from module load until the process exits.
//
// Callers for whom this exists: a host that owns all device memory (a
// framework with its own pool, or a plugin host, that does not let libraries
// call cudaMalloc), and latency-critical loops where cudaMalloc / cudaFree
// would synchronise the device or take the allocator's lock.
//
// Set-up: the first call on a device looks up the array's device address with
// cudaGetSymbolAddress (with that device current) and caches it for the life of
// the process, for device ordinals 0..255 (a higher ordinal is rejected); make
// that first call before any stream capture.  cudaDeviceReset() on a device
// destroys its copy of the array, so the cached address is then stale: do not
// call this entry point on a device after resetting it.
//
// The host-computed constants (twiddles, weights, group offsets, recursion
// seeds: about 15 KB) reach the GPU as one __grid_constant__ kernel parameter,
// which needs the large kernel parameters of CUDA 12.1 and later (up to 32,764
// bytes; checked at compile time below) -- no host-to-device copy, so nothing
// to allocate or pin.  Every call shares the one array and
// each call rewrites all of it before reading it (nothing has to start at
// zero), so two calls that overlap on the GPU -- on different streams, or from
// different host threads -- race and corrupt each other's result: serialise
// them.
//
// This translation unit is compiled with -fmad=false like tables.cu, so the
// Wigner-d table is bit-for-bit the plan path's table.
#include <cmath>
#include <mutex>
#include <string>

#include "../../include/fftso3_gb300.h"
#include "common.cuh"
#include "contract.cuh"
#include "fft.cuh"
#include "tables.cuh"
#include "wigner_rec.cuh"

using namespace fftso3;

namespace {

constexpr int NA_LMAX = FFTSO3_NOALLOC_MAX_LMAX;
constexpr int NA_B = NA_LMAX + 1;
constexpr int NA_N = 2 * NA_B;

constexpr long long na_table_elems()
{
    long long t = 0;
    for (int m = 0; m < NA_B; ++m) t += (long long)(2 * m + 1) * (NA_B - m) * NA_N;
    return t;
}

constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }

// scratch sections (bytes)
constexpr size_t OFF_TW = 0;
constexpr size_t OFF_W = align256(OFF_TW + sizeof(double) * 2 * NA_N);
constexpr size_t OFF_GOFF = align256(OFF_W + sizeof(double) * NA_N);
constexpr size_t OFF_SEEDS = align256(OFF_GOFF + sizeof(long long) * (NA_B * NA_B + 1));
constexpr size_t OFF_TABLE = align256(OFF_SEEDS + sizeof(WignerSeeds) * NA_N);
constexpr size_t OFF_WORK = align256(OFF_TABLE + sizeof(double) * na_table_elems());
constexpr size_t SCRATCH_BYTES = align256(OFF_WORK + sizeof(double2) * (size_t)NA_N * NA_N * NA_N);

static __device__ __align__(256) unsigned char g_noalloc_scratch[SCRATCH_BYTES];

std::mutex na_mutex;
void* na_ptr[256] = {};

// Host-computed constants, passed by value (no host-to-device copy).
struct NAParams {
    double tw[2 * NA_N];
    double w[NA_N];
    long long goff[NA_B * NA_B + 1];
    WignerSeeds seeds[NA_N];
};
static_assert(sizeof(NAParams) <= 32764, "NAParams must fit CUDA's 32,764-byte kernel parameter limit");

__global__ void na_setup_kernel(const __grid_constant__ NAParams P, unsigned char* __restrict__ scratch, int L)
{
    const int B = L + 1, N = 2 * B, ng = B * B;
    double* tw = (double*)(scratch + OFF_TW);
    double* w = (double*)(scratch + OFF_W);
    long long* goff = (long long*)(scratch + OFF_GOFF);
    WignerSeeds* seeds = (WignerSeeds*)(scratch + OFF_SEEDS);
    for (int i = threadIdx.x; i < 2 * N; i += blockDim.x) tw[i] = P.tw[i];
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        w[i] = P.w[i];
        seeds[i] = P.seeds[i];
    }
    for (int i = threadIdx.x; i <= ng; i += blockDim.x) goff[i] = P.goff[i];
}

// One thread per (group, k), the reference recursion (fdcl_FFTSO3.cpp:127-194).
__global__ void na_table_kernel(unsigned char* __restrict__ scratch, int L)
{
    const int B = L + 1, N = 2 * B;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B * B * N) return;
    const int g = (int)(idx / N), k = (int)(idx % N);
    const long long* goff = (const long long*)(scratch + OFF_GOFF);
    const WignerSeeds* seeds = (const WignerSeeds*)(scratch + OFF_SEEDS);
    double* table = (double*)(scratch + OFF_TABLE);
    int m0, n0;
    group_mn(g, m0, n0);
    const WignerSeeds s = seeds[k];
    double* out = table + goff[g] + k;
    auto emit = [&](int l, double v) { out[(long long)(l - m0) * N] = v; };
    wigner_column_faithful(m0, n0, L, s, emit);
}

int na_fail(int code, const std::string& m)
{
    set_last_error(m);  // reported by fftso3_last_error_string()
    return code;
}

}  // namespace

extern "C" int fftso3_forward_noalloc(int l_max, const void* grid, void* coeffs, void* stream)
{
    if (l_max < 0) return na_fail(FFTSO3_ERR_INVALID_ARG, "l_max must be >= 0");
    if (l_max > NA_LMAX)
        return na_fail(FFTSO3_ERR_INVALID_ARG, "l_max " + std::to_string(l_max) +
                                                   " exceeds the allocation-free limit FFTSO3_NOALLOC_MAX_LMAX = " +
                                                   std::to_string(NA_LMAX) + "; use a plan instead");
    if (!grid || !coeffs) return na_fail(FFTSO3_ERR_INVALID_ARG, "grid/coeffs pointer is NULL");
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 256)
        return na_fail(FFTSO3_ERR_NO_DEVICE, std::string("no current CUDA device: ") + cudaGetErrorString(e));
    unsigned char* scratch;
    {
        std::lock_guard<std::mutex> lk(na_mutex);
        if (!na_ptr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p)
                return na_fail(FFTSO3_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            na_ptr[dev] = p;
        }
        scratch = (unsigned char*)na_ptr[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    const int B = l_max + 1, N = 2 * B, ng = B * B;

    // host constants, formed exactly as plan creation forms them
    NAParams P;
    for (int i = 0; i < N; ++i) {
        double a = -2. * M_PI * (double)i / (double)N;
        P.tw[2 * i] = cos(a);
        P.tw[2 * i + 1] = sin(a);
    }
    {
        double factor = M_PI / ((double)(4 * B));
        for (int j = 0; j < N; j++) {
            double sum = 0.0;
            for (int k = 0; k < B; k++)
                sum += 1. / ((double)(2 * k + 1)) * sin((double)((2 * j + 1) * (2 * k + 1)) * factor);
            sum *= 1. / ((double)4 * B * B * B) * sin((double)(2 * j + 1) * factor);
            P.w[j] = sum;
        }
    }
    {
        long long o = 0;
        for (int g = 0; g < ng; ++g) {
            int m0, n0;
            group_mn(g, m0, n0);
            P.goff[g] = o;
            o += (long long)(B - m0) * N;
        }
        P.goff[ng] = o;
    }
    for (int k = 0; k < N; ++k) {
        const double beta = ((double)(2 * k + 1)) * M_PI / 4. / ((double)B);
        WignerSeeds& s = P.seeds[k];
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
    }

    na_setup_kernel<<<1, 256, 0, st>>>(P, scratch, l_max);
    if ((e = cudaGetLastError()) != cudaSuccess) return na_fail(FFTSO3_ERR_CUDA, cudaGetErrorString(e));
    {
        const long long tot = (long long)ng * N;
        na_table_kernel<<<(unsigned)((tot + 127) / 128), 128, 0, st>>>(scratch, l_max);
        if ((e = cudaGetLastError()) != cudaSuccess) return na_fail(FFTSO3_ERR_CUDA, cudaGetErrorString(e));
    }
    double2* work = (double2*)(scratch + OFF_WORK);
    FFTFactors fac;
    make_fft_factors(N, fac);
    FFTLaunch R;
    R.in = grid;
    R.out = work;
    R.fac = fac;
    R.nlines = (long long)N * N;
    R.lpb = 4;
    R.inner = 1;
    R.ostride = N;
    R.istride = 0;
    R.es = 1;
    R.tw = scratch + OFF_TW;
    R.fp64 = true;
    R.real_in = false;
    R.real_out = false;
    R.lines_fastest = false;
    if ((e = launch_fft_lines(R, st)) != cudaSuccess) return na_fail(FFTSO3_ERR_CUDA, cudaGetErrorString(e));
    FFTLaunch C = R;
    C.in = work;
    C.lpb = 8;
    C.inner = N;
    C.ostride = (long long)N * N;
    C.istride = 1;
    C.es = N;
    C.lines_fastest = true;
    if ((e = launch_fft_lines(C, st)) != cudaSuccess) return na_fail(FFTSO3_ERR_CUDA, cudaGetErrorString(e));
    e = launch_so3_fwd_fp64((const double*)(scratch + OFF_TABLE), (const long long*)(scratch + OFF_GOFF), work,
                            (const double*)(scratch + OFF_W), (double2*)coeffs, l_max, N, 1, st);
    if (e != cudaSuccess) return na_fail(FFTSO3_ERR_CUDA, cudaGetErrorString(e));
    return FFTSO3_SUCCESS;
}
