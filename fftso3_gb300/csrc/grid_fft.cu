// The two-dimensional grid FFT stage of the tensor-core SO(3) transforms as
// its own C entry point (declared in include/fftso3_gb300.h): the one-launch
// transposing FFT (fft_grid2d, fft_fast.cu) over caller buffers and a caller
// workspace, with no allocation.
//
// The reference runs this stage inside its forward transforms (Eigen FFTs of
// the rows and then the columns of each beta slice, fdcl_FFTSO3.cpp:689-699
// complex, :805-815 real); the inverse here uses the same transform to
// synthesise whole grids.  Exposed so that callers (and the tests) can use and
// check it alone.
#include <cmath>
#include <string>
#include <vector>

#include "../../include/fftso3_gb300.h"
#include "common.cuh"
#include "fft.cuh"

using namespace fftso3;

namespace {

constexpr size_t ALIGN = 256;
size_t up(size_t x) { return (x + ALIGN - 1) / ALIGN * ALIGN; }

// workspace: [error word][twiddles N double2][control ints][ring]
struct WsLayout {
    size_t tw, ctl, ring, total, ring_elems;
};

WsLayout layout(int N, long long nf)
{
    WsLayout w;
    w.tw = ALIGN;
    w.ctl = w.tw + up(sizeof(double) * 2 * N);
    w.ring = w.ctl + up(sizeof(int) * fft_grid_fused_ctl_ints(nf, N));
    w.ring_elems = fft_grid_fused_ring_elems(N);
    w.total = w.ring + sizeof(float) * 2 * w.ring_elems;
    return w;
}

int gfail(int code, const std::string& m)
{
    set_last_error(m);
    return code;
}

}  // namespace

extern "C" {

size_t fftso3_grid_fft_workspace_bytes(int N, long long nf)
{
    if (!fft_grid_fused_supported(N) || nf < 1) return 0;
    return layout(N, nf).total;
}

int fftso3_grid_fft(int N, long long nf, int dir, int real, const void* in, void* out, void* workspace,
                    void* stream)
{
    if (!fft_grid_fused_supported(N)) return gfail(FFTSO3_ERR_INVALID_ARG, "grid FFT: N must be 64, 128, 256 or 512");
    if (nf < 1 || (long long)nf * (N / 16) > (1LL << 29) / N)
        return gfail(FFTSO3_ERR_INVALID_ARG, "grid FFT: bad number of grids");
    if (dir != 1 && dir != -1) return gfail(FFTSO3_ERR_INVALID_ARG, "grid FFT: dir must be 1 or -1");
    if (!in || !out || !workspace || in == out)
        return gfail(FFTSO3_ERR_INVALID_ARG, "grid FFT: null buffer, or in == out");
    if ((uintptr_t)workspace % ALIGN || (uintptr_t)in % 16 || (uintptr_t)out % 16)
        return gfail(FFTSO3_ERR_INVALID_ARG, "grid FFT: workspace must be 256-byte aligned, buffers 16-byte aligned");
    const WsLayout w = layout(N, nf);
    cudaStream_t st = (cudaStream_t)stream;
    char* ws = (char*)workspace;
    std::vector<double> tw(2 * N);
    for (int i = 0; i < N; ++i) {
        const double a = -2. * M_PI * (double)i / (double)N;
        tw[2 * i] = cos(a);
        tw[2 * i + 1] = sin(a);
    }
    cudaError_t e = cudaMemcpyAsync(ws + w.tw, tw.data(), sizeof(double) * 2 * N, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = launch_fft_grid_fused(in, out, ws + w.ring, w.ring_elems, (int*)(ws + w.ctl), (int*)ws, nf, N, dir,
                                  ws + w.tw, st, real != 0);
    if (e != cudaSuccess) return gfail(FFTSO3_ERR_CUDA, std::string("grid FFT: ") + cudaGetErrorString(e));
    return FFTSO3_SUCCESS;
}

int fftso3_grid_fft_check(const void* workspace, void* stream)
{
    if (!workspace) return gfail(FFTSO3_ERR_INVALID_ARG, "grid FFT check: null workspace");
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, workspace, sizeof(int), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return gfail(FFTSO3_ERR_CUDA, std::string("grid FFT check: ") + cudaGetErrorString(e));
    if (h != 0)
        return gfail(FFTSO3_ERR_CUDA, "grid FFT: a wait on another tile gave up (code " + std::to_string(h) + ")");
    return FFTSO3_SUCCESS;
}

int fftso3_grid_fft_reset(void* workspace, void* stream)
{
    if (!workspace) return gfail(FFTSO3_ERR_INVALID_ARG, "grid FFT reset: null workspace");
    cudaError_t e = cudaMemsetAsync(workspace, 0, sizeof(int), (cudaStream_t)stream);
    if (e != cudaSuccess) return gfail(FFTSO3_ERR_CUDA, std::string("grid FFT reset: ") + cudaGetErrorString(e));
    return FFTSO3_SUCCESS;
}

}  // extern "C"
