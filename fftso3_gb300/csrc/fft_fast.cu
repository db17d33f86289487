// Register-resident FP32 FFT kernels for the tensor-core path, N = 32 R
// (R = 2..32, i.e. N = 64..1024, powers of two).
//
// One warp transforms one line of N points: lane t holds x[t + 32 i],
// i < R.  With n = t + 32 i and K = k1 + R k2,
//   X[K] = sum_t w_N^{t k1} w_32^{t k2} sum_i x[t + 32 i] w_R^{i k1},
// so each lane runs an R-point radix-2 DIF in registers, multiplies by the
// twiddles w_N^{t k1}, and the warp finishes with a 32-point radix-2 DIF across
// lanes (shuffles).  Lane t then holds X[brR(r) + R br5(t)] in register r,
// i.e. R consecutive outputs.  Twiddles come from the host FP64 table
// W[j] = e^{-2 pi i j / N}, staged in shared memory as FP32.
//
// Kernels:
//   fft_rows_reg      lines contiguous (the gamma / q axis), in place or not;
//   fft_pencil_fwd    the alpha axis of [fn][k][j1][q] with the result written
//                     as k-contiguous pencils [fn][p][q][k] (column FFT fused
//                     with the transpose the beta-sum GEMM wants);
//   fft_pencil_inv    the reverse: pencils [fn][p][q][k] -> FFT over p ->
//                     [fn][k][j1][q].
// The pencil kernels stage a tile of KT x QT lines (4 beta indices x 4 columns)
// in shared memory so that both the line reads and the pencil writes move
// whole 32-byte sectors.
#include "common.cuh"
#include "fft.cuh"

namespace fftso3 {

namespace ffast {

constexpr unsigned FULL = 0xffffffffu;

__host__ __device__ constexpr int brev(int x, int bits)
{
    int r = 0;
    for (int b = 0; b < bits; ++b) r |= ((x >> b) & 1) << (bits - 1 - b);
    return r;
}

__host__ __device__ constexpr int ilog2(int x) { return x <= 1 ? 0 : 1 + ilog2(x >> 1); }

__device__ __forceinline__ float2 cmulf(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// R-point radix-2 DIF in registers (natural input, bit-reversed output).
template <int R>
__device__ __forceinline__ void reg_dif(float2 (&v)[R], const float2* __restrict__ W, int N)
{
#pragma unroll
    for (int h = R / 2; h >= 1; h >>= 1) {
#pragma unroll
        for (int j = 0; j < R; j += 2 * h) {
#pragma unroll
            for (int k = 0; k < h; ++k) {
                const float2 a = v[j + k], b = v[j + k + h];
                v[j + k] = make_float2(a.x + b.x, a.y + b.y);
                const float2 d = make_float2(a.x - b.x, a.y - b.y);
                if (k == 0)
                    v[j + k + h] = d;
                else if (4 * k == 2 * h)
                    v[j + k + h] = make_float2(d.y, -d.x);  // w = -i
                else
                    v[j + k + h] = cmulf(d, W[k * (N / (2 * h))]);
            }
        }
    }
}

// Full N = 32 R point FFT of the line held by the warp (see the file comment).
template <int R>
__device__ __forceinline__ void warp_fft(float2 (&v)[R], const float2* __restrict__ W, int lane)
{
    constexpr int N = 32 * R;
    constexpr int LR = ilog2(R);
    reg_dif<R>(v, W, N);
#pragma unroll
    for (int r = 1; r < R; ++r) {
        const int k1 = brev(r, LR);
        v[r] = cmulf(v[r], W[lane * k1]);
    }
#pragma unroll
    for (int h = 16; h >= 1; h >>= 1) {
        const bool upper = (lane & h) != 0;
        const int kk = lane & (h - 1);
        const float2 w = W[kk * (N / (2 * h))];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const float ox = __shfl_xor_sync(FULL, v[r].x, h);
            const float oy = __shfl_xor_sync(FULL, v[r].y, h);
            if (!upper) {
                v[r].x += ox;
                v[r].y += oy;
            } else {
                v[r] = cmulf(make_float2(ox - v[r].x, oy - v[r].y), w);
            }
        }
    }
}

template <int N>
__device__ __forceinline__ void load_twiddles(float2* Ws, const double2* __restrict__ tw)
{
    for (int i = threadIdx.x; i < N; i += blockDim.x) Ws[i] = make_float2((float)tw[i].x, (float)tw[i].y);
}

// Contiguous lines: in[line * N + j] -> out[line * N + K].
template <int R, int WPB, int LPW>
__global__ void __launch_bounds__(32 * WPB) fft_rows_reg(const float2* __restrict__ in, float2* __restrict__ out,
                                                         long long nlines, const double2* __restrict__ tw)
{
    constexpr int N = 32 * R;
    constexpr int LR = ilog2(R);
    __shared__ float2 Ws[N];
    load_twiddles<N>(Ws, tw);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t5 = brev(lane, 5);
    for (int u = 0; u < LPW; ++u) {
        const long long line = ((long long)blockIdx.x * LPW + u) * WPB + warp;
        if (line >= nlines) return;
        const float2* src = in + line * N;
        float2 v[R];
#pragma unroll
        for (int i = 0; i < R; ++i) v[i] = src[lane + 32 * i];
        warp_fft<R>(v, Ws, lane);
        float2* dst = out + line * N + R * t5;
#pragma unroll
        for (int k1 = 0; k1 < R; k1 += 2) {
            const float2 a = v[brev(k1, LR)], b = v[brev(k1 + 1, LR)];
            reinterpret_cast<float4*>(dst)[k1 / 2] = make_float4(a.x, a.y, b.x, b.y);
        }
    }
}

constexpr int KT = 4, QT = 4;        // tile: 4 beta indices x 4 columns = 16 lines
constexpr int PWARPS = 8;            // 2 lines per warp

// padded position of element j in a staged line (one pad slot every R elements)
template <int R>
__device__ __forceinline__ int ppos(int j) { return j + (j >> ilog2(R)); }

// FORWARD = true : in [fn][k][j1][q]  -> FFT over j1 -> out pencils [fn][p][q][k]
// FORWARD = false: in pencils [fn][p][q][k] -> FFT over p -> out [fn][k][j1][q]
template <int R, bool FORWARD>
__global__ void __launch_bounds__(32 * PWARPS) fft_pencil(const float2* __restrict__ in, float2* __restrict__ out,
                                                          long long nf, const double2* __restrict__ tw)
{
    constexpr int N = 32 * R;
    constexpr int LR = ilog2(R);
    constexpr int LP = N + N / R + 1;  // padded staged line
    extern __shared__ float2 smem_f2[];
    float2* Ws = smem_f2;
    float2* T = smem_f2 + N;  // [KT * QT][LP]
    load_twiddles<N>(Ws, tw);

    const long long ntk = N / KT, ntq = N / QT;
    const long long b = blockIdx.x;
    const long long f = b / (ntk * ntq);
    const int k0 = (int)((b / ntq) % ntk) * KT;
    const int q0 = (int)(b % ntq) * QT;
    const long long NN = (long long)N * N;
    const float2* src = in + f * NN * N;
    float2* dst = out + f * NN * N;
    constexpr int NL = KT * QT;
    // load: line = kt * QT + qt
    for (int e = threadIdx.x; e < NL * N; e += blockDim.x) {
        int j, kt, qt;
        long long off;
        if (FORWARD) {  // q fastest, then j1, then k: runs of QT columns
            qt = e % QT;
            j = (e / QT) % N;
            kt = e / (QT * N);
            off = (long long)(k0 + kt) * NN + (long long)j * N + (q0 + qt);
        } else {        // k fastest, then q, then p: runs of KT beta indices
            kt = e % KT;
            qt = (e / KT) % QT;
            j = e / (KT * QT);
            off = (long long)j * NN + (long long)(q0 + qt) * N + (k0 + kt);
        }
        T[(kt * QT + qt) * LP + ppos<R>(j)] = src[off];
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t5 = brev(lane, 5);
    for (int line = warp; line < NL; line += PWARPS) {
        float2* Tl = T + line * LP;
        float2 v[R];
#pragma unroll
        for (int i = 0; i < R; ++i) v[i] = Tl[ppos<R>(lane + 32 * i)];
        warp_fft<R>(v, Ws, lane);
        __syncwarp();
#pragma unroll
        for (int k1 = 0; k1 < R; ++k1) Tl[ppos<R>(k1 + R * t5)] = v[brev(k1, LR)];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < NL * N; e += blockDim.x) {
        int j, kt, qt;
        long long off;
        if (FORWARD) {  // pencils: k fastest, then q, then p
            kt = e % KT;
            qt = (e / KT) % QT;
            j = e / (KT * QT);
            off = (long long)j * NN + (long long)(q0 + qt) * N + (k0 + kt);
        } else {        // rows: q fastest, then j1, then k
            qt = e % QT;
            j = (e / QT) % N;
            kt = e / (QT * N);
            off = (long long)(k0 + kt) * NN + (long long)j * N + (q0 + qt);
        }
        dst[off] = T[(kt * QT + qt) * LP + ppos<R>(j)];
    }
}

template <int R>
static cudaError_t rows_r(const void* in, void* out, long long nlines, const void* tw, cudaStream_t st)
{
    constexpr int WPB = 8, LPW = 4;
    const long long per = (long long)WPB * LPW;
    fft_rows_reg<R, WPB, LPW><<<(unsigned)((nlines + per - 1) / per), 32 * WPB, 0, st>>>(
        (const float2*)in, (float2*)out, nlines, (const double2*)tw);
    return cudaGetLastError();
}

template <int R, bool FWD>
static cudaError_t pencil_r(const void* in, void* out, long long nf, const void* tw, cudaStream_t st)
{
    constexpr int N = 32 * R;
    constexpr int LP = N + N / R + 1;
    const size_t smem = sizeof(float2) * ((size_t)N + (size_t)KT * QT * LP);
    auto k = fft_pencil<R, FWD>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const long long nblk = nf * (N / KT) * (N / QT);
    k<<<(unsigned)nblk, 32 * PWARPS, smem, st>>>((const float2*)in, (float2*)out, nf, (const double2*)tw);
    return cudaGetLastError();
}

}  // namespace ffast

bool fft_fast_supported(int N) { return N == 64 || N == 128 || N == 256 || N == 512 || N == 1024; }

cudaError_t launch_fft_rows_fast(const void* in, void* out, long long nlines, int N, const void* tw, cudaStream_t st)
{
    switch (N) {
        case 64: return ffast::rows_r<2>(in, out, nlines, tw, st);
        case 128: return ffast::rows_r<4>(in, out, nlines, tw, st);
        case 256: return ffast::rows_r<8>(in, out, nlines, tw, st);
        case 512: return ffast::rows_r<16>(in, out, nlines, tw, st);
        case 1024: return ffast::rows_r<32>(in, out, nlines, tw, st);
        default: return cudaErrorNotSupported;
    }
}

cudaError_t launch_fft_pencil(const void* in, void* out, long long nf, int N, bool forward, const void* tw,
                              cudaStream_t st)
{
    switch (N) {
        case 64: return forward ? ffast::pencil_r<2, true>(in, out, nf, tw, st) : ffast::pencil_r<2, false>(in, out, nf, tw, st);
        case 128: return forward ? ffast::pencil_r<4, true>(in, out, nf, tw, st) : ffast::pencil_r<4, false>(in, out, nf, tw, st);
        case 256: return forward ? ffast::pencil_r<8, true>(in, out, nf, tw, st) : ffast::pencil_r<8, false>(in, out, nf, tw, st);
        case 512: return forward ? ffast::pencil_r<16, true>(in, out, nf, tw, st) : ffast::pencil_r<16, false>(in, out, nf, tw, st);
        case 1024: return forward ? ffast::pencil_r<32, true>(in, out, nf, tw, st) : ffast::pencil_r<32, false>(in, out, nf, tw, st);
        default: return cudaErrorNotSupported;
    }
}

}  // namespace fftso3
