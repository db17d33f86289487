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
//   fft_rows_reg  lines contiguous (one axis of a contiguous array);
//   fft_tile      a tile of 16 lines staged in shared memory with one side
//                 contiguous and the other transposed, so a 2-D transform of
//                 the Euler grid is two passes that both read and write whole
//                 128-byte runs, the second one producing the k-contiguous
//                 pencils [fn][p][q][k] the beta-sum GEMM consumes (and the
//                 reverse for the inverse).
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

// Scratch row stride of the line FFT: 32 + P (P = 32 / R), so that step B's
// reads (lane = (k1, h), h < P) fall in distinct banks for each half-warp of
// 8-byte accesses ((32 + P) k1 + h is distinct mod 16).
template <int R>
__host__ __device__ constexpr int scratch_stride() { return 32 + 32 / R; }

// Line FFT through shared memory (far fewer shuffles than warp_fft), in two
// steps on a per-warp scratch line Tl (at least R * scratch_stride<R>() elements):
//   step A: lane t holds x[t + 32 i] (i < R); R-point DFT over i, twiddle
//           w_N^{t k1}, store Y[t][k1] at Tl[k1 * S + t], S = scratch_stride<R>();
//   step B: lane (k1, h) (h < P = 32 / R) loads Y[P s + h][k1] (s < R), R-point
//           DFT over s (index kappa), twiddle w_32^{h kappa}, then a P-point DFT
//           across its P lanes (log2 P shuffle stages).  Register r then holds
//           X[K(r)], K(r) = k1 + R kappa(r) + R^2 brP(h), kappa(r) = brR(r).
template <int R>
__device__ __forceinline__ void line_step_a(float2 (&v)[R], float2* Tl, const float2* __restrict__ W, int lane)
{
    constexpr int N = 32 * R;
    constexpr int LR = ilog2(R);
    reg_dif<R>(v, W, N);
    __syncwarp();
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int k1 = brev(r, LR);
        Tl[k1 * scratch_stride<R>() + lane] = (r == 0) ? v[r] : cmulf(v[r], W[lane * k1]);
    }
    __syncwarp();
}

template <int R>
__device__ __forceinline__ void line_step_b(float2 (&v)[R], const float2* Tl, const float2* __restrict__ W,
                                            int lane)
{
    constexpr int N = 32 * R;
    constexpr int LR = ilog2(R);
    constexpr int P = 32 / R;
    const int k1 = lane / P, h = lane % P;
#pragma unroll
    for (int s2 = 0; s2 < R; ++s2) v[s2] = Tl[k1 * scratch_stride<R>() + P * s2 + h];
    reg_dif<R>(v, W, N);
    if (P > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) {
            const int kappa = brev(r, LR);
            if (h != 0) v[r] = cmulf(v[r], W[(h * kappa) * (N / 32)]);
        }
#pragma unroll
        for (int hh = P / 2; hh >= 1; hh >>= 1) {
            const bool upper = (h & hh) != 0;
            const int kk = h & (hh - 1);
            const float2 w = W[kk * (N / (2 * hh))];
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const float ox = __shfl_xor_sync(FULL, v[r].x, hh);
                const float oy = __shfl_xor_sync(FULL, v[r].y, hh);
                if (!upper) {
                    v[r].x += ox;
                    v[r].y += oy;
                } else {
                    v[r] = cmulf(make_float2(ox - v[r].x, oy - v[r].y), w);
                }
            }
        }
    }
}

template <int R>
__device__ __forceinline__ int line_out_index(int lane, int r)
{
    constexpr int LR = ilog2(R);
    constexpr int P = 32 / R;
    const int k1 = lane / P, h = lane % P;
    return k1 + R * brev(r, LR) + R * R * brev(h, ilog2(P));
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

constexpr int TL = 16;               // lines per CTA tile
constexpr int PWARPS = 8;            // 2 lines per warp

// Padded position of element j in a staged line: one pad slot every R
// elements, plus SH slots every R^2 elements.  The output element K of lane
// (k1, h) in register r is K = k1 + R brR(r) + R^2 brP(h); with
// SH = R/2 - R^2 - R (mod 16) the 16 lanes of a half-warp store to 16
// distinct banks (8-byte elements) for every r.
template <int R>
__host__ __device__ constexpr int pad_sh()
{
    return R >= 32 ? 0 : (((R / 2 - R * R - R) % 16) + 16) % 16;
}
template <int R>
__device__ __forceinline__ int ppos(int j)
{
    return j + (j >> ilog2(R)) + pad_sh<R>() * (j >> (2 * ilog2(R)));
}
// Staged line length: holds every padded position and the line-FFT scratch;
// odd, so the transposed side's pairs of lines (l, l + 1) spread over the banks.
template <int R>
__host__ __device__ constexpr int tile_lp()
{
    constexpr int N = 32 * R;
    constexpr int need = (N - 1) + (N - 1) / R + pad_sh<R>() * ((N - 1) / (R * R)) + 1;
    constexpr int lp = need > R * scratch_stride<R>() ? need : R * scratch_stride<R>();
    return lp | 1;
}

// Geometry of a tiled pass (element offsets).
struct TileGeo {
    long long FS;  // per function (N^3 for SO(3) grids, N^2 for S^2 grids)
    int NO;        // outer index range (N for SO(3), 1 for S^2)
    long long Oc, Ls, Ot, Js;
};

// A tile of TL lines with one side contiguous and the other transposed.
//   contiguous side: line l, element j at  cbase + l * Ls + j
//   transposed side: line l, element j at  tbase + j * Js + l    (TL consecutive l)
// cbase = f FS + o Oc + bb TL Ls,  tbase = f FS + o Ot + bb TL, with the CTA
// index split into (f, o < NO, bb < N / TL).  C2T = true reads the contiguous
// side and writes the transposed one; C2T = false the reverse.  Both sides
// move TL * 8 = 128-byte runs.
// REAL_IO: the contiguous side holds real values (pass 1 reads real samples,
// pass -1 writes the real part only).
template <int R, bool C2T, bool REAL_IO>
__global__ void __launch_bounds__(32 * PWARPS, 3) fft_tile(const float2* __restrict__ in, float2* __restrict__ out,
                                                        const TileGeo g, const double2* __restrict__ tw)
{
    constexpr int N = 32 * R;
    constexpr int LR = ilog2(R);
    constexpr int LP = tile_lp<R>();  // padded staged line
    extern __shared__ float2 smem_f2[];
    float2* Ws = smem_f2;
    float2* T = smem_f2 + N;  // [TL][LP]
    load_twiddles<N>(Ws, tw);

    constexpr int NB = N / TL;
    const long long b = blockIdx.x;
    const long long f = b / ((long long)g.NO * NB);
    const long long o = (b / NB) % g.NO;
    const long long bb = b % NB;
    const long long Ls = g.Ls, Js = g.Js;
    const long long cbase = f * g.FS + o * g.Oc + bb * TL * Ls;
    const long long tbase = f * g.FS + o * g.Ot + bb * TL;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int NV = TL * N / 2 / (32 * PWARPS);  // float4 accesses per thread on the transposed side
    static_assert(TL * N / 2 % (32 * PWARPS) == 0, "tile must split evenly over the threads");
    // REAL_IO: real lines 2p and 2p+1 share one complex transform (staged row p):
    // forward z = x_{2p} + i x_{2p+1}, X = (Z[k] + conj Z[-k]) / 2, Y = (Z[k] - conj Z[-k]) / 2i;
    // inverse z = X_{2p} + i X_{2p+1} (spectra of real lines), lines = Re, Im of its transform.
    constexpr int TLI = REAL_IO ? TL / 2 : TL;  // transforms (staged rows) per tile
    if (C2T) {
        // contiguous input: each warp loads its line(s) straight into registers
        __syncthreads();  // twiddles staged
        for (int row = warp; row < TLI; row += PWARPS) {
            float2* Tl = T + row * LP;
            float2 v[R];
            if (REAL_IO) {
                const float* s0 = reinterpret_cast<const float*>(in) + cbase + (2 * row) * Ls;
                const float* s1 = s0 + Ls;
#pragma unroll
                for (int i = 0; i < R; ++i) v[i] = make_float2(__ldg(s0 + lane + 32 * i), __ldg(s1 + lane + 32 * i));
            } else {
                const float2* src = in + cbase + row * Ls;
#pragma unroll
                for (int i = 0; i < R; ++i) v[i] = __ldg(src + lane + 32 * i);
            }
            line_step_a<R>(v, Tl, Ws, lane);
            line_step_b<R>(v, Tl, Ws, lane);
            __syncwarp();
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int K = line_out_index<R>(lane, r);
                Tl[ppos<R>(K)] = v[r];
            }
        }
        __syncthreads();
        // transposed output: pairs (l, l + 1) of element j as 16-byte stores
        float4* out4 = reinterpret_cast<float4*>(out);
#pragma unroll 4
        for (int u = 0; u < NV; ++u) {
            const int e2 = threadIdx.x + u * 32 * PWARPS;
            const int l = (e2 % (TL / 2)) * 2, j = e2 / (TL / 2);
            float2 a, b;
            if (REAL_IO) {
                const float2 z = T[(l / 2) * LP + ppos<R>(j)];
                const float2 zm = T[(l / 2) * LP + ppos<R>((N - j) & (N - 1))];
                a = make_float2(0.5f * (z.x + zm.x), 0.5f * (z.y - zm.y));
                b = make_float2(0.5f * (z.y + zm.y), -0.5f * (z.x - zm.x));
            } else {
                a = T[l * LP + ppos<R>(j)];
                b = T[(l + 1) * LP + ppos<R>(j)];
            }
            out4[(tbase + (long long)j * Js + l) / 2] = make_float4(a.x, a.y, b.x, b.y);
        }
    } else {
        // transposed input staged through shared memory (16-byte loads, all issued first)
        constexpr int VB = NV < 8 ? NV : 8;
        const float4* in4 = reinterpret_cast<const float4*>(in);
#pragma unroll 1
        for (int u0 = 0; u0 < NV; u0 += VB) {
            float4 buf[VB];
#pragma unroll
            for (int q = 0; q < VB; ++q) {
                const int e2 = threadIdx.x + (u0 + q) * 32 * PWARPS;
                const int l = (e2 % (TL / 2)) * 2, j = e2 / (TL / 2);
                buf[q] = __ldg(in4 + (tbase + (long long)j * Js + l) / 2);
            }
#pragma unroll
            for (int q = 0; q < VB; ++q) {
                const int e2 = threadIdx.x + (u0 + q) * 32 * PWARPS;
                const int l = (e2 % (TL / 2)) * 2, j = e2 / (TL / 2);
                if (REAL_IO) {
                    T[(l / 2) * LP + ppos<R>(j)] = make_float2(buf[q].x - buf[q].w, buf[q].y + buf[q].z);
                } else {
                    T[l * LP + ppos<R>(j)] = make_float2(buf[q].x, buf[q].y);
                    T[(l + 1) * LP + ppos<R>(j)] = make_float2(buf[q].z, buf[q].w);
                }
            }
        }
        __syncthreads();
        // contiguous output straight from registers: runs of R consecutive outputs per lane group
        for (int row = warp; row < TLI; row += PWARPS) {
            float2* Tl = T + row * LP;
            float2 v[R];
#pragma unroll
            for (int i = 0; i < R; ++i) v[i] = Tl[ppos<R>(lane + 32 * i)];
            line_step_a<R>(v, Tl, Ws, lane);
            line_step_b<R>(v, Tl, Ws, lane);
            if (REAL_IO) {
                float* d0 = reinterpret_cast<float*>(out) + cbase + (2 * row) * Ls;
                float* d1 = d0 + Ls;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const int K = line_out_index<R>(lane, r);
                    d0[K] = v[r].x;
                    d1[K] = v[r].y;
                }
            } else {
                float2* dst = out + cbase + row * Ls;
#pragma unroll
                for (int r = 0; r < R; ++r) dst[line_out_index<R>(lane, r)] = v[r];
            }
        }
    }
}

template <int R, bool C2T, bool REAL_IO>
static cudaError_t tile_r(const void* in, void* out, long long nf, const TileGeo& g, const void* tw, cudaStream_t st)
{
    constexpr int N = 32 * R;
    constexpr int LP = tile_lp<R>();
    constexpr int TLI = REAL_IO ? TL / 2 : TL;  // staged rows (real lines go in pairs)
    const size_t smem = sizeof(float2) * ((size_t)N + (size_t)TLI * LP);
    auto k = fft_tile<R, C2T, REAL_IO>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const long long nblk = nf * (long long)g.NO * (N / TL);
    k<<<(unsigned)nblk, 32 * PWARPS, smem, st>>>((const float2*)in, (float2*)out, g, (const double2*)tw);
    return cudaGetLastError();
}

template <bool C2T, bool REAL_IO>
static cudaError_t tile_dispatch(const void* in, void* out, long long nf, int N, const TileGeo& g, const void* tw,
                                 cudaStream_t st)
{
    switch (N) {
        case 64: return tile_r<2, C2T, REAL_IO>(in, out, nf, g, tw, st);
        case 128: return tile_r<4, C2T, REAL_IO>(in, out, nf, g, tw, st);
        case 256: return tile_r<8, C2T, REAL_IO>(in, out, nf, g, tw, st);
        case 512: return tile_r<16, C2T, REAL_IO>(in, out, nf, g, tw, st);
        case 1024: return tile_r<32, C2T, REAL_IO>(in, out, nf, g, tw, st);
        default: return cudaErrorNotSupported;
    }
}

template <bool C2T>
static cudaError_t tile_any(const void* in, void* out, long long nf, int N, const TileGeo& g, const void* tw,
                            cudaStream_t st, bool real_io)
{
    return real_io ? tile_dispatch<C2T, true>(in, out, nf, N, g, tw, st)
                   : tile_dispatch<C2T, false>(in, out, nf, N, g, tw, st);
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

// Forward passes of one batch of N^3 grids (see fft.cuh):
//   pass 1: grid [f][k][j1][j2] -> FFT over j2 -> T1 [f][k][q][j1]
//   pass 2: T1 [f][k][q][j1]    -> FFT over j1 -> pencils [f][p][q][k]
// Inverse passes:
//   pass 2': pencils [f][p][q][k] -> FFT over p  -> T1 [f][k][q][j1]
//   pass 1': T1 [f][k][q][j1]     -> FFT over q  -> grid [f][k][j1][j2]
cudaError_t launch_fft_grid_pass(const void* in, void* out, long long nf, int N, int pass, const void* tw,
                                 cudaStream_t st, bool real_io)
{
    const long long N1 = N, N2 = (long long)N * N, N3 = N2 * N;
    if (real_io && pass != 1 && pass != -1) return cudaErrorInvalidValue;
    const ffast::TileGeo g1{N3, N, N2, N1, N2, N1};  // lines along j2 / q, transposed (q, j1)
    const ffast::TileGeo g2{N3, N, N1, N2, N1, N2};  // lines along j1 / p, transposed (p.., k)
    switch (pass) {
        case 1: return ffast::tile_any<true>(in, out, nf, N, g1, tw, st, real_io);
        case 2: return ffast::tile_any<true>(in, out, nf, N, g2, tw, st, false);
        case -2: return ffast::tile_any<false>(in, out, nf, N, g2, tw, st, false);
        case -1: return ffast::tile_any<false>(in, out, nf, N, g1, tw, st, real_io);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_fft_s2_pass(const void* in, void* out, long long nf, int N, int dir, const void* tw,
                               cudaStream_t st, bool real_io)
{
    const long long N1 = N, N2 = (long long)N * N;
    const ffast::TileGeo g{N2, 1, 0, N1, 0, N1};  // lines along j (contiguous), transposed [p][k]
    if (dir == 1) return ffast::tile_any<true>(in, out, nf, N, g, tw, st, real_io);
    if (dir == -1) return ffast::tile_any<false>(in, out, nf, N, g, tw, st, real_io);
    return cudaErrorInvalidValue;
}

}  // namespace fftso3
