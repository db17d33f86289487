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
#include <algorithm>
#include <cstdlib>

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

// R-point radix-2 DIF in registers (natural input, bit-reversed output);
// tw(k, h) = e^{-2 pi i k / (2h)}, the twiddle of butterfly k of the stage of span h.
template <int R, typename TW>
__device__ __forceinline__ void reg_dif_t(float2 (&v)[R], TW tw)
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
                    v[j + k + h] = cmulf(d, tw(k, h));
            }
        }
    }
}

// ... with the full table W[j] = e^{-2 pi i j / N}
template <int R>
__device__ __forceinline__ void reg_dif(float2 (&v)[R], const float2* __restrict__ W, int N)
{
    reg_dif_t<R>(v, [&](int k, int h) { return W[k * (N / (2 * h))]; });
}

// Twiddles of the tile kernels in shared memory, laid out for their accesses:
//   Wa[k1 * 32 + t] = w_N^{t k1}  (t < 32, k1 < R): step A's per-lane twiddles, consecutive
//                                 lanes on consecutive entries (free of bank conflicts);
//   W32[x] = w_N^{R x} = w_32^x   (x < 32, at Wa + N): every other twiddle of the line FFT
//                                 (warp-uniform, or two values per warp: broadcast reads).
template <int R>
__host__ __device__ constexpr int tile_tw_elems() { return 32 * R + 32; }
template <int R>
__device__ __forceinline__ void load_tile_twiddles(float2* Wt, const double2* __restrict__ tw)
{
    constexpr int N = 32 * R;
    for (int i = threadIdx.x; i < N + 32; i += blockDim.x) {
        const int j = i < N ? (i & 31) * (i >> 5) : (i - N) * R;
        Wt[i] = make_float2((float)tw[j].x, (float)tw[j].y);
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
// Wt: tile twiddles (load_tile_twiddles).
template <int R>
__device__ __forceinline__ void line_step_a(float2 (&v)[R], float2* Tl, const float2* __restrict__ Wt, int lane)
{
    constexpr int N = 32 * R;
    constexpr int LR = ilog2(R);
    const float2* W32 = Wt + N;
    reg_dif_t<R>(v, [&](int k, int h) { return W32[16 * k / h]; });
    __syncwarp();
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int k1 = brev(r, LR);
        Tl[k1 * scratch_stride<R>() + lane] = (r == 0) ? v[r] : cmulf(v[r], Wt[k1 * 32 + lane]);
    }
    __syncwarp();
}

template <int R>
__device__ __forceinline__ void line_step_b(float2 (&v)[R], const float2* Tl, const float2* __restrict__ Wt,
                                            int lane)
{
    constexpr int N = 32 * R;
    constexpr int LR = ilog2(R);
    constexpr int P = 32 / R;
    const float2* W32 = Wt + N;
    const int k1 = lane / P, h = lane % P;
#pragma unroll
    for (int s2 = 0; s2 < R; ++s2) v[s2] = Tl[k1 * scratch_stride<R>() + P * s2 + h];
    reg_dif_t<R>(v, [&](int k, int hs) { return W32[16 * k / hs]; });
    if (P > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) {
            const int kappa = brev(r, LR);
            if (h != 0) v[r] = cmulf(v[r], W32[h * kappa]);
        }
#pragma unroll
        for (int hh = P / 2; hh >= 1; hh >>= 1) {
            const bool upper = (h & hh) != 0;
            const int kk = h & (hh - 1);
            const float2 w = W32[16 * kk / hh];
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

// Padded position of element j in a staged line:
//   ppos(j) = j + PA floor(j / R) + PB floor(j / R^2).
// The accesses to a staged line are the step-B stores of lane (k1, h) into
// K = k1 + R brR(r) + R^2 brP(h), the row loads of element lane + 32 i, and the
// transposed side's reads / writes of element j of 8 (real) or 16 (complex)
// lines.  (PA, PB) = (1, R/2 - R^2 - R mod 16) for R >= 16 and (0, R/2) for
// R = 4, 8 make every half-warp of 8-byte accesses touch 16 distinct banks
// (R = 2: (0, 1), the row loads 2-way); checked for every R by a bank model on
// the CPU.
template <int R>
__host__ __device__ constexpr int pad_a() { return R >= 16 ? 1 : 0; }
template <int R>
__host__ __device__ constexpr int pad_b()
{
    return R >= 32 ? 0 : R >= 16 ? (((R / 2 - R * R - R) % 16) + 16) % 16 : R >= 4 ? R / 2 : 1;
}
template <int R>
__host__ __device__ constexpr int ppos(int j)
{
    return j + pad_a<R>() * (j >> ilog2(R)) + pad_b<R>() * (j >> (2 * ilog2(R)));
}
// Staged line length: holds every padded position and the line-FFT scratch.
// Complex tiles stage 16 lines read in pairs (l, l + 1): odd, so the pairs
// spread over the banks.  Real tiles stage 8 lines (one per real pair), each
// read by two lanes per element: = 2 (mod 16).
template <int R, bool REAL>
__host__ __device__ constexpr int tile_lp()
{
    constexpr int N = 32 * R;
    constexpr int need = ppos<R>(N - 1) + 1;
    constexpr int lp = need > R * scratch_stride<R>() ? need : R * scratch_stride<R>();
    return REAL ? ((lp + 13) / 16) * 16 + 2 : (lp | 1);
}

// Geometry of a tiled pass (element offsets).
struct TileGeo {
    long long FS;  // per function (N^3 for SO(3) grids, N^2 for S^2 grids)
    int NO;        // outer index range (N for SO(3), 1 for S^2)
    long long Oc, Ls, Ot, Js;
};

// Global-memory access modes of a tile's two sides.
//   IO_PLAIN:   read-only loads through the texture path, plain stores (one pass per launch);
//   IO_STREAM:  data touched once (grid, pencils): loads and stores marked first for L2 eviction;
//   IO_SCRATCH: the L2-resident ring between the two passes of a fused launch: stores marked last
//               for eviction, loads coherent at L2 (other CTAs of the same launch wrote them).
enum { IO_PLAIN = 0, IO_STREAM = 1, IO_SCRATCH = 2 };

__device__ __forceinline__ uint64_t l2_policy_first()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ uint64_t l2_policy_last()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}

template <int M>
__device__ __forceinline__ float ld1(const float* p, uint64_t pol)
{
    if constexpr (M == IO_PLAIN) return __ldg(p);
    else if constexpr (M == IO_SCRATCH) return __ldcg(p);
    else {
        float v;
        asm volatile("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol));
        return v;
    }
}
template <int M>
__device__ __forceinline__ float2 ld2(const float2* p, uint64_t pol)
{
    if constexpr (M == IO_PLAIN) return __ldg(p);
    else if constexpr (M == IO_SCRATCH) return __ldcg(p);
    else {
        float2 v;
        asm volatile("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(v.x), "=f"(v.y) : "l"(p), "l"(pol));
        return v;
    }
}
template <int M>
__device__ __forceinline__ float4 ld4(const float4* p, uint64_t pol)
{
    if constexpr (M == IO_PLAIN) return __ldg(p);
    else if constexpr (M == IO_SCRATCH) return __ldcg(p);
    else {
        float4 v;
        asm volatile("ld.global.nc.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
                     : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                     : "l"(p), "l"(pol));
        return v;
    }
}
template <int M>
__device__ __forceinline__ void st1(float* p, float v, uint64_t pol)
{
    if constexpr (M == IO_PLAIN) *p = v;
    else asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(p), "f"(v), "l"(pol) : "memory");
}
template <int M>
__device__ __forceinline__ void st2(float2* p, float2 v, uint64_t pol)
{
    if constexpr (M == IO_PLAIN) *p = v;
    else asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(p), "f"(v.x), "f"(v.y), "l"(pol)
                      : "memory");
}
template <int M>
__device__ __forceinline__ void st4(float4* p, float4 v, uint64_t pol)
{
    if constexpr (M == IO_PLAIN) *p = v;
    else asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p), "f"(v.x), "f"(v.y),
                      "f"(v.z), "f"(v.w), "l"(pol)
                      : "memory");
}
// Drop one 128-byte line from L2 without writing it back (its data is dead).
__device__ __forceinline__ void l2_discard(const void* p)
{
    asm volatile("discard.global.L2 [%0], 128;" ::"l"(p) : "memory");
}

// A tile of TL lines with one side contiguous and the other transposed.
//   contiguous side: line l, element j at  cbase + l * Ls + j
//   transposed side: line l, element j at  tbase + j * Js + l    (TL consecutive l)
// C2T = true reads the contiguous side and writes the transposed one; C2T =
// false the reverse.  Both sides move TL * 8 = 128-byte runs.
// REAL_IO: the contiguous side holds real values (pass 1 reads real samples,
// pass -1 writes the real part only).  IN / OUT: access modes (IO_*) of the
// side read and the side written; an IO_SCRATCH input is dropped from L2
// once the tile holds it (every line of the ring is read by exactly one tile).
// T: staged tile [TL][LP] in shared memory; Ws: twiddles (staged, synchronised).
// mid(): run by every thread right after the barrier between the two halves of
// the tile (the input is consumed, no output written yet).
template <int R, bool C2T, bool REAL_IO, int IN, int OUT, typename MID>
__device__ __forceinline__ void tile_body(const float2* __restrict__ in, float2* __restrict__ out, long long cbase,
                                          long long tbase, long long Ls, long long Js, float2* T,
                                          const float2* Ws, uint64_t pol_in, uint64_t pol_out, MID mid)
{
    constexpr int N = 32 * R;
    constexpr int LP = tile_lp<R, REAL_IO>();  // padded staged line
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int NV = TL * N / 2 / (32 * PWARPS);  // float4 accesses per thread on the transposed side
    static_assert(TL * N / 2 % (32 * PWARPS) == 0, "tile must split evenly over the threads");
    static_assert(!(REAL_IO && IN == IO_SCRATCH && C2T), "the ring holds complex lines");
    // REAL_IO: real lines 2p and 2p+1 share one complex transform (staged row p):
    // forward z = x_{2p} + i x_{2p+1}, X = (Z[k] + conj Z[-k]) / 2, Y = (Z[k] - conj Z[-k]) / 2i;
    // inverse z = X_{2p} + i X_{2p+1} (spectra of real lines), lines = Re, Im of its transform.
    constexpr int TLI = REAL_IO ? TL / 2 : TL;  // transforms (staged rows) per tile
    if (C2T) {
        // contiguous input: each warp loads its line(s) straight into registers
        for (int row = warp; row < TLI; row += PWARPS) {
            float2* Tl = T + row * LP;
            float2 v[R];
            if (REAL_IO) {
                const float* s0 = reinterpret_cast<const float*>(in) + cbase + (2 * row) * Ls;
                const float* s1 = s0 + Ls;
#pragma unroll
                for (int i = 0; i < R; ++i)
                    v[i] = make_float2(ld1<IN>(s0 + lane + 32 * i, pol_in), ld1<IN>(s1 + lane + 32 * i, pol_in));
            } else {
                const float2* src = in + cbase + row * Ls;
#pragma unroll
                for (int i = 0; i < R; ++i) v[i] = ld2<IN>(src + lane + 32 * i, pol_in);
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
        mid();
        if (IN == IO_SCRATCH)
            for (int i = threadIdx.x; i < TL * (N / 16); i += 32 * PWARPS)
                l2_discard(in + cbase + (long long)(i / (N / 16)) * Ls + (i % (N / 16)) * 16);
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
            st4<OUT>(out4 + (tbase + (long long)j * Js + l) / 2, make_float4(a.x, a.y, b.x, b.y), pol_out);
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
                buf[q] = ld4<IN>(in4 + (tbase + (long long)j * Js + l) / 2, pol_in);
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
        mid();
        if (IN == IO_SCRATCH)
            for (int j = threadIdx.x; j < N; j += 32 * PWARPS) l2_discard(in + tbase + (long long)j * Js);
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
                    st1<OUT>(d0 + K, v[r].x, pol_out);
                    st1<OUT>(d1 + K, v[r].y, pol_out);
                }
            } else {
                float2* dst = out + cbase + row * Ls;
#pragma unroll
                for (int r = 0; r < R; ++r) st2<OUT>(dst + line_out_index<R>(lane, r), v[r], pol_out);
            }
        }
    }
}

// One pass over nf functions: the CTA index splits into (f, o < NO, bb < N / TL),
// cbase = f FS + o Oc + bb TL Ls, tbase = f FS + o Ot + bb TL.
template <int R, bool C2T, bool REAL_IO>
__global__ void __launch_bounds__(32 * PWARPS, 3) fft_tile(const float2* __restrict__ in, float2* __restrict__ out,
                                                        const TileGeo g, const double2* __restrict__ tw)
{
    constexpr int N = 32 * R;
    extern __shared__ float2 smem_f2[];
    float2* Ws = smem_f2;
    float2* T = smem_f2 + tile_tw_elems<R>();  // [TL][LP]
    load_tile_twiddles<R>(Ws, tw);
    constexpr int NB = N / TL;
    const long long b = blockIdx.x;
    const long long f = b / ((long long)g.NO * NB);
    const long long o = (b / NB) % g.NO;
    const long long bb = b % NB;
    const long long cbase = f * g.FS + o * g.Oc + bb * TL * g.Ls;
    const long long tbase = f * g.FS + o * g.Ot + bb * TL;
    __syncthreads();  // twiddles staged
    tile_body<R, C2T, REAL_IO, IO_PLAIN, IO_PLAIN>(in, out, cbase, tbase, g.Ls, g.Js, T, Ws, 0, 0, [] {});
}

// ---------------------------------------------------------------------------
// Both passes of one direction of the SO(3) grid transform in one persistent
// launch, with the intermediate held in an L2-resident ring instead of a
// full-size work grid.
//
// The batch splits into chunks c = (f, kb): the TL consecutive beta slices
// k = kb TL + kl of function f.  Phase A of a chunk is the first pass over
// those slices into ring slot c mod S (N tiles), phase B the second pass out
// of the slot (N tiles):
//   forward  A: grid slice rows  -> FFT over j2 -> slot [kl][q][j1]       (tile = (kl, bb))
//            B: slot rows (kl, q) -> FFT over j1 -> pencils [f][p][q][kb TL + kl] (tile = q)
//   inverse  A: pencils            -> FFT over p  -> slot [kl][q][j1]     (tile = q)
//            B: slot              -> FFT over q  -> grid slice rows       (tile = (kl, bb))
// Every phase-B tile needs every phase-A tile of its chunk (a transpose), and
// phase A of chunk c reuses the slot of chunk c - S.  CTAs claim tiles from
// one atomic counter in the order (blocks of N tiles, lookahead D)
//   A(0), ..., A(D-1), A(D), B(0), A(D+1), B(1), ..., B(C-1)
// so a phase-B tile's producers were claimed at least D + 1 blocks earlier
// and a slot is reused 2 (S - D) - 1 blocks after its last reader was claimed;
// D and S are chosen from the number of resident CTAs (about 12 tiles per SM
// are claimed but not yet published at any time) so that dependencies are
// normally complete when checked, while only about D + 1 slots hold live data
// (the rest were dropped from L2 as they were read).  At N = 512 D stays 1 so
// that the live 32 MB slots fit in L2; about a third of the tiles then find
// their dependency incomplete at the first check (a larger D was measured
// slower).  Every tile waits only on tiles claimed before it, by CTAs that are
// running or done, so the launch cannot deadlock and needs no co-residency;
// waits are bounded, and on timeout the launch records an error and every CTA
// stops at its next wait.
//
// Control (thread 0 of each CTA), kept off the critical path where it can be:
// the claim of the tile after next is issued when a tile starts and the next
// tile's dependency counter is read then too, with an acquire load; at the
// tile's middle barrier (its input consumed) one release reduction publishes
// the previous tile, so a tile costs two barriers and no fence (the form with
// one fence.acq_rel for both, and relaxed operations, measured 0.3% slower).
// A dependency still incomplete at that point is read again at the end of the
// tile (one fence if it has completed); only if it is still incomplete is the
// current tile published first, then waited for.
constexpr long long WAIT_LIMIT = 4000000000LL;  // clock64 cycles (~2 s)

struct Grid2DArgs {
    const float2* in;
    float2* out;
    float2* ring;    // nslots slots of TL N^2 complex64
    int* ctl;        // [0] next tile, [1] abort, [2, 2 + C) phase-A done per chunk, [2 + C, 2 + 2C) phase-B done
    int* err;        // first error code (9: dependency wait timed out)
    int nchunks;     // C = nf * N / TL
    int look;        // D
    int nslots;      // S
    int prefetch;    // 1: prefetch the next claimed phase-A tile's input into L2 at each middle barrier
};

__device__ __forceinline__ int ld_relaxed(const int* p)
{
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_acquire(const int* p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void red_add_release(int* p, int v)
{
    asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void fence_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ __forceinline__ void red_add(int* p, int v)
{
    asm volatile("red.relaxed.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// Claim order -> (phase, chunk, tile within the phase).
__device__ __forceinline__ void decode_task(int t, int N, int C, int D, bool& phaseA, int& c, int& u)
{
    const int bi = t / N;
    u = t - bi * N;
    const int P = D < C ? D : C;
    if (bi < P) {
        phaseA = true;
        c = bi;
        return;
    }
    const int j = bi - P, Q = C > D ? C - D : 0;
    if (j < 2 * Q) {
        phaseA = (j & 1) == 0;
        c = (j >> 1) + (phaseA ? D : 0);
        return;
    }
    phaseA = false;
    c = Q + (j - 2 * Q);
}

template <int R, bool FWD, bool REAL_IO>
__global__ void __launch_bounds__(32 * PWARPS, 3) fft_grid2d(const Grid2DArgs a, const double2* __restrict__ tw)
{
    constexpr int N = 32 * R;
    constexpr int NB = N / TL;
    constexpr long long N2 = (long long)N * N, N3 = N2 * N;
    extern __shared__ float2 smem_f2[];
    float2* Ws = smem_f2;
    float2* T = smem_f2 + tile_tw_elems<R>();
    __shared__ int s_cur[2], s_slow;
    __shared__ const char* s_pf;  // input of the next tile to prefetch into L2 (null: none)
    load_tile_twiddles<R>(Ws, tw);
    const uint64_t pol_stream = l2_policy_first(), pol_keep = l2_policy_last();
    const int C = a.nchunks, D = a.look, S = a.nslots;
    const int total = 2 * C * N;
    int* const abort_flag = a.ctl + 1;
    int* const doneA = a.ctl + 2;
    int* const doneB = a.ctl + 2 + C;

    // thread-0 control state
    int nxt = -1, pend = -1, prev = -1, dv = 0;
    const int* dptr = nullptr;  // dependency counter of nxt (null: none)
    bool ready = true;
    // raw claim (checked against total where it is used, so the atomic's latency hides behind a tile)
    auto claim = [&]() -> int { return atomicAdd(a.ctl, 1); };
    auto valid = [&](int t) { return t < total ? t : -1; };
    auto dep_of = [&](int t) -> const int* {
        bool pa;
        int c, u;
        decode_task(t, N, C, D, pa, c, u);
        if (pa) return c >= S ? doneB + (c - S) : nullptr;
        return doneA + c;
    };
    auto signal = [&](int t) {  // after a fence (release pattern)
        bool pa;
        int c, u;
        decode_task(t, N, C, D, pa, c, u);
        red_add(pa ? doneA + c : doneB + c, 1);
    };
    auto signal_release = [&](int t) {  // one release reduction
        bool pa;
        int c, u;
        decode_task(t, N, C, D, pa, c, u);
        red_add_release(pa ? doneA + c : doneB + c, 1);
    };
    // bounded wait for *p >= N (relaxed reads; the caller fences)
    auto spin = [&](const int* p) -> bool {
        const long long t0 = clock64();
        while (ld_relaxed(p) < N) {
            if (*(volatile int*)abort_flag) return false;
            if (clock64() - t0 > WAIT_LIMIT) {
                atomicCAS(a.err, 0, 9);
                atomicExch(abort_flag, 1);
                return false;
            }
            __nanosleep(64);
        }
        return true;
    };
    if (threadIdx.x == 0) {
        int t0 = valid(claim());
        nxt = t0 >= 0 ? valid(claim()) : -1;
        if (t0 >= 0) {
            const int* p = dep_of(t0);
            if (p && !spin(p)) t0 = nxt = -1;
            fence_gpu();
        }
        s_cur[0] = t0;
        dptr = nxt >= 0 ? dep_of(nxt) : nullptr;
    }
    __syncthreads();
    for (int it = 0;; ++it) {
        const int t = s_cur[it & 1];
        if (t < 0) break;
        if (threadIdx.x == 0) {
            pend = nxt >= 0 ? claim() : -1;  // the tile after next
            dv = dptr ? ld_acquire(dptr) : N;  // acquire: the next tile's reads are ordered after it
            // The next tile's input, if it comes from HBM (phase A), is prefetched into L2 by every
            // thread after the middle barrier, a half tile ahead: its loads then wait on L2 instead of
            // HBM.  Phase-B inputs (the ring) are in L2 already.
            const char* pf = nullptr;
            if (a.prefetch && nxt >= 0) {
                bool pa;
                int cn, un;
                decode_task(nxt, N, C, D, pa, cn, un);
                const long long fb = (long long)(cn / NB) * N3, kbn = cn % NB;
                if (pa && FWD)  // TL contiguous grid rows of slice kbn TL + un / NB (as tile_body reads them)
                    pf = reinterpret_cast<const char*>(a.in) +
                         (fb + (kbn * TL + un / NB) * N2 + (long long)(un % NB) * TL * N) * (REAL_IO ? 4 : 8);
                else if (pa)    // N runs of TL pencil entries (128 bytes each, N^2 apart), one per p
                    pf = reinterpret_cast<const char*>(a.in + fb + (long long)un * N + kbn * TL);
            }
            s_pf = pf;
        }
        auto mid = [&] {
            if (threadIdx.x == 0) {
                // publish the previous tile: its stores (every thread's, ordered before this point by the
                // barriers) are released by the reduction
                if (prev >= 0) signal_release(prev);
                prev = -1;
                ready = nxt < 0 || dv >= N;
                s_cur[(it + 1) & 1] = nxt;
                s_slow = !ready;
            }
            // next-tile prefetch (thread 0 after publishing: measured faster than before it, a release
            // would also wait for its prefetches)
            if (const char* pf = s_pf) {
                constexpr int NL = FWD ? TL * N * (REAL_IO ? 4 : 8) / 128 : N;
                constexpr long long STEP = FWD ? 128 : 8 * N2;
#pragma unroll
                for (int i = threadIdx.x; i < NL; i += 32 * PWARPS) prefetch_l2(pf + STEP * i);
            }
        };
        bool phaseA;
        int c, u;
        decode_task(t, N, C, D, phaseA, c, u);
        const long long f = c / NB, kb = c % NB;
        float2* slot = a.ring + (long long)(c % S) * TL * N2;
        const long long fbase = f * N3;
        const int kl = u / NB, bb = u % NB, q = u;  // slice-type tile (kl, bb), q-type tile q
        if (FWD) {
            if (phaseA)
                tile_body<R, true, REAL_IO, IO_STREAM, IO_SCRATCH>(
                    a.in, slot, fbase + (kb * TL + kl) * N2 + (long long)bb * TL * N, kl * N2 + bb * TL, N, N, T,
                    Ws, pol_stream, pol_keep, mid);
            else
                tile_body<R, true, false, IO_SCRATCH, IO_STREAM>(slot, a.out, (long long)q * N,
                                                                  fbase + (long long)q * N + kb * TL, N2, N2, T, Ws,
                                                                  0, pol_stream, mid);
        } else {
            if (phaseA)
                tile_body<R, false, false, IO_STREAM, IO_SCRATCH>(a.in, slot, (long long)q * N,
                                                                   fbase + (long long)q * N + kb * TL, N2, N2, T,
                                                                   Ws, pol_stream, pol_keep, mid);
            else
                tile_body<R, false, REAL_IO, IO_SCRATCH, IO_STREAM>(
                    slot, a.out, fbase + (kb * TL + kl) * N2 + (long long)bb * TL * N, kl * N2 + bb * TL, N, N, T,
                    Ws, 0, pol_stream, mid);
        }
        __syncthreads();  // every thread's stores (and discards) of tile t issued; shared memory free
        if (s_slow) {
            // the next tile's dependency was incomplete at the middle barrier.  Usually it has completed
            // since: re-read it and, if so, one fence (acquire) suffices and t stays unpublished until the
            // next tile's middle barrier.  Otherwise publish t first (it may be one of them) and wait.
            if (threadIdx.x == 0) {
                bool published = false, ok = true;
                if (ld_relaxed(dptr) < N) {
                    fence_gpu();
                    signal(t);
                    published = true;
                    ok = spin(dptr);
                }
                fence_gpu();
                s_cur[(it + 1) & 1] = ok ? nxt : -1;
                if (!ok) pend = -1;
                prev = published ? -1 : t;
            }
            __syncthreads();
        } else if (threadIdx.x == 0) {
            prev = t;
        }
        if (threadIdx.x == 0) {
            nxt = pend >= 0 ? valid(pend) : -1;
            dptr = nxt >= 0 ? dep_of(nxt) : nullptr;
        }
    }
    if (threadIdx.x == 0 && prev >= 0) {
        fence_gpu();
        signal(prev);
    }
}

template <int R, bool C2T, bool REAL_IO>
static cudaError_t tile_r(const void* in, void* out, long long nf, const TileGeo& g, const void* tw, cudaStream_t st)
{
    constexpr int N = 32 * R;
    constexpr int LP = tile_lp<R, REAL_IO>();
    constexpr int TLI = REAL_IO ? TL / 2 : TL;  // staged rows (real lines go in pairs)
    const size_t smem = sizeof(float2) * ((size_t)tile_tw_elems<R>() + (size_t)TLI * LP);
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

// Lookahead D and ring slots S for N on a device of nsm SMs: about W = 12 nsm
// tiles are claimed and not yet published at any time (three resident CTAs per
// SM, each holding up to three claims and one unpublished tile); D and S put
// every dependency at least W tiles back (2 D + 1 and 2 (S - D) - 1 blocks of
// N tiles).  At N = 512 D stays 1 so that the live slots (D + 1, 32 MB each)
// fit in L2; the rare incomplete dependency then takes the slow path.
static void fused_geometry(int N, int nsm, int& D, int& S)
{
    const int W = 12 * nsm;
    D = N >= 512 ? 1 : std::max(1, (W - N + 2 * N - 1) / (2 * N));
    if (const char* ev = getenv("FFTSO3_FFT_LOOKAHEAD")) {  // tuning override of D (1..16)
        const int d = atoi(ev);
        if (d >= 1 && d <= 16) D = d;
    }
    S = D + std::max(2, (W + N + 2 * N - 1) / (2 * N));
}

static int device_sms()
{
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return 0;
    return nsm;
}

template <int R, bool FWD, bool REAL_IO>
static cudaError_t grid2d_r(const Grid2DArgs& a, long long tiles, const void* tw, cudaStream_t st)
{
    // staged tile: 16 complex lines, or 8 rows of real pairs (phase A forward / phase B inverse)
    constexpr size_t rows = std::max<size_t>((size_t)TL * tile_lp<R, false>(), (size_t)(TL / 2) * tile_lp<R, true>());
    const size_t smem = sizeof(float2) * ((size_t)tile_tw_elems<R>() + rows);
    auto k = fft_grid2d<R, FWD, REAL_IO>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, nsm = 0, occ = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, 32 * PWARPS, smem)) != cudaSuccess) return e;
    const long long ctas = std::min<long long>(tiles, (long long)nsm * std::max(occ, 1));
    k<<<(unsigned)ctas, 32 * PWARPS, smem, st>>>(a, (const double2*)tw);
    return cudaGetLastError();
}

template <bool FWD, bool REAL_IO>
static cudaError_t grid2d_dispatch(const Grid2DArgs& a, long long tiles, int N, const void* tw, cudaStream_t st)
{
    switch (N) {
        case 64: return grid2d_r<2, FWD, REAL_IO>(a, tiles, tw, st);
        case 128: return grid2d_r<4, FWD, REAL_IO>(a, tiles, tw, st);
        case 256: return grid2d_r<8, FWD, REAL_IO>(a, tiles, tw, st);
        case 512: return grid2d_r<16, FWD, REAL_IO>(a, tiles, tw, st);
        default: return cudaErrorNotSupported;
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

bool fft_grid_fused_supported(int N) { return N == 64 || N == 128 || N == 256 || N == 512; }
size_t fft_grid_fused_ring_elems(int N)
{
    int D, S;
    ffast::fused_geometry(N, ffast::device_sms(), D, S);
    return (size_t)S * ffast::TL * N * N;
}
size_t fft_grid_fused_ctl_ints(long long nf, int N) { return 2 + 2 * (size_t)nf * (N / ffast::TL); }

// Both passes of one direction (dir 1: grid -> pencils, dir -1: pencils ->
// grid) in one persistent launch through the L2-resident ring (fft_grid2d).
cudaError_t launch_fft_grid_fused(const void* in, void* out, void* ring, size_t ring_elems, int* ctl, int* err,
                                  long long nf, int N, int dir, const void* tw, cudaStream_t st, bool real_io)
{
    if (!fft_grid_fused_supported(N) || (dir != 1 && dir != -1) || nf < 1) return cudaErrorInvalidValue;
    const long long C = nf * (N / ffast::TL);
    if (C > (1LL << 29) / N) return cudaErrorInvalidValue;  // tile indices stay in int
    cudaError_t e = cudaMemsetAsync(ctl, 0, sizeof(int) * fft_grid_fused_ctl_ints(nf, N), st);
    if (e != cudaSuccess) return e;
    int D, S;
    ffast::fused_geometry(N, ffast::device_sms(), D, S);
    if ((size_t)S * ffast::TL * N * N > ring_elems) return cudaErrorInvalidValue;  // ring sized for another device
    const char* pf = getenv("FFTSO3_FFT_PREFETCH");  // 0 turns the next-tile L2 prefetch off (tuning)
    ffast::Grid2DArgs a{(const float2*)in, (float2*)out, (float2*)ring, ctl, err, (int)C, D, S,
                        pf && atoi(pf) == 0 ? 0 : 1};
    const long long tiles = 2 * C * N;
    if (dir == 1)
        return real_io ? ffast::grid2d_dispatch<true, true>(a, tiles, N, tw, st)
                       : ffast::grid2d_dispatch<true, false>(a, tiles, N, tw, st);
    return real_io ? ffast::grid2d_dispatch<false, true>(a, tiles, N, tw, st)
                   : ffast::grid2d_dispatch<false, false>(a, tiles, N, tw, st);
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
